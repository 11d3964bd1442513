// tpss_gpu.hpp -- C++ host interface over the C ABI of tpss_gpu.h.
//
// Mirrors the reference's smoother-path classes with the same names, AdditionalData fields
// and error behaviour (deal.II's AssertThrow throws; here every non-zero status throws
// tpss_gpu::Error):
//   SubdomainHandler           TPSS/subdomain_handler.h:33-262
//   LaplaceOperator            apps/laplace_integrator.h:396-786 (MF::Operator)
//   SchwarzPreconditioner      preconditioner/schwarz_preconditioner.h:88-588
//   SchwarzSmoother            smoother/schwarz_smoother.h:16-52, smoother_richardson.h:14-163
//   MultigridSolver            apps/poisson_problem.h:642-755 (GMG + CG)
//   C0IPBiharmonic             apps/biharmonic_problem.h, biharmonic_integrator.h (C0IP path)
//   MLP, BatchSolver           no counterpart: learned local solver network, concurrent batches
// Vectors are device pointers to FP64 arrays; streams are cudaStream_t passed as void*.
// Header-only; link with libtpss_gpu.so.
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "tpss_gpu.h"

namespace tpss_gpu
{
struct Error : std::runtime_error
{
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc)
{
  if(rc != TPSS_OK)
  {
    const char *m = tpss_last_error();
    throw Error(rc, m ? m : "tpss_gpu error");
  }
}

enum class PatchVariant { cell = TPSS_PATCH_CELL, vertex = TPSS_PATCH_VERTEX };
enum class SmootherVariant { additive = TPSS_ADDITIVE, multiplicative = TPSS_MULTIPLICATIVE };
enum class Precision { fp64 = TPSS_FP64, fp32 = TPSS_FP32 };

/* TPSS::lookup_damping_factor (TPSS/TPSS.h:121-163) */
inline double lookup_damping_factor(PatchVariant pv, SmootherVariant sv, int dim)
{
  if(sv == SmootherVariant::multiplicative) return 1.;
  if(pv == PatchVariant::cell) return 0.7;
  if(dim == 2) return 0.25;
  if(dim == 3) return 0.15;
  throw Error(TPSS_ERR_INVALID_ARGUMENT, "This case is not listed!");
}

class SubdomainHandler
{
public:
  struct AdditionalData
  {
    int dim = 2, degree = 1;
    std::vector<int> n_cells = {2, 2};
    PatchVariant patch_variant = PatchVariant::vertex;
    SmootherVariant smoother_variant = SmootherVariant::additive;
    unsigned int level = 0;
    std::vector<std::vector<double>> cell_h;  // empty: uniform 1/n per direction
    std::vector<int64_t> cell_dof_start;      // empty: lexicographic cell blocks
    std::vector<int32_t> coloring;            // empty: default coloring
    std::vector<double> vertex_coords;        // distorted mesh: (n+1)^dim x dim, empty: Cartesian
    int surrogate_n_q = 5;
  };

  SubdomainHandler() = default;
  explicit SubdomainHandler(const AdditionalData &ad) { reinit(ad); }
  SubdomainHandler(const SubdomainHandler &) = delete;
  SubdomainHandler &operator=(const SubdomainHandler &) = delete;
  ~SubdomainHandler() { clear(); }

  void reinit(const AdditionalData &ad)
  {
    clear();
    tpss_layout_desc d{};
    d.dim = ad.dim;
    d.degree = ad.degree;
    d.dof_layout = TPSS_DOF_DGQ;
    d.patch_variant = static_cast<int>(ad.patch_variant);
    d.smoother_variant = static_cast<int>(ad.smoother_variant);
    for(int i = 0; i < 3; ++i) d.n_cells[i] = i < (int)ad.n_cells.size() ? ad.n_cells[i] : 1;
    for(int i = 0; i < 3 && i < (int)ad.cell_h.size(); ++i)
      d.cell_h[i] = ad.cell_h[i].empty() ? nullptr : ad.cell_h[i].data();
    d.cell_dof_start = ad.cell_dof_start.empty() ? nullptr : ad.cell_dof_start.data();
    d.patch_color = ad.coloring.empty() ? nullptr : ad.coloring.data();
    d.vertex_coords = ad.vertex_coords.empty() ? nullptr : ad.vertex_coords.data();
    d.surrogate_n_q = ad.surrogate_n_q;
    check(tpss_layout_create(&d, &handle_));
    additional_data_ = ad;
  }

  void clear()
  {
    if(handle_) tpss_layout_destroy(handle_);
    handle_ = nullptr;
  }

  int64_t n_dofs() const
  {
    int64_t n = 0;
    check(tpss_layout_info(handle_, &n, nullptr, nullptr));
    return n;
  }
  int64_t n_subdomains() const
  {
    int64_t p = 0;
    check(tpss_layout_info(handle_, nullptr, &p, nullptr));
    return p;
  }
  int n_colors() const
  {
    int c = 0;
    check(tpss_layout_info(handle_, nullptr, nullptr, &c));
    return c;
  }
  const AdditionalData &get_additional_data() const { return additional_data_; }
  tpss_layout *handle() const { return handle_; }

private:
  tpss_layout *handle_ = nullptr;
  AdditionalData additional_data_;
};

class LaplaceOperator
{
public:
  LaplaceOperator(std::shared_ptr<const SubdomainHandler> sh, double ip_factor = 1.,
                  int penalty_mode = TPSS_PENALTY_REFERENCE)
    : sh_(std::move(sh))
  {
    check(tpss_operator_create_penalty(sh_->handle(), ip_factor, penalty_mode, &handle_));
  }
  LaplaceOperator(const LaplaceOperator &) = delete;
  ~LaplaceOperator() { tpss_operator_destroy(handle_); }
  int64_t m() const { return sh_->n_dofs(); }
  int64_t n() const { return m(); }
  void vmult(double *dst, const double *src, void *stream = nullptr) const
  {
    check(tpss_operator_vmult(handle_, dst, src, stream));
  }
  // the same product in FP32 arithmetic (level operator of a single-precision V-cycle)
  void vmult_fp32(double *dst, const double *src, void *stream = nullptr) const
  {
    check(tpss_operator_vmult_fp32(handle_, dst, src, stream));
  }
  void Tvmult(double *dst, const double *src, void *stream = nullptr) const { vmult(dst, src, stream); }
  tpss_operator *handle() const { return handle_; }

private:
  std::shared_ptr<const SubdomainHandler> sh_;
  tpss_operator *handle_ = nullptr;
};

struct TimeInfo
{
  double time;
  std::string description;
  std::string unit = "[s]";
  int64_t n_calls;
};

class SchwarzPreconditioner
{
public:
  struct AdditionalData
  {
    double relaxation = 1.;
    bool reverse = false;
    bool symmetrized = false;
    bool use_ras_weights = false;
    bool use_ras_boolean_weights = false;
    Precision precision = Precision::fp64;
    double ip_factor = 1.;
    bool check_finite = false;
    int kernel_variant = TPSS_KERNEL_AUTO;
    int stream_variant = 0;
    int local_solver = TPSS_LOCAL_FD;  // TPSS_LOCAL_FD / EXACT / KSUM / LEARNED
    const tpss_mlp *model = nullptr;   // trained network for TPSS_LOCAL_LEARNED
    int penalty_mode = TPSS_PENALTY_REFERENCE;  // must match the level operator's
  };

  SchwarzPreconditioner() = default;
  SchwarzPreconditioner(const SchwarzPreconditioner &) = delete;
  SchwarzPreconditioner &operator=(const SchwarzPreconditioner &) = delete;
  ~SchwarzPreconditioner() { clear(); }

  void clear()
  {
    if(handle_) tpss_precond_destroy(handle_);
    handle_ = nullptr;
  }

  void initialize(std::shared_ptr<const SubdomainHandler> sh, LaplaceOperator *op,
                  const AdditionalData &ad)
  {
    clear();
    const tpss_precond_desc d = desc(ad);
    check(tpss_precond_create(sh->handle(), op ? op->handle() : nullptr, &d, &handle_));
    sh_ = std::move(sh);
    additional_data_ = ad;
  }

  /* shallow copy sharing the local solvers (schwarz_preconditioner.templates.h:63-86) */
  void initialize(const SchwarzPreconditioner &other, const AdditionalData &ad)
  {
    clear();
    const tpss_precond_desc d = desc(ad);
    check(tpss_precond_create_shallow(other.handle_, &d, &handle_));
    sh_ = other.sh_;
    additional_data_ = ad;
  }

  void vmult(double *dst, const double *src, void *stream = nullptr) const
  {
    check(tpss_precond_vmult(handle_, dst, src, stream));
  }
  void vmult_add(double *dst, const double *src, void *stream = nullptr) const
  {
    check(tpss_precond_vmult_add(handle_, dst, src, stream));
  }
  void Tvmult(double *dst, const double *src, void *stream = nullptr) const
  {
    check(tpss_precond_Tvmult(handle_, dst, src, stream));
  }
  /* dst and src in host memory (pinned for the copies to overlap the kernel) */
  void vmult_host(double *dst, const double *src, void *stream = nullptr) const
  {
    check(tpss_precond_vmult_host(handle_, dst, src, stream));
  }

  /* times the kernel variants on (src -> dst), keeps the fastest; returns its index */
  int autotune(double *dst, const double *src, int reps = 5, void *stream = nullptr)
  {
    int chosen = 0, nv = 0;
    double ms[8];
    check(tpss_precond_autotune(handle_, dst, src, reps, &chosen, ms, &nv, stream));
    return chosen;
  }

  std::vector<TimeInfo> get_time_data() const
  {
    int n = 0;
    check(tpss_precond_time_info(handle_, nullptr, &n));
    std::vector<tpss_time_info> raw(n);
    check(tpss_precond_time_info(handle_, raw.data(), &n));
    std::vector<TimeInfo> out;
    for(const auto &r : raw) out.push_back({r.time, r.description, "[s]", r.n_calls});
    return out;
  }

  std::shared_ptr<const SubdomainHandler> get_subdomain_handler() const { return sh_; }
  const AdditionalData &get_additional_data() const { return additional_data_; }
  int64_t m() const { return sh_->n_dofs(); }
  int64_t n() const { return m(); }
  tpss_precond *handle() const { return handle_; }

private:
  static tpss_precond_desc desc(const AdditionalData &ad)
  {
    tpss_precond_desc d{};
    d.relaxation = ad.relaxation;
    d.reverse = ad.reverse;
    d.symmetrized = ad.symmetrized;
    d.use_ras_weights = ad.use_ras_weights;
    d.use_ras_boolean_weights = ad.use_ras_boolean_weights;
    d.precision = static_cast<int>(ad.precision);
    d.ip_factor = ad.ip_factor;
    d.check_finite = ad.check_finite;
    d.kernel_variant = ad.kernel_variant;
    d.stream_variant = ad.stream_variant;
    d.local_solver = ad.local_solver;
    d.model = ad.model;
    d.penalty_mode = ad.penalty_mode;
    return d;
  }

  tpss_precond *handle_ = nullptr;
  std::shared_ptr<const SubdomainHandler> sh_;
  AdditionalData additional_data_;
};

class SchwarzSmoother
{
public:
  struct AdditionalData
  {
    unsigned int number_of_smoothing_steps = 1;
    double damping_factor = 1.;
  };

  SchwarzSmoother() = default;
  SchwarzSmoother(const SchwarzSmoother &) = delete;
  ~SchwarzSmoother()
  {
    if(handle_) tpss_smoother_destroy(handle_);
  }

  void initialize(LaplaceOperator &op, std::shared_ptr<SchwarzPreconditioner> p,
                  const AdditionalData &ad)
  {
    if(handle_) tpss_smoother_destroy(handle_);
    handle_ = nullptr;
    check(tpss_smoother_create(op.handle(), p->handle(), (int)ad.number_of_smoothing_steps,
                               ad.damping_factor, &handle_));
    precond_ = std::move(p);
  }
  void step(double *dst, const double *src, void *stream = nullptr) const
  {
    check(tpss_smoother_step(handle_, dst, src, stream));
  }
  void vmult(double *dst, const double *src, void *stream = nullptr) const
  {
    check(tpss_smoother_vmult(handle_, dst, src, stream));
  }

private:
  tpss_smoother *handle_ = nullptr;
  std::shared_ptr<SchwarzPreconditioner> precond_;
};

class MultigridSolver
{
public:
  explicit MultigridSolver(const tpss_mg_desc &d) { check(tpss_mg_create(&d, &handle_)); }
  MultigridSolver(const MultigridSolver &) = delete;
  ~MultigridSolver() { tpss_mg_destroy(handle_); }
  int64_t n_dofs() const
  {
    int64_t n = 0;
    check(tpss_mg_n_dofs(handle_, &n));
    return n;
  }
  void vmult(double *dst, const double *src, void *stream = nullptr) const
  {
    check(tpss_mg_vmult(handle_, dst, src, stream));
  }
  /* returns the CG iteration count; residual norms in `history` (max_iter + 1 entries) */
  int solve(double *u, const double *f, double rel_tol, double abs_tol = 1e-14, int max_iter = 100,
            std::vector<double> *history = nullptr, void *stream = nullptr) const
  {
    int it = 0;
    std::vector<double> h(max_iter + 1);
    check(tpss_mg_cg_solve(handle_, u, f, rel_tol, abs_tol, max_iter, &it, h.data(), stream));
    if(history) *history = std::vector<double>(h.begin(), h.begin() + it + 1);
    return it;
  }

  /* damping of level 1..L and the lambda_max(P A) estimate it was scaled by */
  std::pair<double, double> relaxation(int level) const
  {
    double w = 0, lam = 0;
    check(tpss_mg_relaxation(handle_, level, &w, &lam));
    return {w, lam};
  }
  tpss_mg *handle() const { return handle_; }

private:
  tpss_mg *handle_ = nullptr;
};

/* fully connected tanh network of the learned local solver, trained on the GPU */
class MLP
{
public:
  MLP(int n_in, int n_out, int n_hidden = 64, int n_hidden_layers = 3, uint64_t seed = 0)
  {
    tpss_mlp_desc d{n_in, n_hidden, n_hidden_layers, n_out, seed};
    check(tpss_mlp_create(&d, &handle_));
  }
  MLP(const MLP &) = delete;
  ~MLP() { tpss_mlp_destroy(handle_); }
  /* x, target: device FP32 [rows][n_in], [rows][n_out]; returns the loss after every epoch */
  std::vector<double> train(const float *x, const float *target, int64_t rows, int epochs, int batch = 256,
                            double lr = 1e-3, uint64_t seed = 0, void *stream = nullptr)
  {
    std::vector<double> hist(epochs > 0 ? epochs : 1);
    check(tpss_mlp_train(handle_, x, target, rows, epochs, batch, lr, seed, hist.data(), stream));
    hist.resize(epochs);
    return hist;
  }
  void forward(const float *x, int64_t rows, float *y, void *stream = nullptr)
  {
    check(tpss_mlp_forward(handle_, x, rows, y, stream));
  }
  const tpss_mlp *handle() const { return handle_; }

private:
  tpss_mlp *handle_ = nullptr;
};

/* clamped C0IP biharmonic hierarchy on the unit square (apps/biharmonic_problem.h) */
class C0IPBiharmonic
{
public:
  explicit C0IPBiharmonic(const tpss_c0ip_desc &d) { check(tpss_c0ip_create(&d, &handle_)); }
  C0IPBiharmonic(const C0IPBiharmonic &) = delete;
  ~C0IPBiharmonic() { tpss_c0ip_destroy(handle_); }
  int64_t n_dofs(int level = -1) const
  {
    int64_t n = 0;
    check(tpss_c0ip_info(handle_, level, &n, nullptr));
    return n;
  }
  void vmult(double *dst, const double *src, int level = -1, void *stream = nullptr) const
  {
    check(tpss_c0ip_operator_vmult(handle_, level, dst, src, stream));
  }
  void smooth(double *dst, const double *src, int level = -1, void *stream = nullptr) const
  {
    check(tpss_c0ip_smoother_vmult(handle_, level, dst, src, stream));
  }
  int solve(double *u, const double *f, double rel_tol, double abs_tol = 1e-14, int max_iter = 200,
            void *stream = nullptr) const
  {
    int it = 0;
    check(tpss_c0ip_cg_solve(handle_, u, f, rel_tol, abs_tol, max_iter, &it, nullptr, stream));
    return it;
  }

private:
  tpss_c0ip *handle_ = nullptr;
};

/* many independent CG + GMG problems solved concurrently (device-side CG loops) */
class BatchSolver
{
public:
  BatchSolver(const std::vector<tpss_mg_desc> &problems, int n_streams = 64)
  {
    check(tpss_batch_create(problems.data(), (int)problems.size(), n_streams, &handle_));
    n_ = (int)problems.size();
  }
  BatchSolver(const BatchSolver &) = delete;
  ~BatchSolver() { tpss_batch_destroy(handle_); }
  std::vector<int> solve(const std::vector<double *> &u, const std::vector<const double *> &f, double rel_tol,
                         double abs_tol = 1e-14, int max_iter = 200, void *stream = nullptr)
  {
    std::vector<int> its(n_);
    check(tpss_batch_solve(handle_, u.data(), f.data(), rel_tol, abs_tol, max_iter, its.data(), stream));
    return its;
  }

private:
  tpss_batch *handle_ = nullptr;
  int n_ = 0;
};

}  // namespace tpss_gpu
