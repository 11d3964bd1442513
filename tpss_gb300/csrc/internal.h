// internal.h -- structures shared by the translation units of libtpss_gpu.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/tpss_gpu.h"

namespace tpss
{
// ------------------------------------------------------------------------------------------
// status handling: every C entry point catches tpss::Error and returns its code
// ------------------------------------------------------------------------------------------
struct Error
{
  int code;
  std::string msg;
};

void set_last_error(const std::string &msg);

[[noreturn]] inline void fail(int code, const std::string &msg) { throw Error{code, msg}; }

#define TPSS_CUDA(call)                                                                     \
  do                                                                                        \
  {                                                                                         \
    cudaError_t e_ = (call);                                                                \
    if(e_ != cudaSuccess)                                                                   \
      ::tpss::fail(e_ == cudaErrorMemoryAllocation ? TPSS_ERR_OUT_OF_MEMORY : TPSS_ERR_CUDA, \
                   std::string(#call) + ": " + cudaGetErrorString(e_));                     \
  } while(0)

#define TPSS_REQUIRE(cond, msg)                                    \
  do                                                               \
  {                                                                \
    if(!(cond)) ::tpss::fail(TPSS_ERR_INVALID_ARGUMENT, (msg));    \
  } while(0)

template<typename F>
int guarded(F &&f)
{
  try
  {
    f();
    return TPSS_OK;
  }
  catch(const Error &e)
  {
    set_last_error(e.msg);
    return e.code;
  }
  catch(const std::bad_alloc &)
  {
    set_last_error("host allocation failed");
    return TPSS_ERR_OUT_OF_MEMORY;
  }
  catch(const std::exception &e)
  {
    set_last_error(e.what());
    return TPSS_ERR_STATE;
  }
}

// device buffer with RAII
template<typename T>
struct DeviceBuffer
{
  T *ptr = nullptr;
  size_t n = 0;
  DeviceBuffer() = default;
  explicit DeviceBuffer(size_t count) { resize(count); }
  DeviceBuffer(const DeviceBuffer &) = delete;
  DeviceBuffer &operator=(const DeviceBuffer &) = delete;
  DeviceBuffer(DeviceBuffer &&o) noexcept : ptr(o.ptr), n(o.n)
  {
    o.ptr = nullptr;
    o.n = 0;
  }
  DeviceBuffer &operator=(DeviceBuffer &&o) noexcept
  {
    if(this != &o)
    {
      release();
      ptr = o.ptr;
      n = o.n;
      o.ptr = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DeviceBuffer() { release(); }
  void resize(size_t count)
  {
    release();
    if(count)
    {
      TPSS_CUDA(cudaMalloc(&ptr, count * sizeof(T)));
      n = count;
    }
  }
  void upload(const T *host, size_t count)
  {
    resize(count);
    if(count) TPSS_CUDA(cudaMemcpy(ptr, host, count * sizeof(T), cudaMemcpyHostToDevice));
  }
  void release()
  {
    if(ptr) cudaFree(ptr);
    ptr = nullptr;
    n = 0;
  }
};

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline int ipow(int b, int e)
{
  int r = 1;
  while(e-- > 0) r *= b;
  return r;
}

int num_sms();

// ------------------------------------------------------------------------------------------
// host-side 1-D finite element data (setup.cu)
// ------------------------------------------------------------------------------------------
struct Shape1D
{
  int k = 0, np = 1;
  std::vector<double> qx, qw, nodes;
  std::vector<double> val, grad;        // [i*np + q]
  std::vector<double> fval[2], fgrad[2];  // at x=0 and x=1
};
Shape1D make_shape_1d(int k);
// Effective ip factors of the SIPG faces: interior faces sigma = in * gamma * (1/h_l + 1/h_r)/2,
// Dirichlet faces sigma = 2 * bd * gamma / h, gamma = k(k+1). A plain ip converts to in = bd = ip
// (the reference's penalty).
struct Penalty
{
  double in = 1.0, bd = 1.0;
  Penalty() = default;
  Penalty(double ip) : in(ip), bd(ip) {}
  Penalty(double i, double b) : in(i), bd(b) {}
};
// TPSS_PENALTY_REFERENCE: in = bd = ip; TPSS_PENALTY_2KP1SQ: sigma = ip 2(k+1)^2 (1/h_l+1/h_r)/2
// inside and ip 2(k+1)^2 / h on the boundary
Penalty make_penalty(double ip, int mode, int k);
// 1-D DG patch matrices of the FD local solver (ncp = 1 or 2 cells)
void patch_matrices_1d(const Shape1D &s, int ncp, const double *h, bool bdry_lo, bool bdry_hi,
                       Penalty ip, double *M, double *A);
// global 1-D SIPG blocks of one direction: mass[c][np^2], blk[c][3][np^2]
void operator_blocks_1d(const Shape1D &s, int nc, const double *h, Penalty ip,
                        std::vector<double> &mass, std::vector<double> &blk);
// per-cell 1-D factors of the operator: mass, own block, rank-2 neighbour couplings
std::vector<double> operator_factors_1d(const Shape1D &s, int nc, const double *h, Penalty ip);
// child embedding E[s][i*np+j] = phi_j((z_i+s)/2)
std::vector<double> embedding_1d(const Shape1D &s);

// ------------------------------------------------------------------------------------------
// layout
// ------------------------------------------------------------------------------------------
}  // namespace tpss

struct tpss_layout
{
  int dim = 0, k = 0, np = 0, patch_variant = 0, smoother_variant = 0;
  int ncp = 0;        // cells per patch per direction
  int n = 0;          // 1-D patch size
  int nloc = 0;       // n^dim
  int npc = 0;        // cells per patch
  int cell_dofs = 0;  // (k+1)^dim
  int nc[3] = {1, 1, 1};
  std::vector<double> h[3];
  int64_t n_cells = 0, n_dofs = 0;
  bool lexicographic = true;
  std::vector<int64_t> cell_start;  // host
  int64_t P = 0;
  int n_colors = 0;
  std::vector<int64_t> color_start;  // n_colors + 1
  std::vector<int32_t> lower, color; // host, P*3 and P
  std::vector<int32_t> patch_fd_key; // host: P*dim indices into fd_keys
  struct FdKey
  {
    double h0, h1;
    int lo, hi;
  };
  std::vector<FdKey> fd_keys;
  std::vector<int32_t> cell_multiplicity;  // number of patches covering each cell
  std::vector<int64_t> patch_first;           // host: P*npc first DoF of each patch cell
  std::mutex device_mutex;
  bool on_device = false;
  tpss::DeviceBuffer<int64_t> d_patch_first;  // P*npc first DoF of each patch cell
  tpss::DeviceBuffer<int32_t> d_patch_fd;     // P*dim
  tpss::DeviceBuffer<int64_t> d_cell_start;   // n_cells (empty when lexicographic)
  std::vector<int32_t> vertex_fd[3];           // vertex patches: FD entry of vertex v_d, per d
  bool per_patch_fd = false;                   // FD keys differ per patch (surrogate widths)
  std::vector<double> coords;                  // vertex coordinates of a distorted level (host)
  tpss::DeviceBuffer<int32_t> d_vertex_fd[3];
};

namespace tpss
{
// block-sparse SIPG matrix of a multilinear (distorted) level (mapped.cu)
struct MappedOperator
{
  int nd = 0, nb = 0;     // cell DoFs, blocks per block row (2 dim + 1)
  int64_t n_cells = 0;
  DeviceBuffer<double> coords;  // vertex coordinates
  DeviceBuffer<double> vals;    // n_cells * nb blocks of nd x nd, entry (i, j) at j * nd + i
  DeviceBuffer<float> vals32;   // FP32 copy (single-precision V-cycle), made on first use
  DeviceBuffer<int32_t> col;    // n_cells * nb column cell (lexicographic), -1 = none
  DeviceBuffer<double> fgeo;    // per cell and face: geometry of the face coupling (mapped_tab.cuh)
  int fg = 0;                   // doubles per face record
  DeviceBuffer<float> self32;   // FP32 cell blocks, nd x nd per cell (single-precision V-cycle)
  DeviceBuffer<float> fgeo32;   // FP32 face geometry (single-precision V-cycle)
};
}  // namespace tpss

struct tpss_operator
{
  const tpss_layout *layout = nullptr;
  double ip = 1.0;
  int penalty_mode = TPSS_PENALTY_REFERENCE;
  tpss::DeviceBuffer<double> d_mass[3], d_blk[3];
  tpss::DeviceBuffer<double> d_fac[3];  // operator_factors_1d per direction
  tpss::DeviceBuffer<float> d_fac32[3];  // the same in FP32 (single-precision level operator)
  tpss::DeviceBuffer<float> x32;         // FP32 copy of the source (single-precision operator)
  bool sparse_faces = false;             // face couplings with unit value vectors (operator.cu)
  int nblk_cells[3] = {0, 0, 0};
  std::unique_ptr<tpss::MappedOperator> mapped;  // set on distorted levels
};

namespace tpss
{
// FD tables of a preconditioner (shared between shallow copies)
struct FdTables
{
  const tpss_layout *layout = nullptr;
  int n = 0, n_entries = 0;
  int npad32 = 0, npad64 = 0;
  DeviceBuffer<double> fd64;  // entries: [St n*npad][S n*npad][lam npad]
  DeviceBuffer<float> fd32;
  std::vector<double> S_host, lam_host;  // n_entries * n*n, n_entries * n (FP64 results)
  double setup_seconds = 0.0;
  DeviceBuffer<float> ras_w;  // P*npc weights (1/multiplicity) when RAS is used
  // Even/odd split of mirror-symmetric entries (vertex patches with equal cells and equal
  // boundary flags): per entry [Se^T h x hpad][So^T][Se][So][lambda: even then odd, npad],
  // Se = S_even / sqrt(2); sym[e] = 1 when entry e has this form.
  int hpad32 = 0, hpad64 = 0;
  DeviceBuffer<float> fd32_eo;
  DeviceBuffer<double> fd64_eo;  // the same in FP64 (per-color kernel, FP64 smoother)
  DeviceBuffer<int32_t> sym;
  bool has_eo = false;           // some entry has the even/odd form
  // eigenvalues of every entry in the order the kernels read them (the even/odd order for
  // mirror-symmetric entries), n_entries x n, host
  std::vector<double> lam_kernel;
  // reciprocal eigenvalue sums of keyed entries: for the entry combination c = sum_d e_d E^d
  // (e_d the entry of direction d, E = n_entries) the n^dim values 1 / (lambda_0 + .. +
  // lambda_{dim-1}) in the kernels' eigenvalue order; empty when E^dim n^dim > 4 Mi (many
  // distinct 1-D problems) or for per-patch entries, which keep the division
  // (rcp_E = -1: one table per patch, P x n^dim values -- the product-form eigenvalue
  // combinations 1 / (1 + prod_d mu_d) of the rank-2 Kronecker local solver)
  DeviceBuffer<double> rcp64;
  DeviceBuffer<float> rcp32;
  int rcp_E = 0;
  // RAS boolean weights (restricted prolongation, rscatter_add): per patch its boundary class
  // sum_d (lo_d + 2 hi_d) 4^d, and per class and patch-local DoF 1 when the patch scatters it
  DeviceBuffer<int32_t> keep_class;
  DeviceBuffer<unsigned char> keep_mask;
  // per-patch entries (entry p * dim + d) instead of the layout's shared keys
  DeviceBuffer<int32_t> own_fd;
  DeviceBuffer<int32_t> vpatch;  // streamed smoother on per-patch tables: patch of each vertex
  // exact local inverses (local solver TPSS_LOCAL_EXACT): P x nloc x nloc, transposed
  DeviceBuffer<double> dense64;
  DeviceBuffer<float> dense32;
  bool dense = false;
  int64_t learned_fallbacks = 0;  // fitted / learned solvers: patches kept at the surrogate
};

struct TimerSlot
{
  double time = 0.0;
  int64_t n_calls = 0;
  const char *name = "";
};

struct PendingEvent
{
  cudaEvent_t start, stop;
  int slot;
};

// copy / compute / copy pipeline of the host-buffer smoother entry point
struct HostPipe
{
  cudaStream_t up = nullptr, comp = nullptr, comp2 = nullptr, down = nullptr;
  std::vector<cudaEvent_t> ev;
  DeviceBuffer<double> src, dst;
  cudaEvent_t event(size_t i)
  {
    while(ev.size() <= i)
    {
      cudaEvent_t e;
      TPSS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      ev.push_back(e);
    }
    return ev[i];
  }
  void streams()
  {
    if(up) return;
    TPSS_CUDA(cudaStreamCreateWithFlags(&up, cudaStreamNonBlocking));
    TPSS_CUDA(cudaStreamCreateWithFlags(&comp, cudaStreamNonBlocking));
    TPSS_CUDA(cudaStreamCreateWithFlags(&comp2, cudaStreamNonBlocking));
    TPSS_CUDA(cudaStreamCreateWithFlags(&down, cudaStreamNonBlocking));
  }
  HostPipe() = default;
  HostPipe(const HostPipe &) = delete;
  ~HostPipe()
  {
    for(cudaEvent_t e : ev) cudaEventDestroy(e);
    for(cudaStream_t s : {up, comp, comp2, down})
      if(s) cudaStreamDestroy(s);
  }
};
}  // namespace tpss

struct tpss_precond
{
  std::shared_ptr<tpss::FdTables> tables;
  tpss_operator *op = nullptr;
  tpss_precond_desc desc{};
  tpss::DeviceBuffer<double> residual;  // multiplicative scratch
  tpss::DeviceBuffer<int> flag;         // finiteness check
  tpss::DeviceBuffer<float> halo;       // streamed kernel: partial sums of shared cells
  tpss::DeviceBuffer<int64_t> fix_rec[8];  // streamed kernel: shared-cell list per variant
  int64_t fix_n[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
  std::vector<int64_t> fix_layer[8];
  tpss::HostPipe pipe;                  // host-buffer entry point
  int stream_variant = 0;               // streamed kernel variant (autotuner)
  int color_variant = 0;                // per-color kernel variant: patches per CTA (autotuner)
  std::vector<tpss::TimerSlot> timers;
  std::vector<tpss::PendingEvent> pending;
  std::vector<cudaEvent_t> event_pool;
};

namespace tpss
{
// FD kernel launch (fd_kernels_*.cu). Returns false when (dim, k, ncp) is not instantiated.
struct FdLaunch
{
  const double *src;
  double *dst;
  const int64_t *patch_first;  // first patch of the range
  const int32_t *patch_fd;     // first patch of the range
  const void *fd;              // table of the precision
  const float *ras_w;          // nullptr or first patch of the range
  int64_t n_patches;
  double omega;
  int entry_stride;            // elements per table entry
  const void *fd_eo = nullptr;     // even/odd forms of the mirror-symmetric entries (or nullptr)
  const int32_t *sym = nullptr;    // entry has the even/odd form (or nullptr)
  int eo_stride = 0;               // elements per even/odd entry
  const void *rcp = nullptr;       // reciprocal eigenvalue sums (FdTables::rcp*) or nullptr
  int rcp_E = 0;                   // entries per direction of the rcp combinations
  const unsigned char *keep_mask = nullptr;  // RAS boolean weights (FdTables::keep_mask) or nullptr
  const int32_t *keep_class = nullptr;       // first patch of the range
  int variant = 0;                           // work decomposition (patches per CTA) of the autotuner
};
bool launch_fd_f32(int dim, int k, int ncp, const FdLaunch &a, cudaStream_t s);
bool launch_fd_f64(int dim, int k, int ncp, const FdLaunch &a, cudaStream_t s);
// work decompositions the per-color kernel offers for (dim, k, ncp) in FP32 / FP64
int fd_variants(bool fp32, int dim, int k, int ncp);

// mapped (distorted) levels (mapped.cu)
size_t mapped_smem_bytes(int dim, int np);
void mapped_build(tpss_operator &op, const tpss_layout &L, Penalty ip);
void mapped_apply(const tpss_operator &op, double *dst, const double *src, cudaStream_t s,
                  const double *rhs = nullptr);
// FP32 blocks and source, FP64 result (the level operator of a single-precision V-cycle)
void mapped_apply_f32(tpss_operator &op, double *dst, const double *src, cudaStream_t s,
                      const double *rhs = nullptr);
std::vector<double> mapped_dense(const tpss_operator &op);
// the same product with the face couplings applied matrix-free (mapped_mf.cu); false when the
// level has no face geometry or its degree has no kernel
bool mapped_apply_mf(const tpss_operator &op, double *dst, const double *src, cudaStream_t s,
                     const double *rhs = nullptr);
// its FP32 arithmetic (FP32 copies of the cell blocks, face geometry and source; FP64 result)
bool mapped_apply_mf_f32(tpss_operator &op, double *dst, const double *src, cudaStream_t s,
                         const double *rhs = nullptr);
// FD setup helpers (precond.cu, eigen.cu)
void gen_eig_batched(int n, int n_problems, const std::vector<double> &Ms,
                     const std::vector<double> &As, std::vector<double> &S,
                     std::vector<double> &lam, std::vector<int> *status = nullptr);
// rank-2 Kronecker approximations of the exact patch matrices (local.cu)
std::vector<double> ksvd_fit(const tpss_layout &L, const tpss_operator &op, const std::vector<double> &Mp,
                             const std::vector<double> &Ap, int iters);
void kcp_als(int dim, const int *m, const int *n, int rank, int iters, const double *K_dev, int64_t count,
             double *F_dev, cudaStream_t s);
void key_matrices(const tpss_layout &L, Penalty ip, std::vector<double> &Ms, std::vector<double> &As);
std::vector<double> per_patch(const tpss_layout &L, const std::vector<double> &keyed);
int64_t keep_definite(const tpss_layout &L, const std::vector<double> &Mp, std::vector<double> &Ap,
                      const std::vector<double> &Asur);

// learned local solver (learned.cu, mlp.cu)
using TableMaker = std::function<std::shared_ptr<FdTables>(const std::vector<double> *,
                                                           const std::vector<double> *)>;
std::shared_ptr<FdTables> build_learned_tables(const tpss_layout &L, const tpss_precond_desc &d,
                                               const TableMaker &make);
void mlp_infer(const tpss_mlp &m, const float *x_dev, int64_t rows, float *y_dev, cudaStream_t s);
int mlp_n_in(const tpss_mlp &m);
int mlp_n_out(const tpss_mlp &m);

// local solvers from exact patch matrices (local.cu)
void check_exact_local(const tpss_layout &L, const tpss_operator *op);
void build_dense_inverses(const tpss_layout &L, const tpss_operator &op, bool fp32,
                          DeviceBuffer<double> &inv64, DeviceBuffer<float> &inv32);
void dense_apply_color(const tpss_layout &L, const void *inv, bool fp32, int color, double omega,
                       double *dst, const double *src, cudaStream_t s);
std::vector<double> ksum_fit(const tpss_layout &L, const tpss_operator &op, const std::vector<double> &Ms);
void extract_local_matrices(const tpss_layout &L, const tpss_operator &op, int64_t p0, int64_t count,
                            double *out_dev);

// operator and transfer (operator.cu)
// dst = A src, or with rhs the residual dst = rhs - A src
void operator_apply(tpss_operator *op, double *dst, const double *src, cudaStream_t s,
                    const double *rhs = nullptr);
// the same operator in FP32 arithmetic (FP64 vectors; the source is converted once into a
// scratch copy): for the residuals inside a single-precision V-cycle (distorted levels: FP32
// copy of the block-sparse matrix)
void operator_apply_f32(tpss_operator *op, double *dst, const double *src, cudaStream_t s,
                        const double *rhs = nullptr);
// single: FP32 arithmetic on the FP64 vectors (the transfers of a single-precision V-cycle)
void transfer_apply(int dim, int k, const int *ncc, const double *E_dev, bool restrict_mode,
                    double *coarse, double *fine, cudaStream_t s, bool single = false);

// vector kernels (operator.cu)
void vec_axpby(int64_t n, double a, const double *x, double b, double *y, cudaStream_t s);  // y = a x + b y
void vec_sub(int64_t n, const double *a, double *y, cudaStream_t s);  // y = a - y
// dot products: partial sums into `partial` (device, >= dot_partials()), final into out (device)
int dot_partials();
void vec_dot(int64_t n, const double *x, const double *y, double *partial, double *out,
             cudaStream_t s);

// streamed 3D vertex-patch smoother, FP32 (stream3d.cu)
struct StreamLaunch
{
  const double *src;
  double *dst;
  const float *fd32;
  const float *fd32_eo;
  const int32_t *sym;
  int es_eo;
  double omega;
  int ras;
  DeviceBuffer<float> *halo;  // scratch, grown on demand
  int variant = 0;            // work decomposition chosen by the autotuner
  // shared-cell list of the fix-up pass for this variant (built on first use), or null for
  // the list-free fix-up kernel
  DeviceBuffer<int64_t> *fix_rec = nullptr;
  int64_t *fix_n = nullptr;
  std::vector<int64_t> *fix_layer = nullptr;  // first record of every cell layer (nc_z + 1)
  // per-patch 1-D problems (distorted levels): vertex -> patch map and the patches' FD entries
  bool per_patch = false;
  const int32_t *vpatch = nullptr;
  const int32_t *pfd = nullptr;
};

// pipelined streamed smoother between host buffers: returns false when not applicable
bool launch_stream3d_host(const tpss_layout &L, const StreamLaunch &l, HostPipe &pipe, double *h_dst,
                          const double *h_src, cudaStream_t caller);
bool stream_supported(const tpss_layout &L);
// plane-pass decompositions of the streamed smoother (k = 4; 8 or 4 vertex layers per item)
bool launch_plane3d_bz8(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s);
bool launch_plane3d_bz4(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s);
bool launch_plane3d_host_bz8(const tpss_layout &L, const StreamLaunch &l, HostPipe &pipe, double *h_dst,
                             const double *h_src, cudaStream_t s);
bool launch_plane3d_host_bz4(const tpss_layout &L, const StreamLaunch &l, HostPipe &pipe, double *h_dst,
                             const double *h_src, cudaStream_t s);
// degree-5 decompositions of the streamed smoother (4 x 2 vertex columns, stream_k5.cu)
bool launch_stream3d_k5(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s);
bool launch_stream3d_host_k5(const tpss_layout &L, const StreamLaunch &l, HostPipe &pipe, double *h_dst,
                             const double *h_src, cudaStream_t s);
int stream_variant_count(const tpss_layout &L);
bool launch_stream3d(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s);

// upload the layout's index tables (layout.cu)
void layout_to_device(const tpss_layout &L);

// preconditioner internals (precond.cu)
void precond_vmult(tpss_precond *p, double *dst, const double *src, cudaStream_t s);
// the column-streamed FP32 smoother can serve this preconditioner (layout, precision, tables)
bool stream_eligible(const tpss_precond *p);
}  // namespace tpss
