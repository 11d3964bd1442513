// mg.cu -- geometric multigrid V-cycle and the preconditioned CG outer solver (FP64).
//
// Follows the solver stack the Schwarz smoother runs in (apps/poisson_problem.h:642-755,
// apps/multigrid.h:137-399) with deal.II Multigrid::level_v_step semantics:
//   level l > 0:  x_l = P_l b_l                          (pre-smoothing from zero:
//                                                       SmootherRichardson::vmult with one step)
//                 b_{l-1} = R (b_l - A_l x_l)
//                 V-cycle on l-1
//                 x_l += P x_{l-1}
//                 x_l += P_l (b_l - A_l x_l)           (post-smoothing step)
//   level 0:      coarse solve (CG to an absolute residual, or the dense inverse).
// Outer solver: SolverCG with the V-cycle as preconditioner and ReductionControl
// (stop at ||r|| <= max(abs_tol, rel_tol ||r_0||)).
// The V-cycle can be captured in CUDA graphs: with the dense coarse solver the whole cycle is
// one graph launch; with the CG coarse solver the down- and up-sweeps are two graphs around
// the host-driven coarse iteration. With the dense coarse solver the outer CG loop is a graph
// too: a conditional WHILE node whose body holds one iteration and a one-thread kernel that
// tests the residual and sets the loop condition (single solves and batches).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>

#include "internal.h"

namespace tpss
{
const double *embedding_table(int k);

namespace
{
__global__ void cg_update_xr(int64_t n, double *__restrict__ x, double *__restrict__ r,
                             const double *__restrict__ p, const double *__restrict__ Ap,
                             const double *__restrict__ rz, const double *__restrict__ pAp)
{
  const double alpha = *rz / *pAp;
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
  {
    x[i] = fma(alpha, p[i], x[i]);
    r[i] = fma(-alpha, Ap[i], r[i]);
  }
}

__global__ void cg_update_p(int64_t n, double *__restrict__ p, const double *__restrict__ z,
                            const double *__restrict__ rz_new, const double *__restrict__ rz_old)
{
  const double beta = *rz_new / *rz_old;
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = fma(beta, p[i], z[i]);
}

// State of a CG solve whose iteration loop runs on the device: the loop is a conditional WHILE
// node of a CUDA graph, its body one CG iteration followed by cg_loop_control, which sets the
// condition (no host round trip per iteration).
struct CgLoopState
{
  double tol;
  int it, max_iter, hist_cap, converged;
};

__global__ void cg_loop_init(CgLoopState *st, double tol, int max_iter, int hist_cap)
{
  st->tol = tol;
  st->it = 0;
  st->max_iter = max_iter;
  st->hist_cap = hist_cap;
  st->converged = 0;
}

// p = z + beta p, beta = rz_new / rz_old; beta = 0 in the first iteration, whose p is zero
// (the loop starts from p = 0), so that p = z
__global__ void cg_update_p_loop(int64_t n, double *__restrict__ p, const double *__restrict__ z,
                                 const double *__restrict__ rz_new, const double *__restrict__ rz_old,
                                 const CgLoopState *__restrict__ st)
{
  const double beta = st->it == 0 ? 0.0 : *rz_new / *rz_old;
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = fma(beta, p[i], z[i]);
}

// counts the iteration, records ||r|| and continues the loop while ||r|| > tol and
// it < max_iter (a NaN norm fails the test and runs to max_iter)
__global__ void cg_loop_control(cudaGraphConditionalHandle h, const double *__restrict__ rr,
                                double *__restrict__ hist, CgLoopState *__restrict__ st)
{
  const int it = st->it + 1;
  st->it = it;
  const double res = sqrt(*rr);
  if(it < st->hist_cap) hist[it] = res;
  const bool conv = res <= st->tol;
  st->converged = conv;
  cudaGraphSetConditional(h, (conv || it >= st->max_iter) ? 0u : 1u);
}

__global__ void dense_matvec(int n, const double *__restrict__ A, const double *__restrict__ x,
                             double *__restrict__ y)
{
  // one warp per row
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x % 32;
  if(warp >= n) return;
  double s = 0.0;
  for(int j = lane; j < n; j += 32) s = fma(A[(size_t)warp * n + j], x[j], s);
  for(int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if(lane == 0) y[warp] = s;
}

int grid_for(int64_t n)
{
  const int64_t b = (n + 255) / 256, cap = (int64_t)num_sms() * 8;
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

// Dense SIPG matrix of a small Cartesian level (Kronecker sum of the global 1-D operators),
// FP64 on the host.
std::vector<double> dense_matrix(const tpss_layout &L, Penalty ip)
{
  const Shape1D s = make_shape_1d(L.k);
  const int np = L.np, dim = L.dim;
  std::vector<std::vector<double>> M1(dim), A1(dim);
  std::vector<int> n1(dim);
  for(int d = 0; d < dim; ++d)
  {
    std::vector<double> mass, blk;
    operator_blocks_1d(s, L.nc[d], L.h[d].data(), ip, mass, blk);
    const int n = L.nc[d] * np;
    n1[d] = n;
    M1[d].assign((size_t)n * n, 0.0);
    A1[d].assign((size_t)n * n, 0.0);
    for(int c = 0; c < L.nc[d]; ++c)
      for(int i = 0; i < np; ++i)
        for(int j = 0; j < np; ++j)
        {
          M1[d][(size_t)(c * np + i) * n + c * np + j] = mass[(size_t)c * np * np + i * np + j];
          for(int o = -1; o <= 1; ++o)
          {
            const int cn = c + o;
            if(cn < 0 || cn >= L.nc[d]) continue;
            A1[d][(size_t)(c * np + i) * n + cn * np + j] =
              blk[((size_t)c * 3 + o + 1) * np * np + i * np + j];
          }
        }
  }
  const int64_t N = L.n_dofs;
  std::vector<double> A((size_t)N * N, 0.0);
  // global index of (cell multi-index, dof multi-index) in the layout's numbering
  auto gidx = [&](const int *pos) -> int64_t {
    int c[3] = {0, 0, 0}, e = 0, stride = 1;
    for(int d = 0; d < dim; ++d)
    {
      c[d] = pos[d] / np;
      e += (pos[d] % np) * stride;
      stride *= np;
    }
    const int64_t cell = c[0] + (int64_t)L.nc[0] * (c[1] + (int64_t)L.nc[1] * c[2]);
    return L.cell_start[cell] + e;
  };
  int pr[3] = {0, 0, 0}, pc[3] = {0, 0, 0};
  const int n0 = n1[0], n1d = dim > 1 ? n1[1] : 1, n2 = dim > 2 ? n1[2] : 1;
  for(pr[2] = 0; pr[2] < n2; ++pr[2])
    for(pr[1] = 0; pr[1] < n1d; ++pr[1])
      for(pr[0] = 0; pr[0] < n0; ++pr[0])
      {
        const int64_t row = gidx(pr);
        for(pc[2] = 0; pc[2] < n2; ++pc[2])
          for(pc[1] = 0; pc[1] < n1d; ++pc[1])
            for(pc[0] = 0; pc[0] < n0; ++pc[0])
            {
              double v = 0.0;
              for(int d = 0; d < dim; ++d)
              {
                double t = 1.0;
                for(int e = 0; e < dim; ++e)
                {
                  const auto &B = e == d ? A1[e] : M1[e];
                  t *= B[(size_t)pr[e] * n1[e] + pc[e]];
                  if(t == 0.0) break;
                }
                v += t;
              }
              if(v != 0.0) A[(size_t)row * N + gidx(pc)] = v;
            }
      }
  return A;
}

// inverse of an SPD matrix by Cholesky A = G G^T (lower), A^-1 = G^-T G^-1, FP64 on the host
std::vector<double> cholesky_inverse(const std::vector<double> &A, int64_t N)
{
  std::vector<double> G(A);
  for(int64_t j = 0; j < N; ++j)
  {
    double d = G[(size_t)j * N + j];
    for(int64_t p = 0; p < j; ++p) d -= G[(size_t)j * N + p] * G[(size_t)j * N + p];
    if(!(d > 0.0)) fail(TPSS_ERR_INVALID_ARGUMENT, "coarse matrix is not positive definite");
    const double gjj = std::sqrt(d);
    G[(size_t)j * N + j] = gjj;
    for(int64_t i = j + 1; i < N; ++i)
    {
      double t = G[(size_t)i * N + j];
      const double *gi = &G[(size_t)i * N], *gj = &G[(size_t)j * N];
      for(int64_t p = 0; p < j; ++p) t -= gi[p] * gj[p];
      G[(size_t)i * N + j] = t / gjj;
    }
  }
  // Ginv (lower) by forward substitution, then Ainv = Ginv^T Ginv
  std::vector<double> Gi((size_t)N * N, 0.0);
  for(int64_t c = 0; c < N; ++c)
    for(int64_t i = c; i < N; ++i)
    {
      double t = i == c ? 1.0 : 0.0;
      for(int64_t p = c; p < i; ++p) t -= G[(size_t)i * N + p] * Gi[(size_t)p * N + c];
      Gi[(size_t)i * N + c] = t / G[(size_t)i * N + i];
    }
  std::vector<double> Ainv((size_t)N * N, 0.0);
  for(int64_t i = 0; i < N; ++i)
    for(int64_t j = 0; j <= i; ++j)
    {
      double t = 0.0;
      for(int64_t p = i; p < N; ++p) t += Gi[(size_t)p * N + i] * Gi[(size_t)p * N + j];
      Ainv[(size_t)i * N + j] = t;
      Ainv[(size_t)j * N + i] = t;
    }
  return Ainv;
}
}  // namespace
}  // namespace tpss

using namespace tpss;

struct MgLevel
{
  tpss_layout *L = nullptr;
  tpss_operator *op = nullptr;
  tpss_precond *P = nullptr;
  double lambda_max = 0.0;  // estimate of lambda_max(P A) when the damping is scaled
  DeviceBuffer<double> x, b, t, r;
};

struct tpss_mg
{
  tpss_mg_desc desc{};
  std::vector<MgLevel> lv;
  DeviceBuffer<double> coarse_inv;
  // coarse CG and outer CG work vectors and device scalars
  DeviceBuffer<double> cp, cAp, partial, scal;  // scal: [rz, pAp, rz_new, rr, ...]
  DeviceBuffer<double> r, p, Ap, z;
  double *h_scal = nullptr;  // pinned
  const double *E = nullptr;
  cudaGraphExec_t g_full = nullptr, g_down = nullptr, g_up = nullptr;
  // the CG loop on the device (conditional WHILE node; body: one iteration on ub, r, p, ...)
  cudaGraphExec_t g_loop = nullptr;
  DeviceBuffer<double> ub;              // solution vector the loop graph updates
  DeviceBuffer<double> hist;            // residual norms the loop records
  DeviceBuffer<CgLoopState> loop_state;
  // graphs are captured on and launched into a private stream (capture is not possible on
  // the legacy default stream); events order it after / before the caller's stream
  cudaStream_t gstream = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  int coarse_iters_last = 0;
  ~tpss_mg()
  {
    if(gstream) cudaStreamDestroy(gstream);
    if(ev_in) cudaEventDestroy(ev_in);
    if(ev_out) cudaEventDestroy(ev_out);
    if(g_full) cudaGraphExecDestroy(g_full);
    if(g_down) cudaGraphExecDestroy(g_down);
    if(g_up) cudaGraphExecDestroy(g_up);
    if(g_loop) cudaGraphExecDestroy(g_loop);
    for(auto &l : lv)
    {
      tpss_precond_destroy(l.P);
      tpss_operator_destroy(l.op);
      tpss_layout_destroy(l.L);
    }
    if(h_scal) cudaFreeHost(h_scal);
  }
};

namespace
{
// smoothing residual inside the V-cycle, t = b - A x in one pass over the level (FP32
// arithmetic for a single-precision V-cycle)
void level_residual_op(tpss_mg *mg, MgLevel &c, cudaStream_t s)
{
  if(mg->desc.vcycle_precision == TPSS_FP32)
    operator_apply_f32(c.op, c.t.ptr, c.x.ptr, s, c.b.ptr);
  else
    operator_apply(c.op, c.t.ptr, c.x.ptr, s, c.b.ptr);
}

void down_sweep(tpss_mg *mg, cudaStream_t s)
{
  const int top = (int)mg->lv.size() - 1;
  for(int l = top; l >= 1; --l)
  {
    MgLevel &c = mg->lv[l], &f = mg->lv[l - 1];
    precond_vmult(c.P, c.x.ptr, c.b.ptr, s);
    level_residual_op(mg, c, s);
    TPSS_CUDA(cudaMemsetAsync(f.b.ptr, 0, sizeof(double) * f.L->n_dofs, s));
    transfer_apply(c.L->dim, c.L->k, f.L->nc, mg->E, true, f.b.ptr, c.t.ptr, s,
                   mg->desc.vcycle_precision == TPSS_FP32);
  }
}

void up_sweep(tpss_mg *mg, cudaStream_t s)
{
  const int top = (int)mg->lv.size() - 1;
  for(int l = 1; l <= top; ++l)
  {
    MgLevel &c = mg->lv[l], &f = mg->lv[l - 1];
    transfer_apply(c.L->dim, c.L->k, f.L->nc, mg->E, false, f.x.ptr, c.x.ptr, s,
                   mg->desc.vcycle_precision == TPSS_FP32);
    level_residual_op(mg, c, s);
    precond_vmult(c.P, c.r.ptr, c.t.ptr, s);
    vec_axpby(c.L->n_dofs, 1.0, c.r.ptr, 1.0, c.x.ptr, s);
  }
}

void coarse_dense(tpss_mg *mg, cudaStream_t s)
{
  MgLevel &c = mg->lv[0];
  const int n = (int)c.L->n_dofs;
  dense_matvec<<<(n * 32 + 255) / 256, 256, 0, s>>>(n, mg->coarse_inv.ptr, c.b.ptr, c.x.ptr);
  TPSS_CUDA(cudaGetLastError());
}

// Unpreconditioned CG from zero to ||r|| <= coarse_tol (deal.II SolverCG with
// SolverControl(n, tol), as MGCoarseGridIterativeSolver).
void coarse_cg(tpss_mg *mg, cudaStream_t s)
{
  MgLevel &c = mg->lv[0];
  const int64_t n = c.L->n_dofs;
  double *x = c.x.ptr, *r = c.r.ptr, *p = mg->cp.ptr, *Ap = mg->cAp.ptr;
  double *rz = mg->scal.ptr + 0, *pAp = mg->scal.ptr + 1, *rz_new = mg->scal.ptr + 2;
  TPSS_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, s));
  TPSS_CUDA(cudaMemcpyAsync(r, c.b.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  TPSS_CUDA(cudaMemcpyAsync(p, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  vec_dot(n, r, r, mg->partial.ptr, rz, s);
  TPSS_CUDA(cudaMemcpyAsync(mg->h_scal, rz, sizeof(double), cudaMemcpyDeviceToHost, s));
  TPSS_CUDA(cudaStreamSynchronize(s));
  const double tol = mg->desc.coarse_tol;
  int it = 0;
  if(std::sqrt(mg->h_scal[0]) > tol)
  {
    for(it = 1; it <= n; ++it)
    {
      operator_apply(c.op, Ap, p, s);
      vec_dot(n, p, Ap, mg->partial.ptr, pAp, s);
      cg_update_xr<<<grid_for(n), 256, 0, s>>>(n, x, r, p, Ap, rz, pAp);
      vec_dot(n, r, r, mg->partial.ptr, rz_new, s);
      TPSS_CUDA(cudaMemcpyAsync(mg->h_scal, rz_new, sizeof(double), cudaMemcpyDeviceToHost, s));
      TPSS_CUDA(cudaStreamSynchronize(s));
      if(std::sqrt(mg->h_scal[0]) <= tol) break;
      cg_update_p<<<grid_for(n), 256, 0, s>>>(n, p, r, rz_new, rz);
      TPSS_CUDA(cudaMemcpyAsync(rz, rz_new, sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
    if(it > n) fail(TPSS_ERR_NOT_CONVERGED, "coarse grid CG did not converge");
  }
  mg->coarse_iters_last = it;
}

void capture(tpss_mg *mg, void (*fn)(tpss_mg *, cudaStream_t), cudaGraphExec_t *out)
{
  cudaGraph_t g = nullptr;
  cudaStream_t s = mg->gstream;
  TPSS_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  try
  {
    fn(mg, s);
  }
  catch(...)
  {
    cudaStreamEndCapture(s, &g);
    if(g) cudaGraphDestroy(g);
    throw;
  }
  TPSS_CUDA(cudaStreamEndCapture(s, &g));
  cudaError_t e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  TPSS_CUDA(e);
}

void full_cycle(tpss_mg *mg, cudaStream_t s)
{
  down_sweep(mg, s);
  coarse_dense(mg, s);
  up_sweep(mg, s);
}

void launch_graph(tpss_mg *mg, cudaGraphExec_t g, cudaStream_t s)
{
  TPSS_CUDA(cudaEventRecord(mg->ev_in, s));
  TPSS_CUDA(cudaStreamWaitEvent(mg->gstream, mg->ev_in, 0));
  TPSS_CUDA(cudaGraphLaunch(g, mg->gstream));
  TPSS_CUDA(cudaEventRecord(mg->ev_out, mg->gstream));
  TPSS_CUDA(cudaStreamWaitEvent(s, mg->ev_out, 0));
}

// x_top = V-cycle(b_top)
void vcycle(tpss_mg *mg, cudaStream_t s)
{
  const bool dense = mg->desc.coarse_solver == 1;
  if(mg->desc.use_graph)
  {
    if(dense)
    {
      if(!mg->g_full)
      {
        full_cycle(mg, s);  // eager warm-up: scratch allocations happen outside the capture
        TPSS_CUDA(cudaStreamSynchronize(s));
        capture(mg, full_cycle, &mg->g_full);
      }
      launch_graph(mg, mg->g_full, s);
      return;
    }
    if(!mg->g_down)
    {
      down_sweep(mg, s);
      coarse_cg(mg, s);
      up_sweep(mg, s);
      TPSS_CUDA(cudaStreamSynchronize(s));
      capture(mg, down_sweep, &mg->g_down);
      capture(mg, up_sweep, &mg->g_up);
    }
    launch_graph(mg, mg->g_down, s);
    coarse_cg(mg, s);
    launch_graph(mg, mg->g_up, s);
    return;
  }
  down_sweep(mg, s);
  if(dense)
    coarse_dense(mg, s);
  else
    coarse_cg(mg, s);
  up_sweep(mg, s);
}
}  // namespace

namespace
{
// Damping from the spectrum of the additive smoother: the largest eigenvalue of P A (P the
// undamped Schwarz preconditioner) is 2^dim for exact vertex-patch solvers on a Cartesian level
// (every cell lies in 2^dim patches), where the reference's damping factor is tuned. On a
// distorted level it grows (overlap of non-orthogonal patches, inexact local solvers), and with
// the Cartesian damping the smoothing sweep stops being a contraction, which makes the V-cycle
// indefinite. Power iteration with the Rayleigh quotient in the A inner product,
// lambda = (A x, P A x) / (x, A x), 30 steps, 5% safety margin; the level's damping becomes
// omega * 2^dim / (1.05 lambda) when that is smaller than omega.
void scale_relaxation(tpss_mg &mg, MgLevel &lv)
{
  const tpss_layout &L = *lv.L;
  const int64_t n = L.n_dofs;
  std::vector<double> x0(n);
  uint64_t st = 0x5eedull;
  for(int64_t i = 0; i < n; ++i)
  {
    st = st * 6364136223846793005ull + 1442695040888963407ull;  // LCG (Knuth MMIX constants)
    x0[i] = double(st >> 11) * (1.0 / 9007199254740992.0) - 0.5;
  }
  TPSS_CUDA(cudaMemcpy(lv.x.ptr, x0.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
  const double omega = lv.P->desc.relaxation;
  lv.P->desc.relaxation = 1.0;
  cudaStream_t s = nullptr;
  auto dot = [&](const double *a, const double *b) {
    vec_dot(n, a, b, mg.partial.ptr, mg.scal.ptr, s);
    double h = 0.0;
    TPSS_CUDA(cudaMemcpy(&h, mg.scal.ptr, sizeof(double), cudaMemcpyDeviceToHost));
    return h;
  };
  double lambda = 0.0;
  for(int it = 0; it < 30; ++it)
  {
    operator_apply(lv.op, lv.t.ptr, lv.x.ptr, s);  // t = A x
    precond_vmult(lv.P, lv.r.ptr, lv.t.ptr, s);    // r = P A x
    const double xt = dot(lv.x.ptr, lv.t.ptr), tr = dot(lv.t.ptr, lv.r.ptr), rr = dot(lv.r.ptr, lv.r.ptr);
    if(!(xt > 0.0) || !(rr > 0.0)) break;
    lambda = tr / xt;
    vec_axpby(n, 1.0 / std::sqrt(rr), lv.r.ptr, 0.0, lv.x.ptr, s);  // x = r / |r|
  }
  TPSS_CUDA(cudaDeviceSynchronize());
  const double cart = L.patch_variant == TPSS_PATCH_VERTEX ? double(1 << L.dim) : 1.0;
  double w = omega;
  if(lambda > 0.0) w = std::min(omega, omega * cart / (1.05 * lambda));
  lv.P->desc.relaxation = w;
  lv.lambda_max = lambda;
}

// Autotuned smoother kernels of the levels: the first level of a shape (device, dim, degree,
// cells per direction, patch/smoother variant, precision, local solver) times its kernel's work
// decompositions (tpss_precond_autotune, zero vectors, 3 applications each); later levels of the
// same shape -- e.g. the same level in many problems of a batch -- reuse the choice.
std::mutex g_tune_mutex;
std::map<std::vector<int>, std::pair<int, int>> g_tuned;  // shape -> (stream, color) variant

void autotune_level(MgLevel &lv, const tpss_mg_desc &d)
{
  int dev = 0;
  TPSS_CUDA(cudaGetDevice(&dev));
  const tpss_layout &L = *lv.L;
  const std::vector<int> key = {dev, L.dim, L.k, L.nc[0], L.nc[1], L.nc[2], d.patch_variant,
                                d.smoother_variant, lv.P->desc.precision, d.local_solver,
                                d.vertex_coords != nullptr};
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  auto it = g_tuned.find(key);
  if(it == g_tuned.end())
  {
    TPSS_CUDA(cudaMemset(lv.b.ptr, 0, sizeof(double) * L.n_dofs));
    int chosen = 0;
    const int rc = tpss_precond_autotune(lv.P, lv.x.ptr, lv.b.ptr, 3, &chosen, nullptr, nullptr, nullptr);
    if(rc) fail(rc, tpss_last_error());
    TPSS_CUDA(cudaDeviceSynchronize());
    it = g_tuned.emplace(key, std::make_pair(lv.P->stream_variant, lv.P->color_variant)).first;
  }
  lv.P->stream_variant = it->second.first;
  lv.P->color_variant = it->second.second;
}
}  // namespace

namespace
{
bool device_loop(const tpss_mg *mg);
void prepare_loop(tpss_mg *mg, int max_iter);
}  // namespace

extern "C" int tpss_mg_create(const tpss_mg_desc *d, tpss_mg **out)
{
  return guarded([&] {
    TPSS_REQUIRE(d && out, "null argument");
    *out = nullptr;
    TPSS_REQUIRE(d->dim == 2 || d->dim == 3, "dim must be 2 or 3");
    TPSS_REQUIRE(d->n_rep >= 1 && d->n_cells_fine >= d->n_rep, "invalid mesh sizes");
    int nl = 0;
    for(int nc = d->n_rep; nc <= d->n_cells_fine; nc *= 2) ++nl;
    TPSS_REQUIRE((d->n_rep << (nl - 1)) == d->n_cells_fine, "n_cells_fine must be n_rep * 2^L");
    TPSS_REQUIRE(nl >= 2, "at least two levels are needed");
    TPSS_REQUIRE(d->vcycle_precision == TPSS_FP64 || d->vcycle_precision == TPSS_FP32,
                 "vcycle_precision must be TPSS_FP64 or TPSS_FP32");
    auto mg = std::make_unique<tpss_mg>();
    mg->desc = *d;
    mg->lv.resize(nl);
    std::vector<double> coords;
    for(int l = 0; l < nl; ++l)
    {
      MgLevel &lv = mg->lv[l];
      tpss_layout_desc ld{};
      if(d->vertex_coords)
      {
        // distorted hierarchy: a coarse level keeps every 2^(L-l)-th vertex of the finest
        const int nf = d->n_cells_fine, nv = nf + 1, stride = 1 << (nl - 1 - l);
        const int ncl = d->n_rep << l, nvl = ncl + 1;
        const int nz = d->dim > 2 ? nvl : 1;
        coords.assign((size_t)nvl * nvl * nz * d->dim, 0.0);
        for(int z = 0; z < nz; ++z)
          for(int y = 0; y < nvl; ++y)
            for(int x = 0; x < nvl; ++x)
            {
              const int64_t src = x * stride + (int64_t)nv * (y * stride + (int64_t)nv * z * stride);
              const int64_t dst = x + (int64_t)nvl * (y + (int64_t)nvl * z);
              for(int e = 0; e < d->dim; ++e) coords[dst * d->dim + e] = d->vertex_coords[src * d->dim + e];
            }
        ld.vertex_coords = coords.data();
        ld.surrogate_n_q = d->surrogate_n_q;
      }
      ld.dim = d->dim;
      ld.degree = d->degree;
      ld.dof_layout = TPSS_DOF_DGQ;
      ld.patch_variant = d->patch_variant;
      ld.smoother_variant = d->smoother_variant;
      for(int dd = 0; dd < 3; ++dd) ld.n_cells[dd] = dd < d->dim ? (d->n_rep << l) : 1;
      int rc = tpss_layout_create(&ld, &lv.L);
      if(rc) fail(rc, tpss_last_error());
      rc = tpss_operator_create_penalty(lv.L, d->ip_factor, d->penalty_mode, &lv.op);
      if(rc) fail(rc, tpss_last_error());
      if(l > 0)
      {
        tpss_precond_desc pd{};
        pd.relaxation = d->relaxation;
        pd.precision = (d->fp64_level_mask >> l) & 1 ? TPSS_FP64 : d->precision;
        pd.ip_factor = d->ip_factor;
        pd.penalty_mode = d->penalty_mode;
        pd.local_solver = d->local_solver;
        pd.model = d->model;
        rc = tpss_precond_create(lv.L, lv.op, &pd, &lv.P);
        if(rc) fail(rc, tpss_last_error());
      }
      const int64_t n = lv.L->n_dofs;
      lv.x.resize(n);
      lv.b.resize(n);
      lv.t.resize(n);
      lv.r.resize(n);
    }
    const int64_t n0 = mg->lv[0].L->n_dofs, nt = mg->lv[nl - 1].L->n_dofs;
    if(d->coarse_solver == 1)
    {
      TPSS_REQUIRE(n0 <= 4096, "dense coarse solver limited to 4096 coarse DoFs");
      const tpss_operator &cop = *mg->lv[0].op;
      std::vector<double> inv = cholesky_inverse(
        cop.mapped ? mapped_dense(cop)
                   : dense_matrix(*mg->lv[0].L, make_penalty(d->ip_factor, d->penalty_mode, d->degree)),
        n0);
      mg->coarse_inv.upload(inv.data(), inv.size());
    }
    mg->cp.resize(n0);
    mg->cAp.resize(n0);
    mg->partial.resize(dot_partials());
    mg->scal.resize(16);
    mg->r.resize(nt);
    mg->p.resize(nt);
    mg->Ap.resize(nt);
    mg->z.resize(nt);
    TPSS_CUDA(cudaMallocHost(&mg->h_scal, 16 * sizeof(double)));
    TPSS_CUDA(cudaStreamCreateWithFlags(&mg->gstream, cudaStreamNonBlocking));
    TPSS_CUDA(cudaEventCreateWithFlags(&mg->ev_in, cudaEventDisableTiming));
    TPSS_CUDA(cudaEventCreateWithFlags(&mg->ev_out, cudaEventDisableTiming));
    mg->E = embedding_table(d->degree);
    if(d->auto_relaxation)
      for(int l = 1; l < nl; ++l) scale_relaxation(*mg, mg->lv[l]);
    if(d->autotune)
      for(int l = 1; l < nl; ++l) autotune_level(mg->lv[l], *d);
    // the device CG loop is captured here (after an eager V-cycle on r = 0), so that a solve
    // launches it directly
    if(device_loop(mg.get()))
    {
      TPSS_CUDA(cudaMemset(mg->r.ptr, 0, sizeof(double) * mg->r.n));
      prepare_loop(mg.get(), 1023);
    }
    *out = mg.release();
  });
}

extern "C" int tpss_mg_n_dofs(const tpss_mg *mg, int64_t *n)
{
  return guarded([&] {
    TPSS_REQUIRE(mg && n, "null argument");
    *n = mg->lv.back().L->n_dofs;
  });
}

extern "C" int tpss_mg_n_levels(const tpss_mg *mg, int *n)
{
  return guarded([&] {
    TPSS_REQUIRE(mg && n, "null argument");
    *n = (int)mg->lv.size();
  });
}

extern "C" int tpss_mg_level(tpss_mg *mg, int level, tpss_layout **layout, tpss_operator **op,
                             tpss_precond **precond)
{
  return guarded([&] {
    TPSS_REQUIRE(mg && level >= 0 && level < (int)mg->lv.size(), "invalid level");
    if(layout) *layout = mg->lv[level].L;
    if(op) *op = mg->lv[level].op;
    if(precond) *precond = mg->lv[level].P;
  });
}

extern "C" int tpss_mg_vmult(tpss_mg *mg, double *dst, const double *src, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(mg && dst && src, "null argument");
    cudaStream_t s = as_stream(stream);
    MgLevel &top = mg->lv.back();
    const int64_t n = top.L->n_dofs;
    TPSS_CUDA(cudaMemcpyAsync(top.b.ptr, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    vcycle(mg, s);
    TPSS_CUDA(cudaMemcpyAsync(dst, top.x.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  });
}

namespace
{
// r = f, ||r||^2 into the pinned host slot (u := 0 on the device loop's ub)
void cg_start(tpss_mg *mg, double *u, const double *f, cudaStream_t s)
{
  MgLevel &top = mg->lv.back();
  const int64_t n = top.L->n_dofs;
  TPSS_CUDA(cudaMemsetAsync(u, 0, sizeof(double) * n, s));
  TPSS_CUDA(cudaMemcpyAsync(mg->r.ptr, f, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  vec_dot(n, mg->r.ptr, mg->r.ptr, mg->partial.ptr, mg->scal.ptr + 10, s);
  TPSS_CUDA(cudaMemcpyAsync(mg->h_scal + 4, mg->scal.ptr + 10, sizeof(double), cudaMemcpyDeviceToHost, s));
}

// One CG iteration of the device loop: z = V(r); rz_new = r.z; p = z + beta p (beta = 0 first);
// rz = rz_new; then alpha = rz / p.Ap, ub += alpha p, r -= alpha A p, ||r||^2 -- the order and
// the kernels of the host loop of tpss_mg_cg_solve -- and cg_loop_control.
void loop_body(tpss_mg *mg, cudaGraphConditionalHandle h, cudaStream_t s)
{
  MgLevel &top = mg->lv.back();
  const int64_t n = top.L->n_dofs;
  double *r = mg->r.ptr, *p = mg->p.ptr, *Ap = mg->Ap.ptr, *u = mg->ub.ptr;
  double *d_rz = mg->scal.ptr + 8, *d_pAp = mg->scal.ptr + 9, *d_rr = mg->scal.ptr + 10,
         *d_rz_new = mg->scal.ptr + 11;
  CgLoopState *st = mg->loop_state.ptr;
  TPSS_CUDA(cudaMemcpyAsync(top.b.ptr, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  vcycle(mg, s);
  vec_dot(n, r, top.x.ptr, mg->partial.ptr, d_rz_new, s);
  cg_update_p_loop<<<grid_for(n), 256, 0, s>>>(n, p, top.x.ptr, d_rz_new, d_rz, st);
  TPSS_CUDA(cudaMemcpyAsync(d_rz, d_rz_new, sizeof(double), cudaMemcpyDeviceToDevice, s));
  operator_apply(top.op, Ap, p, s);
  vec_dot(n, p, Ap, mg->partial.ptr, d_pAp, s);
  cg_update_xr<<<grid_for(n), 256, 0, s>>>(n, u, r, p, Ap, d_rz, d_pAp);
  vec_dot(n, r, r, mg->partial.ptr, d_rr, s);
  cg_loop_control<<<1, 1, 0, s>>>(h, d_rr, mg->hist.ptr, st);
  TPSS_CUDA(cudaGetLastError());
}

// The loop graph: one conditional WHILE node (condition 1 at every launch) whose body is
// captured from loop_body with the V-cycle's kernels inline. Captured once per hierarchy after
// an eager V-cycle (its lazy set-up -- scratch, lists -- happens outside the capture).
void capture_loop(tpss_mg *mg, int hist_cap)
{
  MgLevel &top = mg->lv.back();
  const int64_t n = top.L->n_dofs;
  if(mg->ub.n < (size_t)n) mg->ub.resize(n);
  if(mg->loop_state.n == 0) mg->loop_state.resize(1);
  mg->hist.resize(hist_cap);
  if(mg->g_loop)
  {
    TPSS_CUDA(cudaGraphExecDestroy(mg->g_loop));
    mg->g_loop = nullptr;
  }
  cudaStream_t s = mg->gstream;
  TPSS_CUDA(cudaMemcpyAsync(top.b.ptr, mg->r.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  vcycle(mg, s);
  TPSS_CUDA(cudaStreamSynchronize(s));
  cudaGraph_t g = nullptr;
  TPSS_CUDA(cudaGraphCreate(&g, 0));
  const int use_graph = mg->desc.use_graph;
  try
  {
    cudaGraphConditionalHandle h = 0;
    TPSS_CUDA(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    TPSS_CUDA(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    TPSS_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    mg->desc.use_graph = 0;  // V-cycle kernels inline in the body
    try
    {
      loop_body(mg, h, s);
    }
    catch(...)
    {
      cudaGraph_t tmp = nullptr;
      cudaStreamEndCapture(s, &tmp);
      throw;
    }
    mg->desc.use_graph = use_graph;
    cudaGraph_t captured = nullptr;
    TPSS_CUDA(cudaStreamEndCapture(s, &captured));  // the body, owned by the node
    TPSS_CUDA(cudaGraphInstantiate(&mg->g_loop, g, 0));
  }
  catch(...)
  {
    mg->desc.use_graph = use_graph;
    cudaGraphDestroy(g);
    throw;
  }
  cudaGraphDestroy(g);
}

bool device_loop(const tpss_mg *mg) { return mg->desc.use_graph && mg->desc.coarse_solver == 1; }

// ensure the loop graph for max_iter iterations (the residual history holds max_iter + 1)
void prepare_loop(tpss_mg *mg, int max_iter)
{
  const size_t cap = std::max<size_t>(1024, (size_t)max_iter + 1);
  if(!mg->g_loop || mg->hist.n < (size_t)max_iter + 1) capture_loop(mg, (int)cap);
}

// launch the device loop (p := 0, state reset) on stream s; r holds f, ub zero
void launch_loop(tpss_mg *mg, double tol, int max_iter, cudaStream_t s, bool private_stream)
{
  const int64_t n = mg->lv.back().L->n_dofs;
  TPSS_CUDA(cudaMemsetAsync(mg->p.ptr, 0, sizeof(double) * n, s));
  cg_loop_init<<<1, 1, 0, s>>>(mg->loop_state.ptr, tol, max_iter, (int)mg->hist.n);
  TPSS_CUDA(cudaGetLastError());
  if(private_stream)
    launch_graph(mg, mg->g_loop, s);
  else
    TPSS_CUDA(cudaGraphLaunch(mg->g_loop, s));
}
}  // namespace

extern "C" int tpss_mg_cg_solve(tpss_mg *mg, double *u, const double *f, double rel_tol,
                                double abs_tol, int max_iter, int *iterations,
                                double *res_history, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(mg && u && f && iterations, "null argument");
    TPSS_REQUIRE(max_iter >= 0, "max_iter must be non-negative");
    cudaStream_t s = as_stream(stream);
    MgLevel &top = mg->lv.back();
    const int64_t n = top.L->n_dofs;
    double *r = mg->r.ptr, *p = mg->p.ptr, *Ap = mg->Ap.ptr;
    double *d_rz = mg->scal.ptr + 8, *d_pAp = mg->scal.ptr + 9, *d_rr = mg->scal.ptr + 10,
           *d_rz_new = mg->scal.ptr + 11;
    if(device_loop(mg))
    {
      // the iteration loop on the device: one graph launch, one synchronization
      if(mg->ub.n < (size_t)n) mg->ub.resize(n);
      cg_start(mg, mg->ub.ptr, f, s);
      TPSS_CUDA(cudaStreamSynchronize(s));
      const double res0 = std::sqrt(mg->h_scal[4]);
      if(res_history) res_history[0] = res0;
      const double tol = std::max(abs_tol, rel_tol * res0);
      int it = 0;
      bool converged = res0 <= tol;
      if(!converged && max_iter > 0)
      {
        prepare_loop(mg, max_iter);
        launch_loop(mg, tol, max_iter, s, true);
        CgLoopState st{};
        TPSS_CUDA(cudaMemcpyAsync(mg->h_scal + 8, mg->loop_state.ptr, sizeof(CgLoopState),
                                  cudaMemcpyDeviceToHost, s));
        TPSS_CUDA(cudaStreamSynchronize(s));
        std::memcpy(&st, mg->h_scal + 8, sizeof(CgLoopState));
        it = st.it;
        converged = st.converged != 0;
        if(res_history && it > 0)
          TPSS_CUDA(cudaMemcpy(res_history + 1, mg->hist.ptr + 1, sizeof(double) * it, cudaMemcpyDeviceToHost));
      }
      TPSS_CUDA(cudaMemcpyAsync(u, mg->ub.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      *iterations = converged ? it : -1;
      if(!converged) fail(TPSS_ERR_NOT_CONVERGED, "CG did not reach the tolerance within max_iter");
      return;
    }
    TPSS_CUDA(cudaMemsetAsync(u, 0, sizeof(double) * n, s));
    TPSS_CUDA(cudaMemcpyAsync(r, f, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    vec_dot(n, r, r, mg->partial.ptr, d_rr, s);
    TPSS_CUDA(cudaMemcpyAsync(mg->h_scal + 4, d_rr, sizeof(double), cudaMemcpyDeviceToHost, s));
    TPSS_CUDA(cudaStreamSynchronize(s));
    double res = std::sqrt(mg->h_scal[4]);
    if(res_history) res_history[0] = res;
    const double tol = std::max(abs_tol, rel_tol * res);
    int it = 0;
    bool converged = res <= tol;
    if(!converged)
    {
      // z = V(r); p = z; rz = r.z
      TPSS_CUDA(cudaMemcpyAsync(top.b.ptr, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      vcycle(mg, s);
      TPSS_CUDA(cudaMemcpyAsync(p, top.x.ptr, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      vec_dot(n, r, top.x.ptr, mg->partial.ptr, d_rz, s);
      for(it = 1; it <= max_iter; ++it)
      {
        operator_apply(top.op, Ap, p, s);
        vec_dot(n, p, Ap, mg->partial.ptr, d_pAp, s);
        cg_update_xr<<<grid_for(n), 256, 0, s>>>(n, u, r, p, Ap, d_rz, d_pAp);
        vec_dot(n, r, r, mg->partial.ptr, d_rr, s);
        TPSS_CUDA(cudaMemcpyAsync(mg->h_scal + 4, d_rr, sizeof(double), cudaMemcpyDeviceToHost, s));
        TPSS_CUDA(cudaStreamSynchronize(s));
        res = std::sqrt(mg->h_scal[4]);
        if(res_history) res_history[it] = res;
        if(res <= tol)
        {
          converged = true;
          break;
        }
        TPSS_CUDA(cudaMemcpyAsync(top.b.ptr, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        vcycle(mg, s);
        vec_dot(n, r, top.x.ptr, mg->partial.ptr, d_rz_new, s);
        cg_update_p<<<grid_for(n), 256, 0, s>>>(n, p, top.x.ptr, d_rz_new, d_rz);
        TPSS_CUDA(cudaMemcpyAsync(d_rz, d_rz_new, sizeof(double), cudaMemcpyDeviceToDevice, s));
      }
    }
    *iterations = converged ? it : -1;
    if(!converged) fail(TPSS_ERR_NOT_CONVERGED, "CG did not reach the tolerance within max_iter");
  });
}

// ---- batched solves: many independent hierarchies ------------------------------------------
// Every problem's CG runs as its device loop graph (conditional WHILE node), launched once on
// one of n_streams streams: the problems are dealt to the streams largest first, each to the
// stream with the least work so far (estimated as DoFs x (degree + 1) plus a fixed cost per
// problem for its launch-bound small levels); one host synchronization at the end reads all
// iteration counts. A problem stops at its own ReductionControl tolerance
// (apps/rt_parameter.h:39-41).
struct tpss_batch
{
  std::vector<tpss_mg *> mg;
  std::vector<cudaStream_t> streams;
  std::vector<int> stream_of;  // stream of every problem
  std::vector<int> order;      // launch order: estimated work, largest first
  ~tpss_batch()
  {
    for(tpss_mg *m : mg) delete m;
    for(cudaStream_t s : streams) cudaStreamDestroy(s);
  }
};

extern "C" int tpss_batch_create(const tpss_mg_desc *descs, int n_problems, int n_streams, tpss_batch **out)
{
  return guarded([&] {
    TPSS_REQUIRE(descs && out && n_problems >= 1 && n_streams >= 1 && n_streams <= 64, "invalid argument");
    *out = nullptr;
    auto b = std::make_unique<tpss_batch>();
    for(int i = 0; i < n_problems; ++i)
      TPSS_REQUIRE(descs[i].coarse_solver == 1 && descs[i].use_graph,
                   "batched solves run every CG loop as one CUDA graph: they need the dense coarse "
                   "solver (coarse_solver = 1; the coarse CG waits for the host) and use_graph = 1");
    std::vector<double> work(n_problems);
    for(int i = 0; i < n_problems; ++i)
    {
      tpss_mg *m = nullptr;
      const int rc = tpss_mg_create(&descs[i], &m);
      if(rc) fail(rc, std::string("problem ") + std::to_string(i) + ": " + tpss_last_error());
      b->mg.push_back(m);
      work[i] = double(m->lv.back().L->n_dofs) * (descs[i].degree + 1) + 2.0e5;
    }
    for(int i = 0; i < n_streams; ++i)
    {
      cudaStream_t s;
      TPSS_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
      b->streams.push_back(s);
    }
    b->order.resize(n_problems);
    for(int i = 0; i < n_problems; ++i) b->order[i] = i;
    std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) { return work[x] > work[y]; });
    std::vector<double> load(n_streams, 0.0);
    b->stream_of.assign(n_problems, 0);
    for(int i : b->order)
    {
      const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
      b->stream_of[i] = k;
      load[k] += work[i];
    }
    *out = b.release();
  });
}

extern "C" int tpss_batch_problem(tpss_batch *b, int i, tpss_mg **mg)
{
  return guarded([&] {
    TPSS_REQUIRE(b && mg && i >= 0 && i < (int)b->mg.size(), "invalid argument");
    *mg = b->mg[i];
  });
}

extern "C" int tpss_batch_solve(tpss_batch *b, double *const *u, const double *const *f, double rel_tol,
                                double abs_tol, int max_iter, int *iterations, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(b && u && f && iterations && max_iter >= 0, "invalid argument");
    const int P = (int)b->mg.size();
    cudaStream_t caller = as_stream(stream);
    auto st_of = [&](int i) { return b->streams[b->stream_of[i]]; };
    cudaEvent_t ev;
    TPSS_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    TPSS_CUDA(cudaEventRecord(ev, caller));
    for(cudaStream_t s : b->streams) TPSS_CUDA(cudaStreamWaitEvent(s, ev, 0));
    auto sync_all = [&]() {
      for(cudaStream_t s : b->streams) TPSS_CUDA(cudaStreamSynchronize(s));
    };
    for(int i = 0; i < P; ++i)
    {
      TPSS_REQUIRE(u[i] && f[i], "null problem vector");
      tpss_mg *m = b->mg[i];
      const size_t n = (size_t)m->lv.back().L->n_dofs;
      if(m->ub.n < n) m->ub.resize(n);
      cg_start(m, m->ub.ptr, f[i], st_of(i));
    }
    sync_all();
    std::vector<double> tol(P);
    std::vector<char> active(P), converged(P);
    std::vector<int> its(P, 0);
    for(int i = 0; i < P; ++i)
    {
      const double r0 = std::sqrt(b->mg[i]->h_scal[4]);
      tol[i] = std::max(abs_tol, rel_tol * r0);
      converged[i] = r0 <= tol[i];
      active[i] = !converged[i] && max_iter > 0;
    }
    // loop graphs: captured once per problem (after an eager V-cycle on its private stream)
    for(int i = 0; i < P; ++i)
      if(active[i]) prepare_loop(b->mg[i], max_iter);
    for(int i : b->order)
      if(active[i]) launch_loop(b->mg[i], tol[i], max_iter, st_of(i), false);
    for(int i = 0; i < P; ++i)
      if(active[i])
        TPSS_CUDA(cudaMemcpyAsync(b->mg[i]->h_scal + 8, b->mg[i]->loop_state.ptr, sizeof(CgLoopState),
                                  cudaMemcpyDeviceToHost, st_of(i)));
    sync_all();
    for(int i = 0; i < P; ++i)
    {
      if(!active[i]) continue;
      CgLoopState st{};
      std::memcpy(&st, b->mg[i]->h_scal + 8, sizeof(CgLoopState));
      its[i] = st.it;
      converged[i] = st.converged != 0;
    }
    for(int i = 0; i < P; ++i)
    {
      tpss_mg *m = b->mg[i];
      TPSS_CUDA(cudaMemcpyAsync(u[i], m->ub.ptr, sizeof(double) * m->lv.back().L->n_dofs,
                                cudaMemcpyDeviceToDevice, st_of(i)));
    }
    for(cudaStream_t s : b->streams)
    {
      TPSS_CUDA(cudaEventRecord(ev, s));
      TPSS_CUDA(cudaStreamWaitEvent(caller, ev, 0));
    }
    cudaEventDestroy(ev);
    bool all = true;
    for(int i = 0; i < P; ++i)
    {
      iterations[i] = converged[i] ? its[i] : -1;
      all = all && converged[i];
    }
    if(!all) fail(TPSS_ERR_NOT_CONVERGED, "some problems of the batch did not converge");
  });
}

extern "C" void tpss_batch_destroy(tpss_batch *b) { delete b; }

extern "C" void tpss_mg_destroy(tpss_mg *mg) { delete mg; }

extern "C" int tpss_mg_relaxation(const tpss_mg *mg, int level, double *relaxation, double *lambda_max)
{
  return guarded([&] {
    TPSS_REQUIRE(mg && level >= 1 && level < (int)mg->lv.size(), "invalid level (smoothers on 1..L)");
    if(relaxation) *relaxation = mg->lv[level].P->desc.relaxation;
    if(lambda_max) *lambda_max = mg->lv[level].lambda_max;
  });
}
