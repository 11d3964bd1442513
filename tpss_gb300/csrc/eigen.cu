// eigen.cu -- batched FP64 generalized symmetric eigenproblems on the GPU.
//
// For each 1-D patch problem (A_d, M_d) of the fast-diagonalization local solvers this solves
// A s = lambda M s with S^T M S = I, the factorization deal.II's
// TensorProductMatrixSymmetricSum::reinit computes with LAPACK on the CPU (used through
// FD::MatrixIntegrator::assemble_subspace_inverses, apps/laplace_integrator.h:226-250).
// Method: Cholesky M = L L^T, C = L^-1 A L^-T, cyclic Jacobi on C (Golub & Van Loan,
// Matrix Computations, Alg. 8.5.3), S = L^-T V, eigenpairs sorted ascending.
// One warp per problem; the matrices live in shared memory.
#include "internal.h"

namespace tpss
{
namespace
{
constexpr int kMaxN = 32;

__global__ void gen_eig_kernel(int n, int n_problems, const double *__restrict__ Ms,
                               const double *__restrict__ As, double *__restrict__ Ss,
                               double *__restrict__ lams, int *__restrict__ status)
{
  extern __shared__ double sm[];
  const int warps = blockDim.x / 32, w = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int prob = blockIdx.x * warps + w;
  if(prob >= n_problems) return;
  const int nn = n * n;
  double *L = sm + w * 4 * nn, *C = L + nn, *V = C + nn, *X = V + nn;
  const double *M = Ms + (size_t)prob * nn, *A = As + (size_t)prob * nn;
  for(int i = lane; i < nn; i += 32)
  {
    L[i] = 0.0;
    X[i] = A[i];
    C[i] = M[i];  // C holds M during the factorization
    V[i] = (i / n == i % n) ? 1.0 : 0.0;
  }
  __syncwarp();
  // Cholesky, column by column (lanes own rows)
  int bad = 0;
  for(int j = 0; j < n; ++j)
  {
    double d = C[j * n + j];
    for(int p = 0; p < j; ++p) d -= L[j * n + p] * L[j * n + p];
    if(!(d > 0.0)) bad = 1;
    const double ljj = sqrt(fmax(d, 1e-300));
    const int i = j + 1 + lane;
    double lij = 0.0;
    if(i < n)
    {
      double t = C[i * n + j];
      for(int p = 0; p < j; ++p) t -= L[i * n + p] * L[j * n + p];
      lij = t / ljj;
    }
    __syncwarp();
    if(lane == 0) L[j * n + j] = ljj;
    if(i < n) L[i * n + j] = lij;
    __syncwarp();
  }
  // X = L^-1 A (lanes own columns)
  for(int c = lane; c < n; c += 32)
    for(int i = 0; i < n; ++i)
    {
      double t = X[i * n + c];
      for(int p = 0; p < i; ++p) t -= L[i * n + p] * X[p * n + c];
      X[i * n + c] = t / L[i * n + i];
    }
  __syncwarp();
  // C = X L^-T: row r of C solves L y = X[r,:]^T (lanes own rows)
  for(int r = lane; r < n; r += 32)
    for(int i = 0; i < n; ++i)
    {
      double t = X[r * n + i];
      for(int p = 0; p < i; ++p) t -= L[i * n + p] * C[r * n + p];
      C[r * n + i] = t / L[i * n + i];
    }
  __syncwarp();
  for(int idx = lane; idx < nn; idx += 32)
  {
    const int i = idx / n, j = idx % n;
    if(i < j)
    {
      const double t = 0.5 * (C[i * n + j] + C[j * n + i]);
      C[i * n + j] = t;
      C[j * n + i] = t;
    }
  }
  __syncwarp();
  // cyclic Jacobi sweeps
  for(int sweep = 0; sweep < 100; ++sweep)
  {
    double off = 0.0, tot = 0.0;
    for(int idx = lane; idx < nn; idx += 32)
    {
      const double c = C[idx];
      tot += c * c;
      if(idx / n != idx % n) off += c * c;
    }
    for(int o = 16; o > 0; o >>= 1)
    {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    if(off <= 1e-32 * tot) break;
    for(int p = 0; p < n - 1; ++p)
      for(int q = p + 1; q < n; ++q)
      {
        const double apq = C[p * n + q];
        if(apq == 0.0) continue;  // uniform across the warp (same smem value)
        const double tau = (C[q * n + q] - C[p * n + p]) / (2.0 * apq);
        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        const double cs = 1.0 / sqrt(1.0 + t * t), sn = t * cs;
        __syncwarp();
        if(lane < n)
        {
          const int k = lane;
          const double ckp = C[k * n + p], ckq = C[k * n + q];
          C[k * n + p] = cs * ckp - sn * ckq;
          C[k * n + q] = sn * ckp + cs * ckq;
          const double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = cs * vkp - sn * vkq;
          V[k * n + q] = sn * vkp + cs * vkq;
        }
        __syncwarp();
        if(lane < n)
        {
          const int k = lane;
          const double cpk = C[p * n + k], cqk = C[q * n + k];
          C[p * n + k] = cs * cpk - sn * cqk;
          C[q * n + k] = sn * cpk + cs * cqk;
        }
        __syncwarp();
      }
  }
  // S = L^-T V (lanes own columns), written to X
  for(int c = lane; c < n; c += 32)
    for(int i = n - 1; i >= 0; --i)
    {
      double t = V[i * n + c];
      for(int p = i + 1; p < n; ++p) t -= L[p * n + i] * X[p * n + c];
      X[i * n + c] = t / L[i * n + i];
    }
  __syncwarp();
  // sort eigenpairs ascending: rank of each eigenvalue (ties broken by index)
  double *S = Ss + (size_t)prob * nn, *lam = lams + (size_t)prob * n;
  for(int j = lane; j < n; j += 32)
  {
    const double lj = C[j * n + j];
    int rank = 0;
    for(int i = 0; i < n; ++i)
    {
      const double li = C[i * n + i];
      rank += (li < lj) || (li == lj && i < j);
    }
    lam[rank] = lj;
    for(int r = 0; r < n; ++r) S[r * n + rank] = X[r * n + j];
  }
  if(lane == 0) status[prob] = bad;
}
}  // namespace

// Solves all problems; Ms/As/S/lam are host arrays of n_problems * n*n (n) doubles.
// With `status` given, a problem whose M is not positive definite sets its entry (non-zero)
// instead of failing the call.
void gen_eig_batched(int n, int n_problems, const std::vector<double> &Ms,
                     const std::vector<double> &As, std::vector<double> &S,
                     std::vector<double> &lam, std::vector<int> *status)
{
  TPSS_REQUIRE(n >= 1 && n <= kMaxN, "gen_eig_batched: 1-D size out of range");
  if(n_problems == 0)
  {
    S.clear();
    lam.clear();
    return;
  }
  const size_t nn = (size_t)n * n;
  DeviceBuffer<double> dM, dA, dS(n_problems * nn), dl((size_t)n_problems * n);
  DeviceBuffer<int> dst(n_problems);
  dM.upload(Ms.data(), n_problems * nn);
  dA.upload(As.data(), n_problems * nn);
  const int warps = 4;
  const size_t smem = (size_t)warps * 4 * nn * sizeof(double);
  if(smem > 48 * 1024)
    TPSS_CUDA(cudaFuncSetAttribute(gen_eig_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
  const int blocks = (n_problems + warps - 1) / warps;
  gen_eig_kernel<<<blocks, warps * 32, smem>>>(n, n_problems, dM.ptr, dA.ptr, dS.ptr, dl.ptr,
                                               dst.ptr);
  TPSS_CUDA(cudaGetLastError());
  S.resize(n_problems * nn);
  lam.resize((size_t)n_problems * n);
  std::vector<int> st(n_problems);
  TPSS_CUDA(cudaMemcpy(S.data(), dS.ptr, S.size() * sizeof(double), cudaMemcpyDeviceToHost));
  TPSS_CUDA(cudaMemcpy(lam.data(), dl.ptr, lam.size() * sizeof(double), cudaMemcpyDeviceToHost));
  TPSS_CUDA(cudaMemcpy(st.data(), dst.ptr, st.size() * sizeof(int), cudaMemcpyDeviceToHost));
  if(status)
  {
    *status = st;
    return;
  }
  for(int i = 0; i < n_problems; ++i)
    if(st[i]) fail(TPSS_ERR_INVALID_ARGUMENT, "local mass matrix is not positive definite");
}

}  // namespace tpss
