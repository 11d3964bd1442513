// Local solvers built from the exact patch matrices of a distorted level.
//
// The patch matrix A_j = R_j A R_j^T of a vertex patch consists of cell blocks of the
// level's block-sparse SIPG matrix (mapped.cu): the block of two patch cells is the level
// block of the pair when they are equal or share a face, and zero otherwise
// (apps/laplace_integrator.h:226-256 assembles the same submatrices from the level operator).
// From these matrices, batched on the GPU:
//   - the exact local inverse, the reference's dense "basic state" of TensorProductMatrix
//     with its InverseTable (tensor_product_matrix.templates.h:113-124, matrix_helper.h:21-120):
//     Gauss-Jordan in shared memory (FP64, n_loc <= 160), applied per color by a dense
//     matrix-vector kernel with the same gather / damping / scatter-add as the FD path;
//   - a separable approximation for fast diagonalization: the Kronecker sum
//     sum_d M_(D-1) x ... x A_d x ... x M_0 closest to A_j in the Frobenius norm for given
//     1-D masses M_d (the surrogate patch masses), i.e. the low Kronecker-rank approximation
//     of compute_ksvd (kroneckersvd.h:207-402) with the mass factors held fixed, which makes
//     the fit linear:
//        R_d = <A_j, M_e for e != d>  (contraction of every direction but d),
//        S   = <A_j, M_(D-1) x ... x M_0>,  mu_e = ||M_e||_F^2,  c_d = prod_{e != d} mu_e,
//        A_d = R_d / c_d - (D-1)/D * S / prod_e mu_e * M_d
//     (the shifts A_d + a_d M_d with sum_d a_d = 0 leave the sum unchanged; this choice
//     splits them evenly). On a Cartesian patch the fit returns the exact 1-D matrices.
#include "internal.h"

namespace tpss
{
namespace
{
struct LocalMap
{
  int dim, np, n, nloc, npc, ncp;
};

// patch-local lexicographic index r -> (patch cell, DoF in that cell)
__device__ __forceinline__ void local_to_cell(const LocalMap &m, int r, int &cell, int &e)
{
  cell = 0;
  e = 0;
  int sc = 1, se = 1;
  for(int d = 0; d < m.dim; ++d)
  {
    const int l = r % m.n;
    r /= m.n;
    cell += (l / m.np) * sc;
    e += (l % m.np) * se;
    sc *= m.ncp;
    se *= m.np;
  }
}

// slot of the level block coupling patch cells a (row) and b (column), -1 if none
__device__ __forceinline__ int pair_slot(const LocalMap &m, int a, int b)
{
  if(a == b) return 0;
  int diff = -1, side = 0, ndiff = 0;
  for(int d = 0; d < m.dim; ++d)
  {
    const int ca = (a >> d) & 1, cb = (b >> d) & 1;
    if(ca != cb)
    {
      ++ndiff;
      diff = d;
      side = cb > ca;
    }
  }
  return ndiff == 1 ? 1 + 2 * diff + side : -1;
}

struct ExtractArgs
{
  LocalMap m;
  const int32_t *lower;  // P * 3 lower cell of each patch
  int nc[3];
  const double *vals;    // level blocks
  int nd, nb;
  int64_t p0, count;
  double *out;           // count * nloc * nloc, row-major
};

__global__ void __launch_bounds__(256) extract_kernel(const ExtractArgs a)
{
  const int64_t pp = blockIdx.y;
  if(pp >= a.count) return;
  const int64_t p = a.p0 + pp;
  const LocalMap &m = a.m;
  const int64_t nn = (int64_t)m.nloc * m.nloc;
  int lo[3] = {a.lower[p * 3], a.lower[p * 3 + 1], a.lower[p * 3 + 2]};
  for(int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nn;
      idx += (int64_t)gridDim.x * blockDim.x)
  {
    const int r = int(idx / m.nloc), c = int(idx % m.nloc);
    int ca, ea, cb, eb;
    local_to_cell(m, r, ca, ea);
    local_to_cell(m, c, cb, eb);
    const int s = pair_slot(m, ca, cb);
    double v = 0.0;
    if(s >= 0)
    {
      int cc[3] = {lo[0], lo[1], lo[2]};
      for(int d = 0; d < m.dim; ++d) cc[d] += (ca >> d) & 1;
      const int64_t cell = cc[0] + (int64_t)a.nc[0] * (cc[1] + (int64_t)a.nc[1] * cc[2]);
      v = a.vals[((cell * a.nb + s) * a.nd + eb) * a.nd + ea];
    }
    a.out[pp * nn + idx] = v;
  }
}

// In-place Gauss-Jordan inversion of one SPD patch matrix per CTA, in shared memory.
__global__ void __launch_bounds__(512) gj_inverse_kernel(const double *__restrict__ in, int n,
                                                         int64_t count, double *out64,
                                                         float *out32, int64_t p0, int *bad)
{
  extern __shared__ double A[];
  const int64_t pp = blockIdx.x;
  if(pp >= count) return;
  const int64_t nn = (int64_t)n * n;
  for(int64_t i = threadIdx.x; i < nn; i += blockDim.x) A[i] = in[pp * nn + i];
  __syncthreads();
  __shared__ double piv;
  for(int k = 0; k < n; ++k)
  {
    if(threadIdx.x == 0)
    {
      piv = A[k * n + k];
      if(!(piv > 0.0))
      {
        atomicOr(bad, 1);
        piv = 1.0;
      }
    }
    __syncthreads();
    const double p = piv;
    for(int j = threadIdx.x; j < n; j += blockDim.x)
      if(j != k) A[k * n + j] /= p;
    __syncthreads();
    for(int64_t idx = threadIdx.x; idx < nn; idx += blockDim.x)
    {
      const int i = int(idx / n), j = int(idx % n);
      if(i != k && j != k) A[idx] -= A[i * n + k] * A[k * n + j];
    }
    __syncthreads();
    for(int i = threadIdx.x; i < n; i += blockDim.x)
      if(i != k) A[i * n + k] = -A[i * n + k] / p;
    if(threadIdx.x == 0) A[k * n + k] = 1.0 / p;
    __syncthreads();
  }
  const int64_t base = (p0 + pp) * nn;
  for(int64_t i = threadIdx.x; i < nn; i += blockDim.x)
  {
    // store A^-1 transposed, so that output row i reads consecutive addresses in the apply
    const int r = int(i / n), c = int(i % n);
    const double v = A[c * n + r];
    if(out64) out64[base + i] = v;
    if(out32) out32[base + i] = float(v);
  }
}

struct DenseArgs
{
  LocalMap m;
  const double *src;
  double *dst;
  const int64_t *patch_first;  // first patch of the color
  const void *inv;             // P * nloc * nloc (transposed) for the whole level
  int64_t p_begin, n_patches;
  double omega;
};

template<typename T>
__global__ void __launch_bounds__(256) dense_apply_kernel(const DenseArgs a)
{
  extern __shared__ unsigned char smraw[];
  T *r = reinterpret_cast<T *>(smraw);
  const LocalMap &m = a.m;
  const T *inv = reinterpret_cast<const T *>(a.inv);
  for(int64_t pp = blockIdx.x; pp < a.n_patches; pp += gridDim.x)
  {
    const int64_t *first = a.patch_first + pp * m.npc;
    for(int l = threadIdx.x; l < m.nloc; l += blockDim.x)
    {
      int c, e;
      local_to_cell(m, l, c, e);
      r[l] = T(a.src[first[c] + e]);
    }
    __syncthreads();
    const T *Ai = inv + (a.p_begin + pp) * (int64_t)m.nloc * m.nloc;
    for(int i = threadIdx.x; i < m.nloc; i += blockDim.x)
    {
      T acc = 0;
      for(int j = 0; j < m.nloc; ++j) acc += Ai[(int64_t)j * m.nloc + i] * r[j];
      int c, e;
      local_to_cell(m, i, c, e);
      a.dst[first[c] + e] += a.omega * double(acc);
    }
    __syncthreads();
  }
}

// Kronecker-sum fit with fixed masses, one patch per CTA.
struct FitArgs
{
  int dim, n;
  const double *K;      // count * nloc^2 patch matrices (row-major)
  const double *M;      // count * dim * n^2 masses
  double *A;            // count * dim * n^2 fitted 1-D matrices
  int64_t count;
};

__global__ void __launch_bounds__(256) ksum_fit_kernel(const FitArgs a)
{
  extern __shared__ double sm[];
  const int64_t pp = blockIdx.x;
  if(pp >= a.count) return;
  const int n = a.n, n2 = n * n, dim = a.dim;
  int nloc = 1;
  for(int d = 0; d < dim; ++d) nloc *= n;
  const double *K = a.K + pp * (int64_t)nloc * nloc;
  double *M = sm;                 // dim * n2
  double *T = M + dim * n2;       // n^4 intermediate (3D)
  double *R = T + n2 * n2;        // dim * n2
  for(int i = threadIdx.x; i < dim * n2; i += blockDim.x) M[i] = a.M[pp * dim * n2 + i];
  __syncthreads();
  // entry of K with row multi-index (r0, r1, r2) and column multi-index (c0, c1, c2)
  auto Kat = [&](int r0, int r1, int r2, int c0, int c1, int c2) {
    const int row = r0 + n * (r1 + n * r2), col = c0 + n * (c1 + n * c2);
    return K[(int64_t)row * nloc + col];
  };
  for(int d = 0; d < dim; ++d)
  {
    if(dim == 2)
    {
      const int e = 1 - d;
      const double *Me = M + e * n2;
      for(int ij = threadIdx.x; ij < n2; ij += blockDim.x)
      {
        const int i = ij / n, j = ij % n;
        double s = 0.0;
        for(int u = 0; u < n; ++u)
          for(int v = 0; v < n; ++v)
          {
            const double mv = Me[u * n + v];
            s += mv * (d == 0 ? Kat(i, u, 0, j, v, 0) : Kat(u, i, 0, v, j, 0));
          }
        R[d * n2 + ij] = s;
      }
    }
    else
    {
      // the other two directions e1 < e2: contract e1 into T[i, u2, j, v2], then e2
      const int e1 = d == 0 ? 1 : 0, e2 = d == 2 ? 1 : 2;
      const double *M1 = M + e1 * n2, *M2 = M + e2 * n2;
      for(int idx = threadIdx.x; idx < n2 * n2; idx += blockDim.x)
      {
        const int i = idx / (n * n2), u2 = (idx / n2) % n, j = (idx / n) % n, v2 = idx % n;
        double s = 0.0;
        for(int u1 = 0; u1 < n; ++u1)
          for(int v1 = 0; v1 < n; ++v1)
          {
            int r[3], c[3];
            r[d] = i;
            c[d] = j;
            r[e1] = u1;
            c[e1] = v1;
            r[e2] = u2;
            c[e2] = v2;
            s += M1[u1 * n + v1] * Kat(r[0], r[1], r[2], c[0], c[1], c[2]);
          }
        T[idx] = s;
      }
      __syncthreads();
      for(int ij = threadIdx.x; ij < n2; ij += blockDim.x)
      {
        const int i = ij / n, j = ij % n;
        double s = 0.0;
        for(int u2 = 0; u2 < n; ++u2)
          for(int v2 = 0; v2 < n; ++v2) s += M2[u2 * n + v2] * T[((i * n + u2) * n + j) * n + v2];
        R[d * n2 + ij] = s;
      }
      __syncthreads();
    }
  }
  __syncthreads();
  if(threadIdx.x == 0)
  {
    // S = <R_0, M_0>, mu_e = ||M_e||^2
    double S = 0.0, mu[3] = {1.0, 1.0, 1.0}, prod = 1.0;
    for(int i = 0; i < n2; ++i) S += R[i] * M[i];
    for(int d = 0; d < dim; ++d)
    {
      double t = 0.0;
      for(int i = 0; i < n2; ++i) t += M[d * n2 + i] * M[d * n2 + i];
      mu[d] = t;
      prod *= t;
    }
    T[0] = S;
    for(int d = 0; d < dim; ++d) T[1 + d] = mu[d];
    T[4] = prod;
  }
  __syncthreads();
  const double S = T[0], prod = T[4];
  for(int idx = threadIdx.x; idx < dim * n2; idx += blockDim.x)
  {
    const int d = idx / n2, ij = idx % n2, i = ij / n, j = ij % n;
    const double cd = prod / T[1 + d];
    // symmetric part of the fit
    const double rij = 0.5 * (R[d * n2 + i * n + j] + R[d * n2 + j * n + i]);
    a.A[pp * dim * n2 + idx] = rij / cd - double(dim - 1) / dim * S / prod * M[idx];
  }
}

LocalMap local_map(const tpss_layout &L)
{
  LocalMap m;
  m.dim = L.dim;
  m.np = L.np;
  m.n = L.n;
  m.nloc = L.nloc;
  m.npc = L.npc;
  m.ncp = L.ncp;
  return m;
}

// patches per extraction batch: at most ~1 GiB of patch matrices
int64_t batch_patches(const tpss_layout &L)
{
  const int64_t per = (int64_t)L.nloc * L.nloc * (int64_t)sizeof(double);
  int64_t b = ((int64_t)1 << 30) / per;
  if(b < 1) b = 1;
  if(b > 65535) b = 65535;  // the extraction grid's y extent
  return b < L.P ? b : L.P;
}

void extract_batch(const tpss_layout &L, const tpss_operator &op, int64_t p0, int64_t count,
                   const DeviceBuffer<int32_t> &lower, double *out)
{
  ExtractArgs a;
  a.m = local_map(L);
  a.lower = lower.ptr;
  for(int d = 0; d < 3; ++d) a.nc[d] = L.nc[d];
  a.vals = op.mapped->vals.ptr;
  a.nd = op.mapped->nd;
  a.nb = op.mapped->nb;
  a.p0 = p0;
  a.count = count;
  a.out = out;
  const int64_t nn = (int64_t)L.nloc * L.nloc;
  const int gx = (int)std::min<int64_t>((nn + 255) / 256, 64);
  dim3 grid(gx, (unsigned)count);
  extract_kernel<<<grid, 256>>>(a);
  TPSS_CUDA(cudaGetLastError());
}
}  // namespace

void check_exact_local(const tpss_layout &L, const tpss_operator *op)
{
  TPSS_REQUIRE(op && op->layout == &L, "exact local matrices need the level operator of this layout");
  TPSS_REQUIRE(op->mapped != nullptr,
               "exact local matrices are taken from a mapped level operator (give vertex_coords)");
  TPSS_REQUIRE(L.patch_variant == TPSS_PATCH_VERTEX, "exact local matrices: vertex patches only");
}

void build_dense_inverses(const tpss_layout &L, const tpss_operator &op, bool fp32,
                          DeviceBuffer<double> &inv64, DeviceBuffer<float> &inv32)
{
  check_exact_local(L, &op);
  TPSS_REQUIRE(L.nloc <= 160, "dense local inverses are limited to patches of at most 160 DoFs");
  const int64_t nn = (int64_t)L.nloc * L.nloc;
  if(fp32)
    inv32.resize((size_t)(L.P * nn));
  else
    inv64.resize((size_t)(L.P * nn));
  DeviceBuffer<int32_t> lower;
  lower.upload(L.lower.data(), L.lower.size());
  const int64_t B = batch_patches(L);
  DeviceBuffer<double> K((size_t)(B * nn));
  DeviceBuffer<int> bad(1);
  TPSS_CUDA(cudaMemset(bad.ptr, 0, sizeof(int)));
  const size_t smem = sizeof(double) * nn;
  TPSS_CUDA(cudaFuncSetAttribute(gj_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  for(int64_t p0 = 0; p0 < L.P; p0 += B)
  {
    const int64_t cnt = std::min(B, L.P - p0);
    extract_batch(L, op, p0, cnt, lower, K.ptr);
    gj_inverse_kernel<<<(unsigned)cnt, 512, smem>>>(K.ptr, L.nloc, cnt, fp32 ? nullptr : inv64.ptr,
                                                   fp32 ? inv32.ptr : nullptr, p0, bad.ptr);
    TPSS_CUDA(cudaGetLastError());
  }
  int h = 0;
  TPSS_CUDA(cudaMemcpy(&h, bad.ptr, sizeof(int), cudaMemcpyDeviceToHost));
  if(h) fail(TPSS_ERR_INVALID_ARGUMENT, "a local patch matrix is not positive definite");
}

void dense_apply_color(const tpss_layout &L, const void *inv, bool fp32, int color, double omega,
                       double *dst, const double *src, cudaStream_t s)
{
  const int64_t b = L.color_start[color], e = L.color_start[color + 1];
  if(e <= b) return;
  DenseArgs a;
  a.m = local_map(L);
  a.src = src;
  a.dst = dst;
  a.patch_first = L.d_patch_first.ptr + b * L.npc;
  a.inv = inv;
  a.p_begin = b;
  a.n_patches = e - b;
  a.omega = omega;
  const int64_t cap = (int64_t)num_sms() * 8;
  const unsigned grid = (unsigned)std::min<int64_t>(a.n_patches, cap);
  if(fp32)
    dense_apply_kernel<float><<<grid, 256, sizeof(float) * L.nloc, s>>>(a);
  else
    dense_apply_kernel<double><<<grid, 256, sizeof(double) * L.nloc, s>>>(a);
  TPSS_CUDA(cudaGetLastError());
}

std::vector<double> ksum_fit(const tpss_layout &L, const tpss_operator &op, const std::vector<double> &Ms)
{
  check_exact_local(L, &op);
  const int n = L.n, n2 = n * n, dim = L.dim;
  TPSS_REQUIRE(n <= 16, "Kronecker-sum fit: 1-D patch size at most 16");
  const int64_t nn = (int64_t)L.nloc * L.nloc;
  DeviceBuffer<int32_t> lower;
  lower.upload(L.lower.data(), L.lower.size());
  const int64_t B = batch_patches(L);
  DeviceBuffer<double> K((size_t)(B * nn)), dM((size_t)(B * dim * n2)), dA((size_t)(B * dim * n2));
  std::vector<double> out((size_t)L.P * dim * n2);
  const size_t smem = sizeof(double) * ((size_t)dim * n2 + (size_t)n2 * n2 + (size_t)dim * n2 + 8);
  TPSS_REQUIRE(smem <= 220 * 1024, "Kronecker-sum fit: patch too large");
  TPSS_CUDA(cudaFuncSetAttribute(ksum_fit_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  for(int64_t p0 = 0; p0 < L.P; p0 += B)
  {
    const int64_t cnt = std::min(B, L.P - p0);
    extract_batch(L, op, p0, cnt, lower, K.ptr);
    TPSS_CUDA(cudaMemcpy(dM.ptr, &Ms[(size_t)p0 * dim * n2], sizeof(double) * cnt * dim * n2,
                         cudaMemcpyHostToDevice));
    FitArgs a;
    a.dim = dim;
    a.n = n;
    a.K = K.ptr;
    a.M = dM.ptr;
    a.A = dA.ptr;
    a.count = cnt;
    ksum_fit_kernel<<<(unsigned)cnt, 256, smem>>>(a);
    TPSS_CUDA(cudaGetLastError());
    TPSS_CUDA(cudaMemcpy(&out[(size_t)p0 * dim * n2], dA.ptr, sizeof(double) * cnt * dim * n2,
                         cudaMemcpyDeviceToHost));
  }
  return out;
}

void extract_local_matrices(const tpss_layout &L, const tpss_operator &op, int64_t p0, int64_t count,
                            double *out_dev)
{
  check_exact_local(L, &op);
  TPSS_REQUIRE(p0 >= 0 && count >= 0 && p0 + count <= L.P, "patch range out of bounds");
  DeviceBuffer<int32_t> lower;
  lower.upload(L.lower.data(), L.lower.size());
  if(count) extract_batch(L, op, p0, count, lower, out_dev);
}
}  // namespace tpss

using namespace tpss;

extern "C" int tpss_local_matrices(const tpss_layout *layout, const tpss_operator *op, int64_t first,
                                   int64_t count, double *out)
{
  return guarded([&] {
    TPSS_REQUIRE(layout && op && out, "null argument");
    extract_local_matrices(*layout, *op, first, count, out);
    TPSS_CUDA(cudaDeviceSynchronize());
  });
}
