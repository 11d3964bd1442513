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

// The same Gauss-Jordan inversion for patches beyond shared memory (n_loc > 160, e.g. 512 for
// 3D DGQ3 vertex patches): one CTA per patch works in place on the patch's matrix in global
// memory (n^3 FP64 multiply-adds, setup only), then stores the inverse transposed like
// gj_inverse_kernel (out64 / out32 at patch p0 + pp; either may be null).
__global__ void __launch_bounds__(512) gj_inverse_global_kernel(double *__restrict__ A_all, int n, int64_t count,
                                                                double *out64, float *out32, int64_t p0,
                                                                int *bad)
{
  const int64_t pp = blockIdx.x;
  if(pp >= count) return;
  const int64_t nn = (int64_t)n * n;
  double *A = A_all + pp * nn;
  __shared__ double piv;
  for(int k = 0; k < n; ++k)
  {
    if(threadIdx.x == 0)
    {
      piv = A[(int64_t)k * n + k];
      if(!(piv > 0.0))
      {
        atomicOr(bad, 1);
        piv = 1.0;
      }
    }
    __syncthreads();
    const double p = piv;
    for(int j = threadIdx.x; j < n; j += blockDim.x)
      if(j != k) A[(int64_t)k * n + j] /= p;
    __syncthreads();
    // rows i != k: A[i][j] -= A[i][k] A[k][j]; a warp sweeps one row, lanes the columns
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nw = blockDim.x / 32;
    for(int i = warp; i < n; i += nw)
    {
      if(i == k) continue;
      const double aik = A[(int64_t)i * n + k];
      for(int j = lane; j < n; j += 32)
        if(j != k) A[(int64_t)i * n + j] -= aik * A[(int64_t)k * n + j];
    }
    __syncthreads();
    for(int i = threadIdx.x; i < n; i += blockDim.x)
      if(i != k) A[(int64_t)i * n + k] = -A[(int64_t)i * n + k] / p;
    if(threadIdx.x == 0) A[(int64_t)k * n + k] = 1.0 / p;
    __syncthreads();
  }
  const int64_t base = (p0 + pp) * nn;
  for(int64_t i = threadIdx.x; i < nn; i += blockDim.x)
  {
    const int r = int(i / n), c = int(i % n);
    const double v = A[(int64_t)c * n + r];
    if(out64) out64[base + i] = v;
    if(out32) out32[base + i] = float(v);
  }
}

// Dense local inverse of a fast-diagonalization solver, one CTA per (patch, column c):
// column c of S diag(1 / sum_d lambda_d) S^T with S = S_(dim-1) x .. x S_0 is
// S (D (S^T e_c)), where (S^T e_c)_t = prod_d S_d(c_d, t_d) is a product of eigenvector
// components; the outer S is applied by sum factorization. FD entries as in the kernels' FP64
// table: [S^T n x npad][S n x npad][lambda npad]. Output row-major, out[pp][t][c].
struct FdInvArgs
{
  int dim, n, nloc, npad, es;
  const double *fd;
  const int32_t *patch_fd;  // entry of patch p, direction d at p * dim + d
  const double *rcp;        // per-patch reciprocal eigenvalue combinations (P x nloc), or null:
                            // 1 / sum_d lambda_d
  int64_t p0, count;
  double *out;
};

__global__ void __launch_bounds__(512) fd_local_inverse_kernel(const FdInvArgs a)
{
  extern __shared__ double fbuf[];
  double *v = fbuf, *w = fbuf + a.nloc;
  const int64_t pp = blockIdx.y;
  const int c = blockIdx.x, n = a.n;
  if(pp >= a.count || c >= a.nloc) return;
  const int64_t p = a.p0 + pp;
  const double *E[3] = {nullptr, nullptr, nullptr};
  for(int d = 0; d < a.dim; ++d) E[d] = a.fd + (size_t)a.patch_fd[p * a.dim + d] * a.es;
  int cd[3] = {0, 0, 0};
  for(int d = 0, rem = c; d < a.dim; ++d, rem /= n) cd[d] = rem % n;
  for(int t = threadIdx.x; t < a.nloc; t += blockDim.x)
  {
    double prod = 1.0, lsum = 0.0;
    for(int d = 0, rem = t; d < a.dim; ++d, rem /= n)
    {
      const int td = rem % n;
      prod *= E[d][a.n * a.npad + cd[d] * a.npad + td];  // S_d(c_d, t_d): S rows
      lsum += E[d][2 * a.n * a.npad + td];
    }
    v[t] = a.rcp ? prod * a.rcp[p * a.nloc + t] : prod / lsum;
  }
  __syncthreads();
  int stride = 1;
  for(int d = 0; d < a.dim; ++d)
  {
    for(int t = threadIdx.x; t < a.nloc; t += blockDim.x)
    {
      const int td = (t / stride) % n, base = t - td * stride;
      const double *row = E[d] + a.n * a.npad + td * a.npad;  // S_d(t_d, m)
      double s = 0.0;
      for(int m = 0; m < n; ++m) s += row[m] * v[base + m * stride];
      w[t] = s;
    }
    __syncthreads();
    double *x = v;
    v = w;
    w = x;
    stride *= n;
  }
  for(int t = threadIdx.x; t < a.nloc; t += blockDim.x)
    a.out[pp * (int64_t)a.nloc * a.nloc + (int64_t)t * a.nloc + c] = v[t];
}

// Low Kronecker-rank approximation by alternating least squares (the CP/ALS of compute_kcp,
// kroneckersvd.h:501-585; for two factors its fixed point is the truncated SVD of the
// reshuffled matrix that compute_ksvd, kroneckersvd.h:306-402, computes by Lanczos):
//   K ~ sum_r F_{dim-1,r} x ... x F_{0,r},  F_{d,r} of size m_d x n_d,
// K of size (prod m_d) x (prod n_d) with direction 0 fastest in rows and columns. With the
// reshuffled tensor T(a_0, .., a_{dim-1}), a_d = i_d n_d + j_d, a mode-d update is
//   F_d = T_(d) (khatri-rao of the other factors) V^-1,  V = hadamard_{e != d} F_e^T F_e,
// (r x r, inverted directly for r <= 2 with a pseudo-inverse fallback), `iters` sweeps over
// d = 0 .. dim-1 from the given initial factors. One CTA per matrix; the products of the other
// modes' factors are tabulated in shared memory.
struct KcpArgs
{
  int dim, rank, iters;
  int m[3], n[3];
  const double *K;   // count * rows * cols
  double *F;         // count * sum_d rank m_d n_d (in: initial factors, out: result)
  int64_t count;
  int prod_max;      // max over d of prod_{e != d} m_e n_e
};

__global__ void __launch_bounds__(256) kcp_als_kernel(const KcpArgs a)
{
  extern __shared__ double ks[];
  const int64_t pp = blockIdx.x;
  if(pp >= a.count) return;
  const int dim = a.dim, R = a.rank;
  int sz[3] = {1, 1, 1}, off[3] = {0, 0, 0}, total = 0;
  for(int d = 0; d < dim; ++d)
  {
    sz[d] = a.m[d] * a.n[d];
    off[d] = total;
    total += R * sz[d];
  }
  int rows = 1, cols = 1;
  for(int d = 0; d < dim; ++d)
  {
    rows *= a.m[d];
    cols *= a.n[d];
  }
  const double *K = a.K + pp * (int64_t)rows * cols;
  double *F = ks;                     // total
  double *Pt = F + total;             // prod_max * R
  double *V = Pt + (size_t)a.prod_max * R;  // R * R and its inverse
  double *Vi = V + 16;
  for(int i = threadIdx.x; i < total; i += blockDim.x) F[i] = a.F[pp * total + i];
  __syncthreads();
  for(int it = 0; it < a.iters; ++it)
    for(int d = 0; d < dim; ++d)
    {
      // other modes e1 (< e2) and the product table Pt[(ae1 + sz[e1] ae2) R + r]
      int e[2] = {-1, -1}, ne = 0;
      for(int x = 0; x < dim; ++x)
        if(x != d) e[ne++] = x;
      const int s1 = sz[e[0]], s2 = ne > 1 ? sz[e[1]] : 1;
      for(int idx = threadIdx.x; idx < s1 * s2 * R; idx += blockDim.x)
      {
        const int r = idx % R, q = idx / R, a1 = q % s1, a2 = q / s1;
        double v = F[off[e[0]] + r * s1 + a1];
        if(ne > 1) v *= F[off[e[1]] + r * s2 + a2];
        Pt[idx] = v;
      }
      if(threadIdx.x < R * R)
      {
        const int r1 = threadIdx.x / R, r2 = threadIdx.x % R;
        double h = 1.0;
        for(int x = 0; x < ne; ++x)
        {
          double g = 0.0;
          for(int i = 0; i < sz[e[x]]; ++i) g += F[off[e[x]] + r1 * sz[e[x]] + i] * F[off[e[x]] + r2 * sz[e[x]] + i];
          h *= g;
        }
        V[threadIdx.x] = h;
      }
      __syncthreads();
      if(threadIdx.x == 0)
      {
        // inverse of V (R <= 2 directly; singular or larger: diagonal pseudo-inverse)
        if(R == 1)
          Vi[0] = V[0] != 0.0 ? 1.0 / V[0] : 0.0;
        else if(R == 2 && fabs(V[0] * V[3] - V[1] * V[2]) > 1e-14 * fabs(V[0] * V[3]))
        {
          const double det = V[0] * V[3] - V[1] * V[2];
          Vi[0] = V[3] / det;
          Vi[1] = -V[1] / det;
          Vi[2] = -V[2] / det;
          Vi[3] = V[0] / det;
        }
        else
          for(int r1 = 0; r1 < R; ++r1)
            for(int r2 = 0; r2 < R; ++r2) Vi[r1 * R + r2] = (r1 == r2 && V[r1 * R + r1] != 0.0) ? 1.0 / V[r1 * R + r1] : 0.0;
      }
      __syncthreads();
      // G(a_d, r) = sum over the other modes of T(a) Pt; F_d = G Vi
      const int sd = sz[d];
      for(int ad = threadIdx.x; ad < sd; ad += blockDim.x)
      {
        double g[4] = {0.0, 0.0, 0.0, 0.0};
        const int id = ad / a.n[d], jd = ad % a.n[d];
        for(int q = 0; q < s1 * s2; ++q)
        {
          int ai[3], row = 0, col = 0, rs = 1, cs = 1;
          ai[d] = 0;
          ai[e[0]] = q % s1;
          if(ne > 1) ai[e[1]] = q / s1;
          for(int x = 0; x < dim; ++x)
          {
            const int i = x == d ? id : ai[x] / a.n[x], j = x == d ? jd : ai[x] % a.n[x];
            row += i * rs;
            col += j * cs;
            rs *= a.m[x];
            cs *= a.n[x];
          }
          const double t = K[(int64_t)row * cols + col];
          for(int r = 0; r < R; ++r) g[r] += t * Pt[q * R + r];
        }
        for(int r = 0; r < R; ++r)
        {
          double v = 0.0;
          for(int r2 = 0; r2 < R; ++r2) v += g[r2] * Vi[r2 * R + r];
          F[off[d] + r * sd + ad] = v;
        }
      }
      __syncthreads();
    }
  for(int i = threadIdx.x; i < total; i += blockDim.x) a.F[pp * total + i] = F[i];
}

// err[pp] = ||X_pp - Y_pp||_F / ||Y_pp||_F for count pairs of n x n matrices (one CTA each)
__global__ void __launch_bounds__(256) frob_error_kernel(const double *__restrict__ X, const double *__restrict__ Y,
                                                         int64_t nn, int64_t count, double *err)
{
  __shared__ double sd[256], sy[256];
  const int64_t pp = blockIdx.x;
  if(pp >= count) return;
  double a = 0.0, b = 0.0;
  for(int64_t i = threadIdx.x; i < nn; i += blockDim.x)
  {
    const double y = Y[pp * nn + i], d = X[pp * nn + i] - y;
    a += d * d;
    b += y * y;
  }
  sd[threadIdx.x] = a;
  sy[threadIdx.x] = b;
  __syncthreads();
  for(int s = 128; s > 0; s >>= 1)
  {
    if(threadIdx.x < s)
    {
      sd[threadIdx.x] += sd[threadIdx.x + s];
      sy[threadIdx.x] += sy[threadIdx.x + s];
    }
    __syncthreads();
  }
  if(threadIdx.x == 0) err[pp] = sqrt(sd[0] / sy[0]);
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
  TPSS_REQUIRE(L.nloc <= 4096, "dense local inverses are limited to patches of at most 4096 DoFs");
  const int64_t nn = (int64_t)L.nloc * L.nloc;
  TPSS_REQUIRE(L.P <= ((int64_t)1 << 62) / nn, "too many patch matrix entries");
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
  // up to 160 DoFs the matrix lives in shared memory; larger patches are inverted in place in
  // global memory
  const bool in_smem = L.nloc <= 160;
  const size_t smem = sizeof(double) * nn;
  if(in_smem)
    TPSS_CUDA(cudaFuncSetAttribute(gj_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  for(int64_t p0 = 0; p0 < L.P; p0 += B)
  {
    const int64_t cnt = std::min(B, L.P - p0);
    extract_batch(L, op, p0, cnt, lower, K.ptr);
    if(in_smem)
      gj_inverse_kernel<<<(unsigned)cnt, 512, smem>>>(K.ptr, L.nloc, cnt, fp32 ? nullptr : inv64.ptr,
                                                     fp32 ? inv32.ptr : nullptr, p0, bad.ptr);
    else
      gj_inverse_global_kernel<<<(unsigned)cnt, 512>>>(K.ptr, L.nloc, cnt, fp32 ? nullptr : inv64.ptr,
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

namespace
{
__global__ void transpose_copy_kernel(const double *in64, const float *in32, int n, int64_t count, double *out)
{
  const int64_t nn = (int64_t)n * n;
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count * nn; i += (int64_t)gridDim.x * blockDim.x)
  {
    const int64_t pp = i / nn, rc = i % nn, r = rc / n, c = rc % n;
    const int64_t src = pp * nn + c * n + r;
    out[i] = in64 ? in64[src] : double(in32[src]);
  }
}
}  // namespace

// Dense local inverses of patches [p0, p0 + count) as the preconditioner applies them
// (row-major, device FP64): the stored exact inverses, or S D S^T of the FD tables.
void precond_local_inverse(const tpss_precond &p, int64_t p0, int64_t count, double *out_dev)
{
  const FdTables &T = *p.tables;
  const tpss_layout &L = *T.layout;
  TPSS_REQUIRE(p0 >= 0 && count >= 0 && p0 + count <= L.P, "patch range out of bounds");
  if(count == 0) return;
  const int64_t nn = (int64_t)L.nloc * L.nloc;
  if(T.dense)
  {
    const double *in64 = T.dense64.n ? T.dense64.ptr + p0 * nn : nullptr;
    const float *in32 = T.dense64.n ? nullptr : T.dense32.ptr + p0 * nn;
    transpose_copy_kernel<<<(unsigned)std::min<int64_t>((count * nn + 255) / 256, 65535), 256>>>(
      in64, in32, L.nloc, count, out_dev);
    TPSS_CUDA(cudaGetLastError());
    return;
  }
  TPSS_REQUIRE(L.nloc <= 4096, "local inverses: at most 4096 DoFs per patch");
  FdInvArgs a;
  a.dim = L.dim;
  a.n = L.n;
  a.nloc = L.nloc;
  a.npad = T.npad64;
  a.es = (2 * L.n + 1) * T.npad64;
  a.fd = T.fd64.ptr;
  a.patch_fd = T.own_fd.n ? T.own_fd.ptr : L.d_patch_fd.ptr;
  a.rcp = T.rcp_E < 0 ? T.rcp64.ptr : nullptr;
  const size_t smem = 2 * sizeof(double) * L.nloc;
  TPSS_CUDA(cudaFuncSetAttribute(fd_local_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  for(int64_t q = 0; q < count; q += 65535)
  {
    a.p0 = p0 + q;
    a.count = std::min<int64_t>(65535, count - q);
    a.out = out_dev + q * nn;
    fd_local_inverse_kernel<<<dim3((unsigned)L.nloc, (unsigned)a.count), 256, smem>>>(a);
    TPSS_CUDA(cudaGetLastError());
  }
}

// err[i] = ||A_j^-1 - B_j||_F / ||A_j^-1||_F for the patches j = p0 + i, A_j the exact patch
// matrix of the mapped level operator (inverted in FP64) and B_j the preconditioner's local
// inverse
void local_inverse_error(const tpss_precond &p, const tpss_operator &op, int64_t p0, int64_t count,
                         double *err_host)
{
  const tpss_layout &L = *p.tables->layout;
  check_exact_local(L, &op);
  TPSS_REQUIRE(p0 >= 0 && count >= 0 && p0 + count <= L.P, "patch range out of bounds");
  if(count == 0) return;
  const int64_t nn = (int64_t)L.nloc * L.nloc;
  const int64_t B = std::max<int64_t>(1, std::min<int64_t>(count, ((int64_t)1 << 29) / (nn * 8)));
  DeviceBuffer<int32_t> lower;
  lower.upload(L.lower.data(), L.lower.size());
  DeviceBuffer<double> K((size_t)(B * nn)), Ainv((size_t)(B * nn)), Bj((size_t)(B * nn)), err((size_t)B);
  DeviceBuffer<int> bad(1);
  TPSS_CUDA(cudaMemset(bad.ptr, 0, sizeof(int)));
  for(int64_t q = 0; q < count; q += B)
  {
    const int64_t cnt = std::min(B, count - q);
    extract_batch(L, op, p0 + q, cnt, lower, K.ptr);
    // the inverse kernels write patch p0' + pp at (p0' + pp) nn: pass p0' = 0 into Ainv
    gj_inverse_global_kernel<<<(unsigned)cnt, 512>>>(K.ptr, L.nloc, cnt, Ainv.ptr, nullptr, 0, bad.ptr);
    TPSS_CUDA(cudaGetLastError());
    // gj stores the inverse transposed; the inverse of a symmetric matrix is symmetric
    precond_local_inverse(p, p0 + q, cnt, Bj.ptr);
    frob_error_kernel<<<(unsigned)cnt, 256>>>(Bj.ptr, Ainv.ptr, nn, cnt, err.ptr);
    TPSS_CUDA(cudaGetLastError());
    TPSS_CUDA(cudaMemcpy(err_host + q, err.ptr, sizeof(double) * cnt, cudaMemcpyDeviceToHost));
  }
  int h = 0;
  TPSS_CUDA(cudaMemcpy(&h, bad.ptr, sizeof(int), cudaMemcpyDeviceToHost));
  if(h) fail(TPSS_ERR_INVALID_ARGUMENT, "a local patch matrix is not positive definite");
}
}  // namespace tpss

namespace tpss
{
void kcp_als(int dim, const int *m, const int *n, int rank, int iters, const double *K_dev, int64_t count,
             double *F_dev, cudaStream_t s)
{
  TPSS_REQUIRE(dim >= 2 && dim <= 3, "Kronecker approximation: 2 or 3 factors");
  TPSS_REQUIRE(rank >= 1 && rank <= 4, "Kronecker approximation: rank 1..4");
  TPSS_REQUIRE(iters >= 0, "Kronecker approximation: iterations >= 0");
  KcpArgs a;
  a.dim = dim;
  a.rank = rank;
  a.iters = iters;
  int total = 0;
  for(int d = 0; d < 3; ++d)
  {
    a.m[d] = d < dim ? m[d] : 1;
    a.n[d] = d < dim ? n[d] : 1;
    TPSS_REQUIRE(a.m[d] >= 1 && a.n[d] >= 1 && a.m[d] <= 64 && a.n[d] <= 64, "Kronecker approximation: factor size");
    if(d < dim) total += rank * a.m[d] * a.n[d];
  }
  a.prod_max = 1;
  for(int d = 0; d < dim; ++d)
  {
    int p = 1;
    for(int e = 0; e < dim; ++e)
      if(e != d) p *= a.m[e] * a.n[e];
    a.prod_max = std::max(a.prod_max, p);
  }
  const size_t smem = sizeof(double) * ((size_t)total + (size_t)a.prod_max * rank + 32);
  TPSS_REQUIRE(smem <= 200 * 1024, "Kronecker approximation: factors too large for shared memory");
  a.K = K_dev;
  a.F = F_dev;
  a.count = count;
  if(count == 0) return;
  TPSS_CUDA(cudaFuncSetAttribute(kcp_als_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kcp_als_kernel<<<(unsigned)count, 256, smem, s>>>(a);
  TPSS_CUDA(cudaGetLastError());
}

// Rank-2 Kronecker approximation of every exact patch matrix of a mapped level, initialised
// from the patch's surrogate 1-D problems: term 0 = (A_0, M_1[, M_2]), term 1 = (M_0, A_1[, M_2])
// (the Cartesian 2D patch matrix M_1 x A_0 + A_1 x M_0 is reproduced exactly); `iters` ALS
// sweeps. Returns P x dim x 2 x n^2 (direction d, term r at (p dim + d) 2 n^2 + r n^2).
std::vector<double> ksvd_fit(const tpss_layout &L, const tpss_operator &op, const std::vector<double> &Mp,
                             const std::vector<double> &Ap, int iters)
{
  check_exact_local(L, &op);
  const int n = L.n, n2 = n * n, dim = L.dim;
  const int64_t nn = (int64_t)L.nloc * L.nloc;
  DeviceBuffer<int32_t> lower;
  lower.upload(L.lower.data(), L.lower.size());
  const int64_t B = batch_patches(L);
  DeviceBuffer<double> K((size_t)(B * nn)), F((size_t)(B * dim * 2 * n2));
  // kernel layout per patch: direction d block of 2 terms (rank r at d 2 n2 + r n2)
  std::vector<double> out((size_t)L.P * dim * 2 * n2), init((size_t)B * dim * 2 * n2);
  const int mm[3] = {n, n, n};
  for(int64_t p0 = 0; p0 < L.P; p0 += B)
  {
    const int64_t cnt = std::min(B, L.P - p0);
    for(int64_t q = 0; q < cnt; ++q)
      for(int d = 0; d < dim; ++d)
        for(int r = 0; r < 2; ++r)
        {
          const bool lap = (r == 0 && d == 0) || (r == 1 && d == 1);
          const double *src = &(lap ? Ap : Mp)[((size_t)(p0 + q) * dim + d) * n2];
          std::copy(src, src + n2, &init[(((size_t)q * dim + d) * 2 + r) * n2]);
        }
    TPSS_CUDA(cudaMemcpy(F.ptr, init.data(), sizeof(double) * cnt * dim * 2 * n2, cudaMemcpyHostToDevice));
    extract_batch(L, op, p0, cnt, lower, K.ptr);
    kcp_als(dim, mm, mm, 2, iters, K.ptr, cnt, F.ptr, nullptr);
    TPSS_CUDA(cudaMemcpy(&out[(size_t)p0 * dim * 2 * n2], F.ptr, sizeof(double) * cnt * dim * 2 * n2,
                         cudaMemcpyDeviceToHost));
  }
  return out;
}
}  // namespace tpss

extern "C" int tpss_kronecker_approx(const double *mats, int64_t count, int dim, const int *m, const int *n,
                                     int rank, int iterations, double *factors, void *stream)
{
  return tpss::guarded([&] {
    TPSS_REQUIRE(mats && factors && m && n && count >= 0, "invalid argument");
    tpss::kcp_als(dim, m, n, rank, iterations, mats, count, factors, tpss::as_stream(stream));
  });
}

extern "C" int tpss_precond_local_inverse(const tpss_precond *p, int64_t first, int64_t count, double *out)
{
  return tpss::guarded([&] {
    TPSS_REQUIRE(p && out, "null argument");
    tpss::precond_local_inverse(*p, first, count, out);
    TPSS_CUDA(cudaDeviceSynchronize());
  });
}

extern "C" int tpss_local_inverse_error(const tpss_precond *p, const tpss_operator *op, int64_t first,
                                        int64_t count, double *err)
{
  return tpss::guarded([&] {
    TPSS_REQUIRE(p && op && err, "null argument");
    tpss::local_inverse_error(*p, *op, first, count, err);
  });
}

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
