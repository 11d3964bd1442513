// operator.cu -- FP64 matrix-free SIPG operator, DG level transfer and vector kernels.
//
// Operator: MF::Operator::vmult (apps/laplace_integrator.h:578-743) on a Cartesian level.
// With Gauss quadrature of k+1 points per direction the cell and face integrals are exact,
// and on a tensor-product (Cartesian) mesh the SIPG bilinear form is the Kronecker sum
//   A = sum_d M_{dim-1} x .. x A_d x .. x M_0
// of global 1-D operators: block-diagonal cell mass matrices M_e and block-tridiagonal 1-D
// SIPG matrices A_d (cell Laplace, Dirichlet boundary faces with sigma = 2 ip gamma / h,
// interior faces with sigma = ip gamma (1/h_l + 1/h_r)/2, gamma = k(k+1);
// apps/common_integrator.h:30-37).  Each output cell therefore gathers 3*dim neighbour terms
// (left, self, right per direction), each a dim-fold sum-factorized contraction.
//
// Transfer: MGTransferMatrixFree for FE_DGQ -- prolongation embeds the coarse polynomial in
// the 2^dim children (1-D embedding matrices E_0, E_1), restriction is its transpose.
#include <mutex>

#include <map>

#include "internal.h"

namespace tpss
{
namespace
{
__host__ __device__ constexpr int cpow(int b, int e) { return e == 0 ? 1 : b * cpow(b, e - 1); }

// T: arithmetic, shared-memory and source type (double; float for the single-precision level
// operator, whose source is a pre-converted FP32 copy). The result is stored in FP64.
template<typename T>
struct OpArgs
{
  const T *__restrict__ src;
  double *__restrict__ dst;
  const int64_t *__restrict__ cell_start;  // nullptr = lexicographic
  const T *__restrict__ fac[3];            // operator_factors_1d per direction
  int nc[3];
  int64_t n_cells;
  bool sparse_faces;                   // face couplings have unit value vectors (xdir)
  const double *__restrict__ rhs;      // non-null: dst = rhs - A src (the residual)
};

template<int DIM, int NP>
struct OpCfg
{
  static constexpr int ND = cpow(NP, DIM);
  static constexpr int NPENC = ND / NP;
  static constexpr int CPB = NPENC >= 128 ? 1 : 128 / NPENC;  // cells per block
  static constexpr int THREADS = ((CPB * NPENC + 31) / 32) * 32;
  // factors per cell and direction: mass (NP^2), own block (NP^2), couplings (8 NP), then the
  // even/odd form of the (mirror-symmetric) mass used from NP >= 5 (MassEo)
  static constexpr int FS0 = 2 * NP * NP + 8 * NP;
  static constexpr int FS = FS0 + 2 * (NP / 2) * (NP / 2) + 2 * (NP / 2) + 1;
};

// Kronecker-sum application per direction d:
//   X_d = C_d u_c + sum_{r<2} aR_r (bR_r . u_{c+e_d}) + sum_{r<2} aL_r (bL_r . u_{c-e_d})   (along d)
//   out += (mass along the other directions) X_d
// The neighbour couplings are rank two, so a neighbour costs two dot products per pencil
// instead of a full n x n contraction.
// X_d of one pencil along d (the cell's own 1-D block and the rank-2 couplings to the two
// neighbours along d) written to buf. SPARSE: the couplings' value vectors are unit vectors at the
// shared face node (nodal basis with a node on each face, as FE_DGQ on Gauss-Lobatto points):
// aL = aL[0] e_0, bL[n..2n) = c e_(n-1), aR = aR[n-1] e_(n-1), bR[n..2n) = c e_0, which saves
// 2 n - 2 multiply-adds per neighbour and pencil.
template<int DIM, int NP, int D, bool SPARSE, typename T>
__device__ __forceinline__ void xdir(const OpArgs<T> &a, const T *fac, const int64_t *first, int p, T *buf)
{
  constexpr int FS = OpCfg<DIM, NP>::FS;
  constexpr int stride = D == 0 ? 1 : D == 1 ? NP : NP * NP;
  const int base = (p % stride) + (p / stride) * stride * NP;
  const T *F = fac + D * FS;
  const T *Cm = F + NP * NP, *aL = F + 2 * NP * NP, *bL = aL + 2 * NP, *aR = bL + 2 * NP, *bR = aR + 2 * NP;
  T u[NP], x[NP];
  const T *uc = a.src + first[1] + base;
#pragma unroll
  for(int m = 0; m < NP; ++m) u[m] = uc[m * stride];
#pragma unroll
  for(int i = 0; i < NP; ++i)
  {
    T acc = T(0);
#pragma unroll
    for(int m = 0; m < NP; ++m) acc = fma(Cm[i * NP + m], u[m], acc);
    x[i] = acc;
  }
#pragma unroll
  for(int side = 0; side < 2; ++side)
  {
    const int64_t f = first[side == 0 ? 0 : 2];
    if(f < 0) continue;
    const T *an = side == 0 ? aL : aR, *bn = side == 0 ? bL : bR;
    const T *un = a.src + f + base;
    if constexpr(SPARSE)
    {
      const int jn = side == 0 ? NP - 1 : 0;  // neighbour's node on the shared face
      const int jc = side == 0 ? 0 : NP - 1;  // own node on the shared face
      T v[NP];
#pragma unroll
      for(int m = 0; m < NP; ++m) v[m] = un[m * stride];
      T t0 = T(0);
#pragma unroll
      for(int m = 0; m < NP; ++m) t0 = fma(bn[m], v[m], t0);
      const T t1 = bn[NP + jn] * v[jn];
#pragma unroll
      for(int i = 0; i < NP; ++i) x[i] = fma(an[NP + i], t1, x[i]);
      x[jc] = fma(an[jc], t0, x[jc]);
    }
    else
    {
      T t0 = T(0), t1 = T(0);
#pragma unroll
      for(int m = 0; m < NP; ++m)
      {
        const T v = un[m * stride];
        t0 = fma(bn[m], v, t0);
        t1 = fma(bn[NP + m], v, t1);
      }
#pragma unroll
      for(int i = 0; i < NP; ++i) x[i] = fma(an[i], t0, fma(an[NP + i], t1, x[i]));
    }
  }
#pragma unroll
  for(int i = 0; i < NP; ++i) buf[base + i * stride] = x[i];
}

enum MassMode
{
  MASS_WRITE,
  MASS_ADD
};

// Even/odd form of a mirror-symmetric n x n matrix M (M[n-1-i][n-1-j] = M[i][j]), h = n/2, middle
// node m = h for odd n: y_i = A_i + B_i, y_(n-1-i) = A_i - B_i (i < h) with
//   A_i = sum_j Pe[i][j] (r_j + r_(n-1-j)) + Pm[i] r_m,  B_i = sum_j Po[i][j] (r_j - r_(n-1-j)),
//   Pe/Po[i][j] = (M[i][j] +/- M[i][n-1-j]) / 2, Pm[i] = M[i][m], and for odd n
//   y_m = sum_j Mm[j] (r_j + r_(n-1-j)) + Mmm r_m.  Layout: [Pe h*h][Po h*h][Pm h][Mm h][Mmm].
// 2 h^2 + 2 h + 1 multiply-adds and 4 h additions instead of n^2 (21 vs 25 for n = 5, 48 vs 64
// for n = 8); used from n = 5 on.
template<int NP>
struct MassEo
{
  enum : int
  {
    H = NP / 2,
    PE = 0,
    PO = H * H,
    PM = 2 * H * H,
    MM = PM + H,
    MMM = MM + H
  };
  static constexpr bool USE = NP >= 5;
};

// out = (mass along E) in, one pencil along E (out may be in, pencil by pencil); F is the cell's
// factor block of that direction
template<int NP, int E, int MODE, typename T>
__device__ __forceinline__ void mass_pass(const T *F, const T *in, T *out, int p)
{
  constexpr int stride = E == 0 ? 1 : E == 1 ? NP : NP * NP;
  const int base = (p % stride) + (p / stride) * stride * NP;
  T r[NP], y[NP];
#pragma unroll
  for(int m = 0; m < NP; ++m) r[m] = in[base + m * stride];
  if constexpr(MassEo<NP>::USE)
  {
    using X = MassEo<NP>;
    constexpr int H = X::H;
    const T *Q = F + 2 * NP * NP + 8 * NP;
    T e[H], o[H];
#pragma unroll
    for(int j = 0; j < H; ++j)
    {
      e[j] = r[j] + r[NP - 1 - j];
      o[j] = r[j] - r[NP - 1 - j];
    }
#pragma unroll
    for(int i = 0; i < H; ++i)
    {
      T a = T(0), b = T(0);
#pragma unroll
      for(int j = 0; j < H; ++j)
      {
        a = fma(Q[X::PE + i * H + j], e[j], a);
        b = fma(Q[X::PO + i * H + j], o[j], b);
      }
      if constexpr(NP % 2 == 1) a = fma(Q[X::PM + i], r[H], a);
      y[i] = a + b;
      y[NP - 1 - i] = a - b;
    }
    if constexpr(NP % 2 == 1)
    {
      T c = Q[X::MMM] * r[H];
#pragma unroll
      for(int j = 0; j < H; ++j) c = fma(Q[X::MM + j], e[j], c);
      y[H] = c;
    }
  }
  else
  {
#pragma unroll
    for(int i = 0; i < NP; ++i)
    {
      T acc = T(0);
#pragma unroll
      for(int m = 0; m < NP; ++m) acc = fma(F[i * NP + m], r[m], acc);
      y[i] = acc;
    }
  }
#pragma unroll
  for(int i = 0; i < NP; ++i)
  {
    if(MODE == MASS_ADD)
      out[base + i * stride] += y[i];
    else
      out[base + i * stride] = y[i];
  }
}

template<int DIM, int NP, typename T, bool SPARSE>
__global__ void __launch_bounds__(OpCfg<DIM, NP>::THREADS) sipg_kernel(OpArgs<T> a)
{
  using C = OpCfg<DIM, NP>;
  constexpr int ND = C::ND, CPB = C::CPB, NPENC = C::NPENC, FS = C::FS;
  __shared__ T s_x[CPB * ND];
  __shared__ T s_y[CPB * ND];
  __shared__ T s_out[CPB * ND];
  __shared__ T s_fac[CPB * DIM * FS];
  __shared__ int64_t s_first[CPB][3][3];  // [cell][direction][left, self, right]
  __shared__ int s_cc[CPB][3];             // cell coordinates
  const int tid = threadIdx.x, slot = tid / NPENC, p = tid % NPENC;
  for(int64_t c0 = (int64_t)blockIdx.x * CPB; c0 < a.n_cells; c0 += (int64_t)gridDim.x * CPB)
  {
    __syncthreads();
    // cell coordinates of the block's cells (one 64-bit division per cell, not per element)
    if(tid < CPB)
    {
      const int64_t cell = c0 + tid;
      s_cc[tid][0] = (int)(cell % a.nc[0]);
      s_cc[tid][1] = (int)((cell / a.nc[0]) % a.nc[1]);
      s_cc[tid][2] = (int)(cell / ((int64_t)a.nc[0] * a.nc[1]));
    }
    __syncthreads();
    for(int i = tid; i < CPB * DIM * FS; i += C::THREADS)
    {
      const int s = i / (DIM * FS), d = (i / FS) % DIM, o = i % FS;
      T v = T(0);
      if(c0 + s < a.n_cells) v = a.fac[d][(size_t)s_cc[s][d] * FS + o];
      s_fac[i] = v;
    }
    for(int i3 = tid; i3 < CPB * DIM * 3; i3 += C::THREADS)
    {
      const int s = i3 / (DIM * 3), d = (i3 / 3) % DIM, o = i3 % 3 - 1;
      int64_t f = -1;
      if(c0 + s < a.n_cells)
      {
        const int cx = s_cc[s][0] + (d == 0 ? o : 0), cy = s_cc[s][1] + (d == 1 ? o : 0),
                  cz = s_cc[s][2] + (d == 2 ? o : 0);
        const int cdir = d == 0 ? cx : d == 1 ? cy : cz;
        if(cdir >= 0 && cdir < a.nc[d])
        {
          const int64_t nb = cx + (int64_t)a.nc[0] * (cy + (int64_t)a.nc[1] * cz);
          f = a.cell_start ? a.cell_start[nb] : nb * ND;
        }
      }
      s_first[s][d][o + 1] = f;
    }
    __syncthreads();
    const bool active = slot < CPB && c0 + (slot < CPB ? slot : 0) < a.n_cells;
    T *bx = s_x + slot * ND, *by = s_y + slot * ND, *bo = s_out + slot * ND;
    const T *fac = s_fac + slot * DIM * FS;
    // sum_d (masses along e != d) X_d with the masses shared between terms:
    //   2D: out = M_1 X_0 + M_0 X_1
    //   3D: out = M_2 (M_1 X_0 + M_0 X_1) + M_1 (M_0 X_2)   (5 mass passes instead of 6)
    if(active) xdir<DIM, NP, 0, SPARSE>(a, fac, s_first[slot][0], p, bx);
    __syncthreads();
    if(active) mass_pass<NP, 1, MASS_WRITE>(fac + 1 * FS, bx, DIM == 2 ? bo : by, p);
    __syncthreads();
    if(active) xdir<DIM, NP, 1, SPARSE>(a, fac, s_first[slot][1], p, bx);
    __syncthreads();
    if(active) mass_pass<NP, 0, MASS_ADD>(fac, bx, DIM == 2 ? bo : by, p);
    __syncthreads();
    if constexpr(DIM == 3)
    {
      if(active) mass_pass<NP, 2, MASS_WRITE>(fac + 2 * FS, by, bo, p);
      __syncthreads();
      if(active) xdir<DIM, NP, 2, SPARSE>(a, fac, s_first[slot][2], p, bx);
      __syncthreads();
      if(active) mass_pass<NP, 0, MASS_WRITE>(fac, bx, by, p);
      __syncthreads();
      if(active) mass_pass<NP, 1, MASS_ADD>(fac + 1 * FS, by, bo, p);
      __syncthreads();
    }
    for(int i = tid; i < CPB * ND; i += C::THREADS)
    {
      const int s = i / ND;
      const int64_t cell = c0 + s;
      if(cell < a.n_cells)
      {
        const int64_t g = s_first[s][0][1] + i % ND;
        a.dst[g] = a.rhs ? a.rhs[g] - double(s_out[i]) : double(s_out[i]);
      }
    }
  }
}

template<int DIM, int NP, typename T>
void launch_sipg_t(const OpArgs<T> &a, cudaStream_t s)
{
  using C = OpCfg<DIM, NP>;
  const int64_t blocks = (a.n_cells + C::CPB - 1) / C::CPB;
  const int64_t cap = (int64_t)num_sms() * 16;
  const int grid = (int)(blocks < cap ? blocks : cap);
  if(a.sparse_faces)
    sipg_kernel<DIM, NP, T, true><<<grid, C::THREADS, 0, s>>>(a);
  else
    sipg_kernel<DIM, NP, T, false><<<grid, C::THREADS, 0, s>>>(a);
  TPSS_CUDA(cudaGetLastError());
}

template<int DIM, int NP>
void launch_sipg(const OpArgs<double> &a, cudaStream_t s)
{
  launch_sipg_t<DIM, NP, double>(a, s);
}

template<int DIM, int NP>
void launch_sipg32(const OpArgs<float> &a, cudaStream_t s)
{
  launch_sipg_t<DIM, NP, float>(a, s);
}

// ---- transfer: one coarse cell per slot
struct TrArgs
{
  double *coarse;
  double *fine;
  const double *E;  // [2][NP*NP]
  int ncc[3];
  int64_t n_coarse;
};

// out (=, or += with ACC) (I x .. x B x .. x I) in along DIR for one pencil p, B row-major NP x NP
// (TRANS: B^T)
template<int NP, int DIR, bool TRANS, bool ACC, typename T>
__device__ __forceinline__ void pencil_io(const T *in, T *out, const T *B, int p)
{
  constexpr int stride = cpow(NP, DIR);
  const int base = (p % stride) + (p / stride) * stride * NP;
  T r[NP];
#pragma unroll
  for(int m = 0; m < NP; ++m) r[m] = in[base + m * stride];
#pragma unroll
  for(int i = 0; i < NP; ++i)
  {
    T acc = T(0);
#pragma unroll
    for(int m = 0; m < NP; ++m) acc = fma(TRANS ? B[m * NP + i] : B[i * NP + m], r[m], acc);
    if(ACC)
      out[base + i * stride] += acc;
    else
      out[base + i * stride] = acc;
  }
}

// Transfers between a coarse cell and its 2^dim children with the child embeddings E_b along
// each direction (b = the child's bit in that direction), sum-factorized depth first so that the
// contractions are shared between children: prolongation applies E_bx along x (2 passes), E_by
// along y (4) and E_bz along z (8) instead of 3 passes per child (24); restriction runs the
// transposed tree (z: 8, y: 4, x: 2), summing the children on the way up.
// T: arithmetic and shared-memory type (float for the transfers of a single-precision V-cycle:
// FP64 vectors, each value converted once on the way in and out)
template<int DIM, int NP, bool RESTRICT, typename T>
__global__ void __launch_bounds__(OpCfg<DIM, NP>::THREADS) transfer_kernel(TrArgs a)
{
  using C = OpCfg<DIM, NP>;
  constexpr int ND = C::ND, CPB = C::CPB, NPENC = C::NPENC;
  __shared__ T s_u[CPB * ND];   // coarse cell
  __shared__ T s_s[CPB * ND];   // after the x level of the tree
  __shared__ T s_t[CPB * ND];   // after the y level (3D)
  __shared__ T s_c[CPB * ND];   // one child
  __shared__ T s_E[2 * NP * NP];
  __shared__ int s_cc[CPB][3];  // coarse cell coordinates
  const int tid = threadIdx.x, slot = tid / NPENC, p = tid % NPENC;
  for(int i = tid; i < 2 * NP * NP; i += C::THREADS) s_E[i] = T(a.E[i]);
  const int nf0 = 2 * a.ncc[0], nf1 = DIM > 1 ? 2 * a.ncc[1] : 1;
  // fine cell index of child (bx, by, bz) of block cell s
  auto child = [&](int s, int bx, int by, int bz) {
    const int *c = s_cc[s];
    return (int64_t)(2 * c[0] + bx) + (int64_t)nf0 * ((2 * c[1] + by) + (int64_t)nf1 * (DIM == 3 ? 2 * c[2] + bz : 0));
  };
  for(int64_t c0 = (int64_t)blockIdx.x * CPB; c0 < a.n_coarse; c0 += (int64_t)gridDim.x * CPB)
  {
    __syncthreads();
    if(tid < CPB)
    {
      const int64_t cell = c0 + tid;
      s_cc[tid][0] = (int)(cell % a.ncc[0]);
      s_cc[tid][1] = (int)((cell / a.ncc[0]) % a.ncc[1]);
      s_cc[tid][2] = (int)(cell / ((int64_t)a.ncc[0] * a.ncc[1]));
    }
    const bool active = slot < CPB && c0 + (slot < CPB ? slot : 0) < a.n_coarse;
    T *u = s_u + slot * ND, *sx = s_s + slot * ND, *ty = s_t + slot * ND, *ch = s_c + slot * ND;
    // a child's values in s_c <-> the fine vector
    auto load_child = [&](int bx, int by, int bz) {
      for(int i = tid; i < CPB * ND; i += C::THREADS)
      {
        const int s = i / ND;
        s_c[i] = c0 + s < a.n_coarse ? T(a.fine[child(s, bx, by, bz) * ND + i % ND]) : T(0);
      }
    };
    auto add_child = [&](int bx, int by, int bz) {
      for(int i = tid; i < CPB * ND; i += C::THREADS)
      {
        const int s = i / ND;
        if(c0 + s < a.n_coarse) a.fine[child(s, bx, by, bz) * ND + i % ND] += double(s_c[i]);
      }
    };
    if constexpr(!RESTRICT)
    {
      __syncthreads();
      for(int i = tid; i < CPB * ND; i += C::THREADS)
        s_u[i] = c0 + i / ND < a.n_coarse ? T(a.coarse[(c0 + i / ND) * ND + i % ND]) : T(0);
      __syncthreads();
      for(int bx = 0; bx < 2; ++bx)
      {
        if(active) pencil_io<NP, 0, false, false>(u, sx, s_E + bx * NP * NP, p);
        __syncthreads();
        for(int by = 0; by < 2; ++by)
        {
          if constexpr(DIM == 2)
          {
            if(active) pencil_io<NP, 1, false, false>(sx, ch, s_E + by * NP * NP, p);
            __syncthreads();
            add_child(bx, by, 0);
            __syncthreads();
          }
          else
          {
            if(active) pencil_io<NP, 1, false, false>(sx, ty, s_E + by * NP * NP, p);
            __syncthreads();
            for(int bz = 0; bz < 2; ++bz)
            {
              if(active) pencil_io<NP, 2, false, false>(ty, ch, s_E + bz * NP * NP, p);
              __syncthreads();
              add_child(bx, by, bz);
              __syncthreads();
            }
          }
        }
      }
    }
    else
    {
      for(int bx = 0; bx < 2; ++bx)
      {
        for(int by = 0; by < 2; ++by)
        {
          if constexpr(DIM == 2)
          {
            __syncthreads();
            load_child(bx, by, 0);
            __syncthreads();
            if(active)
            {
              if(by == 0) pencil_io<NP, 1, true, false>(ch, sx, s_E, p);
              else pencil_io<NP, 1, true, true>(ch, sx, s_E + NP * NP, p);
            }
          }
          else
          {
            for(int bz = 0; bz < 2; ++bz)
            {
              __syncthreads();
              load_child(bx, by, bz);
              __syncthreads();
              if(active)
              {
                if(bz == 0) pencil_io<NP, 2, true, false>(ch, ty, s_E, p);
                else pencil_io<NP, 2, true, true>(ch, ty, s_E + NP * NP, p);
              }
            }
            __syncthreads();
            if(active)
            {
              if(by == 0) pencil_io<NP, 1, true, false>(ty, sx, s_E, p);
              else pencil_io<NP, 1, true, true>(ty, sx, s_E + NP * NP, p);
            }
          }
        }
        __syncthreads();
        if(active)
        {
          if(bx == 0) pencil_io<NP, 0, true, false>(sx, u, s_E, p);
          else pencil_io<NP, 0, true, true>(sx, u, s_E + NP * NP, p);
        }
      }
      __syncthreads();
      for(int i = tid; i < CPB * ND; i += C::THREADS)
      {
        const int64_t cell = c0 + i / ND;
        if(cell < a.n_coarse) a.coarse[cell * ND + i % ND] += double(s_u[i]);
      }
    }
  }
}

template<int DIM, int NP>
void launch_transfer(const TrArgs &a, bool restrict_mode, bool single, cudaStream_t s)
{
  using C = OpCfg<DIM, NP>;
  const int64_t blocks = (a.n_coarse + C::CPB - 1) / C::CPB;
  const int64_t cap = (int64_t)num_sms() * 16;
  const int grid = (int)(blocks < cap ? blocks : cap);
  if(single)
  {
    if(restrict_mode)
      transfer_kernel<DIM, NP, true, float><<<grid, C::THREADS, 0, s>>>(a);
    else
      transfer_kernel<DIM, NP, false, float><<<grid, C::THREADS, 0, s>>>(a);
  }
  else if(restrict_mode)
    transfer_kernel<DIM, NP, true, double><<<grid, C::THREADS, 0, s>>>(a);
  else
    transfer_kernel<DIM, NP, false, double><<<grid, C::THREADS, 0, s>>>(a);
  TPSS_CUDA(cudaGetLastError());
}

#define TPSS_DISPATCH_NP(dim, np, FN, ...)                                        \
  do                                                                              \
  {                                                                               \
    switch((dim) * 16 + (np))                                                     \
    {                                                                             \
    case 2 * 16 + 2: FN<2, 2>(__VA_ARGS__); break;                                \
    case 2 * 16 + 3: FN<2, 3>(__VA_ARGS__); break;                                \
    case 2 * 16 + 4: FN<2, 4>(__VA_ARGS__); break;                                \
    case 2 * 16 + 5: FN<2, 5>(__VA_ARGS__); break;                                \
    case 2 * 16 + 6: FN<2, 6>(__VA_ARGS__); break;                                \
    case 2 * 16 + 7: FN<2, 7>(__VA_ARGS__); break;                                \
    case 2 * 16 + 8: FN<2, 8>(__VA_ARGS__); break;                                \
    case 3 * 16 + 2: FN<3, 2>(__VA_ARGS__); break;                                \
    case 3 * 16 + 3: FN<3, 3>(__VA_ARGS__); break;                                \
    case 3 * 16 + 4: FN<3, 4>(__VA_ARGS__); break;                                \
    case 3 * 16 + 5: FN<3, 5>(__VA_ARGS__); break;                                \
    case 3 * 16 + 6: FN<3, 6>(__VA_ARGS__); break;                                \
    case 3 * 16 + 7: FN<3, 7>(__VA_ARGS__); break;                                \
    case 3 * 16 + 8: FN<3, 8>(__VA_ARGS__); break;                                \
    default: fail(TPSS_ERR_NOT_IMPLEMENTED, "unsupported (dim, degree)");         \
    }                                                                             \
  } while(0)

// ---- vector kernels
__global__ void axpby_kernel(int64_t n, double a, const double *__restrict__ x, double b,
                             double *__restrict__ y)
{
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}

__global__ void sub_kernel(int64_t n, const double *__restrict__ a, double *__restrict__ y)
{
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a[i] - y[i];
}

__global__ void d2f_kernel(int64_t n, const double *__restrict__ x, float *__restrict__ y)
{
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = float(x[i]);
}

constexpr int kDotBlocks = 1024, kDotThreads = 256;

__global__ void dot_partial_kernel(int64_t n, const double *__restrict__ x,
                                   const double *__restrict__ y, double *__restrict__ part)
{
  __shared__ double sh[kDotThreads];
  double s = 0.0;
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s = fma(x[i], y[i], s);
  sh[threadIdx.x] = s;
  __syncthreads();
  for(int w = kDotThreads / 2; w > 0; w >>= 1)
  {
    if(threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if(threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void dot_final_kernel(const double *__restrict__ part, int n, double *__restrict__ out)
{
  __shared__ double sh[kDotThreads];
  double s = 0.0;
  for(int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for(int w = kDotThreads / 2; w > 0; w >>= 1)
  {
    if(threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if(threadIdx.x == 0) *out = sh[0];
}

int vec_grid(int64_t n)
{
  const int64_t b = (n + 255) / 256, cap = (int64_t)num_sms() * 8;
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}
}  // namespace

namespace
{
template<typename T>
OpArgs<T> op_args(const tpss_operator &op, const T *src, double *dst, const double *rhs)
{
  const tpss_layout &L = *op.layout;
  OpArgs<T> a;
  a.sparse_faces = op.sparse_faces;
  a.rhs = rhs;
  a.src = src;
  a.dst = dst;
  a.cell_start = L.lexicographic ? nullptr : L.d_cell_start.ptr;
  for(int d = 0; d < 3; ++d)
  {
    if constexpr(sizeof(T) == 8)
      a.fac[d] = op.d_fac[d].ptr;
    else
      a.fac[d] = op.d_fac32[d].ptr;
    a.nc[d] = L.nc[d];
  }
  a.n_cells = L.n_cells;
  return a;
}
}  // namespace

void operator_apply(tpss_operator *op, double *dst, const double *src, cudaStream_t s, const double *rhs)
{
  const tpss_layout &L = *op->layout;
  TPSS_REQUIRE(dst && src && dst != src, "operator: invalid vectors");
  if(op->mapped)
  {
    mapped_apply(*op, dst, src, s, rhs);
    return;
  }
  const OpArgs<double> a = op_args<double>(*op, src, dst, rhs);
  TPSS_DISPATCH_NP(L.dim, L.np, launch_sipg, a, s);
}

void operator_apply_f32(tpss_operator *op, double *dst, const double *src, cudaStream_t s, const double *rhs)
{
  const tpss_layout &L = *op->layout;
  TPSS_REQUIRE(dst && src && dst != src, "operator: invalid vectors");
  if(op->mapped)
  {
    mapped_apply_f32(*op, dst, src, s, rhs);
    return;
  }
  const int64_t n = L.n_dofs;
  if(op->x32.n < (size_t)n) op->x32.resize(n);
  d2f_kernel<<<vec_grid(n), 256, 0, s>>>(n, src, op->x32.ptr);
  TPSS_CUDA(cudaGetLastError());
  const OpArgs<float> a = op_args<float>(*op, op->x32.ptr, dst, rhs);
  TPSS_DISPATCH_NP(L.dim, L.np, launch_sipg32, a, s);
}

void transfer_apply(int dim, int k, const int *ncc, const double *E_dev, bool restrict_mode,
                    double *coarse, double *fine, cudaStream_t s, bool single)
{
  TrArgs a;
  a.coarse = coarse;
  a.fine = fine;
  a.E = E_dev;
  a.n_coarse = 1;
  for(int d = 0; d < 3; ++d)
  {
    a.ncc[d] = d < dim ? ncc[d] : 1;
    a.n_coarse *= a.ncc[d];
  }
  TPSS_DISPATCH_NP(dim, k + 1, launch_transfer, a, restrict_mode, single, s);
}

void vec_axpby(int64_t n, double a, const double *x, double b, double *y, cudaStream_t s)
{
  axpby_kernel<<<vec_grid(n), 256, 0, s>>>(n, a, x, b, y);
  TPSS_CUDA(cudaGetLastError());
}

void vec_sub(int64_t n, const double *a, double *y, cudaStream_t s)
{
  sub_kernel<<<vec_grid(n), 256, 0, s>>>(n, a, y);
  TPSS_CUDA(cudaGetLastError());
}

int dot_partials() { return kDotBlocks; }

void vec_dot(int64_t n, const double *x, const double *y, double *partial, double *out,
             cudaStream_t s)
{
  // fixed grid so the summation order (and the result) does not depend on the device
  dot_partial_kernel<<<kDotBlocks, kDotThreads, 0, s>>>(n, x, y, partial);
  dot_final_kernel<<<1, kDotThreads, 0, s>>>(partial, kDotBlocks, out);
  TPSS_CUDA(cudaGetLastError());
}
}  // namespace tpss

using namespace tpss;

extern "C" int tpss_operator_create(const tpss_layout *layout, double ip_factor, tpss_operator **out)
{
  return tpss_operator_create_penalty(layout, ip_factor, TPSS_PENALTY_REFERENCE, out);
}

extern "C" int tpss_operator_create_penalty(const tpss_layout *layout, double ip_factor, int penalty_mode,
                                            tpss_operator **out)
{
  return guarded([&] {
    TPSS_REQUIRE(layout && out, "null argument");
    TPSS_REQUIRE(ip_factor > 0.0, "ip_factor must be positive");
    *out = nullptr;
    const Penalty pen = make_penalty(ip_factor, penalty_mode, layout->k);
    layout_to_device(*layout);
    auto op = std::make_unique<tpss_operator>();
    op->layout = layout;
    op->ip = ip_factor;
    op->penalty_mode = penalty_mode;
    if(!layout->coords.empty())
    {
      // distorted level: block-sparse matrix assembled by quadrature on the mapped cells
      mapped_build(*op, *layout, pen);
      *out = op.release();
      return;
    }
    const Shape1D s = make_shape_1d(layout->k);
    op->sparse_faces = true;
    for(int d = 0; d < layout->dim; ++d)
    {
      const std::vector<double> fac0 = operator_factors_1d(s, layout->nc[d], layout->h[d].data(), pen);
      // per cell: the factors, then the even/odd form of the cell mass (mass_pass)
      const int np = layout->np, q2 = np * np, fs0 = 2 * q2 + 8 * np, hh = np / 2;
      const int fs = fs0 + 2 * hh * hh + 2 * hh + 1;
      std::vector<double> fac((size_t)layout->nc[d] * fs, 0.0);
      for(int c = 0; c < layout->nc[d]; ++c)
      {
        const double *f0 = &fac0[(size_t)c * fs0];
        double *fc = &fac[(size_t)c * fs];
        std::copy(f0, f0 + fs0, fc);
        const double *M = f0;  // cell mass, row-major
        double *Q = fc + fs0;
        for(int i = 0; i < hh; ++i)
        {
          for(int j = 0; j < hh; ++j)
          {
            Q[i * hh + j] = 0.5 * (M[i * np + j] + M[i * np + np - 1 - j]);
            Q[hh * hh + i * hh + j] = 0.5 * (M[i * np + j] - M[i * np + np - 1 - j]);
          }
          if(np % 2 == 1)
          {
            Q[2 * hh * hh + i] = M[i * np + hh];
            Q[2 * hh * hh + hh + i] = M[hh * np + i];
          }
        }
        if(np % 2 == 1) Q[2 * hh * hh + 2 * hh] = M[hh * np + hh];
      }
      // unit value vectors at the shared face nodes (see xdir)
      for(int c = 0; c < layout->nc[d]; ++c)
      {
        const double *aL = &fac[(size_t)c * fs + 2 * q2], *bL = aL + 2 * np, *aR = bL + 2 * np, *bR = aR + 2 * np;
        for(int i = 0; i < np; ++i)
        {
          if(i != 0 && (aL[i] != 0.0 || bR[np + i] != 0.0)) op->sparse_faces = false;
          if(i != np - 1 && (aR[i] != 0.0 || bL[np + i] != 0.0)) op->sparse_faces = false;
        }
      }
      op->d_fac[d].upload(fac.data(), fac.size());
      const std::vector<float> fac32(fac.begin(), fac.end());
      op->d_fac32[d].upload(fac32.data(), fac32.size());
      op->nblk_cells[d] = layout->nc[d];
    }
    *out = op.release();
  });
}

extern "C" int tpss_operator_vmult(tpss_operator *op, double *dst, const double *src, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(op, "null operator");
    operator_apply(op, dst, src, as_stream(stream));
  });
}

extern "C" int tpss_operator_vmult_fp32(tpss_operator *op, double *dst, const double *src, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(op, "null operator");
    operator_apply_f32(op, dst, src, as_stream(stream));
  });
}

extern "C" void tpss_operator_destroy(tpss_operator *op) { delete op; }

namespace
{
// child-embedding table of degree k on the current device (one copy per device and degree,
// kept for the lifetime of the process)
const double *embedding_device(int k)
{
  static std::mutex mu;
  static std::map<std::pair<int, int>, double *> tables;
  int dev = 0;
  TPSS_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  double *&t = tables[{dev, k}];
  if(!t)
  {
    const Shape1D s = make_shape_1d(k);
    const std::vector<double> E = embedding_1d(s);
    double *d = nullptr;
    TPSS_CUDA(cudaMalloc(&d, E.size() * sizeof(double)));
    TPSS_CUDA(cudaMemcpy(d, E.data(), E.size() * sizeof(double), cudaMemcpyHostToDevice));
    t = d;
  }
  return t;
}
}  // namespace

namespace tpss
{
const double *embedding_table(int k) { return embedding_device(k); }
}  // namespace tpss

extern "C" int tpss_transfer_prolongate_add(int dim, int degree, const int *ncc, double *fine,
                                            const double *coarse, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(ncc && fine && coarse, "null argument");
    TPSS_REQUIRE((dim == 2 || dim == 3) && degree >= 1 && degree <= 7, "unsupported dim/degree");
    transfer_apply(dim, degree, ncc, embedding_device(degree), false, const_cast<double *>(coarse),
                   fine, as_stream(stream));
  });
}

extern "C" int tpss_transfer_restrict_add(int dim, int degree, const int *ncc, double *coarse,
                                          const double *fine, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(ncc && fine && coarse, "null argument");
    TPSS_REQUIRE((dim == 2 || dim == 3) && degree >= 1 && degree <= 7, "unsupported dim/degree");
    transfer_apply(dim, degree, ncc, embedding_device(degree), true, coarse,
                   const_cast<double *>(fine), as_stream(stream));
  });
}
