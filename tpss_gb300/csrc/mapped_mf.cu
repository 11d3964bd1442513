// mapped_mf.cu -- SIPG operator of a multilinear (distorted) level with matrix-free face couplings.
//
// y_c = A_cc x_c + sum over the interior faces f of cell c of A_(c, n(f)) x_n(f). The cell block
// A_cc (cell integral and the cell's own face terms) is the assembled diagonal block of mapped.cu;
// the couplings to the face neighbours are applied without their blocks, by sum factorization on
// the face (the evaluation that deal.II's FEFaceEvaluation does for the reference's matrix-free
// operator, apps/laplace_integrator.h:613-743):
//   trace of the neighbour at the shared face points: u+ and its reference gradient, contracted
//   direction by direction from its (k+1)^d values; normal derivative d_n u+ = grad u+ . J_nb^-1 n;
//   test on the cell: y_i += sum_q w_q [ (-sigma u+ - d_n u+ / 2) phi_i + (u+ / 2) d_n phi_i ],
// which is the product with the assembled coupling block -sigma [phi_i psi_j] - {d_n psi_j} phi_i
// + [psi_j] {d_n phi_i} of mapped.cu term by term. Per 3D DGQ3 cell ~10 k FP64 FMAs against
// 28.7 k for the seven dense blocks, and 32 KB of blocks read instead of 224 KB.
#include <mutex>

#include "internal.h"
#include "mapped_tab.cuh"

namespace tpss
{
namespace
{
__host__ __device__ constexpr int ipow_c(int b, int e) { return e == 0 ? 1 : b * ipow_c(b, e - 1); }

// T: arithmetic of the product (double: the level operator; float: the single-precision V-cycle,
// on FP32 copies of the cell blocks, the face geometry and the source). The result is FP64.
template<typename T>
struct MfArgs
{
  const T *vals;               // cell block of cell c at c * self_stride, entry (i, j) at j nd + i
  int64_t self_stride;
  const int32_t *col;          // face neighbour of slot 1 + f, -1 at the boundary
  const T *fgeo;               // face geometry records
  const int64_t *cell_start;   // null: lexicographic cell blocks
  const T *src;
  double *dst;
  const double *rhs;           // non-null: dst = rhs - A src
  int64_t n_cells;
  int nb, fg;
};

// the 1-D tables in the arithmetic type
template<typename T>
struct MapTabT
{
  T V[kMapMaxNp * kMapMaxNp], D[kMapMaxNp * kMapMaxNp], F[2 * kMapMaxNp], G[2 * kMapMaxNp];
};

template<typename T>
MapTabT<T> tab_as(const MapTab &t)
{
  MapTabT<T> o{};
  for(int i = 0; i < kMapMaxNp * kMapMaxNp; ++i)
  {
    o.V[i] = T(t.V[i]);
    o.D[i] = T(t.D[i]);
  }
  for(int i = 0; i < 2 * kMapMaxNp; ++i)
  {
    o.F[i] = T(t.F[i]);
    o.G[i] = T(t.G[i]);
  }
  return o;
}

template<int DIM, int NP>
struct MfShape
{
  static constexpr int ND = ipow_c(NP, DIM);      // cell DoFs
  static constexpr int NF = ipow_c(NP, DIM - 1);  // face points = tangential DoFs
  static constexpr int NFACE = 2 * DIM;
  static constexpr int WORK = NFACE * NF;
  static constexpr int THREADS = ((ND > WORK ? ND : WORK) + 31) / 32 * 32;
  // shared memory (values of the arithmetic type): cell and neighbour values, then the per-face
  // arrays
  static constexpr int OFF_X = 0;                           // (1 + NFACE) * ND
  static constexpr int OFF_T = OFF_X + (1 + NFACE) * ND;    // T0, T1
  static constexpr int OFF_P = OFF_T + 2 * WORK;            // P0V, P0D, P1V (3D)
  static constexpr int OFF_C = OFF_P + 3 * WORK;            // a, c_t1, c_t2, c_d
  static constexpr int OFF_R = OFF_C + 4 * WORK;            // R0V, R0D, R1V (3D)
  static constexpr int OFF_A = OFF_R + 3 * WORK;            // A0, A1
  static constexpr int VALUES = OFF_A + 2 * WORK;
  template<typename T>
  static constexpr size_t smem_bytes() { return sizeof(T) * VALUES + sizeof(int) * 8; }
};

template<typename T, int DIM, int NP>
__global__ void __launch_bounds__(MfShape<DIM, NP>::THREADS) mf_apply_kernel(const MfArgs<T> a, const MapTabT<T> t)
{
  using S = MfShape<DIM, NP>;
  constexpr int ND = S::ND, NF = S::NF, NFACE = S::NFACE, WORK = S::WORK, NT = S::THREADS;
  extern __shared__ __align__(16) unsigned char smraw[];
  T *smd = reinterpret_cast<T *>(smraw);
  T *xs = smd + S::OFF_X;  // [0]: the cell, [1 + f]: neighbour of face f
  T *T0 = smd + S::OFF_T, *T1 = T0 + WORK;
  T *P0V = smd + S::OFF_P, *P0D = P0V + WORK, *P1V = P0D + WORK;
  T *Ca = smd + S::OFF_C, *C1 = Ca + WORK, *C2 = C1 + WORK, *Cd = C2 + WORK;
  T *R0V = smd + S::OFF_R, *R0D = R0V + WORK, *R1V = R0D + WORK;
  T *A0 = smd + S::OFF_A, *A1 = A0 + WORK;
  int *nbr = reinterpret_cast<int *>(smd + S::VALUES);
  const int tid = threadIdx.x;
  const int64_t cell = blockIdx.x;
  if(cell >= a.n_cells) return;
  const int64_t off = a.cell_start ? a.cell_start[cell] : cell * ND;
  if(tid < NFACE) nbr[tid] = a.col[cell * a.nb + 1 + tid];
  __syncthreads();
  // the cell's and the neighbours' values
  for(int w = tid; w < (1 + NFACE) * ND; w += NT)
  {
    const int s = w / ND, j = w % ND;
    const int64_t c = s == 0 ? cell : (int64_t)nbr[s - 1];
    if(c >= 0) xs[w] = __ldg(a.src + (a.cell_start ? a.cell_start[c] : c * ND) + j);
  }
  __syncthreads();
  // tangential directions of face direction d (ascending), and the stride of a direction
  auto tang = [](int d, int k) { return k < d ? k : k + 1; };
  auto stride = [](int e) { return e == 0 ? 1 : e == 1 ? NP : NP * NP; };
  // S1: contract the normal direction of the neighbour with its face values / derivatives
  for(int w = tid; w < WORK; w += NT)
  {
    const int f = w / NF, it = w % NF, d = f / 2, s = f % 2;
    T t0 = T(0), t1 = T(0);
    if(nbr[f] >= 0)
    {
      // tangential DoF index it = i_t1 + NP i_t2 -> offset in the neighbour's values
      int base = 0, r = it;
      for(int k = 0; k < DIM - 1; ++k)
      {
        base += (r % NP) * stride(tang(d, k));
        r /= NP;
      }
      const int stride_d = stride(d);
      const T *un = xs + (1 + f) * ND;
      const int ns = 1 - s;  // the neighbour's side of the shared face
#pragma unroll
      for(int id = 0; id < NP; ++id)
      {
        const T u = un[base + id * stride_d];
        t0 = fma(t.F[ns * NP + id], u, t0);
        t1 = fma(t.G[ns * NP + id], u, t1);
      }
    }
    T0[w] = t0;
    T1[w] = t1;
  }
  __syncthreads();
  if constexpr(DIM == 3)
  {
    // S2: first tangential direction to the Gauss points, index q1 + NP i2
    for(int w = tid; w < WORK; w += NT)
    {
      const int f = w / NF, q1 = (w % NF) % NP, i2 = (w % NF) / NP;
      const T *t0 = T0 + f * NF + NP * i2, *t1 = T1 + f * NF + NP * i2;
      T pv = T(0), pd = T(0), p1 = T(0);
#pragma unroll
      for(int i1 = 0; i1 < NP; ++i1)
      {
        pv = fma(t.V[i1 * NP + q1], t0[i1], pv);
        pd = fma(t.D[i1 * NP + q1], t0[i1], pd);
        p1 = fma(t.V[i1 * NP + q1], t1[i1], p1);
      }
      P0V[w] = pv;
      P0D[w] = pd;
      P1V[w] = p1;
    }
    __syncthreads();
  }
  // S3: values and reference gradients at the face points; coefficients of the test functions
  for(int w = tid; w < WORK; w += NT)
  {
    const int f = w / NF, q = w % NF, d = f / 2;
    T ca = T(0), c1 = T(0), c2 = T(0), cd = T(0);
    if(nbr[f] >= 0)
    {
      T val = T(0), g1 = T(0), g2 = T(0), gd = T(0);
      if constexpr(DIM == 3)
      {
        const int q1 = q % NP, q2 = q / NP;
        const T *pv = P0V + f * NF + q1, *pd = P0D + f * NF + q1, *p1 = P1V + f * NF + q1;
#pragma unroll
        for(int i2 = 0; i2 < NP; ++i2)
        {
          const T v = t.V[i2 * NP + q2], dd = t.D[i2 * NP + q2];
          val = fma(v, pv[NP * i2], val);
          g1 = fma(v, pd[NP * i2], g1);
          g2 = fma(dd, pv[NP * i2], g2);
          gd = fma(v, p1[NP * i2], gd);
        }
      }
      else
      {
        const T *t0 = T0 + f * NF, *t1 = T1 + f * NF;
#pragma unroll
        for(int i1 = 0; i1 < NP; ++i1)
        {
          val = fma(t.V[i1 * NP + q], t0[i1], val);
          g1 = fma(t.D[i1 * NP + q], t0[i1], g1);
          gd = fma(t.V[i1 * NP + q], t1[i1], gd);
        }
      }
      const T *rec = a.fgeo + ((size_t)cell * NFACE + f) * a.fg;
      const T wq = rec[q], sigma = rec[NF * (1 + 2 * DIM)];
      const T *cnc = rec + NF + q * DIM, *cnn = rec + NF + NF * DIM + q * DIM;
      // normal derivative of the neighbour: reference gradient (d: gd, t1: g1, t2: g2) . J_nb^-1 n
      T dn = gd * cnn[d] + g1 * cnn[tang(d, 0)];
      if constexpr(DIM == 3) dn = fma(g2, cnn[tang(d, 1)], dn);
      ca = wq * (-sigma * val - T(0.5) * dn);
      const T b = T(0.5) * wq * val;
      cd = b * cnc[d];
      c1 = b * cnc[tang(d, 0)];
      if constexpr(DIM == 3) c2 = b * cnc[tang(d, 1)];
    }
    Ca[w] = ca;
    C1[w] = c1;
    C2[w] = c2;
    Cd[w] = cd;
  }
  __syncthreads();
  if constexpr(DIM == 3)
  {
    // S4: transpose of the second tangential direction, index q1 + NP i2
    for(int w = tid; w < WORK; w += NT)
    {
      const int f = w / NF, q1 = (w % NF) % NP, i2 = (w % NF) / NP;
      const T *ca = Ca + f * NF + q1, *c1 = C1 + f * NF + q1, *c2 = C2 + f * NF + q1,
                   *cd = Cd + f * NF + q1;
      T r0v = T(0), r0d = T(0), r1v = T(0);
#pragma unroll
      for(int q2 = 0; q2 < NP; ++q2)
      {
        const T v = t.V[i2 * NP + q2], dd = t.D[i2 * NP + q2];
        r0v = fma(v, ca[NP * q2], r0v);
        r0v = fma(dd, c2[NP * q2], r0v);
        r0d = fma(v, c1[NP * q2], r0d);
        r1v = fma(v, cd[NP * q2], r1v);
      }
      R0V[w] = r0v;
      R0D[w] = r0d;
      R1V[w] = r1v;
    }
    __syncthreads();
    // S5: transpose of the first tangential direction, index i1 + NP i2
    for(int w = tid; w < WORK; w += NT)
    {
      const int f = w / NF, i1 = (w % NF) % NP, i2 = (w % NF) / NP;
      const T *r0v = R0V + f * NF + NP * i2, *r0d = R0D + f * NF + NP * i2, *r1v = R1V + f * NF + NP * i2;
      T a0 = T(0), a1 = T(0);
#pragma unroll
      for(int q1 = 0; q1 < NP; ++q1)
      {
        a0 = fma(t.V[i1 * NP + q1], r0v[q1], a0);
        a0 = fma(t.D[i1 * NP + q1], r0d[q1], a0);
        a1 = fma(t.V[i1 * NP + q1], r1v[q1], a1);
      }
      A0[w] = a0;
      A1[w] = a1;
    }
  }
  else
  {
    // S5 (2D): transpose of the tangential direction
    for(int w = tid; w < WORK; w += NT)
    {
      const int f = w / NF, i1 = w % NF;
      const T *ca = Ca + f * NF, *c1 = C1 + f * NF, *cd = Cd + f * NF;
      T a0 = T(0), a1 = T(0);
#pragma unroll
      for(int q = 0; q < NP; ++q)
      {
        a0 = fma(t.V[i1 * NP + q], ca[q], a0);
        a0 = fma(t.D[i1 * NP + q], c1[q], a0);
        a1 = fma(t.V[i1 * NP + q], cd[q], a1);
      }
      A0[w] = a0;
      A1[w] = a1;
    }
  }
  __syncthreads();
  // S6: cell block times the cell's values, plus the face couplings expanded in the normal
  // direction of each face
  if(tid < ND)
  {
    const int i = tid;
    const T *blk = a.vals + cell * a.self_stride + i;
    T y = T(0);
#pragma unroll 8
    for(int j = 0; j < ND; ++j) y = fma(blk[(size_t)j * ND], xs[j], y);
    int idx[3] = {i % NP, (i / NP) % NP, DIM == 3 ? i / (NP * NP) : 0};
#pragma unroll
    for(int f = 0; f < NFACE; ++f)
    {
      if(nbr[f] < 0) continue;
      const int d = f / 2, s = f % 2;
      int it = idx[tang(d, 0)];
      if constexpr(DIM == 3) it += NP * idx[tang(d, 1)];
      y = fma(t.F[s * NP + idx[d]], A0[f * NF + it], y);
      y = fma(t.G[s * NP + idx[d]], A1[f * NF + it], y);
    }
    a.dst[off + i] = a.rhs ? a.rhs[off + i] - (double)y : (double)y;
  }
}

template<typename T, int DIM, int NP>
void launch_mf(const MfArgs<T> &a, const MapTabT<T> &t, cudaStream_t s)
{
  using S = MfShape<DIM, NP>;
  constexpr size_t smem = S::template smem_bytes<T>();
  static std::mutex mu;
  static bool attr[64] = {false};
  int dev = 0;
  TPSS_CUDA(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> lock(mu);
    if(smem > 48 * 1024 && dev >= 0 && dev < 64 && !attr[dev])
    {
      TPSS_CUDA(cudaFuncSetAttribute(mf_apply_kernel<T, DIM, NP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
      attr[dev] = true;
    }
  }
  mf_apply_kernel<T, DIM, NP><<<(unsigned)a.n_cells, S::THREADS, smem, s>>>(a, t);
  TPSS_CUDA(cudaGetLastError());
}

template<typename T, int DIM>
bool dispatch_np(int np, const MfArgs<T> &a, const MapTabT<T> &t, cudaStream_t s)
{
  switch(np)
  {
  case 2: launch_mf<T, DIM, 2>(a, t, s); return true;
  case 3: launch_mf<T, DIM, 3>(a, t, s); return true;
  case 4: launch_mf<T, DIM, 4>(a, t, s); return true;
  case 5: launch_mf<T, DIM, 5>(a, t, s); return true;
  case 6: launch_mf<T, DIM, 6>(a, t, s); return true;
  case 7: launch_mf<T, DIM, 7>(a, t, s); return true;
  case 8: launch_mf<T, DIM, 8>(a, t, s); return true;
  default: return false;
  }
}

// 1-D tables per degree, in both arithmetic types, built once
template<typename T>
const MapTabT<T> &tables(int k)
{
  static std::mutex mu;
  static MapTabT<T> tabs[kMapMaxNp + 1];
  static bool have[kMapMaxNp + 1] = {false};
  std::lock_guard<std::mutex> lock(mu);
  if(!have[k + 1])
  {
    tabs[k + 1] = tab_as<T>(make_tab(k));
    have[k + 1] = true;
  }
  return tabs[k + 1];
}

template<typename T>
bool launch(const tpss_layout &L, const MfArgs<T> &a, cudaStream_t s)
{
  if(L.np < 2 || L.np > kMapMaxNp) return false;
  const MapTabT<T> &t = tables<T>(L.k);
  return L.dim == 2 ? dispatch_np<T, 2>(L.np, a, t, s) : L.dim == 3 ? dispatch_np<T, 3>(L.np, a, t, s) : false;
}

__global__ void mf_d2f_kernel(int64_t n, const double *__restrict__ x, float *__restrict__ y)
{
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = float(x[i]);
}

// FP32 copies of the cell blocks (compact: nd x nd per cell) and of the face geometry
__global__ void mf_self32_kernel(int64_t n_cells, int nb, int nd2, const double *__restrict__ vals,
                                 float *__restrict__ out)
{
  const int64_t n = n_cells * nd2;
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
  {
    const int64_t c = i / nd2, e = i % nd2;
    out[i] = float(vals[c * nb * nd2 + e]);
  }
}

int grid_of(int64_t n)
{
  const int64_t b = (n + 255) / 256, cap = (int64_t)num_sms() * 8;
  return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}
}  // namespace

bool mapped_apply_mf(const tpss_operator &op, double *dst, const double *src, cudaStream_t s, const double *rhs)
{
  const tpss_layout &L = *op.layout;
  const MappedOperator &M = *op.mapped;
  if(M.fgeo.n == 0) return false;
  MfArgs<double> a;
  a.vals = M.vals.ptr;
  a.self_stride = (int64_t)M.nb * M.nd * M.nd;
  a.col = M.col.ptr;
  a.fgeo = M.fgeo.ptr;
  a.cell_start = L.lexicographic ? nullptr : L.d_cell_start.ptr;
  a.src = src;
  a.dst = dst;
  a.rhs = rhs;
  a.n_cells = M.n_cells;
  a.nb = M.nb;
  a.fg = M.fg;
  return launch<double>(L, a, s);
}

bool mapped_apply_mf_f32(tpss_operator &op, double *dst, const double *src, cudaStream_t s, const double *rhs)
{
  const tpss_layout &L = *op.layout;
  MappedOperator &M = *op.mapped;
  if(M.fgeo.n == 0 || L.np < 2 || L.np > kMapMaxNp) return false;
  const int64_t nd2 = (int64_t)M.nd * M.nd;
  if(M.self32.n != (size_t)(M.n_cells * nd2))
  {
    // FP32 copies made on first use (the single-precision V-cycle's level operator)
    M.self32.resize(M.n_cells * nd2);
    mf_self32_kernel<<<grid_of(M.n_cells * nd2), 256, 0, s>>>(M.n_cells, M.nb, (int)nd2, M.vals.ptr,
                                                                M.self32.ptr);
    TPSS_CUDA(cudaGetLastError());
    M.fgeo32.resize(M.fgeo.n);
    mf_d2f_kernel<<<grid_of((int64_t)M.fgeo.n), 256, 0, s>>>((int64_t)M.fgeo.n, M.fgeo.ptr, M.fgeo32.ptr);
    TPSS_CUDA(cudaGetLastError());
  }
  const int64_t n = L.n_dofs;
  if(op.x32.n < (size_t)n) op.x32.resize(n);
  mf_d2f_kernel<<<grid_of(n), 256, 0, s>>>(n, src, op.x32.ptr);
  TPSS_CUDA(cudaGetLastError());
  MfArgs<float> a;
  a.vals = M.self32.ptr;
  a.self_stride = nd2;
  a.col = M.col.ptr;
  a.fgeo = M.fgeo32.ptr;
  a.cell_start = L.lexicographic ? nullptr : L.d_cell_start.ptr;
  a.src = op.x32.ptr;
  a.dst = dst;
  a.rhs = rhs;
  a.n_cells = M.n_cells;
  a.nb = M.nb;
  a.fg = M.fg;
  return launch<float>(L, a, s);
}
}  // namespace tpss
