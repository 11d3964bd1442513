// fd_kernels.cuh -- fused per-color Schwarz kernel: gather -> FD inverse -> damping -> scatter.
//
// One color of SchwarzPreconditioner::apply_local_solvers
// (preconditioner/schwarz_preconditioner.templates.h:585-662) for DG patches:
//   r_j = R_j src            PatchTransfer::gather (TPSS/patch_transfer.templates.h:3-23)
//   u_j = A_j^-1 r_j          TensorProductMatrixSymmetricSum::apply_inverse (deal.II),
//                            u = S Lambda^-1 S^T r with S = S_{d-1} x .. x S_0
//   u_j *= omega             (schwarz_preconditioner.templates.h:631-633)
//   dst += R_j^T u_j          PatchTransfer::scatter_add (patch_transfer.templates.h:54-116)
// Patches of one color share no cell, so the scatter is a plain read-modify-write.
//
// Mapping: a CTA holds PPC patches in shared memory (patch-local lexicographic order,
// direction 0 fastest).  Gather/scatter move whole cells: each cell's (k+1)^d DoFs are
// contiguous in the global vector, so consecutive threads touch consecutive doubles.
// The sum-factorized contractions run pencil-wise: a thread owns one 1-D pencil of a patch,
// keeps it in registers, and contracts it against the 1-D matrix held in shared memory (rows
// read as 16-byte vectors that all lanes of a warp share).  The last forward direction, the
// division by the eigenvalue sums and the first backward direction are fused in registers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace tpss
{
namespace fd
{
template<typename T>
struct VecOf;
template<>
struct VecOf<float>
{
  using type = float4;
  static constexpr int W = 4;
};
template<>
struct VecOf<double>
{
  using type = double2;
  static constexpr int W = 2;
};

__host__ __device__ constexpr int cpow(int b, int e) { return e == 0 ? 1 : b * cpow(b, e - 1); }

template<typename T, int N>
struct Pad
{
  static constexpr int W = VecOf<T>::W;
  static constexpr int value = ((N + W - 1) / W) * W;
};

// o[i] = sum_m B[i][m] r[m], B row-major N x NPAD in shared memory.
template<typename T, int N, int NPAD>
__device__ __forceinline__ void rowmat(const T *__restrict__ B, const T (&r)[N], T (&o)[N])
{
  using V = typename VecOf<T>::type;
  constexpr int W = VecOf<T>::W;
#pragma unroll
  for(int i = 0; i < N; ++i)
  {
    const V *row = reinterpret_cast<const V *>(B + i * NPAD);
    T acc = T(0);
#pragma unroll
    for(int m4 = 0; m4 < NPAD / W; ++m4)
    {
      const V v = row[m4];
      if constexpr(W == 4)
      {
        if(m4 * 4 + 0 < N) acc = fma(v.x, r[m4 * 4 + 0 < N ? m4 * 4 + 0 : 0], acc);
        if(m4 * 4 + 1 < N) acc = fma(v.y, r[m4 * 4 + 1 < N ? m4 * 4 + 1 : 0], acc);
        if(m4 * 4 + 2 < N) acc = fma(v.z, r[m4 * 4 + 2 < N ? m4 * 4 + 2 : 0], acc);
        if(m4 * 4 + 3 < N) acc = fma(v.w, r[m4 * 4 + 3 < N ? m4 * 4 + 3 : 0], acc);
      }
      else
      {
        if(m4 * 2 + 0 < N) acc = fma(v.x, r[m4 * 2 + 0 < N ? m4 * 2 + 0 : 0], acc);
        if(m4 * 2 + 1 < N) acc = fma(v.y, r[m4 * 2 + 1 < N ? m4 * 2 + 1 : 0], acc);
      }
    }
    o[i] = acc;
  }
}

// Per-entry layout of the FD table: [S^T: N x NPAD][S: N x NPAD][lambda: NPAD].
template<typename T, int N>
struct Entry
{
  static constexpr int NPAD = Pad<T, N>::value;
  static constexpr int ST = 0, S = N * NPAD, LAM = 2 * N * NPAD;
  static constexpr int size = (2 * N + 1) * NPAD;
};

// Even/odd form of a mirror-symmetric entry (n = 2h): [Se^T h x HPAD][So^T][Se][So][lambda: NPAD,
// even then odd], Se = S_even / sqrt(2) (the host builds it in precond.cu)
template<typename T, int N>
struct EoEntry
{
  static constexpr int H = N / 2;
  static constexpr int HPAD = Pad<T, (H > 0 ? H : 1)>::value;
  static constexpr int SOT = H * HPAD, SE = 2 * H * HPAD, SO = 3 * H * HPAD, LAM = 4 * H * HPAD;
  static constexpr int size = LAM + Pad<T, N>::value;
};

// h x h matrix rows (stride HPAD) times a vector: o[k] = sum_i B[k][i] v[i]
template<typename T, int H, int HPAD>
__device__ __forceinline__ T eo_row(const T *__restrict__ row, const T (&v)[H])
{
  T acc = T(0);
#pragma unroll
  for(int i = 0; i < H; ++i) acc = fma(row[i], v[i], acc);
  return acc;
}

// forward transform of one pencil: o = [Se^T (r_i + r_{n-1-i}) ; So^T (r_i - r_{n-1-i})]
template<typename T, int N>
__device__ __forceinline__ void eo_fwd(const T *__restrict__ E, const T (&r)[N], T (&o)[N])
{
  using X = EoEntry<T, N>;
  constexpr int H = X::H;
  T a[H], b[H];
#pragma unroll
  for(int i = 0; i < H; ++i)
  {
    a[i] = r[i] + r[N - 1 - i];
    b[i] = r[i] - r[N - 1 - i];
  }
#pragma unroll
  for(int k = 0; k < H; ++k)
  {
    o[k] = eo_row<T, H, X::HPAD>(E + k * X::HPAD, a);
    o[H + k] = eo_row<T, H, X::HPAD>(E + X::SOT + k * X::HPAD, b);
  }
}

// backward transform: u_i = (Se t_e)_i + (So t_o)_i, u_{n-1-i} = (Se t_e)_i - (So t_o)_i
template<typename T, int N>
__device__ __forceinline__ void eo_bwd(const T *__restrict__ E, const T (&t)[N], T (&u)[N])
{
  using X = EoEntry<T, N>;
  constexpr int H = X::H;
  T te[H], to[H];
#pragma unroll
  for(int k = 0; k < H; ++k)
  {
    te[k] = t[k];
    to[k] = t[H + k];
  }
#pragma unroll
  for(int i = 0; i < H; ++i)
  {
    const T e = eo_row<T, H, X::HPAD>(E + X::SE + i * X::HPAD, te);
    const T o = eo_row<T, H, X::HPAD>(E + X::SO + i * X::HPAD, to);
    u[i] = e + o;
    u[N - 1 - i] = e - o;
  }
}

template<typename T, int DIM, int NCP, int K1>
struct Cfg
{
  static constexpr int N = NCP * K1;
  static constexpr int NLOC = cpow(N, DIM);
  static constexpr int NPENCIL = NLOC / N;
  static constexpr int NCELL = cpow(NCP, DIM);
  static constexpr int CELLDOFS = cpow(K1, DIM);
  // a slot holds the dense entry or, for a mirror-symmetric direction, its even/odd form
  static constexpr int ESIZE = Entry<T, N>::size > EoEntry<T, N>::size ? Entry<T, N>::size : EoEntry<T, N>::size;
  // patches per CTA: enough pencils for >= 128 threads, bounded by shared memory
  static constexpr int PPC_WANT = NPENCIL >= 128 ? 1 : (128 + NPENCIL - 1) / NPENCIL;
  static constexpr int SLOT_BYTES = NLOC * sizeof(T) + DIM * ESIZE * sizeof(T) + NCELL * 12;
  static constexpr int PPC_MEM = (96 * 1024) / SLOT_BYTES > 0 ? (96 * 1024) / SLOT_BYTES : 1;
  static constexpr int PPC = PPC_WANT < PPC_MEM ? PPC_WANT : PPC_MEM;
  // Work decompositions for the autotuner: variant v holds ppc(v) = PPC << v patches per CTA
  // (more patches per CTA: fewer, larger blocks and more pencils per barrier); a variant is
  // offered when it fits MAX_THREADS threads and MAX_SMEM bytes of shared memory.
  static constexpr int MAX_THREADS = 512, MAX_SMEM = 200 * 1024, MAX_VARIANTS = 3;
  static constexpr int ppc(int v) { return PPC << v; }
  static constexpr int threads(int ppc_) { return ((ppc_ * NPENCIL + 31) / 32) * 32 < 64 ? 64 : ((ppc_ * NPENCIL + 31) / 32) * 32; }
  // shared memory carve-up for ppc_ patches per CTA (byte offsets, each 16-byte aligned)
  static constexpr size_t al16(size_t x) { return (x + 15) / 16 * 16; }
  struct Lay
  {
    size_t fd, first, w, sym, combo, cls, data, bytes;
  };
  static constexpr Lay lay(int ppc_)
  {
    Lay l{};
    l.fd = 0;
    l.first = al16(l.fd + (size_t)ppc_ * DIM * ESIZE * sizeof(T));
    l.w = al16(l.first + (size_t)ppc_ * NCELL * 8);
    l.sym = al16(l.w + (size_t)ppc_ * NCELL * 4);      // ppc * DIM ints
    l.combo = al16(l.sym + (size_t)ppc_ * DIM * 4);     // ppc ints
    l.cls = al16(l.combo + (size_t)ppc_ * 4);           // ppc ints
    l.data = al16(l.cls + (size_t)ppc_ * 4);
    l.bytes = al16(l.data + (size_t)ppc_ * NLOC * sizeof(T));
    return l;
  }
  static constexpr bool variant_ok(int v)
  {
    return v >= 0 && v < MAX_VARIANTS && threads(ppc(v)) <= MAX_THREADS && lay(ppc(v)).bytes <= (size_t)MAX_SMEM;
  }
  static constexpr int n_variants() { return variant_ok(2) ? 3 : variant_ok(1) ? 2 : 1; }
};

// patch-local index of DoF e of patch cell cn
template<int DIM, int NCP, int K1>
__device__ __forceinline__ int patch_index(int cn, int e)
{
  constexpr int N = NCP * K1;
  int idx = 0, stride = 1;
#pragma unroll
  for(int d = 0; d < DIM; ++d)
  {
    const int cd = NCP == 1 ? 0 : (cn % NCP);
    const int id = e % K1;
    cn /= NCP;
    e /= K1;
    idx += (cd * K1 + id) * stride;
    stride *= N;
  }
  return idx;
}

// pencil base offset and stride for direction DIR
template<int DIM, int N, int DIR>
__device__ __forceinline__ int pencil_base(int p)
{
  constexpr int stride = cpow(N, DIR);
  return (p % stride) + (p / stride) * stride * N;
}

// TRANSPOSED: S^T (forward), else S (backward); sym: the entry is in even/odd form
template<typename T, int DIM, int N, int DIR, bool TRANSPOSED>
__device__ __forceinline__ void pass(T *__restrict__ data, const T *__restrict__ entry, bool sym, int p,
                                     T scale)
{
  constexpr int NPAD = Entry<T, N>::NPAD;
  constexpr int stride = cpow(N, DIR);
  const int base = pencil_base<DIM, N, DIR>(p);
  T r[N], o[N];
#pragma unroll
  for(int m = 0; m < N; ++m) r[m] = data[base + m * stride];
  if constexpr(N % 2 == 0)
  {
    if(sym)
    {
      if constexpr(TRANSPOSED)
        eo_fwd<T, N>(entry, r, o);
      else
        eo_bwd<T, N>(entry, r, o);
    }
    else
      rowmat<T, N, NPAD>(entry + (TRANSPOSED ? Entry<T, N>::ST : Entry<T, N>::S), r, o);
  }
  else
    rowmat<T, N, NPAD>(entry + (TRANSPOSED ? Entry<T, N>::ST : Entry<T, N>::S), r, o);
#pragma unroll
  for(int i = 0; i < N; ++i) data[base + i * stride] = o[i] * scale;
}

// last direction: S^T along DIM-1, divide by sum of eigenvalues, S along DIM-1
// (the eigenvalues of an even/odd entry are in the transformed order its forward pass produces).
// rcp (or nullptr): the patch's table of reciprocal eigenvalue sums, n^DIM values with direction
// 0 fastest; the division becomes a multiplication.
template<typename T, int DIM, int N, int ES>
__device__ __forceinline__ void pass_last(T *__restrict__ data, const T *__restrict__ entries,
                                          const int *sym, int p, const T *__restrict__ rcp)
{
  constexpr int NPAD = Entry<T, N>::NPAD;
  constexpr int DIR = DIM - 1;
  constexpr int stride = cpow(N, DIR);
  const int base = pencil_base<DIM, N, DIR>(p);
  T r[N], o[N];
#pragma unroll
  for(int m = 0; m < N; ++m) r[m] = data[base + m * stride];
  const T *eL = entries + DIR * ES;
  const bool symL = N % 2 == 0 && sym[DIR];
  if constexpr(N % 2 == 0)
  {
    if(symL)
      eo_fwd<T, N>(eL, r, o);
    else
      rowmat<T, N, NPAD>(eL + Entry<T, N>::ST, r, o);
  }
  else
    rowmat<T, N, NPAD>(eL + Entry<T, N>::ST, r, o);
  if(rcp)
  {
    // p enumerates i_0 [+ N i_1]; i runs along the last direction
#pragma unroll
    for(int i = 0; i < N; ++i) o[i] *= __ldg(rcp + p + i * stride);
  }
  else
  {
    // eigenvalue sum of the other directions (p enumerates i_0 [+ N i_1])
    T lsum = T(0);
    int rem = p;
#pragma unroll
    for(int d = 0; d < DIM - 1; ++d)
    {
      const int lam = N % 2 == 0 && sym[d] ? EoEntry<T, N>::LAM : Entry<T, N>::LAM;
      lsum += entries[d * ES + lam + rem % N];
      rem /= N;
    }
    const T *lamL = eL + (symL ? EoEntry<T, N>::LAM : Entry<T, N>::LAM);
#pragma unroll
    for(int i = 0; i < N; ++i) o[i] = o[i] / (lsum + lamL[i]);
  }
  if constexpr(N % 2 == 0)
  {
    if(symL)
      eo_bwd<T, N>(eL, o, r);
    else
      rowmat<T, N, NPAD>(eL + Entry<T, N>::S, o, r);
  }
  else
    rowmat<T, N, NPAD>(eL + Entry<T, N>::S, o, r);
#pragma unroll
  for(int i = 0; i < N; ++i) data[base + i * stride] = r[i];
}

struct KernelArgs
{
  const double *__restrict__ src;
  double *__restrict__ dst;
  const int64_t *__restrict__ patch_first;
  const int32_t *__restrict__ patch_fd;
  const void *__restrict__ fd;
  const float *__restrict__ ras_w;
  int64_t n_patches;
  double omega;
  int entry_stride;
  const void *__restrict__ fd_eo;     // even/odd forms (nullptr: none)
  const int32_t *__restrict__ sym;    // entry is mirror-symmetric (nullptr: none)
  int eo_stride;                      // elements per even/odd entry
  const void *__restrict__ rcp;       // reciprocal eigenvalue combinations (or nullptr)
  int rcp_E;                          // > 0: tables per entry combination, E entries per
                                      // direction; < 0: one table per patch of the range
  const unsigned char *__restrict__ keep_mask;  // RAS boolean: [class][NLOC] 1 = scatter (or nullptr)
  const int32_t *__restrict__ keep_class;       // RAS boolean: class of each patch of the range
  int ppc;                                      // patches per CTA (Cfg::ppc of the variant)
};

template<typename T, int DIM, int NCP, int K1>
__global__ void __launch_bounds__(Cfg<T, DIM, NCP, K1>::MAX_THREADS)
  schwarz_color_kernel(KernelArgs a)
{
  using C = Cfg<T, DIM, NCP, K1>;
  constexpr int N = C::N, NLOC = C::NLOC, NCELL = C::NCELL;
  constexpr int CELLDOFS = C::CELLDOFS, ES = C::ESIZE;
  const int PPC = a.ppc, NTHR = blockDim.x;
  const typename C::Lay lay = C::lay(PPC);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *s_fd = reinterpret_cast<T *>(smem_raw + lay.fd);                 // PPC * DIM * ES
  int64_t *s_first = reinterpret_cast<int64_t *>(smem_raw + lay.first);  // PPC * NCELL
  float *s_w = reinterpret_cast<float *>(smem_raw + lay.w);             // PPC * NCELL
  T *s_data = reinterpret_cast<T *>(smem_raw + lay.data);              // PPC * NLOC
  int *s_sym = reinterpret_cast<int *>(smem_raw + lay.sym);             // PPC * DIM
  int *s_combo = reinterpret_cast<int *>(smem_raw + lay.combo);         // PPC
  int *s_cls = reinterpret_cast<int *>(smem_raw + lay.cls);             // PPC
  const T *rcp = reinterpret_cast<const T *>(a.rcp);

  const T *fd = reinterpret_cast<const T *>(a.fd);
  const T *fd_eo = reinterpret_cast<const T *>(a.fd_eo);
  const int tid = threadIdx.x;
  const int slot = tid / C::NPENCIL, pencil = tid % C::NPENCIL;
  const T omega = T(a.omega);

  for(int64_t p0 = (int64_t)blockIdx.x * PPC; p0 < a.n_patches; p0 += (int64_t)gridDim.x * PPC)
  {
    const int64_t left = a.n_patches - p0;
    const int nvalid = left < PPC ? (int)left : PPC;
    // --- patch metadata and the 1-D eigenbases
    for(int i = tid; i < PPC * NCELL; i += NTHR)
    {
      const int s = i / NCELL;
      if(s < nvalid)
      {
        s_first[i] = a.patch_first[p0 * NCELL + i];
        s_w[i] = a.ras_w ? a.ras_w[p0 * NCELL + i] : 1.0f;
      }
    }
    for(int i = tid; i < PPC * DIM * ES; i += NTHR)
    {
      const int sd = i / ES, s = sd / DIM, o = i % ES;
      if(s < nvalid)
      {
        const int e = a.patch_fd[p0 * DIM + sd];
        const bool sy = N % 2 == 0 && a.sym && a.sym[e];
        if(sy)
          s_fd[i] = o < EoEntry<T, N>::size ? fd_eo[(size_t)e * a.eo_stride + o] : T(0);
        else
          s_fd[i] = o < Entry<T, N>::size ? fd[(size_t)e * a.entry_stride + o] : T(0);
        if(o == 0) s_sym[sd] = sy;
      }
    }
    if(rcp && tid < nvalid)
    {
      int c = 0;
      if(a.rcp_E < 0)
        c = int(p0 + tid);  // one table per patch
      else
#pragma unroll
        for(int d = DIM - 1; d >= 0; --d) c = c * a.rcp_E + a.patch_fd[(p0 + tid) * DIM + d];
      s_combo[tid] = c;
    }
    if(a.keep_mask && tid < nvalid) s_cls[tid] = a.keep_class[p0 + tid];
    __syncthreads();
    // --- gather: whole cells, coalesced
    for(int i = tid; i < PPC * NCELL * CELLDOFS; i += NTHR)
    {
      const int s = i / (NCELL * CELLDOFS);
      const int rem = i % (NCELL * CELLDOFS);
      const int cn = rem / CELLDOFS, e = rem % CELLDOFS;
      if(s < nvalid)
        s_data[s * NLOC + patch_index<DIM, NCP, K1>(cn, e)] = T(a.src[s_first[s * NCELL + cn] + e]);
    }
    __syncthreads();
    const bool active = slot < nvalid;
    T *my = s_data + slot * NLOC;
    const T *ent = s_fd + slot * DIM * ES;
    const int *sy = s_sym + slot * DIM;
    // --- forward S^T along directions 0..DIM-2
    if(active) pass<T, DIM, N, 0, true>(my, ent + 0 * ES, sy[0], pencil, T(1));
    __syncthreads();
    if constexpr(DIM == 3)
    {
      if(active) pass<T, DIM, N, 1, true>(my, ent + 1 * ES, sy[1], pencil, T(1));
      __syncthreads();
    }
    // --- last direction fused with the eigenvalue division
    if(active)
      pass_last<T, DIM, N, ES>(my, ent, sy, pencil, rcp ? rcp + (size_t)s_combo[slot] * NLOC : nullptr);
    __syncthreads();
    // --- backward S along directions DIM-2..0, damping folded into direction 0
    if constexpr(DIM == 3)
    {
      if(active) pass<T, DIM, N, 1, false>(my, ent + 1 * ES, sy[1], pencil, T(1));
      __syncthreads();
    }
    if(active) pass<T, DIM, N, 0, false>(my, ent + 0 * ES, sy[0], pencil, omega);
    __syncthreads();
    // --- scatter-add: whole cells, coalesced read-modify-write
    for(int i = tid; i < PPC * NCELL * CELLDOFS; i += NTHR)
    {
      const int s = i / (NCELL * CELLDOFS);
      const int rem = i % (NCELL * CELLDOFS);
      const int cn = rem / CELLDOFS, e = rem % CELLDOFS;
      if(s < nvalid)
      {
        const int64_t g = s_first[s * NCELL + cn] + e;
        const int pidx = patch_index<DIM, NCP, K1>(cn, e);
        // RAS boolean weights (rscatter_add): only the patch that owns the DoF adds it
        if(a.keep_mask && !a.keep_mask[s_cls[s] * NLOC + pidx]) continue;
        const double v = double(s_data[s * NLOC + pidx]);
        a.dst[g] += a.ras_w ? v * double(s_w[s * NCELL + cn]) : v;
      }
    }
    __syncthreads();
  }
}

template<typename T, int DIM, int NCP, int K1>
bool launch(KernelArgs a, cudaStream_t s, int n_sms, int variant)
{
  using C = Cfg<T, DIM, NCP, K1>;
  if(!C::variant_ok(variant)) variant = 0;
  a.ppc = C::ppc(variant);
  const int threads = C::threads(a.ppc);
  const size_t smem = C::lay(a.ppc).bytes;
  static int per_sm[C::MAX_VARIANTS] = {};  // occupancy per variant, queried once
  if(per_sm[variant] == 0)
  {
    const size_t smem_max = C::lay(C::ppc(C::n_variants() - 1)).bytes;
    if(cudaFuncSetAttribute(schwarz_color_kernel<T, DIM, NCP, K1>,
                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max) != cudaSuccess)
      return false;
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, schwarz_color_kernel<T, DIM, NCP, K1>, threads, smem);
    per_sm[variant] = occ < 1 ? 1 : occ;
  }
  if(a.n_patches <= 0) return true;
  const int64_t batches = (a.n_patches + a.ppc - 1) / a.ppc;
  const int64_t cap = (int64_t)n_sms * per_sm[variant] * 8;
  const int grid = (int)(batches < cap ? batches : cap);
  schwarz_color_kernel<T, DIM, NCP, K1><<<grid, threads, smem, s>>>(a);
  return cudaGetLastError() == cudaSuccess;
}

}  // namespace fd
}  // namespace tpss
