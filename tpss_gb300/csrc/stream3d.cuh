// stream3d.cuh -- additive vertex-patch Schwarz smoother in 3D, FP32, streamed by columns.
//
// Same mathematics as one SchwarzPreconditioner::vmult with additive vertex patches
// (preconditioner/schwarz_preconditioner.templates.h:585-688): dst = omega sum_j R_j^T A_j^-1
// R_j src, A_j^-1 by fast diagonalization.  Instead of one launch per color, which streams
// src and dst through HBM once per color, the work is organized for GB300:
//
//  - a work item is a column of BX x BY vertices (patches) and BZ vertex layers; persistent
//    CTAs take items round-robin (one CTA per SM);
//  - the item's cells are staged layer by layer in shared memory: each cell layer lands as FP64
//    (cp.async, issued one vertex layer ahead) and is converted once to an FP32 layer;
//  - the BX x BY patches of a vertex layer are solved together; each thread owns NPT pencils of one
//    patch, so every 1-D matrix row read from shared memory feeds NPT pencils;
//  - patch results are summed per cell in a shared-memory accumulator (each accumulator cell
//    adds the up to four patches of the vertex layer that touch it, in a fixed order); a cell
//    layer is final once the vertex layer above it is done and is written out once: cells owned
//    by the item go straight to dst, cells on the item's faces shared with neighbouring items go
//    to a halo buffer (scratch), which a fix-up kernel sums in a fixed order -- the result is
//    deterministic.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "fd_kernels.cuh"

namespace tpss
{
namespace stream
{
using fd::cpow;
using fd::Entry;

// base offset of the pencil along DIR through (a, b) -- (y, z), (x, z) or (x, y) -- in the padded
// layout x + SX y + SXY z
template<int SX, int SXY>
__host__ __device__ constexpr int pencil_addr(int dir, int a, int b)
{
  return dir == 0 ? SX * a + SXY * b : dir == 1 ? a + SXY * b : a + SX * b;
}

// the plain order puts the pencils of every warp instruction in distinct banks (one patch per warp)
template<int N, int SX, int SXY, int NPT, int TPP, int DIR>
__host__ __device__ constexpr bool plain_order_conflict_free()
{
  for(int j = 0; j < NPT; ++j)
  {
    int cnt[32] = {};
    for(int q = 0; q < TPP; ++q)
    {
      const int p = q + j * TPP;
      if(++cnt[pencil_addr<SX, SXY>(DIR, p % N, p / N) % 32] > 1) return false;
    }
  }
  return true;
}

// no bank holds more than NPT pencils along DIR: the bank-sorted order is conflict free
template<int N, int SX, int SXY, int NPT, int DIR>
__host__ __device__ constexpr bool bank_order_conflict_free()
{
  int cnt[32] = {};
  for(int p = 0; p < N * N; ++p)
    if(++cnt[pencil_addr<SX, SXY>(DIR, p % N, p / N) % 32] > NPT) return false;
  return true;
}

template<int K1_, int BX_, int BY_, int BZ_, int NPT_, bool WARP_PER_PATCH_ = false, bool PP_ = false>
struct SCfg
{
  static constexpr int K1 = K1_, BX = BX_, BY = BY_, BZ = BZ_, NPT = NPT_;
  static constexpr bool WARP_PER_PATCH = WARP_PER_PATCH_;
  // PP: every patch has its own 1-D problems (distorted levels: surrogate, fitted or learned
  // local solvers): the table slots hold the 3 directions of each patch of the vertex layer and
  // are refilled per vertex layer (cp.async, issued while the previous layer's results are
  // accumulated); otherwise one slot per vertex coordinate of the item
  static constexpr bool PP = PP_;
  static constexpr bool PLANE = false;  // pencil passes (plane3d.cuh holds the plane kernel)
  static constexpr int N = 2 * K1;
  static constexpr int NLOC = N * N * N;
  static constexpr int NPENCIL = N * N;
  static_assert(NPENCIL % NPT == 0, "pencils must split evenly");
  static constexpr int TPP = NPENCIL / NPT;  // threads per patch
  static constexpr int CD = K1 * K1 * K1;     // DoFs per cell
  static constexpr int NPATCH = BX * BY;      // patches per vertex layer
  // lanes per patch slot: TPP, or a whole warp per patch (lanes >= TPP idle in the FD passes),
  // which keeps one patch's pencils alone in a warp and their shared-memory accesses in
  // distinct banks
  static_assert(!WARP_PER_PATCH_ || TPP <= 32, "a warp per patch needs TPP <= 32");
  static constexpr int LPP = WARP_PER_PATCH_ ? 32 : TPP;
  static constexpr int THREADS = NPATCH * LPP;
  static constexpr int CX = BX + 1, CY = BY + 1;
  static constexpr int LCELLS = CX * CY;  // cells per cell layer of a column
  static constexpr int LAYER = LCELLS * CD;
  static constexpr int ES = Entry<float, N>::size;
  static constexpr int NPAD = Entry<float, N>::NPAD;
  // even/odd entries of mirror-symmetric 1-D problems: [Se^T][So^T][Se][So] (h x hpad) + lambda
  static constexpr int H = N / 2;
  static constexpr int HPAD = ((H + 3) / 4) * 4;
  static constexpr int EO_SOT = H * HPAD, EO_SE = 2 * H * HPAD, EO_SO = 3 * H * HPAD;
  static constexpr int EO_LAM = 4 * H * HPAD;
  static constexpr int ES_EO = EO_LAM + NPAD;
  static constexpr int ESLOT = ((ES > ES_EO ? ES : ES_EO) + 3) / 4 * 4;  // shared slot size
  // padded patch layout (x + SX y + SXY z): chosen so that the pencils of a warp fall into
  // distinct shared-memory banks in all three directions (at most 2-way conflicts)
  static constexpr int SX = N == 10 ? 13 : N == 8 ? 9 : N == 6 ? 6 : N == 4 ? 5 : N;
  static constexpr int SXY = N == 10 ? 137 : N == 8 ? 72 : N == 6 ? 39 : N == 4 ? 21 : N * N;
  // floats per patch work buffer; for N = 8 two patches share a warp (TPP 16) and a stride of
  // 576 = 0 mod 32 would put them on the same banks, so it is shifted by half a bank row
  static constexpr int PSTRIDE = SXY * N + (N == 8 && !WARP_PER_PATCH_ && TPP == 16 ? 16 : 0);
  // element loops give every thread one fixed cell-local DoF e (no div/mod per element)
  static constexpr int G = THREADS / CD;   // thread groups sharing an e
  static_assert(G >= 1, "need at least one thread per cell DoF");
  // shared memory carve-up (in floats; the staged FP64 cell layers take two floats per value)
  static constexpr int NSLOT = PP_ ? 3 * BX * BY : BX + BY + BZ;     // 1-D table slots
  static constexpr int OFF_FD = 0;                                   // NSLOT entries
  static constexpr int OFF_SYM = OFF_FD + NSLOT * ESLOT;             // int flags
  // PP: table entry code of every slot of the item's vertex layers (2 entry + mirror-symmetric
  // flag, -1 none), looked up once per item
  static constexpr int OFF_EN = OFF_SYM + NSLOT;
  // cell layers are copied in as FP64 (two landing layers) and converted once to FP32 (two
  // layers, rows of cells padded by RPAD floats so that the x pass reads conflict free)
  static constexpr int RPAD = K1 == 5 ? 4 : K1 == 4 ? 1 : K1 == 3 ? (WARP_PER_PATCH_ ? 0 : 6) : (WARP_PER_PATCH_ ? 5 : 1);
  static constexpr int RSTRIDE = CX * CD + RPAD;                     // floats per row of cells
  static constexpr int LAYERF = ((CY * RSTRIDE + 3) / 4) * 4;        // floats per FP32 layer
  static constexpr int OFF_RAW = ((OFF_EN + (PP_ ? BZ * NSLOT : 0) + 3) / 4) * 4;  // 2 FP64 layers
  static constexpr int OFF_F32 = OFF_RAW + 2 * 2 * LAYER;            // 2 FP32 cell layers
  static constexpr int OFF_ACC = OFF_F32 + 2 * LAYERF;               // 2 FP32 accumulator layers
  static constexpr int OFF_WORK = OFF_ACC + 2 * LAYER;               // NPATCH patches
  // per-item cell tables (ints): global xy index of each column cell (-1 outside the item),
  // its x/y-shared flag, and for each of the 2 LCELLS accumulator cells the offsets of the (up
  // to) 4 patches of a vertex layer that touch it (-1: none)
  static constexpr int OFF_TAB = ((OFF_WORK + NPATCH * PSTRIDE + 3) / 4) * 4;
  static constexpr int OFF_AOFF = OFF_TAB + ((2 * LCELLS + 3) / 4) * 4;  // int4 aligned
  // pencil order tables of the directions whose plain order has bank conflicts (warp per patch)
  static constexpr bool MAP0 = WARP_PER_PATCH_ && !plain_order_conflict_free<N, SX, SXY, NPT, TPP, 0>() &&
                               bank_order_conflict_free<N, SX, SXY, NPT, 0>();
  static constexpr bool MAP1 = WARP_PER_PATCH_ && !plain_order_conflict_free<N, SX, SXY, NPT, TPP, 1>() &&
                               bank_order_conflict_free<N, SX, SXY, NPT, 1>();
  static constexpr bool MAP2 = WARP_PER_PATCH_ && !plain_order_conflict_free<N, SX, SXY, NPT, TPP, 2>() &&
                               bank_order_conflict_free<N, SX, SXY, NPT, 2>();
  static constexpr int OFF_PMAP = OFF_AOFF + 8 * LCELLS;
  static constexpr int FLOATS = OFF_PMAP + (MAP0 || MAP1 || MAP2 ? 3 * NPENCIL : 0);
  static constexpr size_t smem_bytes() { return (size_t)FLOATS * 4; }
  static_assert((size_t)FLOATS * 4 <= 227 * 1024, "shared memory per CTA exceeds 227 KB");
};

struct StreamArgs
{
  const double *__restrict__ src;
  double *__restrict__ dst;
  float *__restrict__ halo;
  const int64_t *__restrict__ cell_start;  // nullptr: lexicographic cells
  const float *__restrict__ fd;            // FP32 FD table
  const float *__restrict__ fd_eo;         // even/odd table (valid where sym[e])
  const int32_t *__restrict__ sym;         // entry is mirror-symmetric
  int es_eo;                               // elements per even/odd entry
  const int32_t *__restrict__ vfd[3];      // FD entry of vertex v per direction
  int nc[3];                               // cells per direction
  int T[3];                                // items per direction
  float omega;
  int ras;                                 // scale by 1/multiplicity
  int item_begin, item_end;                // items of this launch (z-major item order)
  // per-patch 1-D problems (SCfg::PP): patch index of each vertex (lexicographic over the
  // (n+1)^3 vertices, -1 on the boundary) and the patches' FD entries (3 per patch)
  const int32_t *__restrict__ vpatch;
  const int32_t *__restrict__ pfd;
};

// tiles (t, local index l) of direction d that contain cell c; returns the count (1 or 2)
__host__ __device__ __forceinline__ int tiles_of(int c, int W, int T, int *t, int *l)
{
  int n = 0;
  const int tt = c / W;
  if(tt <= T - 1)
  {
    t[n] = tt;
    l[n] = c - W * tt;
    ++n;
  }
  if(c % W == 0 && tt >= 1)
  {
    t[n] = tt - 1;
    l[n] = W;
    ++n;
  }
  return n;
}

__host__ __device__ __forceinline__ float multiplicity(int c, int n)
{
  return float((c >= 1 ? 1 : 0) + (c + 1 <= n - 1 ? 1 : 0));
}

// Pencil idx = q + j TPP of a thread (pencil group q, j-th of its NPT pencils) along DIR. Plain
// order: a = idx % N, b = idx / N. Mapped order (MAP): read from the table pm, which deals the
// pencils sorted by shared-memory bank round-robin to the NPT groups, so that the TPP pencils one
// warp instruction touches lie in distinct banks (entries: offset | a << 16 | b << 24).
template<bool MAP, int N, int SX, int SXY, int DIR>
__device__ __forceinline__ int pencil_of(const int *__restrict__ pm, int idx, int &a, int &b)
{
  if constexpr(MAP)
  {
    const int v = pm[idx];
    a = (v >> 16) & 0xff;
    b = v >> 24;
    return v & 0xffff;
  }
  else
  {
    a = idx % N;
    b = idx / N;
    return pencil_addr<SX, SXY>(DIR, a, b);
  }
}


template<bool MAP, bool SCALED, int N, int SX, int SXY, int NPAD, int DIR, int NPT, int TPP>
__device__ __forceinline__ void mpass(float *__restrict__ data, const float *__restrict__ B,
                                      const int *__restrict__ pm, int q, float scale)
{
  constexpr int stride = DIR == 0 ? 1 : DIR == 1 ? SX : SXY;
  float r[NPT][N];
  int base[NPT];
#pragma unroll
  for(int j = 0; j < NPT; ++j)
  {
    int pa, pb;
    base[j] = pencil_of<MAP, N, SX, SXY, DIR>(pm, q + j * TPP, pa, pb);
#pragma unroll
    for(int m = 0; m < N; ++m) r[j][m] = data[base[j] + m * stride];
  }
#pragma unroll
  for(int i = 0; i < N; ++i)
  {
    const float4 *row = reinterpret_cast<const float4 *>(B + i * NPAD);
    float acc[NPT];
#pragma unroll
    for(int j = 0; j < NPT; ++j) acc[j] = 0.f;
#pragma unroll
    for(int m4 = 0; m4 < NPAD / 4; ++m4)
    {
      const float4 v = row[m4];
      const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for(int w = 0; w < 4; ++w)
        if(m4 * 4 + w < N)
#pragma unroll
          for(int j = 0; j < NPT; ++j) acc[j] = fmaf(vv[w], r[j][m4 * 4 + w < N ? m4 * 4 + w : 0], acc[j]);
    }
#pragma unroll
    for(int j = 0; j < NPT; ++j) data[base[j] + i * stride] = SCALED ? acc[j] * scale : acc[j];
  }
}

// Even/odd passes of mirror-symmetric directions (n = 2h): forward t_e = Se^T (r_i + r_{n-1-i}),
// t_o = So^T (r_i - r_{n-1-i}) stored at transformed positions [0,h) and [h,n); backward
// u_i = Se t_e + So t_o, u_{n-1-i} = Se t_e - So t_o.  Half the FMAs of a full n x n pass.
// NPT pencils of N values in pairs of registers: pencils 2p and 2p+1 share the float2 v[p][m]
// (for odd NPT the last pair's y half is a spare), so the even/odd passes below run on packed
// FP32 instructions (FFMA2 / FADD2: two pencils per instruction, the same rounding as two scalar
// operations)
template<int NPT, int N>
struct Pencils
{
  static constexpr int P = (NPT + 1) / 2;
  float2 v[P][N];
  __device__ __forceinline__ float &at(int j, int m) { return (j & 1) ? v[j >> 1][m].y : v[j >> 1][m].x; }
};

__device__ __forceinline__ float2 bcast2(float x) { return make_float2(x, x); }

template<int H, int HPAD, int NPT>
__device__ __forceinline__ void eo_forward(Pencils<NPT, 2 * H> &r, const float *__restrict__ eo,
                                           Pencils<NPT, 2 * H> &t)
{
  constexpr int P = Pencils<NPT, 2 * H>::P;
  const float2 m1 = bcast2(-1.f);
#pragma unroll
  for(int p = 0; p < P; ++p)
#pragma unroll
    for(int i = 0; i < H; ++i)
    {
      const float2 a = r.v[p][i], b = r.v[p][2 * H - 1 - i];
      r.v[p][i] = __fadd2_rn(a, b);
      r.v[p][2 * H - 1 - i] = __ffma2_rn(b, m1, a);  // a - b, stored mirrored
    }
#pragma unroll
  for(int par = 0; par < 2; ++par)
#pragma unroll
    for(int k = 0; k < H; ++k)
    {
      const float4 *row = reinterpret_cast<const float4 *>(eo + (par * H + k) * HPAD);
      float2 acc[P];
#pragma unroll
      for(int p = 0; p < P; ++p) acc[p] = bcast2(0.f);
#pragma unroll
      for(int m4 = 0; m4 < HPAD / 4; ++m4)
      {
        const float4 v = row[m4];
        const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for(int w = 0; w < 4; ++w)
          if(m4 * 4 + w < H)
          {
            const int i = m4 * 4 + w < H ? m4 * 4 + w : 0;
            const float2 c = bcast2(vv[w]);
#pragma unroll
            for(int p = 0; p < P; ++p) acc[p] = __ffma2_rn(c, r.v[p][par == 0 ? i : 2 * H - 1 - i], acc[p]);
          }
      }
#pragma unroll
      for(int p = 0; p < P; ++p) t.v[p][par * H + k] = acc[p];
    }
}

template<int H, int HPAD, int NPT>
__device__ __forceinline__ void eo_backward(const Pencils<NPT, 2 * H> &t, const float *__restrict__ eo,
                                            Pencils<NPT, 2 * H> &u)
{
  constexpr int P = Pencils<NPT, 2 * H>::P;
  const float2 m1 = bcast2(-1.f);
#pragma unroll
  for(int i = 0; i < H; ++i)
  {
    const float4 *re = reinterpret_cast<const float4 *>(eo + (2 * H + i) * HPAD);
    const float4 *ro = reinterpret_cast<const float4 *>(eo + (3 * H + i) * HPAD);
    float2 E[P], O[P];
#pragma unroll
    for(int p = 0; p < P; ++p) E[p] = O[p] = bcast2(0.f);
#pragma unroll
    for(int m4 = 0; m4 < HPAD / 4; ++m4)
    {
      const float4 ve = re[m4], vo = ro[m4];
      const float ee[4] = {ve.x, ve.y, ve.z, ve.w}, oo[4] = {vo.x, vo.y, vo.z, vo.w};
#pragma unroll
      for(int w = 0; w < 4; ++w)
        if(m4 * 4 + w < H)
        {
          const int k = m4 * 4 + w < H ? m4 * 4 + w : 0;
          const float2 ce = bcast2(ee[w]), co = bcast2(oo[w]);
#pragma unroll
          for(int p = 0; p < P; ++p)
          {
            E[p] = __ffma2_rn(ce, t.v[p][k], E[p]);
            O[p] = __ffma2_rn(co, t.v[p][H + k], O[p]);
          }
        }
    }
#pragma unroll
    for(int p = 0; p < P; ++p)
    {
      u.v[p][i] = __fadd2_rn(E[p], O[p]);
      u.v[p][2 * H - 1 - i] = __ffma2_rn(O[p], m1, E[p]);
    }
  }
}

// full or even/odd pass along DIR (in place in the padded patch layout)
// (SCALED: the outputs are multiplied by scale)
template<bool SYM, bool FWD, bool MAP, bool SCALED, int N, int SX, int SXY, int NPAD, int HPAD, int DIR, int NPT,
         int TPP>
__device__ __forceinline__ void spass(float *__restrict__ data, const float *__restrict__ ent,
                                      const int *__restrict__ pm, int q, float scale)
{
  if constexpr(!SYM)
    mpass<MAP, SCALED, N, SX, SXY, NPAD, DIR, NPT, TPP>(
      data, ent + (FWD ? Entry<float, N>::ST : Entry<float, N>::S), pm, q, scale);
  else
  {
    constexpr int H = N / 2;
    constexpr int stride = DIR == 0 ? 1 : DIR == 1 ? SX : SXY;
    Pencils<NPT, N> r, o;
    int base[NPT];
#pragma unroll
    for(int j = 0; j < NPT; ++j)
    {
      int pa, pb;
      base[j] = pencil_of<MAP, N, SX, SXY, DIR>(pm, q + j * TPP, pa, pb);
#pragma unroll
      for(int m = 0; m < N; ++m) r.at(j, m) = data[base[j] + m * stride];
    }
    if constexpr(NPT % 2 == 1)
#pragma unroll
      for(int m = 0; m < N; ++m) r.at(NPT, m) = 0.f;
    if constexpr(FWD)
      eo_forward<H, HPAD, NPT>(r, ent, o);
    else
      eo_backward<H, HPAD, NPT>(r, ent, o);
#pragma unroll
    for(int j = 0; j < NPT; ++j)
#pragma unroll
      for(int i = 0; i < N; ++i) data[base[j] + i * stride] = SCALED ? o.at(j, i) * scale : o.at(j, i);
  }
}

// direction 0, forward, reading the patch straight from the two staged FP64 cell layers:
// pencil (y, z) of patch (px, py) covers cells (px, px+1) of row (py + y/K1) in layer z/K1
template<bool SYM, bool MAP, int K1, int N, int SX, int SXY, int NPAD, int HPAD, int NPT, int TPP, int RS, int CD>
__device__ __forceinline__ void mpass_x_from_layers(float *__restrict__ data, const float *__restrict__ lo,
                                                    const float *__restrict__ hi,
                                                    const float *__restrict__ St, const int *__restrict__ pm,
                                                    int px, int py, int q)
{
  int base[NPT], row[NPT];
  const float *layer[NPT];
#pragma unroll
  for(int j = 0; j < NPT; ++j)
  {
    int y, z;
    base[j] = pencil_of<MAP, N, SX, SXY, 0>(pm, q + j * TPP, y, z);
    layer[j] = z >= K1 ? hi : lo;
    row[j] = px * CD + RS * (py + y / K1) + K1 * (y % K1) + K1 * K1 * (z % K1);
  }
  if constexpr(SYM)
  {
    Pencils<NPT, N> r, t;
#pragma unroll
    for(int j = 0; j < NPT; ++j)
#pragma unroll
      for(int m = 0; m < N; ++m) r.at(j, m) = layer[j][row[j] + (m / K1) * CD + (m % K1)];
    if constexpr(NPT % 2 == 1)
#pragma unroll
      for(int m = 0; m < N; ++m) r.at(NPT, m) = 0.f;
    eo_forward<N / 2, HPAD, NPT>(r, St, t);
#pragma unroll
    for(int j = 0; j < NPT; ++j)
#pragma unroll
      for(int i = 0; i < N; ++i) data[base[j] + i] = t.at(j, i);
  }
  else
  {
    float r[NPT][N];
#pragma unroll
    for(int j = 0; j < NPT; ++j)
#pragma unroll
      for(int m = 0; m < N; ++m) r[j][m] = layer[j][row[j] + (m / K1) * CD + (m % K1)];
#pragma unroll
    for(int i = 0; i < N; ++i)
    {
      const float4 *rw = reinterpret_cast<const float4 *>(St + i * NPAD);
      float acc[NPT];
#pragma unroll
      for(int j = 0; j < NPT; ++j) acc[j] = 0.f;
#pragma unroll
      for(int m4 = 0; m4 < NPAD / 4; ++m4)
      {
        const float4 v = rw[m4];
        const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for(int w = 0; w < 4; ++w)
          if(m4 * 4 + w < N)
#pragma unroll
            for(int j = 0; j < NPT; ++j) acc[j] = fmaf(vv[w], r[j][m4 * 4 + w < N ? m4 * 4 + w : 0], acc[j]);
      }
#pragma unroll
      for(int j = 0; j < NPT; ++j) data[base[j] + i] = acc[j];
    }
  }
}

// 1/x by the hardware's approximate reciprocal (PTX rcp.approx.ftz.f32, max. 1 ulp); the divisors
// here are sums of positive eigenvalues
__device__ __forceinline__ float rcp_approx(float x)
{
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// direction 2 in registers: S^T along z, division by the eigenvalue sums, S along z -- the
// pencil a thread transforms forward is the one it transforms back, so the intermediate never
// goes through shared memory
template<bool SYM, bool MAP, int N, int SX, int SXY, int NPAD, int HPAD, int NPT, int TPP>
__device__ __forceinline__ void zpass_solve(float *__restrict__ data, const float *__restrict__ lamx,
                                            const float *__restrict__ lamy, const float *__restrict__ ez,
                                            const float *__restrict__ lamz, const int *__restrict__ pm, int q)
{
  constexpr int stride = SXY;
  float lxy[NPT];
  int base[NPT];
#pragma unroll
  for(int j = 0; j < NPT; ++j)
  {
    int px_, py_;
    base[j] = pencil_of<MAP, N, SX, SXY, 2>(pm, q + j * TPP, px_, py_);
    lxy[j] = lamx[px_] + lamy[py_];
  }
  if constexpr(SYM)
  {
    Pencils<NPT, N> r, t;
#pragma unroll
    for(int j = 0; j < NPT; ++j)
#pragma unroll
      for(int m = 0; m < N; ++m) r.at(j, m) = data[base[j] + m * stride];
    if constexpr(NPT % 2 == 1)
#pragma unroll
      for(int m = 0; m < N; ++m) r.at(NPT, m) = 0.f;
    eo_forward<N / 2, HPAD, NPT>(r, ez, t);
#pragma unroll
    for(int i = 0; i < N; ++i)
    {
      const float lz = lamz[i];
#pragma unroll
      for(int j = 0; j < NPT; ++j) t.at(j, i) = t.at(j, i) * rcp_approx(lxy[j] + lz);
    }
    eo_backward<N / 2, HPAD, NPT>(t, ez, r);
#pragma unroll
    for(int j = 0; j < NPT; ++j)
#pragma unroll
      for(int i = 0; i < N; ++i) data[base[j] + i * stride] = r.at(j, i);
  }
  else
  {
    float r[NPT][N], t[NPT][N];
#pragma unroll
    for(int j = 0; j < NPT; ++j)
#pragma unroll
      for(int m = 0; m < N; ++m) r[j][m] = data[base[j] + m * stride];
#pragma unroll
    for(int i = 0; i < N; ++i)
    {
      const float4 *row = reinterpret_cast<const float4 *>(ez + Entry<float, N>::ST + i * NPAD);
      float acc[NPT];
#pragma unroll
      for(int j = 0; j < NPT; ++j) acc[j] = 0.f;
#pragma unroll
      for(int m4 = 0; m4 < NPAD / 4; ++m4)
      {
        const float4 v = row[m4];
        const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for(int w = 0; w < 4; ++w)
          if(m4 * 4 + w < N)
#pragma unroll
            for(int j = 0; j < NPT; ++j) acc[j] = fmaf(vv[w], r[j][m4 * 4 + w < N ? m4 * 4 + w : 0], acc[j]);
      }
      const float lz = lamz[i];
#pragma unroll
      for(int j = 0; j < NPT; ++j) t[j][i] = acc[j] * rcp_approx(lxy[j] + lz);
    }
#pragma unroll
    for(int i = 0; i < N; ++i)
    {
      const float4 *row = reinterpret_cast<const float4 *>(ez + Entry<float, N>::S + i * NPAD);
      float acc[NPT];
#pragma unroll
      for(int j = 0; j < NPT; ++j) acc[j] = 0.f;
#pragma unroll
      for(int m4 = 0; m4 < NPAD / 4; ++m4)
      {
        const float4 v = row[m4];
        const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for(int w = 0; w < 4; ++w)
          if(m4 * 4 + w < N)
#pragma unroll
            for(int j = 0; j < NPT; ++j) acc[j] = fmaf(vv[w], t[j][m4 * 4 + w < N ? m4 * 4 + w : 0], acc[j]);
      }
#pragma unroll
      for(int j = 0; j < NPT; ++j) data[base[j] + i * stride] = acc[j];
    }
  }
}

// barrier between two FD passes: a warp that owns its patch alone only waits for itself
template<class C>
__device__ __forceinline__ void pass_sync()
{
  if constexpr(C::WARP_PER_PATCH)
    __syncwarp();
  else
    __syncthreads();
}

// first DoF of the cell with lexicographic index xy + nx ny cz
template<class C>
__device__ __forceinline__ int64_t cell_first_xy(const StreamArgs &a, int xy, int cz)
{
  const int64_t cell = xy + (int64_t)a.nc[0] * a.nc[1] * cz;
  return a.cell_start ? a.cell_start[cell] : cell * C::CD;
}

// The element loops below give a thread the cells g, g + G, g + 2G, ... of a layer (DoF e of
// each). They are unrolled in phases -- all shared-memory reads first, then the dependent work --
// so that a thread's reads are in flight together instead of one round trip per cell.

// asynchronous copy (cp.async, 8 bytes) of cell layer cz of the column (the item's cells of
// the table cxy) into the FP64 staging buffer; cells outside are zero-filled
template<class C>
__device__ __forceinline__ void copy_layer_async(const StreamArgs &a, const int *cxy, int cz, double *raw,
                                                 int e, int g)
{
  constexpr int IT = (C::LCELLS + C::G - 1) / C::G;
  if(g < C::G)
  {
    int xy[IT];
#pragma unroll
    for(int it = 0; it < IT; ++it)
    {
      const int cell = g + it * C::G;
      xy[it] = cell < C::LCELLS ? cxy[cell] : -2;
    }
#pragma unroll
    for(int it = 0; it < IT; ++it)
    {
      const int cell = g + it * C::G, i = cell * C::CD + e;
      if(xy[it] >= 0)
      {
        const double *src = a.src + cell_first_xy<C>(a, xy[it], cz) + e;
        const unsigned saddr = (unsigned)__cvta_generic_to_shared(raw + i);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(saddr), "l"(src) : "memory");
      }
      else if(xy[it] == -1)
        raw[i] = 0.0;
    }
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

__device__ __forceinline__ void wait_async_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// asynchronous copy (cp.async, 16 bytes) of one vertex layer's per-patch 1-D problems into the
// table slots (SCfg::PP): slot sl takes the full or even/odd entry of code en[sl], zero-filled
// beyond the entry and for en[sl] < 0; the mirror-symmetric flags are stored directly
template<class C>
__device__ __forceinline__ void fill_tables_async(const StreamArgs &a, float *s_fd, int *s_sym, const int *en,
                                                  int tid)
{
  constexpr int Q = C::ESLOT / 4;  // 16-byte chunks per slot
  for(int i = tid; i < C::NSLOT * Q; i += C::THREADS)
  {
    const int sl = i / Q, o = 4 * (i % Q), code = en[sl];
    const float *src = a.fd;
    int bytes = 0;
    if(code >= 0)
    {
      const int e = code >> 1;
      if(code & 1)
      {
        if(o < C::ES_EO) { src = a.fd_eo + (size_t)e * a.es_eo + o; bytes = 16; }
      }
      else if(o < C::ES) { src = a.fd + (size_t)e * C::ES + o; bytes = 16; }
    }
    const unsigned saddr = (unsigned)__cvta_generic_to_shared(s_fd + sl * C::ESLOT + o);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(saddr), "l"(src), "r"(bytes) : "memory");
    if(o == 0) s_sym[sl] = code >= 0 ? (code & 1) : 0;
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// FP64 landing layer -> FP32 cell layer (rows padded to RSTRIDE). Each thread converts the values
// its own copy_layer_async put there (same cell/DoF assignment), so after its wait_async_all no
// barrier is needed in between.
template<class C>
__device__ __forceinline__ void convert_layer(const double *raw, float *f32, int e, int g)
{
  constexpr int IT = (C::LCELLS + C::G - 1) / C::G;
  if(g < C::G)
  {
    double v[IT];
#pragma unroll
    for(int it = 0; it < IT; ++it)
    {
      const int cell = g + it * C::G;
      v[it] = cell < C::LCELLS ? raw[cell * C::CD + e] : 0.0;
    }
#pragma unroll
    for(int it = 0; it < IT; ++it)
    {
      const int cell = g + it * C::G;
      if(cell < C::LCELLS)
      {
        const int lx = cell % C::CX, ly = cell / C::CX;
        f32[lx * C::CD + ly * C::RSTRIDE + e] = float(v[it]);
      }
    }
  }
}

// write one completed cell layer: cells owned by the item to dst, shared cells to the halo
template<class C>
__device__ __forceinline__ void write_layer(const StreamArgs &a, float *accl, int item, int lz, int cz,
                                            bool zshared, const int *cxy, const int *cshared, int e,
                                            int g, bool clear)
{
  constexpr int IT = (C::LCELLS + C::G - 1) / C::G;
  if(g >= C::G) return;
  int xy[IT], sh[IT];
  float v[IT];
#pragma unroll
  for(int it = 0; it < IT; ++it)
  {
    const int cell = g + it * C::G;
    xy[it] = cell < C::LCELLS ? cxy[cell] : -1;
    sh[it] = cell < C::LCELLS ? cshared[cell] : 0;
    v[it] = cell < C::LCELLS ? accl[cell * C::CD + e] : 0.f;
  }
#pragma unroll
  for(int it = 0; it < IT; ++it)
  {
    const int cell = g + it * C::G;
    if(xy[it] < 0) continue;
    float w = v[it];
    if(sh[it] || zshared)
      a.halo[((size_t)item * (C::BZ + 1) * C::LCELLS + (size_t)lz * C::LCELLS + cell) * C::CD + e] = w;
    else
    {
      if(a.ras)
      {
        const int cx = xy[it] % a.nc[0], cy = xy[it] / a.nc[0];
        w /= multiplicity(cx, a.nc[0]) * multiplicity(cy, a.nc[1]) * multiplicity(cz, a.nc[2]);
      }
      a.dst[cell_first_xy<C>(a, xy[it], cz) + e] = double(w);
    }
  }
  if(clear)
#pragma unroll
    for(int it = 0; it < IT; ++it)
      if(xy[it] >= 0) accl[(g + it * C::G) * C::CD + e] = 0.f;
}

template<class C>
__global__ void __launch_bounds__(C::THREADS, 1) stream_kernel(StreamArgs a)
{
  constexpr int K1 = C::K1, N = C::N, CD = C::CD, ES = C::ES, NPAD = C::NPAD;
  constexpr int BX = C::BX, BY = C::BY, BZ = C::BZ, TPP = C::TPP, NPT = C::NPT;
  constexpr int SX = C::SX, SXY = C::SXY, PS = C::PSTRIDE;
  extern __shared__ __align__(16) float sm[];
  float *s_fd = sm + C::OFF_FD;
  int *s_sym = reinterpret_cast<int *>(sm + C::OFF_SYM);
  int *s_en = reinterpret_cast<int *>(sm + C::OFF_EN);
  double *s_raw = reinterpret_cast<double *>(sm + C::OFF_RAW);
  float *s_f32 = sm + C::OFF_F32;
  float *s_acc = sm + C::OFF_ACC;
  float *s_work = sm + C::OFF_WORK;
  int *s_cxy = reinterpret_cast<int *>(sm + C::OFF_TAB);
  int *s_cshared = s_cxy + C::LCELLS;
  int *s_aoff = reinterpret_cast<int *>(sm + C::OFF_AOFF);
  int *s_pmap = reinterpret_cast<int *>(sm + C::OFF_PMAP);
  const int tid = threadIdx.x;
  const int slot = tid / C::LPP, q = tid % C::LPP;  // FD passes: patch slot (px + BX py), pencil group
  const int px = slot % BX, py = slot / BX;
  // element loops: fixed cell-local DoF e and its patch-local offset
  const int e = tid % CD, g = tid / CD;
  const int e_patch = (e % K1) + SX * ((e / K1) % K1) + SXY * (e / (K1 * K1));
  const int n_items = a.T[0] * a.T[1] * a.T[2];
  if constexpr(C::MAP0 || C::MAP1 || C::MAP2)
  {
    // pencil order tables: rank the pencils by (bank, index), deal rank i to thread q = i / NPT as
    // its (i % NPT)-th pencil; a bank holds at most NPT pencils, so every warp instruction's
    // pencils lie in distinct banks (read after the barrier at the top of the item loop)
    constexpr int NP = C::NPENCIL;
    for(int t = tid; t < 3 * NP; t += C::THREADS)
    {
      const int dir = t / NP, p = t % NP;
      if(!(dir == 0 ? C::MAP0 : dir == 1 ? C::MAP1 : C::MAP2)) continue;
      const int addr = pencil_addr<SX, SXY>(dir, p % N, p / N), bank = addr % 32;
      int rank = 0;
      for(int p2 = 0; p2 < NP; ++p2)
      {
        const int b2 = pencil_addr<SX, SXY>(dir, p2 % N, p2 / N) % 32;
        rank += b2 < bank || (b2 == bank && p2 < p);
      }
      s_pmap[dir * NP + rank / NPT + (rank % NPT) * TPP] = addr | (p % N) << 16 | (p / N) << 24;
    }
  }
  const int *pm0 = s_pmap, *pm1 = s_pmap + C::NPENCIL, *pm2 = s_pmap + 2 * C::NPENCIL;
  constexpr bool M0 = C::MAP0, M1 = C::MAP1, M2 = C::MAP2;

  for(int item = a.item_begin + blockIdx.x; item < a.item_end && item < n_items; item += gridDim.x)
  {
    const int tx = item % a.T[0], ty = (item / a.T[0]) % a.T[1], tz = item / (a.T[0] * a.T[1]);
    // vertices of the item: v_d in [1 + W t, min(W (t+1), n_d - 1)]
    const int bx = min(BX, a.nc[0] - 1 - BX * tx), by = min(BY, a.nc[1] - 1 - BY * ty);
    const int bz = min(BZ, a.nc[2] - 1 - BZ * tz);
    const int x0 = BX * tx, y0 = BY * ty, z0 = BZ * tz;  // first cell of the item
    __syncthreads();  // the previous item is done with shared memory
    if constexpr(C::PP)
    {
      // entry codes of the item's patches, per vertex layer and slot (3 directions per patch);
      // the slots are filled per vertex layer by fill_tables_async
      const int nvx = a.nc[0] + 1, nvy = a.nc[1] + 1;
      for(int i = tid; i < BZ * C::NSLOT; i += C::THREADS)
      {
        const int jj = i / C::NSLOT, sl = i % C::NSLOT, pp = sl / 3, d = sl % 3;
        const int ppx = pp % BX, ppy = pp / BX;
        int code = -1;
        if(jj < bz && ppx < bx && ppy < by)
        {
          const int32_t patch =
            a.vpatch[(x0 + 1 + ppx) + (int64_t)nvx * ((y0 + 1 + ppy) + (int64_t)nvy * (z0 + 1 + jj))];
          const int32_t en = patch >= 0 ? a.pfd[(int64_t)patch * 3 + d] : -1;
          if(en >= 0) code = 2 * en + (a.sym[en] ? 1 : 0);
        }
        s_en[i] = code;
      }
    }
    // 1-D eigenbases of the item's x, y and z vertices: full entry or even/odd split
    for(int i = tid; i < (C::PP ? 0 : (BX + BY + BZ) * C::ESLOT); i += C::THREADS)
    {
      const int sl = i / C::ESLOT, o = i % C::ESLOT;
      int en = -1;
      if(sl < BX) { if(sl < bx) en = a.vfd[0][x0 + 1 + sl]; }
      else if(sl < BX + BY) { if(sl - BX < by) en = a.vfd[1][y0 + 1 + (sl - BX)]; }
      else if(sl - BX - BY < bz) en = a.vfd[2][z0 + 1 + (sl - BX - BY)];
      float v = 0.f;
      if(en >= 0)
      {
        if(a.sym[en]) { if(o < C::ES_EO) v = a.fd_eo[(size_t)en * a.es_eo + o]; }
        else if(o < ES) v = a.fd[(size_t)en * ES + o];
      }
      s_fd[i] = v;
      if(o == 0) s_sym[sl] = en >= 0 ? a.sym[en] : 0;
    }
    // cell tables of the item (read by the element loops below, which then need no index
    // arithmetic of their own)
    for(int i = tid; i < C::LCELLS; i += C::THREADS)
    {
      const int lx = i % C::CX, ly = i / C::CX;
      s_cxy[i] = (lx <= bx && ly <= by) ? (x0 + lx) + a.nc[0] * (y0 + ly) : -1;
      s_cshared[i] = (lx == 0 && tx > 0) || (lx == bx && tx < a.T[0] - 1) || (ly == 0 && ty > 0) ||
                     (ly == by && ty < a.T[1] - 1);
    }
    for(int i = tid; i < 2 * C::LCELLS; i += C::THREADS)
    {
      const int L = i >= C::LCELLS, cell = i - L * C::LCELLS;
      const int lx = cell % C::CX, ly = cell / C::CX;
      int k = 0;
      for(int oy = 1; oy >= 0; --oy)
        for(int ox = 1; ox >= 0; --ox, ++k)
        {
          const int sx = lx - ox, sy = ly - oy;
          s_aoff[4 * i + k] = (sx >= 0 && sx < bx && sy >= 0 && sy < by)
                                ? (sx + BX * sy) * PS + K1 * (ox + SX * oy + SXY * L)
                                : -1;
        }
    }
    __syncthreads();
    copy_layer_async<C>(a, s_cxy, z0, s_raw, e, g);
    copy_layer_async<C>(a, s_cxy, z0 + 1, s_raw + C::LAYER, e, g);
    if constexpr(C::PP) fill_tables_async<C>(a, s_fd, s_sym, s_en, tid);
    for(int i = tid; i < 2 * C::LAYER; i += C::THREADS) s_acc[i] = 0.f;
    wait_async_all();
    convert_layer<C>(s_raw, s_f32, e, g);
    convert_layer<C>(s_raw + C::LAYER, s_f32 + C::LAYERF, e, g);
    __syncthreads();

    for(int j = 0; j < bz; ++j)
    {
      // layer j+2 streams in while this vertex layer is solved (its ring slot held layer j-1)
      const bool more = j + 2 <= bz;
      // (cell layer j+2 lands in the FP64 slot of layer j, converted at the end of iteration j-2)
      if(more) copy_layer_async<C>(a, s_cxy, z0 + j + 2, s_raw + (j % 2) * C::LAYER, e, g);
      // (PP: the slots hold this vertex layer's 1-D problems, copied during iteration j-1)
      const float *lo = s_f32 + (j % 2) * C::LAYERF, *hi = s_f32 + ((j + 1) % 2) * C::LAYERF;
      const bool active = px < bx && py < by && q < TPP;
      float *my = s_work + slot * PS;
      constexpr int ESL = C::ESLOT, HP = C::HPAD;
      const int slx = C::PP ? 3 * slot : px, sly = C::PP ? 3 * slot + 1 : BX + py,
                slz = C::PP ? 3 * slot + 2 : BX + BY + j;
      const float *ex = s_fd + slx * ESL, *ey = s_fd + sly * ESL, *ez = s_fd + slz * ESL;
      const bool sx = s_sym[slx], sy = s_sym[sly], sz = s_sym[slz];
      const float *lamx = ex + (sx ? C::EO_LAM : Entry<float, N>::LAM);
      const float *lamy = ey + (sy ? C::EO_LAM : Entry<float, N>::LAM);
      const float *lamz = ez + (sz ? C::EO_LAM : Entry<float, N>::LAM);
      if(active)
      {
        if(sx)
          mpass_x_from_layers<true, M0, K1, N, SX, SXY, NPAD, HP, NPT, TPP, C::RSTRIDE, CD>(my, lo, hi, ex, pm0, px, py, q);
        else
          mpass_x_from_layers<false, M0, K1, N, SX, SXY, NPAD, HP, NPT, TPP, C::RSTRIDE, CD>(my, lo, hi, ex, pm0, px, py, q);
      }
      pass_sync<C>();
      if(active)
      {
        if(sy) spass<true, true, M1, false, N, SX, SXY, NPAD, HP, 1, NPT, TPP>(my, ey, pm1, q, 1.f);
        else spass<false, true, M1, false, N, SX, SXY, NPAD, HP, 1, NPT, TPP>(my, ey, pm1, q, 1.f);
      }
      pass_sync<C>();
      if(active)
      {
        if(sz) zpass_solve<true, M2, N, SX, SXY, NPAD, HP, NPT, TPP>(my, lamx, lamy, ez, lamz, pm2, q);
        else zpass_solve<false, M2, N, SX, SXY, NPAD, HP, NPT, TPP>(my, lamx, lamy, ez, lamz, pm2, q);
      }
      pass_sync<C>();
      if(active)
      {
        if(sy) spass<true, false, M1, false, N, SX, SXY, NPAD, HP, 1, NPT, TPP>(my, ey, pm1, q, 1.f);
        else spass<false, false, M1, false, N, SX, SXY, NPAD, HP, 1, NPT, TPP>(my, ey, pm1, q, 1.f);
      }
      pass_sync<C>();
      if(active)
      {
        if(sx) spass<true, false, M0, true, N, SX, SXY, NPAD, HP, 0, NPT, TPP>(my, ex, pm0, q, a.omega);
        else spass<false, false, M0, true, N, SX, SXY, NPAD, HP, 0, NPT, TPP>(my, ex, pm0, q, a.omega);
      }
      __syncthreads();
      // PP: the passes are done with the slots; the next vertex layer's 1-D problems stream in
      // behind the accumulation and the write (waited for at the end of this iteration)
      if constexpr(C::PP)
        if(j + 1 < bz) fill_tables_async<C>(a, s_fd, s_sym, s_en + (j + 1) * C::NSLOT, tid);
      // accumulate per cell: the (up to) 4 patches of this layer touching the cell, fixed order
      float *alo = s_acc + (j % 2) * C::LAYER, *ahi = s_acc + ((j + 1) % 2) * C::LAYER;
      if(g < C::G)
      {
        constexpr int IT = (2 * C::LCELLS + C::G - 1) / C::G;
        float sum[IT], old[IT];
#pragma unroll
        for(int it = 0; it < IT; ++it)
        {
          const int cl = g + it * C::G;
          sum[it] = 0.f;
          if(cl < 2 * C::LCELLS)
          {
            const int4 o = reinterpret_cast<const int4 *>(s_aoff)[cl];
            if(o.x >= 0) sum[it] += s_work[o.x + e_patch];
            if(o.y >= 0) sum[it] += s_work[o.y + e_patch];
            if(o.z >= 0) sum[it] += s_work[o.z + e_patch];
            if(o.w >= 0) sum[it] += s_work[o.w + e_patch];
          }
        }
#pragma unroll
        for(int it = 0; it < IT; ++it)
        {
          const int cl = g + it * C::G, L = cl >= C::LCELLS, cell = cl - L * C::LCELLS;
          old[it] = cl < 2 * C::LCELLS ? (L ? ahi : alo)[cell * CD + e] : 0.f;
        }
#pragma unroll
        for(int it = 0; it < IT; ++it)
        {
          const int cl = g + it * C::G, L = cl >= C::LCELLS, cell = cl - L * C::LCELLS;
          if(cl < 2 * C::LCELLS) (L ? ahi : alo)[cell * CD + e] = old[it] + sum[it];
        }
      }
      __syncthreads();
      // cell layer j is complete: write it, clear its accumulator for layer j+2
      write_layer<C>(a, alo, item, j, z0 + j, j == 0 && tz > 0, s_cxy, s_cshared, e, g, true);
      if(more || C::PP) wait_async_all();
      if(more) convert_layer<C>(s_raw + (j % 2) * C::LAYER, s_f32 + (j % 2) * C::LAYERF, e, g);
      __syncthreads();
    }
    // last cell layer of the item
    write_layer<C>(a, s_acc + (bz % 2) * C::LAYER, item, bz, z0 + bz, tz < a.T[2] - 1, s_cxy, s_cshared,
                   e, g, false);
  }
}

// dst of the cells shared between items = sum of the items' halo partials (fixed order)
template<class C>
__global__ void fixup_kernel(StreamArgs a)
{
  constexpr int CD = C::CD;
  const int64_t n_cells = (int64_t)a.nc[0] * a.nc[1] * a.nc[2];
  for(int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_cells * CD;
      i += (int64_t)gridDim.x * blockDim.x)
  {
    const int64_t cell = i / CD;
    const int e = (int)(i % CD);
    const int cx = (int)(cell % a.nc[0]), cy = (int)((cell / a.nc[0]) % a.nc[1]),
              cz = (int)(cell / ((int64_t)a.nc[0] * a.nc[1]));
    int tx[2], lx[2], ty[2], ly[2], tz[2], lz[2];
    const int nx = tiles_of(cx, C::BX, a.T[0], tx, lx);
    const int ny = tiles_of(cy, C::BY, a.T[1], ty, ly);
    const int nz = tiles_of(cz, C::BZ, a.T[2], tz, lz);
    if(nx * ny * nz == 1) continue;  // written by the streaming kernel
    float s = 0.f;
    for(int kz = 0; kz < nz; ++kz)
      for(int ky = 0; ky < ny; ++ky)
        for(int kx = 0; kx < nx; ++kx)
        {
          const int item = tx[kx] + a.T[0] * (ty[ky] + a.T[1] * tz[kz]);
          const int lcell = lx[kx] + C::CX * ly[ky];
          s += a.halo[((size_t)item * (C::BZ + 1) * C::LCELLS + (size_t)lz[kz] * C::LCELLS + lcell) * CD + e];
        }
    if(a.ras)
      s /= multiplicity(cx, a.nc[0]) * multiplicity(cy, a.nc[1]) * multiplicity(cz, a.nc[2]);
    a.dst[(a.cell_start ? a.cell_start[cell] : cell * CD) + e] = double(s);
  }
}

// The same sums from a precomputed list of the shared cells: per record (10 int64) the first
// dst DoF of the cell, the partial count (low 32 bits) and the RAS scale bits (high 32 bits),
// then up to 8 halo offsets in the fixup_kernel order. Blocks of fixup_threads<C>() threads (128,
// or CD rounded up to a warp multiple when a cell has more than 128 DoFs) take
// fixup_threads / CD cells at a time, one thread per cell DoF; no index arithmetic per DoF.
constexpr int kFixRec = 10;

template<class C>
__host__ __device__ constexpr int fixup_threads()
{
  return C::CD <= 128 ? 128 : (C::CD + 31) / 32 * 32;
}

template<class C>
__global__ void __launch_bounds__(fixup_threads<C>()) fixup_list_kernel(const int64_t *__restrict__ rec, int64_t n,
                                                                        const float *__restrict__ halo,
                                                                        double *__restrict__ dst)
{
  constexpr int CD = C::CD;
  constexpr int PER = fixup_threads<C>() / CD;
  static_assert(PER >= 1, "a block covers at least one cell");
  const int lc = threadIdx.x / CD, e = threadIdx.x % CD;
  if(lc >= PER) return;
  for(int64_t r = (int64_t)blockIdx.x * PER + lc; r < n; r += (int64_t)gridDim.x * PER)
  {
    const int64_t *f = rec + r * kFixRec;
    const int64_t meta = f[1];
    const int count = int(meta & 0xffffffff);
    const float scale = __int_as_float(int(uint64_t(meta) >> 32));
    float s = 0.f;
    for(int k = 0; k < count; ++k) s += halo[f[2 + k] + e];
    dst[f[0] + e] = double(s * scale);
  }
}

}  // namespace stream
}  // namespace tpss
