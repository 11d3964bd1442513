// plane3d.cuh -- additive vertex-patch Schwarz smoother in 3D, FP32, streamed by columns, with the
// fast-diagonalization passes done on whole planes held in registers.
//
// Same mathematics and the same column streaming as stream3d.cuh (a work item is a column of
// BX x BY vertices and BZ vertex layers; cell layers staged in shared memory; per-cell
// accumulation; cells shared between items summed by the fix-up kernel), but a patch is solved by
// N = 2(k+1) threads of one warp, thread t owning a whole 2-D plane of the patch tensor (N x N
// values in registers):
//
//   A  plane z = t (read from the staged cell layers): S_x^T and S_y^T in registers, store
//   B  plane y = t: S_z^T, division by the eigenvalue sums, S_z, S_x in registers, store
//   C  plane z = t: S_y in registers, omega-scaled sum into the cell accumulator
//
// so the patch goes through shared memory twice (A -> B, B -> C) instead of once per pass, and a
// 1-D matrix loaded into registers serves N pencils. The three patches of a warp use only that
// warp's lanes, so A, B and C need warp barriers only. The shared-memory strides are chosen so
// that every warp-wide access of A, B and C (30 lanes: 3 patches x 10 planes for k = 4) touches
// 30 distinct banks.
//
// Measured on GB300 (3D DGQ4, 48^3 cells, one launch): ~350 shared-memory wavefronts per patch
// against ~860 for the pencil passes of stream3d.cuh, but a plane of 100 values per thread takes
// 255 registers, so an SM holds 8 warps; the kernel is latency-bound (issue active ~25 %, stalls on
// fixed-latency dependencies and instruction fetch) and runs at 0.70 ms against 0.50 ms. It stays
// a decomposition the autotuner measures (stream variants 6 and 7).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "stream3d.cuh"

namespace tpss
{
namespace stream
{
// smallest m >= n with m = r (mod 32)
__host__ __device__ constexpr int up_to_residue(int n, int r) { return n + (((r - n) % 32) + 32) % 32; }

template<int K1_, int BY_, int BZ_>
struct PCfg
{
  static_assert(K1_ == 5, "the plane kernel is laid out for k = 4 (10 x 10 x 10 patches)");
  static constexpr bool PLANE = true;
  static constexpr int K1 = K1_, N = 2 * K1, H = K1;
  static constexpr int PPW = 32 / N;                  // patches per warp (3)
  static constexpr int BX = PPW, BY = BY_, BZ = BZ_;  // a warp solves one row of BX patches
  static constexpr int NPATCH = BX * BY;
  static constexpr int THREADS = 32 * BY;
  static constexpr int CD = K1 * K1 * K1;
  static constexpr int CX = BX + 1, CY = BY + 1;
  static constexpr int LCELLS = CX * CY;
  static constexpr int LAYER = LCELLS * CD;
  static constexpr int G = THREADS / CD;
  static_assert(G >= 1, "need at least one thread per cell DoF");
  static constexpr int RSTRIDE = CX * CD;  // rows of cells unpadded: cell index lx + CX ly
  // FP32 cell layers and accumulator layers: stride = 16 (mod 32), so that the lanes of the
  // planes z < k+1 (lower cell layer) and z >= k+1 (upper) fall into disjoint banks
  static constexpr int LAYERF = up_to_residue(LAYER, 16);
  // 1-D tables: even/odd [Se^T][So^T][Se][So][lambda] with rows padded to HPAD, full [S^T][S][lambda]
  static constexpr int HPAD = ((H + 3) / 4) * 4;
  static constexpr int EO_LAM = 4 * H * HPAD;
  static constexpr int NPAD = Entry<float, N>::NPAD;
  static constexpr int ES = Entry<float, N>::size;
  // patch work buffer: value (x, y, z) at y + WX x + WZ z; patch p of a warp at p * PS. With
  // WZ = 111 = 15 and PS = 10 (mod 32) the lanes (p, t) of a plane access (t along z: 15 t + 10 p)
  // and of a y-plane access (t along y: t + 10 p) each hit 30 distinct banks
  static constexpr int WX = N, WZ = 111;
  static constexpr int PS = up_to_residue(WZ * (N - 1) + WX * (N - 1) + N, 10);
  // shared memory carve-up (floats)
  static constexpr int OFF_TAB = 0;                                     // cxy, cshared (ints)
  static constexpr int OFF_RAW = ((2 * LCELLS + 3) / 4) * 4;            // one FP64 landing layer
  static constexpr int OFF_F32 = OFF_RAW + 2 * LAYER;                   // 2 FP32 cell layers
  static constexpr int OFF_ACC = OFF_F32 + 2 * LAYERF;                  // 2 accumulator layers
  static constexpr int OFF_WORK = OFF_ACC + 2 * LAYERF;                 // NPATCH patch tensors
  static constexpr int FLOATS = OFF_WORK + NPATCH * PS;
  static_assert(2 * LAYERF >= 2 * LAYER, "the accumulator doubles as the second landing layer");
  static constexpr size_t smem_bytes() { return (size_t)FLOATS * 4; }
  static_assert((size_t)FLOATS * 4 <= 227 * 1024, "shared memory per CTA exceeds 227 KB");
};

// One h x h block of an even/odd 1-D table in registers: c[k][i] = row k of block par (Se^T for
// par 0, So^T for par 1). The backward passes use the same numbers transposed (Se = (Se^T)^T), so
// one block (h^2 = 25 floats for k = 4) is live at a time.
template<int H, int HPAD>
__device__ __forceinline__ void load_block(const float *__restrict__ E, int par, float (&c)[H][H])
{
  static_assert(HPAD % 4 == 0 && H <= HPAD, "rows are read as float4");
#pragma unroll
  for(int k = 0; k < H; ++k)
  {
    // the padded row (HPAD floats, 16-byte aligned) is read whole
    const float *row = E + (par * H + k) * HPAD;
    float tmp[HPAD];
#pragma unroll
    for(int i4 = 0; i4 < HPAD / 4; ++i4)
    {
      const float4 q = __ldg(reinterpret_cast<const float4 *>(row) + i4);
      tmp[4 * i4] = q.x;
      tmp[4 * i4 + 1] = q.y;
      tmp[4 * i4 + 2] = q.z;
      tmp[4 * i4 + 3] = q.w;
    }
#pragma unroll
    for(int i = 0; i < H; ++i) c[k][i] = tmp[i];
  }
}

// out[k] = sum_i c[k][i] in[i] (TR: sum_i c[i][k] in[i]) on one pencil pair, in place: the inputs
// are read from positions ip(i), the outputs written to op(k) after all are formed
template<int H, bool TR, int IB, int IS, int OB, int OS>
__device__ __forceinline__ void block_pair(float2 (&r)[2 * H], const float (&c)[H][H])
{
  float2 o[H];
#pragma unroll
  for(int k = 0; k < H; ++k)
  {
    o[k] = __fmul2_rn(bcast2(TR ? c[0][k] : c[k][0]), r[IB]);
#pragma unroll
    for(int i = 1; i < H; ++i) o[k] = __ffma2_rn(bcast2(TR ? c[i][k] : c[k][i]), r[IB + IS * i], o[k]);
  }
#pragma unroll
  for(int k = 0; k < H; ++k) r[OB + OS * k] = o[k];
}

// Forward even/odd transform of the N/2 pencil pairs of a plane, in place: r_i + r_{n-1-i} at i and
// r_i - r_{n-1-i} at n-1-i, then Se^T (even sums) to [0, h) and So^T (odd differences, read
// mirrored) to [h, n)
template<int H, int HPAD>
__device__ __forceinline__ void plane_eo_fwd(float2 (&v)[H][2 * H], const float *__restrict__ E)
{
  const float2 m1 = bcast2(-1.f);
#pragma unroll
  for(int a = 0; a < H; ++a)
#pragma unroll
    for(int i = 0; i < H; ++i)
    {
      const float2 x = v[a][i], y = v[a][2 * H - 1 - i];
      v[a][i] = __fadd2_rn(x, y);
      v[a][2 * H - 1 - i] = __ffma2_rn(y, m1, x);
    }
  float c[H][H];
  load_block<H, HPAD>(E, 0, c);
#pragma unroll
  for(int a = 0; a < H; ++a) block_pair<H, false, 0, 1, 0, 1>(v[a], c);
  load_block<H, HPAD>(E, 1, c);
#pragma unroll
  for(int a = 0; a < H; ++a) block_pair<H, false, 2 * H - 1, -1, H, 1>(v[a], c);
}

// Backward: E_i = Se t_e to i, O_i = So t_o to n-1-i, then u_i = E_i + O_i, u_{n-1-i} = E_i - O_i
template<int H, int HPAD>
__device__ __forceinline__ void plane_eo_bwd(float2 (&v)[H][2 * H], const float *__restrict__ E)
{
  float c[H][H];
  load_block<H, HPAD>(E, 0, c);
#pragma unroll
  for(int a = 0; a < H; ++a) block_pair<H, true, 0, 1, 0, 1>(v[a], c);
  load_block<H, HPAD>(E, 1, c);
#pragma unroll
  for(int a = 0; a < H; ++a) block_pair<H, true, H, 1, 2 * H - 1, -1>(v[a], c);
  const float2 m1 = bcast2(-1.f);
#pragma unroll
  for(int a = 0; a < H; ++a)
#pragma unroll
    for(int i = 0; i < H; ++i)
    {
      const float2 e = v[a][i], o = v[a][2 * H - 1 - i];
      v[a][i] = __fadd2_rn(e, o);
      v[a][2 * H - 1 - i] = __ffma2_rn(o, m1, e);
    }
}

// table pointers of one direction's 1-D problem
struct DirTab
{
  bool sym;
  const float *eo;    // even/odd entry (sym)
  const float *full;  // full entry (!sym)
  const float *lam;   // eigenvalues, transformed order
};

template<class C>
__device__ __forceinline__ DirTab dir_tab(const StreamArgs &a, int en)
{
  DirTab d;
  d.sym = __ldg(a.sym + en) != 0;
  d.eo = a.fd_eo + (size_t)en * a.es_eo;
  d.full = a.fd + (size_t)en * C::ES;
  d.lam = d.sym ? d.eo + C::EO_LAM : d.full + Entry<float, C::N>::LAM;
  return d;
}

// 16-byte read-only load that the compiler may not merge with the same load for another pencil
// pair (merged, the whole n x n matrix would stay live in registers across the pairs)
__device__ __forceinline__ float4 ld_nc_v4(const float *p)
{
  float4 q;
  asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(q.x), "=f"(q.y), "=f"(q.z), "=f"(q.w) : "l"(p));
  return q;
}

// Full n x n pass (1-D problems without mirror symmetry, at the domain boundary) on the pencil
// pairs of a plane, in registers: out = B in, column m of B read per pair (cols points at the
// transposed matrix, rows padded to NPAD: row m of cols = column m of B)
template<int N, int NPAD>
__device__ __forceinline__ void full_pass(float2 (&v)[N / 2][N], const float *__restrict__ cols)
{
  static_assert(NPAD % 4 == 0, "rows are read as float4");
#pragma unroll
  for(int a = 0; a < N / 2; ++a)
  {
    float2 o[N];
#pragma unroll
    for(int m = 0; m < N; ++m)
    {
      float c[NPAD];
#pragma unroll
      for(int i4 = 0; i4 < NPAD / 4; ++i4)
      {
        const float4 q = ld_nc_v4(cols + m * NPAD + 4 * i4);
        c[4 * i4] = q.x;
        c[4 * i4 + 1] = q.y;
        c[4 * i4 + 2] = q.z;
        c[4 * i4 + 3] = q.w;
      }
#pragma unroll
      for(int k = 0; k < N; ++k)
        o[k] = m == 0 ? __fmul2_rn(bcast2(c[k]), v[a][0]) : __ffma2_rn(bcast2(c[k]), v[a][m], o[k]);
    }
#pragma unroll
    for(int k = 0; k < N; ++k) v[a][k] = o[k];
  }
}

// one 1-D pass over the N/2 pencil pairs of a plane: even/odd (fwd: S^T, else S) or full, in
// registers; the full pass reads S^T's columns from the S rows and S's columns from the S^T rows
template<class C>
__device__ __forceinline__ void plane_pass(float2 (&v)[C::N / 2][C::N], const DirTab &d, bool fwd)
{
  constexpr int N = C::N;
  if(d.sym)
  {
    if(fwd)
      plane_eo_fwd<C::H, C::HPAD>(v, d.eo);
    else
      plane_eo_bwd<C::H, C::HPAD>(v, d.eo);
  }
  else
    full_pass<N, C::NPAD>(v, d.full + (fwd ? Entry<float, N>::S : Entry<float, N>::ST));
}

// 2 x 2 block transpose of a pair-packed plane, in place: before, pair v[a][b] holds elements
// (2a, b) and (2a+1, b); after, v[b'][m] holds (m, 2b') and (m, 2b'+1)
template<int N>
__device__ __forceinline__ void repack(float2 (&v)[N / 2][N])
{
  float2 w[N / 2][N];
#pragma unroll
  for(int a = 0; a < N / 2; ++a)
#pragma unroll
    for(int b = 0; b < N / 2; ++b)
    {
      const float2 p = v[a][2 * b], q = v[a][2 * b + 1];
      w[b][2 * a] = make_float2(p.x, q.x);
      w[b][2 * a + 1] = make_float2(p.y, q.y);
    }
#pragma unroll
  for(int a = 0; a < N / 2; ++a)
#pragma unroll
    for(int m = 0; m < N; ++m) v[a][m] = w[a][m];
}

// Moves of a plane between registers and shared memory (k = 4 layout of PCfg):
//   A in:  plane z = t from the staged cell layers, pairs of y rows: v[a][x] = (y = 2a, 2a + 1)
//   A out / C in: plane z = t of the patch buffer, pairs of x columns: v[b][y] = (x = 2b, 2b + 1)
//   B in:  plane y = t, pairs of x columns: v[b][z] = (x = 2b, 2b + 1)
//   B out: plane y = t, pairs of z rows: v[a][x] = (z = 2a, 2a + 1)
template<class C>
__device__ __forceinline__ void plane_load_layers(float2 (&v)[C::N / 2][C::N], const float *lay)
{
  constexpr int K1 = C::K1, N = C::N, CD = C::CD, RS = C::RSTRIDE;
#pragma unroll
  for(int a2 = 0; a2 < N / 2; ++a2)
#pragma unroll
    for(int x = 0; x < N; ++x)
    {
      const int y0 = 2 * a2, y1 = 2 * a2 + 1;
      v[a2][x].x = lay[(x / K1) * CD + (y0 / K1) * RS + x % K1 + K1 * (y0 % K1)];
      v[a2][x].y = lay[(x / K1) * CD + (y1 / K1) * RS + x % K1 + K1 * (y1 % K1)];
    }
}

// plane z = t <-> v[b][y] = (x = 2b, 2b + 1): p = patch buffer + WZ t
template<class C, bool STORE>
__device__ __forceinline__ void plane_z(float2 (&v)[C::N / 2][C::N], float *p)
{
  constexpr int N = C::N, WX = C::WX;
#pragma unroll
  for(int b = 0; b < N / 2; ++b)
#pragma unroll
    for(int y = 0; y < N; ++y)
    {
      if constexpr(STORE)
      {
        p[y + WX * (2 * b)] = v[b][y].x;
        p[y + WX * (2 * b + 1)] = v[b][y].y;
      }
      else
      {
        v[b][y].x = p[y + WX * (2 * b)];
        v[b][y].y = p[y + WX * (2 * b + 1)];
      }
    }
}

// plane y = t -> v[b][z] = (x = 2b, 2b + 1): p = patch buffer + t
template<class C>
__device__ __forceinline__ void plane_y_load(float2 (&v)[C::N / 2][C::N], const float *p)
{
  constexpr int N = C::N, WX = C::WX, WZ = C::WZ;
#pragma unroll
  for(int b = 0; b < N / 2; ++b)
#pragma unroll
    for(int z = 0; z < N; ++z)
    {
      v[b][z].x = p[WX * (2 * b) + WZ * z];
      v[b][z].y = p[WX * (2 * b + 1) + WZ * z];
    }
}

// v[a][x] = (z = 2a, 2a + 1) -> plane y = t
template<class C>
__device__ __forceinline__ void plane_y_store(const float2 (&v)[C::N / 2][C::N], float *p)
{
  constexpr int N = C::N, WX = C::WX, WZ = C::WZ;
#pragma unroll
  for(int a2 = 0; a2 < N / 2; ++a2)
#pragma unroll
    for(int x = 0; x < N; ++x)
    {
      p[WX * x + WZ * (2 * a2)] = v[a2][x].x;
      p[WX * x + WZ * (2 * a2 + 1)] = v[a2][x].y;
    }
}

// 1 / (lambda_x + lambda_y + lambda_z) on the transformed plane y = t, v[b][z] = (x = 2b, 2b + 1)
template<class C>
__device__ __forceinline__ void plane_scale(float2 (&v)[C::N / 2][C::N], const DirTab &dx, const DirTab &dy,
                                            const DirTab &dz, int t)
{
  constexpr int N = C::N;
  const float ly = __ldg(dy.lam + t);
  float lz[N];
#pragma unroll
  for(int z = 0; z < N; ++z) lz[z] = __ldg(dz.lam + z) + ly;
#pragma unroll
  for(int b = 0; b < N / 2; ++b)
  {
    const float lx0 = __ldg(dx.lam + 2 * b), lx1 = __ldg(dx.lam + 2 * b + 1);
#pragma unroll
    for(int z = 0; z < N; ++z)
      v[b][z] = __fmul2_rn(v[b][z], make_float2(rcp_approx(lx0 + lz[z]), rcp_approx(lx1 + lz[z])));
  }
}

template<class C>
__global__ void __launch_bounds__(C::THREADS, 1) plane_kernel(StreamArgs a)
{
  constexpr int K1 = C::K1, N = C::N, CD = C::CD, H2 = N / 2;
  constexpr int BX = C::BX, BY = C::BY, BZ = C::BZ;
  constexpr int WZ = C::WZ, PS = C::PS, RS = C::RSTRIDE, LF = C::LAYERF;
  extern __shared__ __align__(16) float sm[];
  int *s_cxy = reinterpret_cast<int *>(sm + C::OFF_TAB);
  int *s_cshared = s_cxy + C::LCELLS;
  double *s_raw = reinterpret_cast<double *>(sm + C::OFF_RAW);
  float *s_f32 = sm + C::OFF_F32;
  float *s_acc = sm + C::OFF_ACC;
  float *s_work = sm + C::OFF_WORK;
  const int tid = threadIdx.x;
  const int lane = tid % 32, py = tid / 32;
  const int px = lane / N, t = lane % N;  // patch of the warp's row, plane index
  const bool lane_ok = lane < BX * N;
  float *my = s_work + (py * BX + (lane_ok ? px : 0)) * PS;
  const int e = tid % CD, g = tid / CD;
  const int n_items = a.T[0] * a.T[1] * a.T[2];

  for(int item = a.item_begin + blockIdx.x; item < a.item_end && item < n_items; item += gridDim.x)
  {
    const int tx = item % a.T[0], ty = (item / a.T[0]) % a.T[1], tz = item / (a.T[0] * a.T[1]);
    const int bx = min(BX, a.nc[0] - 1 - BX * tx), by = min(BY, a.nc[1] - 1 - BY * ty);
    const int bz = min(BZ, a.nc[2] - 1 - BZ * tz);
    const int x0 = BX * tx, y0 = BY * ty, z0 = BZ * tz;
    __syncthreads();  // the previous item is done with shared memory
    for(int i = tid; i < C::LCELLS; i += C::THREADS)
    {
      const int lx = i % C::CX, ly = i / C::CX;
      s_cxy[i] = (lx <= bx && ly <= by) ? (x0 + lx) + a.nc[0] * (y0 + ly) : -1;
      s_cshared[i] = (lx == 0 && tx > 0) || (lx == bx && tx < a.T[0] - 1) || (ly == 0 && ty > 0) ||
                     (ly == by && ty < a.T[1] - 1);
    }
    __syncthreads();
    // the first two cell layers land in the FP64 slot and in the (not yet used) accumulator
    copy_layer_async<C>(a, s_cxy, z0, s_raw, e, g);
    copy_layer_async<C>(a, s_cxy, z0 + 1, reinterpret_cast<double *>(s_acc), e, g);
    wait_async_all();
    convert_layer<C>(s_raw, s_f32, e, g);
    convert_layer<C>(reinterpret_cast<double *>(s_acc), s_f32 + LF, e, g);
    __syncthreads();
    for(int i = tid; i < 2 * LF; i += C::THREADS) s_acc[i] = 0.f;
    // 1-D tables of the patch's x and y vertices (fixed for the item)
    const bool active_xy = lane_ok && px < bx && py < by;
    DirTab dx{}, dy{};
    if(active_xy)
    {
      dx = dir_tab<C>(a, a.vfd[0][x0 + 1 + px]);
      dy = dir_tab<C>(a, a.vfd[1][y0 + 1 + py]);
    }
    __syncthreads();

    for(int j = 0; j < bz; ++j)
    {
      const bool more = j + 2 <= bz;
      if(more) copy_layer_async<C>(a, s_cxy, z0 + j + 2, s_raw, e, g);
      const float *lo = s_f32 + (j % 2) * LF, *hi = s_f32 + ((j + 1) % 2) * LF;
      float *alo = s_acc + (j % 2) * LF, *ahi = s_acc + ((j + 1) % 2) * LF;
      float2 v[H2][N];
      const DirTab dz = active_xy ? dir_tab<C>(a, a.vfd[2][z0 + 1 + j]) : DirTab{};
      float *pz = my + WZ * t, *pyp = my + t;
      const float *lay = (t < K1 ? lo : hi) + px * CD + py * RS + K1 * K1 * (t % K1);
      // Six 1-D passes as a loop (one copy of the pass code keeps the kernel small for the
      // instruction caches): step 0 S_x^T, 1 S_y^T (plane z = t), 2 S_z^T and the eigenvalue
      // division, 3 S_z, 4 S_x (plane y = t), 5 S_y (plane z = t); v moves through the patch
      // buffer before steps 0, 2 and 5
#pragma unroll 1
      for(int st = 0; st < 6; ++st)
      {
        if(st == 0 && active_xy) plane_load_layers<C>(v, lay);
        if(st == 2)
        {
          if(active_xy) plane_z<C, true>(v, pz);
          __syncwarp();
          if(active_xy) plane_y_load<C>(v, pyp);
        }
        if(st == 5)
        {
          if(active_xy) plane_y_store<C>(v, pyp);
          __syncwarp();
          if(active_xy) plane_z<C, false>(v, pz);
        }
        if(active_xy)
        {
          const DirTab &d = (st == 0 || st == 4) ? dx : (st == 1 || st == 5) ? dy : dz;
          plane_pass<C>(v, d, st <= 2);
          if(st == 2) plane_scale<C>(v, dx, dy, dz, t);
          if(st == 0 || st == 3) repack<N>(v);
        }
      }
      float2 (&w)[H2][N] = v;  // v[b][y] = (x = 2b, x = 2b + 1) of plane z = t
      // omega-scaled sum into the accumulator, one of the patch's 2 x 2 cells per sub-step:
      // in sub-step (cx, cy) patch (px, py) adds to cell (px + cx, py + cy), so no two patches
      // write a cell at once and every cell sums its patches in a fixed order
      float *acc_t = (t < K1 ? alo : ahi) + px * CD + py * RS + K1 * K1 * (t % K1);
#pragma unroll
      for(int s = 0; s < 4; ++s)
      {
        const int cx = s & 1, cy = s >> 1;
        if(active_xy)
        {
          float old[K1 * K1];
#pragma unroll
          for(int ey = 0; ey < K1; ++ey)
#pragma unroll
            for(int ex = 0; ex < K1; ++ex) old[ex + K1 * ey] = acc_t[cx * CD + cy * RS + ex + K1 * ey];
#pragma unroll
          for(int ey = 0; ey < K1; ++ey)
#pragma unroll
            for(int ex = 0; ex < K1; ++ex)
            {
              const int x = K1 * cx + ex, y = K1 * cy + ey;
              const float u = (x & 1) ? w[x >> 1][y].y : w[x >> 1][y].x;
              acc_t[cx * CD + cy * RS + ex + K1 * ey] = fmaf(a.omega, u, old[ex + K1 * ey]);
            }
        }
        __syncthreads();
      }
      // cell layer j is complete: write it, clear its accumulator for layer j + 2
      write_layer<C>(a, alo, item, j, z0 + j, j == 0 && tz > 0, s_cxy, s_cshared, e, g, true);
      if(more)
      {
        wait_async_all();
        convert_layer<C>(s_raw, s_f32 + (j % 2) * LF, e, g);
      }
      __syncthreads();
    }
    write_layer<C>(a, s_acc + (bz % 2) * LF, item, bz, z0 + bz, tz < a.T[2] - 1, s_cxy, s_cshared, e, g,
                   false);
  }
}

}  // namespace stream
}  // namespace tpss
