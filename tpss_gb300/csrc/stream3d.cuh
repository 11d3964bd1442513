// stream3d.cuh -- additive vertex-patch Schwarz smoother in 3D, FP32, streamed by columns.
//
// Same mathematics as one SchwarzPreconditioner::vmult with additive vertex patches
// (preconditioner/schwarz_preconditioner.templates.h:585-688): dst = omega sum_j R_j^T A_j^-1
// R_j src, A_j^-1 by fast diagonalization.  Instead of one launch per color, which streams
// src and dst through HBM once per color, the work is organized for GB300:
//
//  - a work item is a column of BX x BY vertices (patches) and BZ vertex layers; persistent
//    CTAs take items round-robin (one CTA per SM);
//  - the item's cells are staged layer by layer in shared memory (FP32), the next layer is
//    prefetched into registers while the current vertex layer is solved;
//  - the 16 patches of a vertex layer are solved together; each thread owns NPT pencils of one
//    patch, so every 1-D matrix row read from shared memory feeds NPT pencils;
//  - patch results are summed in a shared-memory accumulator (x/y parity sub-steps, so no
//    two patches write the same cell at once); a cell layer is final once the vertex layer
//    above it is done and is written out once: cells owned by the item go straight to dst,
//    cells on the item's faces shared with neighbouring items go to a halo buffer (scratch),
//    which a fix-up kernel sums in a fixed order -- the result is deterministic.
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

template<int K1_, int BX_, int BY_, int BZ_, int NPT_>
struct SCfg
{
  static constexpr int K1 = K1_, BX = BX_, BY = BY_, BZ = BZ_, NPT = NPT_;
  static constexpr int N = 2 * K1;
  static constexpr int NLOC = N * N * N;
  static constexpr int NPENCIL = N * N;
  static_assert(NPENCIL % NPT == 0, "pencils must split evenly");
  static constexpr int TPP = NPENCIL / NPT;  // threads per patch
  static constexpr int CD = K1 * K1 * K1;     // DoFs per cell
  static constexpr int NPATCH = BX * BY;      // patches per vertex layer
  static constexpr int THREADS = NPATCH * TPP;
  static constexpr int CX = BX + 1, CY = BY + 1;
  static constexpr int LCELLS = CX * CY;  // cells per cell layer of a column
  static constexpr int LAYER = LCELLS * CD;
  static constexpr int ES = Entry<float, N>::size;
  static constexpr int NPAD = Entry<float, N>::NPAD;
  // shared memory carve-up (in floats; the staged FP64 cell layers take two floats per value)
  static constexpr int OFF_FD = 0;                                   // (BX + BY + BZ) entries
  static constexpr int OFF_RAW = ((OFF_FD + (BX + BY + BZ) * ES + 3) / 4) * 4;  // 3 FP64 layers
  static constexpr int OFF_ACC = OFF_RAW + 3 * 2 * LAYER;            // 2 FP32 layers
  static constexpr int OFF_WORK = OFF_ACC + 2 * LAYER;               // NPATCH patches
  static constexpr int FLOATS = OFF_WORK + NPATCH * NLOC;
  static constexpr size_t smem_bytes() { return (size_t)FLOATS * 4; }
};

struct StreamArgs
{
  const double *__restrict__ src;
  double *__restrict__ dst;
  float *__restrict__ halo;
  const int64_t *__restrict__ cell_start;  // nullptr: lexicographic cells
  const float *__restrict__ fd;            // FP32 FD table
  const int32_t *__restrict__ vfd[3];      // FD entry of vertex v per direction
  int nc[3];                               // cells per direction
  int T[3];                                // items per direction
  float omega;
  int ras;                                 // scale by 1/multiplicity
};

// tiles (t, local index l) of direction d that contain cell c; returns the count (1 or 2)
__device__ __forceinline__ int tiles_of(int c, int W, int T, int *t, int *l)
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

__device__ __forceinline__ float multiplicity(int c, int n)
{
  return float((c >= 1 ? 1 : 0) + (c + 1 <= n - 1 ? 1 : 0));
}

template<int N, int NPAD, int DIR, int NPT, int TPP>
__device__ __forceinline__ void mpass(float *__restrict__ data, const float *__restrict__ B, int q,
                                      float scale)
{
  constexpr int stride = cpow(N, DIR);
  float r[NPT][N];
  int base[NPT];
#pragma unroll
  for(int j = 0; j < NPT; ++j)
  {
    base[j] = fd::pencil_base<3, N, DIR>(q + j * TPP);
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
    for(int j = 0; j < NPT; ++j) data[base[j] + i * stride] = acc[j] * scale;
  }
}

// direction 2, forward: S^T along z, then division by the eigenvalue sums
// lambda_x[i0] + lambda_y[i1] + lambda_z[i2]
template<int N, int NPAD, int NPT, int TPP>
__device__ __forceinline__ void mpass_divide(float *__restrict__ data, const float *__restrict__ ex,
                                             const float *__restrict__ ey, const float *__restrict__ ez,
                                             int q)
{
  constexpr int stride = N * N;
  float r[NPT][N];
  float lxy[NPT];
#pragma unroll
  for(int j = 0; j < NPT; ++j)
  {
    const int p = q + j * TPP;  // pencil along z: i0 + N i1
    lxy[j] = ex[Entry<float, N>::LAM + p % N] + ey[Entry<float, N>::LAM + p / N];
#pragma unroll
    for(int m = 0; m < N; ++m) r[j][m] = data[p + m * stride];
  }
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
    const float lz = ez[Entry<float, N>::LAM + i];
#pragma unroll
    for(int j = 0; j < NPT; ++j) data[q + j * TPP + i * stride] = acc[j] / (lxy[j] + lz);
  }
}

template<class C>
__device__ __forceinline__ int64_t cell_first(const StreamArgs &a, int cx, int cy, int cz)
{
  const int64_t cell = cx + (int64_t)a.nc[0] * (cy + (int64_t)a.nc[1] * cz);
  return a.cell_start ? a.cell_start[cell] : cell * C::CD;
}

// asynchronous copy (cp.async, 8 bytes) of cell layer cz of the column (cells x in
// [x0, x0+bx], y in [y0, y0+by]) into the FP64 staging buffer; cells outside are zero-filled
template<class C>
__device__ __forceinline__ void copy_layer_async(const StreamArgs &a, int x0, int y0, int bx, int by,
                                                 int cz, double *raw)
{
  for(int i = threadIdx.x; i < C::LAYER; i += C::THREADS)
  {
    const int cell = i / C::CD, e = i % C::CD;
    const int lx = cell % C::CX, ly = cell / C::CX;
    if(lx <= bx && ly <= by)
    {
      const double *g = a.src + cell_first<C>(a, x0 + lx, y0 + ly, cz) + e;
      const unsigned saddr = (unsigned)__cvta_generic_to_shared(raw + i);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(saddr), "l"(g) : "memory");
    }
    else
      raw[i] = 0.0;
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

__device__ __forceinline__ void wait_async_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

template<class C>
__global__ void __launch_bounds__(C::THREADS, 1) stream_kernel(StreamArgs a)
{
  constexpr int K1 = C::K1, N = C::N, NLOC = C::NLOC, CD = C::CD, ES = C::ES, NPAD = C::NPAD;
  constexpr int BX = C::BX, BY = C::BY, BZ = C::BZ, TPP = C::TPP, NPT = C::NPT;
  extern __shared__ __align__(16) float sm[];
  float *s_fd = sm + C::OFF_FD;
  double *s_raw = reinterpret_cast<double *>(sm + C::OFF_RAW);
  float *s_acc = sm + C::OFF_ACC;
  float *s_work = sm + C::OFF_WORK;
  const int tid = threadIdx.x;
  const int slot = tid / TPP, q = tid % TPP;  // patch slot (px + BX py) and pencil group
  const int px = slot % BX, py = slot / BX;
  const int n_items = a.T[0] * a.T[1] * a.T[2];

  for(int item = blockIdx.x; item < n_items; item += gridDim.x)
  {
    const int tx = item % a.T[0], ty = (item / a.T[0]) % a.T[1], tz = item / (a.T[0] * a.T[1]);
    // vertices of the item: v_d in [1 + W t, min(W (t+1), n_d - 1)]
    const int bx = min(BX, a.nc[0] - 1 - BX * tx), by = min(BY, a.nc[1] - 1 - BY * ty);
    const int bz = min(BZ, a.nc[2] - 1 - BZ * tz);
    const int x0 = BX * tx, y0 = BY * ty, z0 = BZ * tz;  // first cell of the item
    __syncthreads();  // previous item done with shared memory
    // FD entries: x vertices, y vertices, z vertices of the item
    for(int i = tid; i < (BX + BY + BZ) * ES; i += C::THREADS)
    {
      const int s = i / ES, o = i % ES;
      int e = -1;
      if(s < BX) { if(s < bx) e = a.vfd[0][x0 + 1 + s]; }
      else if(s < BX + BY) { if(s - BX < by) e = a.vfd[1][y0 + 1 + (s - BX)]; }
      else if(s - BX - BY < bz) e = a.vfd[2][z0 + 1 + (s - BX - BY)];
      s_fd[i] = e >= 0 ? a.fd[(size_t)e * ES + o] : 0.f;
    }
    // cell layers 0 and 1 of the item, zero accumulators
    copy_layer_async<C>(a, x0, y0, bx, by, z0, s_raw);
    copy_layer_async<C>(a, x0, y0, bx, by, z0 + 1, s_raw + C::LAYER);
    for(int i = tid; i < 2 * C::LAYER; i += C::THREADS) s_acc[i] = 0.f;
    wait_async_all();
    __syncthreads();

    for(int j = 0; j < bz; ++j)
    {
      // vertex layer j: cell layers j (ring slot j%3 / acc j%2) and j+1
      // layer j+2 streams in while this vertex layer is solved (its ring slot held layer j-1)
      const bool more = j + 2 <= bz;
      if(more) copy_layer_async<C>(a, x0, y0, bx, by, z0 + j + 2, s_raw + ((j + 2) % 3) * C::LAYER);
      const double *lo = s_raw + (j % 3) * C::LAYER, *hi = s_raw + ((j + 1) % 3) * C::LAYER;
      // gather the BX x BY patches of this layer into the work buffers
      for(int i = tid; i < C::NPATCH * NLOC; i += C::THREADS)
      {
        const int s = i / NLOC, r = i % NLOC;
        const int sx = s % BX, sy = s / BX;
        const int ix = r % N, iy = (r / N) % N, iz = r / (N * N);
        const int ox = ix / K1, oy = iy / K1, oz = iz / K1;
        const int e = (ix % K1) + K1 * ((iy % K1) + K1 * (iz % K1));
        const double *layer = oz ? hi : lo;
        s_work[i] = (sx < bx && sy < by) ? float(layer[((sx + ox) + C::CX * (sy + oy)) * CD + e]) : 0.f;
      }
      __syncthreads();
      const bool active = px < bx && py < by;
      float *my = s_work + slot * NLOC;
      const float *ex = s_fd + px * ES, *ey = s_fd + (BX + py) * ES, *ez = s_fd + (BX + BY + j) * ES;
      if(active) mpass<N, NPAD, 0, NPT, TPP>(my, ex + Entry<float, N>::ST, q, 1.f);
      __syncthreads();
      if(active) mpass<N, NPAD, 1, NPT, TPP>(my, ey + Entry<float, N>::ST, q, 1.f);
      __syncthreads();
      if(active) mpass_divide<N, NPAD, NPT, TPP>(my, ex, ey, ez, q);
      __syncthreads();
      if(active) mpass<N, NPAD, 2, NPT, TPP>(my, ez + Entry<float, N>::S, q, 1.f);
      __syncthreads();
      if(active) mpass<N, NPAD, 1, NPT, TPP>(my, ey + Entry<float, N>::S, q, 1.f);
      __syncthreads();
      if(active) mpass<N, NPAD, 0, NPT, TPP>(my, ex + Entry<float, N>::S, q, a.omega);
      __syncthreads();
      // accumulate: four x/y parity classes, patches within a class do not share cells
      float *alo = s_acc + (j % 2) * C::LAYER, *ahi = s_acc + ((j + 1) % 2) * C::LAYER;
#pragma unroll 1
      for(int par = 0; par < 4; ++par)
      {
        for(int i = tid; i < C::NPATCH * NLOC; i += C::THREADS)
        {
          const int s = i / NLOC, r = i % NLOC;
          const int sx = s % BX, sy = s / BX;
          if((sx & 1) + 2 * (sy & 1) != par || sx >= bx || sy >= by) continue;
          const int ix = r % N, iy = (r / N) % N, iz = r / (N * N);
          const int ox = ix / K1, oy = iy / K1, oz = iz / K1;
          const int e = (ix % K1) + K1 * ((iy % K1) + K1 * (iz % K1));
          float *layer = oz ? ahi : alo;
          layer[((sx + ox) + C::CX * (sy + oy)) * CD + e] += s_work[i];
        }
        __syncthreads();
      }
      // cell layer j is complete: write it out, clear its accumulator for layer j+2
      {
        const int lz = j, cz = z0 + j;
        const bool zshared = (lz == 0 && tz > 0);  // lz == bz handled after the loop
        for(int i = tid; i < C::LAYER; i += C::THREADS)
        {
          const int cell = i / CD, e = i % CD;
          const int lx = cell % C::CX, ly = cell / C::CX;
          if(lx > bx || ly > by) continue;
          const bool xs = (lx == 0 && tx > 0) || (lx == bx && tx < a.T[0] - 1);
          const bool ys = (ly == 0 && ty > 0) || (ly == by && ty < a.T[1] - 1);
          float v = alo[i];
          if(xs || ys || zshared)
          {
            float *h = a.halo + ((size_t)item * (BZ + 1) * C::LCELLS + (size_t)lz * C::LCELLS + cell) * CD;
            h[e] = v;
          }
          else
          {
            const int cx = x0 + lx, cy = y0 + ly;
            if(a.ras)
              v /= multiplicity(cx, a.nc[0]) * multiplicity(cy, a.nc[1]) * multiplicity(cz, a.nc[2]);
            a.dst[cell_first<C>(a, cx, cy, cz) + e] = double(v);
          }
          alo[i] = 0.f;
        }
      }
      if(more) wait_async_all();
      __syncthreads();
    }
    // last cell layer bz
    {
      const int lz = bz, cz = z0 + bz;
      const bool zshared = tz < a.T[2] - 1;
      const float *alast = s_acc + (bz % 2) * C::LAYER;
      for(int i = tid; i < C::LAYER; i += C::THREADS)
      {
        const int cell = i / CD, e = i % CD;
        const int lx = cell % C::CX, ly = cell / C::CX;
        if(lx > bx || ly > by) continue;
        const bool xs = (lx == 0 && tx > 0) || (lx == bx && tx < a.T[0] - 1);
        const bool ys = (ly == 0 && ty > 0) || (ly == by && ty < a.T[1] - 1);
        float v = alast[i];
        if(xs || ys || zshared)
        {
          float *h = a.halo + ((size_t)item * (BZ + 1) * C::LCELLS + (size_t)lz * C::LCELLS + cell) * CD;
          h[e] = v;
        }
        else
        {
          const int cx = x0 + lx, cy = y0 + ly;
          if(a.ras)
            v /= multiplicity(cx, a.nc[0]) * multiplicity(cy, a.nc[1]) * multiplicity(cz, a.nc[2]);
          a.dst[cell_first<C>(a, cx, cy, cz) + e] = double(v);
        }
      }
    }
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

}  // namespace stream
}  // namespace tpss
