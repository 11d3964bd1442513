// stream_launch.cuh -- host-side launch glue shared by the streamed smoother kernels
// (stream3d.cuh: pencil passes, plane3d.cuh: plane passes): work-item arguments, the list of cells
// shared between items, resident-CTA count, device-buffer and host-buffer launches.
#pragma once

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "internal.h"
#include "plane3d.cuh"
#include "stream3d.cuh"

namespace tpss
{
// (templates only: every translation unit that includes this header instantiates the same
// definitions, and each launch configuration keeps one per-device cache in stream_cap)

// the kernel of a decomposition: pencil passes (SCfg) or plane passes (PCfg)
template<class C>
constexpr void (*kernel_of())(stream::StreamArgs)
{
  if constexpr(C::PLANE)
    return stream::plane_kernel<C>;
  else
    return stream::stream_kernel<C>;
}

// records of the cells shared between items (stream::fixup_list_kernel), same order of the
// partials as stream::fixup_kernel
template<class C>
void build_fixup_list(const tpss_layout &L, const stream::StreamArgs &a, DeviceBuffer<int64_t> &out,
                      int64_t &n_out, std::vector<int64_t> *layer_start)
{
  std::vector<int64_t> rec;
  if(layer_start) layer_start->assign(L.nc[2] + 1, 0);
  for(int cz = 0; cz < L.nc[2]; ++cz)
  {
    if(layer_start) (*layer_start)[cz] = (int64_t)(rec.size() / stream::kFixRec);
    for(int cy = 0; cy < L.nc[1]; ++cy)
      for(int cx = 0; cx < L.nc[0]; ++cx)
      {
        int tx[2], lx[2], ty[2], ly[2], tz[2], lz[2];
        const int nx = stream::tiles_of(cx, C::BX, a.T[0], tx, lx);
        const int ny = stream::tiles_of(cy, C::BY, a.T[1], ty, ly);
        const int nz = stream::tiles_of(cz, C::BZ, a.T[2], tz, lz);
        if(nx * ny * nz == 1) continue;
        const int64_t cell = cx + (int64_t)L.nc[0] * (cy + (int64_t)L.nc[1] * cz);
        float scale = 1.f;
        if(a.ras)
          scale = 1.f / (stream::multiplicity(cx, L.nc[0]) * stream::multiplicity(cy, L.nc[1]) *
                         stream::multiplicity(cz, L.nc[2]));
        uint32_t bits;
        std::memcpy(&bits, &scale, sizeof(bits));
        const size_t r0 = rec.size();
        rec.resize(r0 + stream::kFixRec, 0);
        rec[r0] = L.cell_start[cell];
        rec[r0 + 1] = int64_t(uint64_t(nx * ny * nz) | (uint64_t(bits) << 32));
        int k = 0;
        for(int kz = 0; kz < nz; ++kz)
          for(int ky = 0; ky < ny; ++ky)
            for(int kx = 0; kx < nx; ++kx)
            {
              const int64_t item = tx[kx] + (int64_t)a.T[0] * (ty[ky] + (int64_t)a.T[1] * tz[kz]);
              const int lcell = lx[kx] + C::CX * ly[ky];
              rec[r0 + 2 + k++] =
                ((item * (C::BZ + 1) + lz[kz]) * C::LCELLS + lcell) * (int64_t)C::CD;
            }
      }
  }
  n_out = (int64_t)(rec.size() / stream::kFixRec);
  if(layer_start) (*layer_start)[L.nc[2]] = n_out;
  out.upload(rec.data(), rec.size());
}

template<class C>
stream::StreamArgs make_args(const tpss_layout &L, const StreamLaunch &l)
{
  stream::StreamArgs a;
  a.src = l.src;
  a.dst = l.dst;
  a.cell_start = L.lexicographic ? nullptr : L.d_cell_start.ptr;
  a.fd = l.fd32;
  a.fd_eo = l.fd32_eo;
  a.sym = l.sym;
  a.es_eo = l.es_eo;
  for(int d = 0; d < 3; ++d)
  {
    a.vfd[d] = L.d_vertex_fd[d].ptr;
    a.nc[d] = L.nc[d];
  }
  a.T[0] = (L.nc[0] - 1 + C::BX - 1) / C::BX;
  a.T[1] = (L.nc[1] - 1 + C::BY - 1) / C::BY;
  a.T[2] = (L.nc[2] - 1 + C::BZ - 1) / C::BZ;
  a.omega = (float)l.omega;
  a.ras = l.ras;
  a.vpatch = l.vpatch;
  a.pfd = l.pfd;
  if constexpr(!C::PLANE)
    if(C::PP)
      TPSS_REQUIRE(l.vpatch && l.pfd && l.es_eo % 4 == 0,
                   "per-patch streamed smoother: vertex-patch map, patch entries and 16-byte table rows");
  const int64_t n_items = (int64_t)a.T[0] * a.T[1] * a.T[2];
  a.item_begin = 0;
  a.item_end = (int)n_items;
  const size_t halo_floats = (size_t)n_items * (C::BZ + 1) * C::LCELLS * C::CD;
  if(l.halo->n < halo_floats) l.halo->resize(halo_floats);
  a.halo = l.halo->ptr;
  return a;
}

// resident CTAs of the streamed kernel (sets its shared-memory attribute once)
template<class C>
int64_t stream_cap()
{
  // the shared-memory attribute and the occupancy are set / queried once per device
  static std::mutex mu;
  static int per_sm[64] = {0};
  int dev = 0;
  TPSS_CUDA(cudaGetDevice(&dev));
  TPSS_REQUIRE(dev >= 0 && dev < 64, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(mu);
  if(per_sm[dev] == 0)
  {
    TPSS_CUDA(cudaFuncSetAttribute(kernel_of<C>(), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)C::smem_bytes()));
    int occ = 0;
    TPSS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel_of<C>(), C::THREADS,
                                                            C::smem_bytes()));
    per_sm[dev] = occ < 1 ? 1 : occ;
  }
  return (int64_t)num_sms() * per_sm[dev];
}

template<class C>
void launch_fixup_range(const stream::StreamArgs &a, const int64_t *rec, int64_t n, cudaStream_t s)
{
  if(n <= 0) return;
  constexpr int threads = stream::fixup_threads<C>(), per = threads / C::CD;
  static_assert(per >= 1, "a block covers at least one cell");
  const int64_t fb = (n + per - 1) / per, fcap = (int64_t)num_sms() * 16;
  stream::fixup_list_kernel<C><<<(int)(fb < fcap ? fb : fcap), threads, 0, s>>>(rec, n, a.halo, a.dst);
}

// src and dst in host memory: the level is cut into chunks of z-items; per chunk the cell layers
// it reads are copied in (stream up), its items are solved and the shared cells of the layers it
// completes are summed (compute streams, alternating between two so that a chunk's items fill
// the SMs left idle by the previous chunk's last wave), and those finished layers are copied out
// (stream down). The fix-up of chunk c also waits for chunk c - 1's items: the cell layer
// between them holds partials of both.
template<class C>
bool launch_stream_host(const tpss_layout &L, const StreamLaunch &l0, HostPipe &pp, double *h_dst,
                        const double *h_src, cudaStream_t caller)
{
  if(!L.lexicographic || !l0.fix_rec) return false;
  StreamLaunch l = l0;
  l.src = pp.src.ptr;
  l.dst = pp.dst.ptr;
  stream::StreamArgs a = make_args<C>(L, l);
  if(*l.fix_n < 0) build_fixup_list<C>(L, a, *l.fix_rec, *l.fix_n, l.fix_layer);
  const std::vector<int64_t> &ls = *l.fix_layer;
  const int64_t layer = (int64_t)L.nc[0] * L.nc[1] * C::CD;  // DoFs of one cell layer
  const int nz = L.nc[2], T2 = a.T[2];
  const int64_t items_per_z = (int64_t)a.T[0] * a.T[1];
  const int per = 1;  // one z-item per chunk: the shortest pipeline fill and drain
  const int64_t cap = stream_cap<C>();
  pp.streams();
  size_t e = 0;
  cudaEvent_t start = pp.event(e++);
  TPSS_CUDA(cudaEventRecord(start, caller));
  for(cudaStream_t st : {pp.up, pp.comp, pp.comp2, pp.down}) TPSS_CUDA(cudaStreamWaitEvent(st, start, 0));
  int copied = 0, fixed = 0, chunk = 0;
  cudaEvent_t prev_items = nullptr;
  for(int z0 = 0; z0 < T2; z0 += per, ++chunk)
  {
    cudaStream_t cs = (chunk % 2) ? pp.comp2 : pp.comp;
    const int z1 = std::min(T2, z0 + per);
    const bool last = z1 == T2;
    const int need = last ? nz : std::min(z1 * C::BZ + 1, nz);  // cell layers read so far
    if(need > copied)
      TPSS_CUDA(cudaMemcpyAsync(pp.src.ptr + copied * layer, h_src + copied * layer,
                                sizeof(double) * (size_t)(need - copied) * layer, cudaMemcpyHostToDevice, pp.up));
    copied = need;
    cudaEvent_t up_done = pp.event(e++);
    TPSS_CUDA(cudaEventRecord(up_done, pp.up));
    TPSS_CUDA(cudaStreamWaitEvent(cs, up_done, 0));
    a.item_begin = (int)(z0 * items_per_z);
    a.item_end = (int)(z1 * items_per_z);
    const int64_t n_items = a.item_end - a.item_begin;
    kernel_of<C>()<<<(int)std::min(n_items, cap), C::THREADS, C::smem_bytes(), cs>>>(a);
    TPSS_CUDA(cudaGetLastError());
    cudaEvent_t items_done = pp.event(e++);
    TPSS_CUDA(cudaEventRecord(items_done, cs));
    if(prev_items) TPSS_CUDA(cudaStreamWaitEvent(cs, prev_items, 0));
    prev_items = items_done;
    const int bound = last ? nz : z1 * C::BZ;  // cell layers final after this chunk
    launch_fixup_range<C>(a, l.fix_rec->ptr + ls[fixed] * stream::kFixRec, ls[bound] - ls[fixed], cs);
    TPSS_CUDA(cudaGetLastError());
    cudaEvent_t comp_done = pp.event(e++);
    TPSS_CUDA(cudaEventRecord(comp_done, cs));
    TPSS_CUDA(cudaStreamWaitEvent(pp.down, comp_done, 0));
    if(bound > fixed)
      TPSS_CUDA(cudaMemcpyAsync(h_dst + fixed * layer, pp.dst.ptr + fixed * layer,
                                sizeof(double) * (size_t)(bound - fixed) * layer, cudaMemcpyDeviceToHost, pp.down));
    fixed = bound;
  }
  cudaEvent_t done = pp.event(e++);
  TPSS_CUDA(cudaEventRecord(done, pp.down));
  TPSS_CUDA(cudaStreamWaitEvent(caller, done, 0));
  return true;
}

template<class C>
bool launch_stream(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s)
{
  stream::StreamArgs a = make_args<C>(L, l);
  const int64_t n_items = (int64_t)a.item_end;
  const int64_t cap = stream_cap<C>();
  const int grid = (int)(n_items < cap ? n_items : cap);
  const size_t smem = C::smem_bytes();
  kernel_of<C>()<<<grid, C::THREADS, smem, s>>>(a);
  TPSS_CUDA(cudaGetLastError());
  if(l.fix_rec)
  {
    if(*l.fix_n < 0) build_fixup_list<C>(L, a, *l.fix_rec, *l.fix_n, l.fix_layer);
    launch_fixup_range<C>(a, l.fix_rec->ptr, *l.fix_n, s);
  }
  else
  {
    const int64_t work = L.n_cells * C::CD;
    const int64_t fb = (work + 255) / 256, fcap = (int64_t)num_sms() * 8;
    stream::fixup_kernel<C><<<(int)(fb < fcap ? fb : fcap), 256, 0, s>>>(a);
  }
  TPSS_CUDA(cudaGetLastError());
  return true;
}
}  // namespace tpss
