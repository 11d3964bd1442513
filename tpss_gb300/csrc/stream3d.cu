// stream3d.cu -- launcher of the streamed 3D vertex-patch smoother (see stream3d.cuh).
#include "internal.h"
#include "stream3d.cuh"

namespace tpss
{
namespace
{
template<int K1>
using Cfg3 = stream::SCfg<K1, 4, 4, 8, 4>;

template<class C>
bool launch_stream(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s)
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
  const int64_t n_items = (int64_t)a.T[0] * a.T[1] * a.T[2];
  const size_t halo_floats = (size_t)n_items * (C::BZ + 1) * C::LCELLS * C::CD;
  if(l.halo->n < halo_floats) l.halo->resize(halo_floats);
  a.halo = l.halo->ptr;
  static int per_sm = 0;
  const size_t smem = C::smem_bytes();
  if(per_sm == 0)
  {
    TPSS_CUDA(cudaFuncSetAttribute(stream::stream_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
    int occ = 0;
    TPSS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, stream::stream_kernel<C>, C::THREADS, smem));
    per_sm = occ < 1 ? 1 : occ;
  }
  const int64_t cap = (int64_t)num_sms() * per_sm;
  const int grid = (int)(n_items < cap ? n_items : cap);
  stream::stream_kernel<C><<<grid, C::THREADS, smem, s>>>(a);
  TPSS_CUDA(cudaGetLastError());
  const int64_t work = L.n_cells * C::CD;
  const int64_t fb = (work + 255) / 256, fcap = (int64_t)num_sms() * 8;
  stream::fixup_kernel<C><<<(int)(fb < fcap ? fb : fcap), 256, 0, s>>>(a);
  TPSS_CUDA(cudaGetLastError());
  return true;
}
}  // namespace

bool stream_supported(const tpss_layout &L)
{
  return L.dim == 3 && L.patch_variant == TPSS_PATCH_VERTEX && !L.per_patch_fd && L.k >= 1 && L.k <= 4 &&
         L.nc[0] >= 2 && L.nc[1] >= 2 && L.nc[2] >= 2;
}

bool launch_stream3d(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s)
{
  switch(L.k)
  {
  case 1: return launch_stream<Cfg3<2>>(L, l, s);
  case 2: return launch_stream<Cfg3<3>>(L, l, s);
  case 3: return launch_stream<Cfg3<4>>(L, l, s);
  case 4: return launch_stream<Cfg3<5>>(L, l, s);
  default: return false;
  }
}
}  // namespace tpss
