// stream3d.cu -- launcher of the streamed 3D vertex-patch smoother (see stream3d.cuh).
#include <cstring>
#include <mutex>
#include <string>

#include "internal.h"
#include "stream3d.cuh"

namespace tpss
{
namespace
{
template<int K1>
using Cfg3 = stream::SCfg<K1, 4, 4, 8, 4>;

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
    TPSS_CUDA(cudaFuncSetAttribute(stream::stream_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)C::smem_bytes()));
    int occ = 0;
    TPSS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, stream::stream_kernel<C>, C::THREADS,
                                                            C::smem_bytes()));
    per_sm[dev] = occ < 1 ? 1 : occ;
  }
  return (int64_t)num_sms() * per_sm[dev];
}

template<class C>
void launch_fixup_range(const stream::StreamArgs &a, const int64_t *rec, int64_t n, cudaStream_t s)
{
  if(n <= 0) return;
  constexpr int per = 128 / C::CD;
  const int64_t fb = (n + per - 1) / per, fcap = (int64_t)num_sms() * 16;
  stream::fixup_list_kernel<C><<<(int)(fb < fcap ? fb : fcap), 128, 0, s>>>(rec, n, a.halo, a.dst);
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
    stream::stream_kernel<C><<<(int)std::min(n_items, cap), C::THREADS, C::smem_bytes(), cs>>>(a);
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
  stream::stream_kernel<C><<<grid, C::THREADS, smem, s>>>(a);
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
}  // namespace

bool stream_supported(const tpss_layout &L)
{
  return L.dim == 3 && L.patch_variant == TPSS_PATCH_VERTEX && !L.per_patch_fd && L.k >= 1 && L.k <= 4 &&
         L.nc[0] >= 2 && L.nc[1] >= 2 && L.nc[2] >= 2;
}

// Variants the autotuner chooses from (same mathematics, different work decomposition):
//   0: 4x4 vertex columns, 8 vertex layers per item, 4 pencils per thread
//   1: 4x4 columns, 8 layers, 5 (k = 4) or 2 (k <= 3) pencils per thread
//   2: 4x4 columns, 4 layers per item (more items, more z-shared layers)
//   3: 4x4 columns, 16 layers per item (fewer items, fewer z-shared layers)
//   4: as 0 with a whole warp per patch (no two patches' pencils in one warp)
//   5: as 2 with a whole warp per patch
int stream_variant_count(const tpss_layout &L) { return stream_supported(L) ? 6 : 0; }

template<int K1, int V>
struct VariantCfg;
template<int K1>
struct VariantCfg<K1, 0>
{
  using type = stream::SCfg<K1, 4, 4, 8, 4>;
};
template<int K1>
struct VariantCfg<K1, 1>
{
  using type = stream::SCfg<K1, 4, 4, 8, K1 == 5 ? 5 : 2>;
};
template<int K1>
struct VariantCfg<K1, 2>
{
  using type = stream::SCfg<K1, 4, 4, 4, 4>;
};
template<int K1>
struct VariantCfg<K1, 3>
{
  using type = stream::SCfg<K1, 4, 4, 16, 4>;
};
// pencils per thread that fill most of a warp with one patch: (2 (k+1))^2 / NPT <= 32
template<int K1>
constexpr int npt_warp() { return K1 == 5 ? 4 : K1 == 4 ? 2 : K1 == 3 ? 2 : 1; }
template<int K1>
struct VariantCfg<K1, 4>
{
  using type = stream::SCfg<K1, 4, 4, 8, npt_warp<K1>(), true>;
};
template<int K1>
struct VariantCfg<K1, 5>
{
  using type = stream::SCfg<K1, 4, 4, 4, npt_warp<K1>(), true>;
};

template<int K1>
bool launch_variant(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s, int v)
{
  switch(v)
  {
  case 0: return launch_stream<typename VariantCfg<K1, 0>::type>(L, l, s);
  case 1: return launch_stream<typename VariantCfg<K1, 1>::type>(L, l, s);
  case 2: return launch_stream<typename VariantCfg<K1, 2>::type>(L, l, s);
  case 3: return launch_stream<typename VariantCfg<K1, 3>::type>(L, l, s);
  case 4: return launch_stream<typename VariantCfg<K1, 4>::type>(L, l, s);
  case 5: return launch_stream<typename VariantCfg<K1, 5>::type>(L, l, s);
  default: return false;
  }
}

template<int K1>
bool launch_variant_host(const tpss_layout &L, const StreamLaunch &l, HostPipe &pp, double *h_dst,
                         const double *h_src, cudaStream_t s, int v)
{
  switch(v)
  {
  case 0: return launch_stream_host<typename VariantCfg<K1, 0>::type>(L, l, pp, h_dst, h_src, s);
  case 1: return launch_stream_host<typename VariantCfg<K1, 1>::type>(L, l, pp, h_dst, h_src, s);
  case 2: return launch_stream_host<typename VariantCfg<K1, 2>::type>(L, l, pp, h_dst, h_src, s);
  case 3: return launch_stream_host<typename VariantCfg<K1, 3>::type>(L, l, pp, h_dst, h_src, s);
  case 4: return launch_stream_host<typename VariantCfg<K1, 4>::type>(L, l, pp, h_dst, h_src, s);
  case 5: return launch_stream_host<typename VariantCfg<K1, 5>::type>(L, l, pp, h_dst, h_src, s);
  default: return false;
  }
}

bool launch_stream3d_host(const tpss_layout &L, const StreamLaunch &l, HostPipe &pp, double *h_dst,
                          const double *h_src, cudaStream_t s)
{
  const int v = l.variant;
  switch(L.k)
  {
  case 1: return launch_variant_host<2>(L, l, pp, h_dst, h_src, s, v);
  case 2: return launch_variant_host<3>(L, l, pp, h_dst, h_src, s, v);
  case 3: return launch_variant_host<4>(L, l, pp, h_dst, h_src, s, v);
  case 4: return launch_variant_host<5>(L, l, pp, h_dst, h_src, s, v);
  default: return false;
  }
}

bool launch_stream3d(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s)
{
  const int v = l.variant;
  switch(L.k)
  {
  case 1: return launch_variant<2>(L, l, s, v);
  case 2: return launch_variant<3>(L, l, s, v);
  case 3: return launch_variant<4>(L, l, s, v);
  case 4: return launch_variant<5>(L, l, s, v);
  default: return false;
  }
}
}  // namespace tpss

// ------------------------------------------------------------------------------------------
// Allocation-free variant of the streamed smoother (tpss_precond_vmult_static_scratch).
//
// The regular vmult keeps the halo partial sums in a buffer that it grows with cudaMalloc
// on first use.  This variant uses a fixed scratch array in device global memory instead,
// defined at file scope below, so the call itself allocates and frees nothing.
// ------------------------------------------------------------------------------------------
namespace tpss
{
namespace
{
// maximum halo size of the allocation-free entry point: 8 Mi floats = 32 MiB per device
constexpr size_t kStaticHaloFloats = size_t(8) << 20;
}  // namespace
}  // namespace tpss

// Every GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) float g_static_halo[tpss::kStaticHaloFloats];

namespace tpss
{
namespace
{
// Host code cannot use g_static_halo directly (its name is a host-side stand-in); the
// device address is looked up once per device with that device current.
std::mutex g_static_halo_mu;
float *g_static_halo_ptr[64] = {nullptr};

float *static_halo_address()
{
  int dev = 0;
  TPSS_CUDA(cudaGetDevice(&dev));
  TPSS_REQUIRE(dev >= 0 && dev < 64, "device index out of range");
  std::lock_guard<std::mutex> lock(g_static_halo_mu);
  if(!g_static_halo_ptr[dev])
  {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_static_halo);
    if(e != cudaSuccess || !ptr)
      fail(TPSS_ERR_CUDA, std::string("cudaGetSymbolAddress(g_static_halo): ") + cudaGetErrorString(e));
    g_static_halo_ptr[dev] = static_cast<float *>(ptr);
  }
  return g_static_halo_ptr[dev];
}

template<class C>
void launch_stream_static(const tpss_layout &L, const tpss_precond &p, const double *src, double *dst,
                          cudaStream_t s)
{
  stream::StreamArgs a;
  a.src = src;
  a.dst = dst;
  a.cell_start = L.lexicographic ? nullptr : L.d_cell_start.ptr;
  a.fd = p.tables->fd32.ptr;
  a.fd_eo = p.tables->fd32_eo.ptr;
  a.sym = p.tables->sym.ptr;
  a.es_eo = 4 * (L.n / 2) * p.tables->hpad32 + p.tables->npad32;
  for(int d = 0; d < 3; ++d)
  {
    a.vfd[d] = L.d_vertex_fd[d].ptr;
    a.nc[d] = L.nc[d];
  }
  a.T[0] = (L.nc[0] - 1 + C::BX - 1) / C::BX;
  a.T[1] = (L.nc[1] - 1 + C::BY - 1) / C::BY;
  a.T[2] = (L.nc[2] - 1 + C::BZ - 1) / C::BZ;
  a.omega = (float)p.desc.relaxation;
  a.ras = p.desc.use_ras_weights != 0;
  const int64_t n_items = (int64_t)a.T[0] * a.T[1] * a.T[2];
  a.item_begin = 0;
  a.item_end = (int)n_items;
  const size_t halo_floats = (size_t)n_items * (C::BZ + 1) * C::LCELLS * C::CD;
  if(halo_floats > kStaticHaloFloats)
    fail(TPSS_ERR_INVALID_ARGUMENT,
         "level too large for the allocation-free smoother: its halo needs " +
           std::to_string(halo_floats) + " floats, the static scratch holds " +
           std::to_string(kStaticHaloFloats) + " (32 MiB)");
  a.halo = static_halo_address();
  const size_t smem = C::smem_bytes();
  const int64_t cap = stream_cap<C>();
  const int grid = (int)(n_items < cap ? n_items : cap);
  stream::stream_kernel<C><<<grid, C::THREADS, smem, s>>>(a);
  TPSS_CUDA(cudaGetLastError());
  const int64_t work = L.n_cells * C::CD;
  const int64_t fb = (work + 255) / 256, fcap = (int64_t)num_sms() * 8;
  stream::fixup_kernel<C><<<(int)(fb < fcap ? fb : fcap), 256, 0, s>>>(a);
  TPSS_CUDA(cudaGetLastError());
}
}  // namespace
}  // namespace tpss

extern "C" int tpss_precond_vmult_static_scratch(tpss_precond *p, double *dst, const double *src,
                                                 void *stream)
{
  return tpss::guarded([&] {
    TPSS_REQUIRE(p && dst && src, "null argument");
    TPSS_REQUIRE(dst != src, "dst and src must not alias");
    const tpss_layout &L = *p->tables->layout;
    if(!tpss::stream_eligible(p))
      tpss::fail(TPSS_ERR_INVALID_ARGUMENT,
                 "the allocation-free smoother needs additive 3D vertex patches on a Cartesian level, "
                 "FP32 arithmetic, degree <= 4 and fast-diagonalization local solvers");
    // options that would need memory or a second kernel path are refused rather than ignored
    TPSS_REQUIRE(!p->desc.check_finite,
                 "the allocation-free smoother has no finiteness check (its flag would need a buffer); "
                 "create the preconditioner with check_finite = 0");
    TPSS_REQUIRE(p->desc.kernel_variant != TPSS_KERNEL_COLOR,
                 "the allocation-free smoother is the column-streamed kernel; kernel_variant asks for "
                 "the per-color kernel");
    cudaStream_t s = tpss::as_stream(stream);
    switch(L.k)
    {
    case 1: tpss::launch_stream_static<tpss::Cfg3<2>>(L, *p, src, dst, s); break;
    case 2: tpss::launch_stream_static<tpss::Cfg3<3>>(L, *p, src, dst, s); break;
    case 3: tpss::launch_stream_static<tpss::Cfg3<4>>(L, *p, src, dst, s); break;
    case 4: tpss::launch_stream_static<tpss::Cfg3<5>>(L, *p, src, dst, s); break;
    default: tpss::fail(TPSS_ERR_INVALID_ARGUMENT, "degree must be <= 4");
    }
  });
}
