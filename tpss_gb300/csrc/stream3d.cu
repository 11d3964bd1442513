// stream3d.cu -- launcher of the streamed 3D vertex-patch smoother (see stream3d.cuh).
#include <cstring>
#include <mutex>
#include <string>

#include "internal.h"
#include "stream_launch.cuh"

namespace tpss
{
namespace
{
template<int K1>
using Cfg3 = stream::SCfg<K1, 4, 4, 8, 4>;

}  // namespace

bool stream_supported(const tpss_layout &L)
{
  // per-patch 1-D problems (distorted levels) up to k = 3: their table slots for the 16 patches
  // of a vertex layer fit next to the staged layers
  return L.dim == 3 && L.patch_variant == TPSS_PATCH_VERTEX && (!L.per_patch_fd || L.k <= 3) && L.k >= 1 &&
         L.k <= 5 && L.nc[0] >= 2 && L.nc[1] >= 2 && L.nc[2] >= 2;
}

// the same decomposition with per-patch 1-D problems (registers hold these kernels to one CTA per
// SM, so the 48 table slots of 4 x 4 vertex columns cost no occupancy)
template<class C>
struct WithPP;
template<int K1, int BX, int BY, int BZ, int NPT, bool W>
struct WithPP<stream::SCfg<K1, BX, BY, BZ, NPT, W, false>>
{
  using type = stream::SCfg<K1, BX, BY, BZ, NPT, W, true>;
};

// Variants the autotuner chooses from (same mathematics, different work decomposition):
//   0: 4x4 vertex columns, 8 vertex layers per item, 4 pencils per thread
//   1: 4x4 columns, 8 layers, 5 (k = 4) or 2 (k <= 3) pencils per thread
//   2: 4x4 columns, 4 layers per item (more items, more z-shared layers)
//   3: 4x4 columns, 16 layers per item (fewer items, fewer z-shared layers)
//   4: as 0 with a whole warp per patch (no two patches' pencils in one warp)
//   5: as 2 with a whole warp per patch
//   6: (k = 4) plane passes in registers, 3 x 8 vertex columns, 8 layers per item
//   7: (k = 4) as 6 with 4 layers per item
int stream_variant_count(const tpss_layout &L) { return stream_supported(L) ? (L.k == 4 ? 8 : 6) : 0; }

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
// variant V with keyed or per-patch tables
template<int K1, int V>
bool launch_kv(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s)
{
  using C = typename VariantCfg<K1, V>::type;
  if(!l.per_patch) return launch_stream<C>(L, l, s);
  if constexpr(K1 <= 4)
    return launch_stream<typename WithPP<C>::type>(L, l, s);
  else
    return false;
}

template<int K1, int V>
bool launch_kv_host(const tpss_layout &L, const StreamLaunch &l, HostPipe &pp, double *h_dst,
                    const double *h_src, cudaStream_t s)
{
  using C = typename VariantCfg<K1, V>::type;
  if(!l.per_patch) return launch_stream_host<C>(L, l, pp, h_dst, h_src, s);
  if constexpr(K1 <= 4)
    return launch_stream_host<typename WithPP<C>::type>(L, l, pp, h_dst, h_src, s);
  else
    return false;
}

template<int K1>
bool launch_variant(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s, int v)
{
  switch(v)
  {
  case 0: return launch_kv<K1, 0>(L, l, s);
  case 1: return launch_kv<K1, 1>(L, l, s);
  case 2: return launch_kv<K1, 2>(L, l, s);
  case 3: return launch_kv<K1, 3>(L, l, s);
  case 4: return launch_kv<K1, 4>(L, l, s);
  case 5: return launch_kv<K1, 5>(L, l, s);
  case 6:
  case 7:
    // plane passes (k = 4, keyed tables only), compiled in plane_inst.cu
    if constexpr(K1 == 5)
      return !l.per_patch && (v == 6 ? launch_plane3d_bz8(L, l, s) : launch_plane3d_bz4(L, l, s));
    else
      return false;
  default: return false;
  }
}

template<int K1>
bool launch_variant_host(const tpss_layout &L, const StreamLaunch &l, HostPipe &pp, double *h_dst,
                         const double *h_src, cudaStream_t s, int v)
{
  switch(v)
  {
  case 0: return launch_kv_host<K1, 0>(L, l, pp, h_dst, h_src, s);
  case 1: return launch_kv_host<K1, 1>(L, l, pp, h_dst, h_src, s);
  case 2: return launch_kv_host<K1, 2>(L, l, pp, h_dst, h_src, s);
  case 3: return launch_kv_host<K1, 3>(L, l, pp, h_dst, h_src, s);
  case 4: return launch_kv_host<K1, 4>(L, l, pp, h_dst, h_src, s);
  case 5: return launch_kv_host<K1, 5>(L, l, pp, h_dst, h_src, s);
  case 6:
  case 7:
    if constexpr(K1 == 5)
      return !l.per_patch && (v == 6 ? launch_plane3d_host_bz8(L, l, pp, h_dst, h_src, s)
                                     : launch_plane3d_host_bz4(L, l, pp, h_dst, h_src, s));
    else
      return false;
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
  case 5: return launch_stream3d_host_k5(L, l, pp, h_dst, h_src, s);  // stream_k5.cu
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
  case 5: return launch_stream3d_k5(L, l, s);  // stream_k5.cu
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
  a.vpatch = nullptr;
  a.pfd = nullptr;
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
    TPSS_REQUIRE(!L.per_patch_fd && p->tables->own_fd.n == 0,
                 "the allocation-free smoother runs on levels whose patches share their 1-D problems "
                 "(Cartesian levels with fast-diagonalization tables)");
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
