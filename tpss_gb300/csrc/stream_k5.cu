// stream_k5.cu -- the streamed smoother's decompositions for degree 5 (N = 12), compiled in two
// parts (-DK5_PART=0: variants 0-2, -DK5_PART=1: variants 3-5) so that the large kernels build in
// parallel.
//
// A 4 x 4 vertex column does not fit: its two FP64 landing layers, two FP32 layers, two
// accumulator layers (25 cells of 216 DoFs each) and 16 patch buffers of 12^3 values need about
// 300 KB of shared memory. Columns of 4 x 2 vertices need 172-177 KB (one CTA per SM).
#include "internal.h"
#include "stream_launch.cuh"

#ifndef K5_PART
#error "K5_PART must be defined"
#endif

namespace tpss
{
bool launch_stream3d_k5_part0(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s);
bool launch_stream3d_k5_part1(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s);
bool launch_stream3d_host_k5_part0(const tpss_layout &L, const StreamLaunch &l, HostPipe &pp, double *h_dst,
                                   const double *h_src, cudaStream_t s);
bool launch_stream3d_host_k5_part1(const tpss_layout &L, const StreamLaunch &l, HostPipe &pp, double *h_dst,
                                   const double *h_src, cudaStream_t s);

namespace
{
template<int V>
struct K5Cfg;
// 0: 8 vertex layers per item, a warp per patch, 6 pencils per thread (24 lanes busy)
template<>
struct K5Cfg<0>
{
  using type = stream::SCfg<6, 4, 2, 8, 6, true>;
};
// 1: 8 layers, 36 threads per patch with 4 pencils each (patches share warps)
template<>
struct K5Cfg<1>
{
  using type = stream::SCfg<6, 4, 2, 8, 4>;
};
// 2: as 1 with 4 layers per item
template<>
struct K5Cfg<2>
{
  using type = stream::SCfg<6, 4, 2, 4, 4>;
};
// 3: as 0 with 16 layers per item
template<>
struct K5Cfg<3>
{
  using type = stream::SCfg<6, 4, 2, 16, 6, true>;
};
// 4: 8 layers, a warp per patch, 8 pencils per thread (18 lanes busy)
template<>
struct K5Cfg<4>
{
  using type = stream::SCfg<6, 4, 2, 8, 8, true>;
};
// 5: as 0 with 4 layers per item
template<>
struct K5Cfg<5>
{
  using type = stream::SCfg<6, 4, 2, 4, 6, true>;
};

constexpr int kFirst = 3 * K5_PART;
}  // namespace

#define TPSS_CAT2(a, b) a##b
#define TPSS_CAT(a, b) TPSS_CAT2(a, b)

bool TPSS_CAT(launch_stream3d_k5_part, K5_PART)(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s)
{
  switch(l.variant - kFirst)
  {
  case 0: return launch_stream<typename K5Cfg<kFirst + 0>::type>(L, l, s);
  case 1: return launch_stream<typename K5Cfg<kFirst + 1>::type>(L, l, s);
  case 2: return launch_stream<typename K5Cfg<kFirst + 2>::type>(L, l, s);
  default: return false;
  }
}

bool TPSS_CAT(launch_stream3d_host_k5_part, K5_PART)(const tpss_layout &L, const StreamLaunch &l,
                                                     HostPipe &pp, double *h_dst, const double *h_src,
                                                     cudaStream_t s)
{
  switch(l.variant - kFirst)
  {
  case 0: return launch_stream_host<typename K5Cfg<kFirst + 0>::type>(L, l, pp, h_dst, h_src, s);
  case 1: return launch_stream_host<typename K5Cfg<kFirst + 1>::type>(L, l, pp, h_dst, h_src, s);
  case 2: return launch_stream_host<typename K5Cfg<kFirst + 2>::type>(L, l, pp, h_dst, h_src, s);
  default: return false;
  }
}

#if K5_PART == 0
bool launch_stream3d_k5(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s)
{
  if(l.per_patch) return false;  // per-patch tables: degree <= 3
  return l.variant < 3 ? launch_stream3d_k5_part0(L, l, s) : launch_stream3d_k5_part1(L, l, s);
}

bool launch_stream3d_host_k5(const tpss_layout &L, const StreamLaunch &l, HostPipe &pp, double *h_dst,
                             const double *h_src, cudaStream_t s)
{
  if(l.per_patch) return false;
  return l.variant < 3 ? launch_stream3d_host_k5_part0(L, l, pp, h_dst, h_src, s)
                       : launch_stream3d_host_k5_part1(L, l, pp, h_dst, h_src, s);
}
#endif
}  // namespace tpss
