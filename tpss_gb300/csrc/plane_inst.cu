// plane_inst.cu -- launchers of the plane-pass streamed smoother (plane3d.cuh) for one column
// depth, compiled once per depth (-DPLANE_BZ=8, -DPLANE_BZ=4) so that the two large kernels build
// in parallel.
#include "internal.h"
#include "stream_launch.cuh"

#ifndef PLANE_BZ
#error "PLANE_BZ must be defined"
#endif

#define TPSS_CAT2(a, b) a##b
#define TPSS_CAT(a, b) TPSS_CAT2(a, b)

namespace tpss
{
using PlaneCfgBZ = stream::PCfg<5, 8, PLANE_BZ>;

bool TPSS_CAT(launch_plane3d_bz, PLANE_BZ)(const tpss_layout &L, const StreamLaunch &l, cudaStream_t s)
{
  return launch_stream<PlaneCfgBZ>(L, l, s);
}

bool TPSS_CAT(launch_plane3d_host_bz, PLANE_BZ)(const tpss_layout &L, const StreamLaunch &l, HostPipe &pipe,
                                                double *h_dst, const double *h_src, cudaStream_t s)
{
  return launch_stream_host<PlaneCfgBZ>(L, l, pipe, h_dst, h_src, s);
}
}  // namespace tpss
