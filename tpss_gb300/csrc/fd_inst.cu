// fd_inst.cu -- instantiations of the fused Schwarz color kernel for one arithmetic type and
// dimension.  Compiled once per (FD_T, FD_DIM) pair (float/double x 2/3), so the four
// translation units build in parallel.
#include "fd_kernels.cuh"
#include "internal.h"

#ifndef FD_T
#error "FD_T must be defined (float or double)"
#endif
#ifndef FD_DIM
#error "FD_DIM must be defined (2 or 3)"
#endif

#define TPSS_CAT2(a, b) a##b
#define TPSS_CAT(a, b) TPSS_CAT2(a, b)
#define TPSS_FD_FN TPSS_CAT(TPSS_CAT(launch_fd_, FD_T), TPSS_CAT(_, FD_DIM))

namespace tpss
{
bool TPSS_FD_FN(int k, int ncp, const FdLaunch &l, cudaStream_t s)
{
  fd::KernelArgs a;
  a.src = l.src;
  a.dst = l.dst;
  a.patch_first = l.patch_first;
  a.patch_fd = l.patch_fd;
  a.fd = l.fd;
  a.ras_w = l.ras_w;
  a.n_patches = l.n_patches;
  a.omega = l.omega;
  a.entry_stride = l.entry_stride;
  a.fd_eo = l.fd_eo;
  a.sym = l.sym;
  a.eo_stride = l.eo_stride;
  a.rcp = l.rcp;
  a.rcp_E = l.rcp_E;
  a.keep_mask = l.keep_mask;
  a.keep_class = l.keep_class;
  const int sms = num_sms();
#define TPSS_FD_CASE(NCP, K1) \
  if(ncp == NCP && k + 1 == K1) return fd::launch<FD_T, FD_DIM, NCP, K1>(a, s, sms, l.variant);
  TPSS_FD_CASE(1, 2) TPSS_FD_CASE(1, 3) TPSS_FD_CASE(1, 4) TPSS_FD_CASE(1, 5)
  TPSS_FD_CASE(1, 6) TPSS_FD_CASE(1, 7) TPSS_FD_CASE(1, 8)
  TPSS_FD_CASE(2, 2) TPSS_FD_CASE(2, 3) TPSS_FD_CASE(2, 4) TPSS_FD_CASE(2, 5)
  TPSS_FD_CASE(2, 6) TPSS_FD_CASE(2, 7) TPSS_FD_CASE(2, 8)
#undef TPSS_FD_CASE
  return false;
}

// work decompositions (patches per CTA) the kernel of (k, ncp) offers to the autotuner
int TPSS_CAT(TPSS_CAT(fd_variants_, FD_T), TPSS_CAT(_, FD_DIM))(int k, int ncp)
{
#define TPSS_FD_CASE(NCP, K1) \
  if(ncp == NCP && k + 1 == K1) return fd::Cfg<FD_T, FD_DIM, NCP, K1>::n_variants();
  TPSS_FD_CASE(1, 2) TPSS_FD_CASE(1, 3) TPSS_FD_CASE(1, 4) TPSS_FD_CASE(1, 5)
  TPSS_FD_CASE(1, 6) TPSS_FD_CASE(1, 7) TPSS_FD_CASE(1, 8)
  TPSS_FD_CASE(2, 2) TPSS_FD_CASE(2, 3) TPSS_FD_CASE(2, 4) TPSS_FD_CASE(2, 5)
  TPSS_FD_CASE(2, 6) TPSS_FD_CASE(2, 7) TPSS_FD_CASE(2, 8)
#undef TPSS_FD_CASE
  return 1;
}
}  // namespace tpss
