// diag.cu -- measurement helper: FMA-pipe throughput of this GPU (FP32 or FP64).
//
// The Schwarz FD kernel is bound by the FP32 (or FP64) FMA pipes, not by tensor cores, so its
// roofline denominator is the CUDA-core FMA rate.  This kernel runs eight independent FMA
// chains per thread on every SM and is timed with CUDA events on the caller's stream.
#include "internal.h"

namespace tpss
{
namespace
{
template<typename T>
__global__ void __launch_bounds__(256) fma_peak_kernel(T *out, int iters, T a, T b)
{
  T x[8];
#pragma unroll
  for(int j = 0; j < 8; ++j) x[j] = T(threadIdx.x + j) * T(1e-3);
  for(int i = 0; i < iters; ++i)
  {
#pragma unroll
    for(int j = 0; j < 8; ++j) x[j] = fma(x[j], a, b);
  }
  T s = T(0);
#pragma unroll
  for(int j = 0; j < 8; ++j) s += x[j];
  if(s == T(-1.2345)) out[0] = s;  // keeps the chains alive; never true in practice
}

template<typename T>
double run(int iters, cudaStream_t s)
{
  const int blocks = num_sms() * 8, threads = 256;
  DeviceBuffer<T> out(1);
  cudaEvent_t e0, e1;
  TPSS_CUDA(cudaEventCreate(&e0));
  TPSS_CUDA(cudaEventCreate(&e1));
  fma_peak_kernel<T><<<blocks, threads, 0, s>>>(out.ptr, iters / 8, T(0.999999), T(1e-7));  // warm-up
  TPSS_CUDA(cudaEventRecord(e0, s));
  fma_peak_kernel<T><<<blocks, threads, 0, s>>>(out.ptr, iters, T(0.999999), T(1e-7));
  TPSS_CUDA(cudaEventRecord(e1, s));
  TPSS_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  TPSS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return 2.0 * 8.0 * iters * double(blocks) * threads / (ms * 1e-3);
}
}  // namespace
}  // namespace tpss

using namespace tpss;

extern "C" int tpss_diag_fma_peak(int precision, int iters, double *flops_per_second, void *stream)
{
  return guarded([&] {
    TPSS_REQUIRE(flops_per_second && iters > 0, "invalid argument");
    *flops_per_second = precision == TPSS_FP32 ? run<float>(iters, as_stream(stream))
                                               : run<double>(iters, as_stream(stream));
  });
}
