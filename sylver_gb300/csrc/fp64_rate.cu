// Measured FP64 FMA rate of the device: the denominator of the FP64 path's
// roofline (the GPU's FP64 rate is far below its tensor rates, and no vendor
// figure is read here).  Every thread runs eight independent chains of
// a = fma(a, x, y) with |x| < 1, so the values stay bounded; launches of
// eight CTAs of 256 threads per SM are timed with CUDA events after a
// warm-up launch, and the fastest of three counts.
#include <cuda_runtime.h>

#include "../../include/sylver_gb300.h"
#include "numeric.hpp"

using namespace sylver_gb300;

namespace {

constexpr int FMA_CHAINS = 8;

__global__ void __launch_bounds__(256) k_dfma_loop(int iters, double x, double y, double* out) {
  double a[FMA_CHAINS];
#pragma unroll
  for (int c = 0; c < FMA_CHAINS; ++c) a[c] = 1.0 + 1e-3 * (threadIdx.x + c);
#pragma unroll 4
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int c = 0; c < FMA_CHAINS; ++c) a[c] = fma(a[c], x, y);
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < FMA_CHAINS; ++c) s += a[c];
  // never true for bounded values; keeps the chains live
  if (s == 12345.678) out[blockIdx.x] = s;
}

}  // namespace

extern "C" int sylver_gb300_fp64_fma_rate(double* tflops) {
  if (!tflops) return SYLVER_ERROR_UNKNOWN;
  *tflops = 0.0;
  Runtime& rt = Runtime::get();
  if (!rt.init()) return SYLVER_ERROR_CUDA_UNKNOWN;
  try {
    int nsm = 0;
    SG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, rt.device));
    const int blocks = nsm * 8, threads = 256, iters = 1 << 14;
    DevMem out;
    out.ensure((size_t)blocks * sizeof(double));
    cudaEvent_t e0, e1;
    SG_CUDA(cudaEventCreate(&e0));
    SG_CUDA(cudaEventCreate(&e1));
    k_dfma_loop<<<blocks, threads, 0, rt.stream>>>(iters / 8, 0.999999, 1e-7, out.as<double>());
    SG_CUDA(cudaGetLastError());
    float ms = 0.f;
    for (int rep = 0; rep < 3; ++rep) {
      SG_CUDA(cudaEventRecord(e0, rt.stream));
      k_dfma_loop<<<blocks, threads, 0, rt.stream>>>(iters, 0.999999, 1e-7, out.as<double>());
      SG_CUDA(cudaGetLastError());
      SG_CUDA(cudaEventRecord(e1, rt.stream));
      SG_CUDA(cudaEventSynchronize(e1));
      float t = 0.f;
      SG_CUDA(cudaEventElapsedTime(&t, e0, e1));
      if (rep == 0 || t < ms) ms = t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flops = 2.0 * FMA_CHAINS * (double)iters * blocks * threads;
    *tflops = ms > 0.f ? flops / (ms * 1e-3) / 1e12 : 0.0;
    return SYLVER_SUCCESS;
  } catch (const std::exception&) {
    return SYLVER_ERROR_CUDA_UNKNOWN;
  }
}
