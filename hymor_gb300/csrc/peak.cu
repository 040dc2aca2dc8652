// FP64 throughput of this GPU, for the roofline of the FP64-bound kernels (hymor_fp64_peak).
//
// On GB300 the FP64 pipe, not HBM, bounds the residual and the stencil operators: a
// kernel of this path issues ~150 FP64 instructions per cell against ~200 bytes. The
// denominator of their roofline is measured here the way a copy kernel measures HBM:
// independent DFMA chains in every thread of a grid that fills every SM, timed with
// CUDA events.
#include <cuda_runtime.h>

#include "kernels.h"

namespace hymor {
cudaStream_t ctx_stream(hymor_ctx* c);
int ctx_select_device(hymor_ctx* c);
namespace {

constexpr int kPeakIlp = 8;       // independent chains per thread
constexpr int kPeakIters = 1024;  // DFMA per chain (~5 ms per launch on GB300)
constexpr int kPeakThreads = 256;

__global__ void __launch_bounds__(kPeakThreads) k_dfma_peak(double* out, double a, double b) {
  double x[kPeakIlp];
#pragma unroll
  for (int k = 0; k < kPeakIlp; ++k) x[k] = threadIdx.x * 1e-3 + k;
  for (int it = 0; it < kPeakIters; ++it) {
#pragma unroll
    for (int k = 0; k < kPeakIlp; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < kPeakIlp; ++k) s += x[k];
  if (s == 12345.678) out[0] = s;  // keeps the chains live; never true for these inputs
}

}  // namespace
}  // namespace hymor

using namespace hymor;

extern "C" int hymor_fp64_peak(hymor_ctx* ctx, double* tflops) {
  if (!ctx || !tflops) return HYMOR_ERR_INVALID;
  int dev = 0, sms = 0;
  if (ctx_select_device(ctx) || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return HYMOR_ERR_CUDA;
  cudaStream_t st = ctx_stream(ctx);
  const int blocks = sms * 8;
  double* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = 0;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess) {
    rc = HYMOR_ERR_CUDA;
  } else {
    k_dfma_peak<<<blocks, kPeakThreads, 0, st>>>(out, 0.999999, 1e-7);  // warm-up
    cudaEventRecord(e0, st);
    constexpr int kReps = 5;
    for (int r = 0; r < kReps; ++r) k_dfma_peak<<<blocks, kPeakThreads, 0, st>>>(out, 0.999999, 1e-7);
    cudaEventRecord(e1, st);
    float ms = 0;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0) {
      rc = HYMOR_ERR_CUDA;
    } else {
      const double flop = 2.0 * kPeakIlp * kPeakIters * (double)kPeakThreads * blocks * kReps;
      *tflops = flop / (ms * 1e-3) / 1e12;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  return rc;
}
