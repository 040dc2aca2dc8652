// FP64 throughput of this GPU, for the roofline of the FP64-bound kernels (hymor_fp64_peak).
//
// On GB300 the FP64 pipe, not HBM, bounds the residual and the stencil operators: a
// kernel of this path issues ~150 FP64 instructions per cell against ~200 bytes. The
// denominator of their roofline is measured here the way a copy kernel measures HBM:
// independent DFMA chains in every thread of a grid that fills every SM, timed with
// CUDA events.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.h"

namespace hymor {
cudaStream_t ctx_stream(hymor_ctx* c);
int ctx_select_device(hymor_ctx* c);
namespace {

constexpr int kPeakThreads = 256;
constexpr long kPeakFmaPerThread = 8192;  // DFMA per thread per launch (~5 ms on GB300)

// ILP independent DFMA chains per thread, kPeakFmaPerThread / ILP each
template <int ILP>
__global__ void __launch_bounds__(kPeakThreads) k_dfma_peak(double* out, double a, double b) {
  double x[ILP];
#pragma unroll
  for (int k = 0; k < ILP; ++k) x[k] = threadIdx.x * 1e-3 + k;
  for (int it = 0; it < (int)(kPeakFmaPerThread / ILP); ++it) {
#pragma unroll
    for (int k = 0; k < ILP; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < ILP; ++k) s += x[k];
  if (s == 12345.678) out[0] = s;  // keeps the chains live; never true for these inputs
}

// the same with a distinct multiplier and addend per chain (three distinct source
// registers per DFMA, as in a matvec's coefficient x vector + accumulator)
template <int ILP>
__global__ void __launch_bounds__(kPeakThreads) k_dfma_peak_ops(double* out, double a, double b) {
  double x[ILP], m[ILP], c[ILP];
#pragma unroll
  for (int k = 0; k < ILP; ++k) {
    x[k] = threadIdx.x * 1e-3 + k;
    m[k] = a - k * 1e-9;
    c[k] = b + k * 1e-9;
  }
  for (int it = 0; it < (int)(kPeakFmaPerThread / ILP); ++it) {
#pragma unroll
    for (int k = 0; k < ILP; ++k) x[k] = fma(x[k], m[k], c[k]);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < ILP; ++k) s += x[k];
  if (s == 12345.678) out[0] = s;
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
  double* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = 0;
  double best = 0;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess) {
    rc = HYMOR_ERR_CUDA;
  } else {
    // the best of a sweep over chains per thread and resident blocks per SM: the rate a
    // well-fed FP64 pipe sustains, whichever latency-hiding mix reaches it
    void (*kern[6])(double*, double, double) = {k_dfma_peak<4>,     k_dfma_peak<8>,     k_dfma_peak<16>,
                                                k_dfma_peak_ops<4>, k_dfma_peak_ops<8>, k_dfma_peak_ops<16>};
    const int per_sm[4] = {4, 8, 16, 32};
    for (int ki = 0; ki < 6 && !rc; ++ki)
      for (int bi = 0; bi < 4 && !rc; ++bi) {
        const int blocks = sms * per_sm[bi];
        kern[ki]<<<blocks, kPeakThreads, 0, st>>>(out, 0.999999, 1e-7);  // warm-up
        cudaEventRecord(e0, st);
        constexpr int kReps = 3;
        for (int r = 0; r < kReps; ++r) kern[ki]<<<blocks, kPeakThreads, 0, st>>>(out, 0.999999, 1e-7);
        cudaEventRecord(e1, st);
        float ms = 0;
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0) {
          rc = HYMOR_ERR_CUDA;
        } else {
          const double flop = 2.0 * kPeakFmaPerThread * (double)kPeakThreads * blocks * kReps;
          best = std::max(best, flop / (ms * 1e-3) / 1e12);
        }
      }
    if (!rc) *tflops = best;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  return rc;
}
