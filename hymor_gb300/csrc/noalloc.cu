// Allocation-free variant of the Taylor propagator (hymor_expm_apply_dev).
//
// Who needs it: callers that cannot call cudaMalloc while they run, for example a
// service that reserves its whole device-memory budget at start-up and treats any
// allocation during a solve as a failure, or a host runtime whose own pool allocator
// owns the device memory and must not see a second allocator take from it.
// hymor_expm_apply_dev allocates work vectors (and, with the shock-position unknowns,
// instantiates a CUDA graph of one Taylor step); this entry point takes its work
// vectors from one fixed, file-scope device array and launches every Taylor step
// directly, so the call itself allocates nothing.
//
// Limits and sharing rules:
//   * the array holds 3 x kNoAllocVec doubles (24 MiB) and is held by every GPU
//     that loads libhymor until the process exits;
//   * one call needs 3 work vectors of n * k doubles (n = 4 * Nchi * Neta, plus Nchi
//     with the shock-position unknowns), so n * k <= kNoAllocVec (1 048 576), e.g.
//     Nchi * Neta <= 262 144 for one vector; larger requests return HYMOR_ERR_INVALID
//     before any device work;
//   * all calls in the process share the array and it keeps the last call's
//     contents; nothing in it has to start at zero (each call first copies its input
//     into the work vectors). Calls whose GPU work overlaps (other streams, other
//     contexts on the same device, other host threads) race on the array: serialise
//     them;
//   * the device address of the array is looked up once per device, on the first
//     call for a context on that device (cudaGetSymbolAddress, with the context's
//     device made current first). Make that first call before any stream capture.
//     The lookup is guarded by a mutex, so first calls from several host threads are
//     safe.
#include <atomic>
#include <cstdio>
#include <mutex>

#include "kernels.h"

namespace hymor {
DevCtx& ctx_dev(hymor_ctx* c);
cudaStream_t ctx_stream(hymor_ctx* c);
int ctx_fail(hymor_ctx* c, int code, const char* msg);
int ctx_select_device(hymor_ctx* c);
}  // namespace hymor

using namespace hymor;

namespace {

constexpr long kNoAllocVec = 1L << 20;  // doubles per work vector
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_expm_scratch[3 * kNoAllocVec];

// device address of g_expm_scratch, per device (null until the first call there)
std::atomic<double*> g_scratch_addr[kMaxDevices];
std::mutex g_scratch_mu;

// Makes the context's device current and returns the array's address on it.
int scratch_for_ctx_device(hymor_ctx* ctx, double** out) {
  int dev = -1;
  if (ctx_select_device(ctx) || cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return ctx_fail(ctx, HYMOR_ERR_CUDA, "cannot make the context's device current for the allocation-free propagator");
  double* p = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!p) {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    p = g_scratch_addr[dev].load(std::memory_order_relaxed);
    if (!p) {
      void* a = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&a, g_expm_scratch);
      if (e != cudaSuccess || !a) {
        char msg[256];
        snprintf(msg, sizeof msg, "cudaGetSymbolAddress of the propagator scratch failed: %s", cudaGetErrorString(e));
        return ctx_fail(ctx, HYMOR_ERR_CUDA, msg);
      }
      p = static_cast<double*>(a);
      g_scratch_addr[dev].store(p, std::memory_order_release);
    }
  }
  *out = p;
  return 0;
}

}  // namespace

extern "C" int hymor_expm_apply_dev_noalloc(hymor_ctx* ctx, int k, double dt, int nsteps, int order,
                                            const double* dX, double* dY, int transpose) {
  if (!ctx || k < 1 || nsteps < 0 || order < 1 || order > 20 || !dX || !dY) return HYMOR_ERR_INVALID;
  DevCtx& d = ctx_dev(ctx);
  if (!d.coef) return ctx_fail(ctx, HYMOR_ERR_NOT_READY, "no Jacobian: call hymor_linearize or hymor_jacobian_set");
  const long n = op_size(d) * (long)k;
  if (n > kNoAllocVec) {
    char msg[256];
    snprintf(msg, sizeof msg,
             "allocation-free propagator: (operator size) * k = %ld exceeds its fixed work size of %ld doubles; "
             "use hymor_expm_apply_dev",
             n, kNoAllocVec);
    return ctx_fail(ctx, HYMOR_ERR_INVALID, msg);
  }
  double* work = nullptr;
  int r = scratch_for_ctx_device(ctx, &work);
  if (r) return r;
  // launch_expm uses work[0, 3n): v, and the two alternating Taylor terms; every Taylor
  // step is launched directly (graph_ok false), also with the shock-position blocks
  launch_expm(d, k, dt, nsteps, order, dX, dY, transpose, work, ctx_stream(ctx), false);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return ctx_fail(ctx, HYMOR_ERR_CUDA, cudaGetErrorString(e));
  return 0;
}
