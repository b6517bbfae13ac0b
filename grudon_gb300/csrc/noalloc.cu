// grd_aggregate_values_noalloc: grd_aggregate_values without any device
// allocation.
//
// Some callers cannot call cudaMalloc when they feed aggregates in:
//  * a serving process that reserved the device's memory up front for its own
//    pool, so a new allocation would fail or evict that pool;
//  * a latency-bound caller that must not take the allocator's implicit
//    device synchronisation.
// grd_aggregate_values allocates its device staging buffer on first use and
// whenever a larger batch arrives.  This variant stages the (gid, value) pairs
// in the file-scope device array below instead, so it never allocates; the
// array (2 MiB) is held by every GPU that loads the library until the process
// exits.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "ctx.hpp"
#include "kernels.cuh"

using namespace grd;

namespace {

// Staging for up to GRD_NOALLOC_MAX_VALUES pairs: gids, then values.
static __device__ __align__(256) uint32_t g_noalloc_stage[2 * GRD_NOALLOC_MAX_VALUES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
uint32_t* g_stage_addr[kMaxDevices] = {};  // device address of g_noalloc_stage, per device

// Once per device, with that device current: the host-side symbol is only a
// stand-in, the kernel needs the array's device address.
int stage_address(grd_ctx* ctx, uint32_t** out) {
  if (ctx->device < 0 || ctx->device >= kMaxDevices) {
    ctx->err = "device index beyond the no-alloc set-up table";
    return GRD_E_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_stage_addr[ctx->device]) {
    void* p = nullptr;
    CK(cudaGetSymbolAddress(&p, g_noalloc_stage));
    g_stage_addr[ctx->device] = static_cast<uint32_t*>(p);
  }
  *out = g_stage_addr[ctx->device];
  return GRD_OK;
}

}  // namespace

extern "C" int grd_aggregate_values_noalloc(grd_ctx* ctx, const uint32_t* gids, const uint32_t* values, size_t n) {
  TRY(grd_check_ready(ctx));   // the same readiness rules as grd_aggregate_values
  TRY(grd_wait(ctx, nullptr));  // a queued run first: the call changes the ctx
  if (n == 0) return GRD_OK;
  if (!gids || !values) return GRD_E_INVALID;
  if (n > GRD_NOALLOC_MAX_VALUES) {
    ctx->err = "grd_aggregate_values_noalloc: " + std::to_string(n) + " pairs exceed the maximum of " +
               std::to_string(GRD_NOALLOC_MAX_VALUES) + " per call";
    return GRD_E_INVALID;
  }
  for (size_t i = 0; i < n; ++i)
    if (gids[i] >= ctx->L.V) {
      ctx->err = "gid " + std::to_string(gids[i]) + " out of range";
      return GRD_E_INVALID;
    }
  CK(cudaSetDevice(ctx->device));
  uint32_t* stage = nullptr;
  TRY(stage_address(ctx, &stage));
  // Every entry that the kernel reads is written here first, so nothing in
  // the shared array has to start at zero.
  CK(cudaMemcpyAsync(stage, gids, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(stage + GRD_NOALLOC_MAX_VALUES, values, sizeof(uint32_t) * n, cudaMemcpyHostToDevice,
                     ctx->stream));
  const uint32_t blocks = (uint32_t)std::min<size_t>((n + 255) / 256, (size_t)ctx->num_sms * 8);
  const uint32_t* g = stage;
  const uint32_t* v = stage + GRD_NOALLOC_MAX_VALUES;
  switch (ctx->algo) {
    case GRD_PR_DELTA:
    case GRD_PR_PULL: k_aggregate_values<A_PR_DELTA><<<blocks, 256, 0, ctx->stream>>>(ctx->st, g, v, (uint32_t)n); break;
    case GRD_CC: k_aggregate_values<A_CC><<<blocks, 256, 0, ctx->stream>>>(ctx->st, g, v, (uint32_t)n); break;
    case GRD_SSSP_HOP: k_aggregate_values<A_SSSP_HOP><<<blocks, 256, 0, ctx->stream>>>(ctx->st, g, v, (uint32_t)n); break;
    case GRD_SSSP_W: k_aggregate_values<A_SSSP_W><<<blocks, 256, 0, ctx->stream>>>(ctx->st, g, v, (uint32_t)n); break;
    default: return GRD_E_INVALID;
  }
  CK_LAUNCH();
  ctx->stats.kernel_launches += 1;
  CK(cudaStreamSynchronize(ctx->stream));  // the shared array is free again
  return GRD_OK;
}
