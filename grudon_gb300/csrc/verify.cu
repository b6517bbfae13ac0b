// The reference's verify() validators as device kernels over the ctx's
// resident layout (cc.cpp:139-177, sssp.cpp:145-189, pr.cpp:179-205):
//   CC    every edge joins two vertices of the same label;
//   SSSP  no reachable vertex u has an out-edge (u,v) with
//         dist[v] > dist[u] + w(u,v) (w = 1 for the hop count), plus the
//         count of reachable vertices and the largest distance;
//   PR    the 20 largest pr_vals (the reference prints them).
// Every edge of the graph is checked once: a vertex's out-edges are the row
// of its owned slot, and slot_gid maps each destination slot to its gid.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/grudon_gpu.h"
#include "ctx.hpp"
#include "kernels.cuh"

using namespace grd;

namespace {

constexpr int TOPK = GRD_VERIFY_TOPK;
constexpr uint32_t INF = 0xFFFFFFFFu;

// One warp per owned row; lanes stride its edges.  out[0] errors, out[1]
// edges checked, out[2] visited / components, out[3] max distance.
template <int A>
__global__ void __launch_bounds__(256) k_verify_edges(DevGraph g, DevState st, unsigned long long* out) {
  const uint32_t lane = lane_id();
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  unsigned long long bad = 0, checked = 0, count = 0, mx = 0;
  for (uint64_t s = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < g.S; s += nw) {
    const uint32_t p = g.tile_part[s / K_TILE_SLOTS];
    if (s - g.part_base[p] >= g.part_owned[p]) continue;  // proxy or padding: no row
    const uint32_t u = __ldg(&g.slot_gid[s]);
    const uint32_t du = st.prop[u];
    if (A == A_CC) {
      if (lane == 0 && du == u) ++count;  // one root per component
    } else {
      if (du == INF) continue;  // the reference skips unreached sources
      if (lane == 0) {
        ++count;
        mx = max(mx, (unsigned long long)du);
      }
    }
    const uint32_t e0 = __ldg(&g.row_off[s]), e1 = __ldg(&g.row_off[s + 1]);
    for (uint32_t e = e0 + lane; e < e1; e += 32) {
      const uint32_t v = __ldg(&g.slot_gid[__ldg(&g.col[e])]);
      const uint32_t dv = st.prop[v];
      ++checked;
      if (A == A_CC) {
        bad += dv != du;
      } else {
        const unsigned long long w = A == A_SSSP_W ? __ldg(&g.wgt[e]) : 1ull;
        bad += (unsigned long long)dv > (unsigned long long)du + w;
      }
    }
  }
  // warp sums, one atomic per warp
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    bad += __shfl_xor_sync(FULL, bad, o);
    checked += __shfl_xor_sync(FULL, checked, o);
  }
  if (lane == 0) {
    if (bad) atomicAdd(&out[0], bad);
    if (checked) atomicAdd(&out[1], checked);
    if (count) atomicAdd(&out[2], count);
    if (mx) atomicMax(&out[3], mx);
  }
}

// Ranks ordered by value, then by lower gid: a larger key ranks first.
__device__ __forceinline__ unsigned long long rank_key(float r, uint32_t v) {
  // pr_vals are >= 0, so the float bits order like the values
  return ((unsigned long long)__float_as_uint(r) << 32) | (unsigned long long)(0xFFFFFFFFu - v);
}

// Top TOPK keys of a stride of the ranks, per block: every thread keeps its
// own sorted TOPK, the block merges them in shared memory.
__global__ void __launch_bounds__(256) k_topk_blocks(const float* ranks, uint32_t V, unsigned long long* out) {
  __shared__ unsigned long long s_keys[256 * TOPK];
  unsigned long long top[TOPK];
#pragma unroll
  for (int i = 0; i < TOPK; ++i) top[i] = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const unsigned long long k = rank_key(ranks[v], v);
    if (k <= top[TOPK - 1]) continue;
    // insert, keeping top[] descending
    int i = TOPK - 1;
    while (i > 0 && top[i - 1] < k) {
      top[i] = top[i - 1];
      --i;
    }
    top[i] = k;
  }
  for (int i = 0; i < TOPK; ++i) s_keys[threadIdx.x * TOPK + i] = top[i];
  __syncthreads();
  if (threadIdx.x == 0) {  // select the block's TOPK largest (fixed order)
    for (int r = 0; r < TOPK; ++r) {
      unsigned long long best = 0;
      int at = -1;
      for (int j = 0; j < 256 * TOPK; ++j)
        if (s_keys[j] > best) best = s_keys[j], at = j;
      out[(size_t)blockIdx.x * TOPK + r] = best;
      if (at >= 0) s_keys[at] = 0;
    }
  }
}

}  // namespace

extern "C" int grd_verify(grd_ctx* ctx, grd_verify_result* out) {
  if (!ctx || !out) return GRD_E_INVALID;
  if (ctx->algo < 0 || !ctx->inited) {
    ctx->err = "grd_verify needs a ctx after grd_init / grd_run";
    return GRD_E_INVALID;
  }
  CK(cudaSetDevice(ctx->device));
  std::memset(out, 0, sizeof(*out));
  if (ctx->algo == GRD_PR_DELTA || ctx->algo == GRD_PR_PULL) {
    const uint32_t blocks = (uint32_t)std::min<uint64_t>((ctx->L.V + 255) / 256, (uint64_t)ctx->num_sms);
    unsigned long long* keys = nullptr;
    if (ctx->verify_cap < (size_t)blocks * TOPK) {
      void* p = nullptr;
      TRY(grd_dev_alloc_bytes(ctx, &p, sizeof(unsigned long long) * (size_t)blocks * TOPK));
      ctx->verify_buf = static_cast<unsigned long long*>(p);
      ctx->verify_cap = (size_t)blocks * TOPK;
    }
    keys = ctx->verify_buf;
    k_topk_blocks<<<blocks, 256, 0, ctx->stream>>>(ctx->st.ranks, ctx->L.V, keys);
    CK_LAUNCH();
    std::vector<unsigned long long> h((size_t)blocks * TOPK);
    CK(cudaMemcpyAsync(h.data(), keys, sizeof(unsigned long long) * h.size(), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    std::sort(h.begin(), h.end(), [](unsigned long long a, unsigned long long b) { return a > b; });
    const uint32_t n = (uint32_t)std::min<uint64_t>(TOPK, ctx->L.V);
    for (uint32_t i = 0; i < n; ++i) {
      const uint32_t bits = (uint32_t)(h[i] >> 32);
      float r;
      std::memcpy(&r, &bits, sizeof r);
      out->top_ids[i] = 0xFFFFFFFFu - (uint32_t)(h[i] & 0xFFFFFFFFull);
      out->top_values[i] = r;
    }
    out->num_top = n;
    return GRD_OK;
  }
  if (ctx->algo == GRD_SSSP_W && !ctx->L.weighted) return GRD_E_INVALID;
  unsigned long long* acc = ctx->st.counters + C_VERIFY;
  CK(cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * 4, ctx->stream));
  const uint32_t blocks = (uint32_t)ctx->num_sms * 8;
  switch (ctx->algo) {
    case GRD_CC: k_verify_edges<A_CC><<<blocks, 256, 0, ctx->stream>>>(ctx->g, ctx->st, acc); break;
    case GRD_SSSP_HOP: k_verify_edges<A_SSSP_HOP><<<blocks, 256, 0, ctx->stream>>>(ctx->g, ctx->st, acc); break;
    case GRD_SSSP_W: k_verify_edges<A_SSSP_W><<<blocks, 256, 0, ctx->stream>>>(ctx->g, ctx->st, acc); break;
    default: return GRD_E_INVALID;
  }
  CK_LAUNCH();
  unsigned long long h[4];
  CK(cudaMemcpyAsync(h, acc, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  out->errors = h[0];
  out->edges_checked = h[1];
  out->count = h[2];
  out->max_value = h[3];
  return GRD_OK;
}
