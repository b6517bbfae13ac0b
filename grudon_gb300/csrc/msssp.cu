// grd_sssp_multi: SSSP from up to 64 sources at once over one resident CSR.
//
// Every vertex keeps 64 distance lanes (dist[v][l], one per source) and a
// 64-bit mask of the lanes whose distance changed in the last round.  A round
// relaxes the out-edges of every vertex with a non-empty mask, for all of
// its changed lanes together: the edge's column and weight are read once,
// and the 64 lanes of the source row (256 contiguous bytes) go to the 64
// lanes of the destination row with atomicMin, the lanes that lowered setting
// the destination's next mask.  Per lane this is the reference's SSSP round
// (src/graph_algorithms/sssp.cpp:61-113: relax from the vertices whose
// distance changed, keep the minimum), seeded from many sources instead of
// one (sssp.cpp:40-46); distances are the same minimum fixed point, so they
// equal per-source runs bit for bit whatever the order of the relaxations.
//
// The edges are those of the ctx's partitioned layout: a vertex's row is
// the CSR row of its owned slot, and each destination slot is mapped to its
// vertex through the slot map, as in NO_OFFLOAD rounds (the compute side
// reads the owners' rows directly; no memory-side copies).
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "ctx.hpp"
#include "kernels.cuh"

using namespace grd;

namespace {

constexpr uint32_t MS_LANES = 64;
constexpr uint32_t INF = 0xFFFFFFFFu;

struct MsState {
  uint32_t* dist;            // [V][64]
  unsigned long long* cur;   // [V] lanes changed in the last round
  unsigned long long* nxt;   // [V] lanes changed in this round
  uint32_t* act;             // [V] vertices with a non-empty mask
  uint32_t* pre;             // [V + 1] their out-degrees, then the exclusive prefix
  uint32_t* count;           // [1] active vertices
  uint32_t* sources;         // [64]
};

__global__ void __launch_bounds__(256) k_ms_init(uint32_t* dist, unsigned long long* cur, unsigned long long* nxt,
                                                 uint32_t V) {
  const uint64_t n = (uint64_t)V * MS_LANES;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    dist[i] = INF;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    cur[v] = 0;
    nxt[v] = 0;
  }
}

__global__ void k_ms_seed(uint32_t* dist, unsigned long long* cur, const uint32_t* src, uint32_t n) {
  const uint32_t l = threadIdx.x;
  if (l < n) {
    dist[(uint64_t)src[l] * MS_LANES + l] = 0;
    atomicOr(cur + src[l], 1ull << l);
  }
}

// Active vertices (non-empty mask) and their out-degrees, appended in any
// order (each entry keeps its own degree beside it).
__global__ void __launch_bounds__(256) k_ms_collect(DevGraph g, const unsigned long long* cur, uint32_t* act,
                                                    uint32_t* deg, uint32_t* count) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += gridDim.x * blockDim.x) {
    if (!cur[v]) continue;
    namespace cg = cooperative_groups;
    cg::coalesced_group grp = cg::coalesced_threads();
    uint32_t base = 0;
    if (grp.thread_rank() == 0) base = atomicAdd(count, grp.size());
    base = grp.shfl(base, 0);
    const uint32_t j = base + grp.thread_rank();
    act[j] = v;
    deg[j] = g.outdeg[v];
  }
}

// One warp per 32 consecutive edges of the frontier's flattened out-edges:
// each lane finds its edge (binary search in the degree prefix), then the
// warp walks the 32 edges, four at a time, each lane handling source lanes l
// and l + 32 of the edge's source row.
template <bool kWeighted>
__global__ void __launch_bounds__(256) k_ms_relax(DevGraph g, DevState st, MsState ms, uint32_t K, uint64_t m) {
  const uint32_t lane = lane_id();
  const uint64_t nchunks = (m + 31) / 32;
  const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t c = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < nchunks; c += nw) {
    const uint64_t e = c * 32 + lane;
    uint32_t u = 0, v = 0, w = 1;
    if (e < m) {
      uint32_t lo = 0, hi = K;  // last i with pre[i] <= e
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (ms.pre[mid] <= e) lo = mid; else hi = mid;
      }
      u = ms.act[lo];
      const uint32_t r = g.row_off[st.own_slot[u]] + (uint32_t)(e - ms.pre[lo]);
      v = __ldg(&g.slot_gid[__ldg(&g.col[r])]);
      if (kWeighted) w = __ldg(&g.wgt[r]);
    }
    const uint32_t cnt = (uint32_t)(m - c * 32 < 32 ? m - c * 32 : 32);
    for (uint32_t j0 = 0; j0 < cnt; j0 += 4) {
      uint32_t uj[4], vj[4], wj[4];
      unsigned long long mk[4];
      uint32_t du[4][2], dv[4][2];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const uint32_t j = min(j0 + q, cnt - 1);  // repeats the last edge: a second relaxation changes nothing
        uj[q] = __shfl_sync(FULL, u, j);
        vj[q] = __shfl_sync(FULL, v, j);
        wj[q] = __shfl_sync(FULL, w, j);
        mk[q] = __ldcg(ms.cur + uj[q]);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const uint32_t s = lane + 32u * h;
          const bool on = (mk[q] >> s) & 1ull;
          du[q][h] = on ? __ldcg(&ms.dist[(uint64_t)uj[q] * MS_LANES + s]) : INF;
          dv[q][h] = on ? __ldcg(&ms.dist[(uint64_t)vj[q] * MS_LANES + s]) : 0u;
        }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const uint32_t s = lane + 32u * h;
          const uint32_t cand = sat_add(du[q][h], wj[q]);
          bool low = false;
          if (cand < dv[q][h]) low = cand < atomicMin(&ms.dist[(uint64_t)vj[q] * MS_LANES + s], cand);
          const uint32_t b = __ballot_sync(FULL, low);
          if (lane == 0 && b) atomicOr(ms.nxt + vj[q], (unsigned long long)b << (32u * h));
        }
    }
  }
}

// dist[v][l] -> out[l][v] for the first n lanes.
__global__ void __launch_bounds__(256) k_ms_transpose(const uint32_t* dist, uint32_t V, uint32_t n, uint32_t* out) {
  const uint64_t total = (uint64_t)V * n;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t l = (uint32_t)(i / V), v = (uint32_t)(i % V);
    out[i] = dist[(uint64_t)v * MS_LANES + l];
  }
}

template <class T>
int alloc(grd_ctx* ctx, T** p, size_t count) {
  void* d = nullptr;
  TRY(grd_dev_alloc_bytes(ctx, &d, sizeof(T) * std::max<size_t>(count, 1)));
  *p = static_cast<T*>(d);
  return GRD_OK;
}

}  // namespace

extern "C" int grd_sssp_multi(grd_ctx* ctx, const uint32_t* sources, uint32_t n, uint32_t* dist_out,
                              grd_stats* stats) {
  TRY(grd_check_ready(ctx));
  if (ctx->algo != GRD_SSSP_HOP && ctx->algo != GRD_SSSP_W) {
    ctx->err = "grd_sssp_multi needs GRD_SSSP_HOP or GRD_SSSP_W as the ctx's algorithm";
    return GRD_E_INVALID;
  }
  if (!sources || !dist_out || n == 0 || n > MS_LANES) {
    ctx->err = "grd_sssp_multi takes 1.." + std::to_string(MS_LANES) + " sources and an output array";
    return GRD_E_INVALID;
  }
  const uint32_t V = ctx->L.V;
  for (uint32_t l = 0; l < n; ++l)
    if (sources[l] >= V) {
      ctx->err = "source " + std::to_string(sources[l]) + " out of range";
      return GRD_E_INVALID;
    }
  CK(cudaSetDevice(ctx->device));
  TRY(grd_wait(ctx, nullptr));
  MsState ms{};
  // resident scratch of the ctx, allocated on first use
  static_assert(MS_LANES == 64, "one 64-bit mask per vertex");
  if (!ctx->ms_dist) {
    TRY(alloc(ctx, &ctx->ms_dist, (size_t)V * MS_LANES));
    TRY(alloc(ctx, &ctx->ms_mask, 2 * (size_t)V));
    TRY(alloc(ctx, &ctx->ms_list, 3 * (size_t)V + 2 + MS_LANES));
  }
  ms.dist = ctx->ms_dist;
  ms.cur = ctx->ms_mask;
  ms.nxt = ctx->ms_mask + V;
  ms.act = ctx->ms_list;
  ms.pre = ctx->ms_list + V;
  ms.count = ctx->ms_list + 2 * (size_t)V + 1;
  ms.sources = ctx->ms_list + 2 * (size_t)V + 2;
  cudaStream_t s = ctx->stream;
  const uint32_t grid = (uint32_t)ctx->num_sms * 8;
  CK(cudaMemcpyAsync(ms.sources, sources, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s));
  k_ms_init<<<grid, 256, 0, s>>>(ms.dist, ms.cur, ms.nxt, V);
  k_ms_seed<<<1, MS_LANES, 0, s>>>(ms.dist, ms.cur, ms.sources, n);
  CK_LAUNCH();
  const bool weighted = ctx->algo == GRD_SSSP_W;
  grd_stats st{};
  uint64_t launches = 2;
  uint32_t h[2];
  while (st.rounds < ctx->params.max_rounds) {
    CK(cudaMemsetAsync(ms.count, 0, sizeof(uint32_t), s));
    k_ms_collect<<<grid, 256, 0, s>>>(ctx->g, ms.cur, ms.act, ms.pre, ms.count);
    CK_LAUNCH();
    CK(cudaMemcpyAsync(&h[0], ms.count, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const uint32_t K = h[0];
    launches += 1;
    if (K == 0) {
      st.converged = 1;
      break;
    }
    TRY(grd_scan_add_u32(ctx, ms.pre, ms.pre, K, true));
    CK(cudaMemcpyAsync(&h[1], ms.pre + K, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const uint64_t m = h[1];
    if (m) {
      const uint64_t chunks = (m + 31) / 32;
      const uint32_t rg = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((chunks + 7) / 8, grid));
      if (weighted)
        k_ms_relax<true><<<rg, 256, 0, s>>>(ctx->g, ctx->st, ms, K, m);
      else
        k_ms_relax<false><<<rg, 256, 0, s>>>(ctx->g, ctx->st, ms, K, m);
      CK_LAUNCH();
      launches += 4;  // the scan's three kernels and the relaxation
    }
    st.edges_scanned += m;
    st.rounds++;
    st.push_rounds++;
    st.actives_total += K;
    std::swap(ms.cur, ms.nxt);
    CK(cudaMemsetAsync(ms.nxt, 0, sizeof(unsigned long long) * V, s));
  }
  if (!st.converged) {  // the cap: report whether any lane is still changing
    CK(cudaMemsetAsync(ms.count, 0, sizeof(uint32_t), s));
    k_ms_collect<<<grid, 256, 0, s>>>(ctx->g, ms.cur, ms.act, ms.pre, ms.count);
    CK_LAUNCH();
    CK(cudaMemcpyAsync(&h[0], ms.count, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    st.converged = h[0] == 0;
    launches += 1;
  }
  // source-major copy for the host, through a buffer allocated once
  const size_t need = (size_t)V * n;
  if (ctx->ms_out_cap < need) {
    TRY(alloc(ctx, &ctx->ms_out, need));
    ctx->ms_out_cap = need;
  }
  k_ms_transpose<<<grid, 256, 0, s>>>(ms.dist, V, n, ctx->ms_out);
  CK_LAUNCH();
  CK(cudaMemcpyAsync(dist_out, ctx->ms_out, sizeof(uint32_t) * need, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  st.kernel_launches = launches + 1;
  if (stats) *stats = st;
  return GRD_OK;
}
