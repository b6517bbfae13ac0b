// C ABI of the per-round graph operator: context lifetime, layout upload and
// the round stages.  See include/grudon_gpu.h for the contract and the
// reference interface each entry point replaces.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/grudon_gpu.h"
#include "ctx.hpp"
#include "kernels.cuh"

using namespace grd;

static thread_local std::string g_create_error;

int grd_dev_alloc_bytes(grd_ctx* ctx, void** p, size_t bytes) {
  void* d = nullptr;
  cudaError_t e = cudaMalloc(&d, std::max<size_t>(bytes, 4));
  if (e != cudaSuccess) {
    ctx->err = "cudaMalloc(" + std::to_string(bytes) + " B): " + cudaGetErrorString(e);
    (void)cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? GRD_E_OOM : GRD_E_CUDA;
  }
  ctx->allocs.push_back(d);
  *p = d;
  return GRD_OK;
}

namespace {

template <class T>
int dev_alloc(grd_ctx* ctx, T** p, size_t count) {
  void* d = nullptr;
  int rc = grd_dev_alloc_bytes(ctx, &d, sizeof(T) * std::max<size_t>(count, 1));
  if (rc == GRD_OK) *p = static_cast<T*>(d);
  return rc;
}

// Stream-ordered scratch (cudaMallocAsync), for set-up passes.
template <class T>
int dev_alloc_async(grd_ctx* ctx, T** p, size_t count) {
  void* d = nullptr;
  const cudaError_t e = cudaMallocAsync(&d, sizeof(T) * std::max<size_t>(count, 1), ctx->stream);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    ctx->err = std::string("scratch allocation: ") + cudaGetErrorString(e);
    return GRD_E_OOM;
  }
  *p = static_cast<T*>(d);
  return GRD_OK;
}

template <class T>
int upload(grd_ctx* ctx, T* dst, const std::vector<T>& src) {
  if (src.empty()) return GRD_OK;
  const auto it = ctx->pinned_twin.find(src.data());
  const bool twin = it != ctx->pinned_twin.end() && it->second.bytes == sizeof(T) * src.size();
  const void* from = twin ? it->second.p : (const void*)src.data();
  CK(cudaMemcpyAsync(dst, from, sizeof(T) * src.size(), cudaMemcpyHostToDevice, ctx->stream));
  ctx->upload_bytes += sizeof(T) * src.size();
  return GRD_OK;
}

// Blocks of the degree-scan kernels (fixed grid, segments sized on device).
uint32_t lbs_blocks(const grd_ctx* ctx) { return (uint32_t)ctx->num_sms * 4; }

}  // namespace

// Allocates every resident array from the layout's sizes (the host build
// uploads into them, the device build fills them).
int grd_alloc_resident(grd_ctx* ctx) {
  const Layout& L = ctx->L;
  DevGraph& g = ctx->g;
  DevState& st = ctx->st;
  g.V = L.V;
  g.M = L.M;
  g.S = L.S;
  g.num_tiles = (uint32_t)L.num_tiles();
  g.num_hubs = (uint32_t)L.hubs.size();
  g.E = L.E;
  g.bv_bytes = g.bv_refbytes = 0;
  for (uint32_t p = 0; p < L.M; ++p) {
    const unsigned long long words64 = ((unsigned long long)L.T(p) + 63ull) / 64ull;
    g.bv_bytes += words64 * 8ull;
    g.bv_refbytes += words64 * 64ull;
  }
  const size_t V = L.V, S = L.S, E = L.E, M = L.M, T = L.num_tiles();
  const size_t VW = (V + 31) / 32, SW = S / 32;
  TRY(dev_alloc(ctx, (uint32_t**)&g.slot_gid, S));
  TRY(dev_alloc(ctx, (uint32_t**)&g.row_off, S + 1));
  TRY(dev_alloc(ctx, (uint32_t**)&g.col, std::max<size_t>(E, 4)));
  if (L.weighted) TRY(dev_alloc(ctx, (uint32_t**)&g.wgt, std::max<size_t>(E, 4)));
  TRY(dev_alloc(ctx, (uint32_t**)&g.outdeg, V));
  if (!ctx->device_layout) TRY(dev_alloc(ctx, (HubChunkD**)&g.hubs, L.hubs.size()));  // device: sized when built
  TRY(dev_alloc(ctx, (uint32_t**)&g.tile_part, T));
  TRY(dev_alloc(ctx, (uint32_t**)&g.part_base, M));
  TRY(dev_alloc(ctx, (uint32_t**)&g.part_T, M));
  TRY(dev_alloc(ctx, (uint32_t**)&g.part_owned, M));
  TRY(dev_alloc(ctx, &st.prop, V));
  TRY(dev_alloc(ctx, &st.upd, V));
  TRY(dev_alloc(ctx, &st.ranks, V));
  TRY(dev_alloc(ctx, &st.F, VW));
  TRY(dev_alloc(ctx, &st.UD, VW));
  TRY(dev_alloc(ctx, &st.mprop, S));
  TRY(dev_alloc(ctx, &st.mupd, S));
  TRY(dev_alloc(ctx, &st.snap, S));
  TRY(dev_alloc(ctx, &st.FB, SW));
  TRY(dev_alloc(ctx, &st.MD, SW));
  TRY(dev_alloc(ctx, &st.FV, S));
  TRY(dev_alloc(ctx, &st.BV, S));
  TRY(dev_alloc(ctx, &st.AL, S));
  TRY(dev_alloc(ctx, &st.tile_cnt, T));
  TRY(dev_alloc(ctx, &st.tile_deg, T));
  TRY(dev_alloc(ctx, &st.warp_deg, 8 * (size_t)T));
  TRY(dev_alloc(ctx, &st.DP, S + 1));
  TRY(dev_alloc(ctx, &st.RB, S));
  TRY(dev_alloc(ctx, &st.SV, S));
  TRY(dev_alloc(ctx, &st.chunk_start, E / LBS_CHUNK + 2));
  TRY(dev_alloc(ctx, &st.blk_sum, lbs_blocks(ctx)));
  TRY(dev_alloc(ctx, &st.counters, NUM_COUNTERS));
  TRY(dev_alloc(ctx, &st.FL, V));
  TRY(dev_alloc(ctx, &st.DL, S));
  TRY(dev_alloc(ctx, &st.UL, V));
  TRY(dev_alloc(ctx, &st.own_slot, V));
  TRY(dev_alloc(ctx, &st.lc, NUM_LIST_COUNTERS));
  CK(cudaMemsetAsync(st.counters, 0, sizeof(unsigned long long) * NUM_COUNTERS, ctx->stream));
  CK(cudaMemsetAsync(st.lc, 0, sizeof(uint32_t) * NUM_LIST_COUNTERS, ctx->stream));
  return GRD_OK;
}

// Vertex arrays that follow from the slot map and the row offsets: every
// owned slot s of gid v gives own_slot[v] = s and outdeg[v] = its row length.
static __global__ void __launch_bounds__(256) k_derive_vertex_arrays(DevGraph g, uint32_t* own_slot,
                                                                     uint32_t* outdeg) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < g.S; s += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t p = g.tile_part[s / K_TILE_SLOTS];
    if (s - g.part_base[p] >= g.part_owned[p]) continue;
    const uint32_t v = g.slot_gid[s];
    own_slot[v] = (uint32_t)s;
    outdeg[v] = g.row_off[s + 1] - g.row_off[s];
  }
}

// Weights sent as bytes (every weight below 256) widened to the resident
// u32 array.
static __global__ void __launch_bounds__(256) k_widen_weights(const uint8_t* __restrict__ w8, uint64_t n,
                                                              uint32_t* w) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    w[i] = w8[i];
}

// The out-edge columns and the edge weights of both views (out-edge weights
// below 256 travel as bytes and are widened on the device).
static int upload_out_edges(grd_ctx* ctx) {
  const Layout& L = ctx->L;
  DevGraph& g = ctx->g;
  TRY(upload(ctx, (uint32_t*)g.col, L.col));
  if (L.weighted && !ctx->wgt8_host.empty()) {
    TRY(upload(ctx, ctx->wgt8_dev, ctx->wgt8_host));
    k_widen_weights<<<(uint32_t)ctx->num_sms * 8, 256, 0, ctx->stream>>>(ctx->wgt8_dev, L.E, (uint32_t*)g.wgt);
    CK_LAUNCH();
  } else if (L.weighted) {
    TRY(upload(ctx, (uint32_t*)g.wgt, L.wgt));
  }
  if (ctx->in_edges_alloc && L.weighted) TRY(upload(ctx, (uint32_t*)g.in_wgt, L.in_wgt));
  ctx->out_edges_stale = false;
  return GRD_OK;
}

int grd_ensure_out_edges(grd_ctx* ctx) {
  if (!ctx->out_edges_stale) return GRD_OK;
  const uint64_t b = ctx->upload_bytes;
  TRY(upload_out_edges(ctx));
  ctx->upload_bytes = b;  // not part of the caller's upload
  return GRD_OK;
}

int grd_upload_layout(grd_ctx* ctx) {
  const Layout& L = ctx->L;
  DevGraph& g = ctx->g;
  ctx->upload_bytes = 0;
  ctx->layout_gen++;  // derived arrays (PR_PULL) are rebuilt from the new copy
  TRY(upload(ctx, (uint32_t*)g.slot_gid, L.slot_gid));
  TRY(upload(ctx, (uint32_t*)g.row_off, L.row_off));
  // A Jacobi PageRank ctx reads the in-edge sources, the row offsets
  // (out-degrees) and the slot map only: its out-edges and weights follow
  // when another algorithm or a layout read needs them (grd_ensure_out_edges).
  const bool pr_pull_only = ctx->algo == GRD_PR_PULL && ctx->in_edges_alloc;
  if (pr_pull_only)
    ctx->out_edges_stale = true;
  else
    TRY(upload_out_edges(ctx));
  // the small tables, from their pinned copy (a pageable copy would block
  // the caller until the stream's earlier copies are done)
  static_assert(sizeof(HubChunk) == sizeof(HubChunkD), "hub chunk layout");
  const unsigned char* sm = ctx->h_small;
  const size_t nh = sizeof(HubChunk) * L.hubs.size(), nt = sizeof(uint32_t) * L.tile_part.size(),
               nm = sizeof(uint32_t) * L.M;
  if (nh) CK(cudaMemcpyAsync((void*)g.hubs, sm, nh, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync((void*)g.tile_part, sm + nh, nt, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync((void*)g.part_base, sm + nh + nt, nm, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync((void*)g.part_T, sm + nh + nt + nm, nm, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync((void*)g.part_owned, sm + nh + nt + 2 * nm, nm, cudaMemcpyHostToDevice, ctx->stream));
  ctx->upload_bytes += nh + nt + 3 * nm;
  k_derive_vertex_arrays<<<(uint32_t)ctx->num_sms * 8, 256, 0, ctx->stream>>>(g, ctx->st.own_slot, (uint32_t*)g.outdeg);
  CK_LAUNCH();
  if (ctx->in_edges_alloc) {
    TRY(upload(ctx, (uint32_t*)g.in_off, L.in_off));
    TRY(upload(ctx, (uint32_t*)g.in_src, L.in_src));
  }
  // stream-ordered: the pinned host arrays belong to the ctx and outlive the
  // copies; the small pageable ones are staged before the copy call returns
  return GRD_OK;
}

int grd_ensure_in_edges(grd_ctx* ctx) {
  if (ctx->in_edges_alloc) return GRD_OK;
  if (ctx->device_layout) return grd_device_in_edges(ctx);
  build_in_edges(ctx->L);
  const Layout& L = ctx->L;
  TRY(dev_alloc(ctx, (uint32_t**)&ctx->g.in_off, L.S + 1));
  TRY(dev_alloc(ctx, (uint32_t**)&ctx->g.in_src, std::max<size_t>(L.E, 4)));
  if (L.weighted) TRY(dev_alloc(ctx, (uint32_t**)&ctx->g.in_wgt, std::max<size_t>(L.E, 4)));
  ctx->in_edges_alloc = true;
  for (const auto* v : {&ctx->L.in_off, &ctx->L.in_src, &ctx->L.in_wgt})
    grd_pin_twin(ctx, v->data(), v->size() * sizeof(uint32_t));
  TRY(upload(ctx, (uint32_t*)ctx->g.in_off, L.in_off));
  TRY(upload(ctx, (uint32_t*)ctx->g.in_src, L.in_src));
  if (L.weighted) TRY(upload(ctx, (uint32_t*)ctx->g.in_wgt, L.in_wgt));
  ctx->pull.num_in_hubs = (uint32_t)L.in_hubs.size();
  TRY(dev_alloc(ctx, &ctx->pull.in_hubs, std::max<size_t>(L.in_hubs.size(), 1)));
  if (!L.in_hubs.empty())
    CK(cudaMemcpyAsync(ctx->pull.in_hubs, L.in_hubs.data(), sizeof(HubChunkD) * L.in_hubs.size(),
                       cudaMemcpyHostToDevice, ctx->stream));
  ctx->pull.num_in_meds = (uint32_t)L.in_meds.size();
  TRY(dev_alloc(ctx, &ctx->pull.in_meds, std::max<size_t>(L.in_meds.size(), 1)));
  if (!L.in_meds.empty())
    CK(cudaMemcpyAsync(ctx->pull.in_meds, L.in_meds.data(), sizeof(HubChunkD) * L.in_meds.size(),
                       cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return GRD_OK;
}

// Delta PageRank sums every list of more than 32 in-edges grid-wide by
// 32-edge chunks: the table lists those slots (slot, first edge, end), per
// list its first chunk, and per chunk its list.  Built on the device from the
// in-edge view whenever the layout changed.
static __global__ void __launch_bounds__(256) k_prd_mark(DevGraph g, uint32_t* flag, uint32_t* nch) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < g.S; s += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t n = g.in_off[s + 1] - g.in_off[s];
    const bool lng = n > K_PRD_SHORT;
    flag[s] = lng ? 1u : 0u;
    nch[s] = lng ? (n + 31) / 32 : 0u;
  }
}

static __global__ void __launch_bounds__(256) k_prd_fill(DevGraph g, const uint32_t* flag, const uint32_t* pos,
                                                         const uint32_t* cpos, HubChunkD* lists, uint32_t* coff,
                                                         uint32_t* chunk_list) {
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < g.S; s += (uint64_t)gridDim.x * blockDim.x) {
    if (!flag[s]) continue;
    const uint32_t k = pos[s], a = g.in_off[s], b = g.in_off[s + 1];
    lists[k] = HubChunkD{(uint32_t)s, a, b};
    coff[k] = cpos[s];
    const uint32_t q1 = cpos[s] + (b - a + 31) / 32;
    for (uint32_t q = cpos[s]; q < q1; ++q) chunk_list[q] = k;
  }
}

int grd_pr_delta_hubs(grd_ctx* ctx) {
  PullState& P = ctx->pull;
  if (P.hub_gen == ctx->layout_gen) return GRD_OK;
  const uint64_t S = ctx->L.S;
  cudaStream_t s = ctx->stream;
  uint32_t *flag = nullptr, *nch = nullptr, *pos = nullptr, *cpos = nullptr;
  TRY(dev_alloc_async(ctx, &flag, S));
  TRY(dev_alloc_async(ctx, &nch, S));
  TRY(dev_alloc_async(ctx, &pos, S + 1));
  TRY(dev_alloc_async(ctx, &cpos, S + 1));
  const uint32_t grid = (uint32_t)ctx->num_sms * 8;
  k_prd_mark<<<grid, 256, 0, s>>>(ctx->g, flag, nch);
  CK_LAUNCH();
  int rc = grd_scan_add_u32(ctx, flag, pos, S, true);
  if (rc == GRD_OK) rc = grd_scan_add_u32(ctx, nch, cpos, S, true);
  uint32_t tot[2] = {0, 0};
  if (rc == GRD_OK) {
    CK(cudaMemcpyAsync(&tot[0], pos + S, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&tot[1], cpos + S, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  const uint32_t nl = tot[0], nc = tot[1];
  if (rc == GRD_OK && (nl > P.prd_list_cap || !P.prd_lists)) {
    rc = dev_alloc(ctx, &P.prd_lists, std::max<size_t>(nl, 1));
    if (rc == GRD_OK) rc = dev_alloc(ctx, &P.hub_coff, (size_t)nl + 1);
    if (rc == GRD_OK) P.prd_list_cap = nl;
  }
  if (rc == GRD_OK && (nc > P.hub_chunk_cap || !P.chunk_hub)) {
    rc = dev_alloc(ctx, &P.chunk_hub, std::max<size_t>(nc, 1));
    if (rc == GRD_OK) rc = dev_alloc(ctx, &P.chunk_sum, std::max<size_t>(nc, 1));
    if (rc == GRD_OK) P.hub_chunk_cap = nc;
  }
  if (rc == GRD_OK) {
    k_prd_fill<<<grid, 256, 0, s>>>(ctx->g, flag, pos, cpos, P.prd_lists, P.hub_coff, P.chunk_hub);
    CK_LAUNCH();
    CK(cudaMemcpyAsync(P.hub_coff + nl, &nc, sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));  // nc lives on this stack frame
  }
  for (void* p : {(void*)flag, (void*)nch, (void*)pos, (void*)cpos}) cudaFreeAsync(p, s);
  TRY(rc);
  P.num_prd_lists = nl;
  P.num_hub_chunks = nc;
  P.hub_gen = ctx->layout_gen;
  return GRD_OK;
}

// ---------------------------------------------------------------- stages --
namespace {

template <class F>
int dispatch(int algo, F&& f) {
  switch (algo) {
    case GRD_PR_DELTA: return f(std::integral_constant<int, A_PR_DELTA>{});
    case GRD_CC: return f(std::integral_constant<int, A_CC>{});
    case GRD_SSSP_HOP: return f(std::integral_constant<int, A_SSSP_HOP>{});
    case GRD_SSSP_W: return f(std::integral_constant<int, A_SSSP_W>{});
    default: return GRD_E_INVALID;
  }
}

int check_ready(grd_ctx* ctx) {
  if (!ctx) return GRD_E_INVALID;
  if (!ctx->layout_valid) {
    ctx->err = "the layout was left incomplete by a failed grd_ingest: ingest a matching graph first";
    return GRD_E_INVALID;
  }
  if (ctx->algo < 0) {
    ctx->err = "no algorithm selected (grd_set_algo)";
    return GRD_E_INVALID;
  }
  if (!ctx->inited) {
    ctx->err = "grd_init has not been called";
    return GRD_E_INVALID;
  }
  return GRD_OK;
}

uint32_t grid_for(grd_ctx* ctx, uint32_t blocks_per_sm) { return (uint32_t)ctx->num_sms * blocks_per_sm; }

// One full wave of a grid-stride kernel: SMs x resident 256-thread blocks.
template <class Kernel>
uint32_t resident_grid(grd_ctx* ctx, Kernel k) {
  int per_sm = 0;
  if (ctx->params.push_blocks_per_sm) return (uint32_t)ctx->num_sms * ctx->params.push_blocks_per_sm;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, 0) != cudaSuccess || per_sm <= 0) {
    (void)cudaGetLastError();
    per_sm = 4;
  }
  return (uint32_t)ctx->num_sms * (uint32_t)per_sm;
}

// Round format.  Bitvector rounds sync through per-partition bitvectors
// (O(slots) scans) and track dirty slots densely (reductions, then one linear
// diff pass); list rounds sync through (slot, value) lists and track dirty
// slots with returned atomics (O(frontier + its edges)).  The fixed rule
// takes the bitvector form when the frontier entering the round holds at
// least 1/dense_div of the slots or of the edges.  GRD_FMT_BITVEC /
// GRD_FMT_LIST force it.  k_policy applies the same rule on the device.
bool use_dense(const grd_ctx* ctx) {
  if (ctx->params.frontier_format == GRD_FMT_BITVEC) return true;
  if (ctx->params.frontier_format == GRD_FMT_LIST) return false;
  const uint64_t d = ctx->params.dense_div;
  return ctx->last_frontier * d >= ctx->g.S || ctx->last_fedges * d >= ctx->L.E;
}

// Direction: the pull map reads every in-edge once; the push map reads only
// the frontier's out-edges (load-balanced).  Measured on RMAT, push wins even
// for full frontiers, so the fixed rule pulls only when at least 1/pull_div of
// the vertices are active and the in-edge view exists (it is built when pull
// is requested).
// Pull rounds are available when the in-edge view exists; delta PageRank
// always has it (its fixed-order sums read it), but pulls only when asked to
// (GRD_DIR_PULL, or the learned policy), so the plain method stays the push
// method.
bool pull_available(const grd_ctx* ctx) {
  if (!ctx->in_edges_alloc) return false;
  if (ctx->algo != GRD_PR_DELTA) return true;
  const grd_params& p = ctx->params;
  return p.direction == GRD_DIR_PULL || (p.policy == GRD_POLICY_LEARNED && p.direction == GRD_DIR_AUTO);
}

bool use_pull(const grd_ctx* ctx) {
  if (!pull_available(ctx)) return false;
  if (ctx->params.direction == GRD_DIR_PULL) return true;
  if (ctx->params.direction == GRD_DIR_PUSH) return false;
  return ctx->last_frontier * ctx->params.pull_div >= ctx->g.V;
}

}  // namespace

int grd_check_ready(grd_ctx* ctx) { return check_ready(ctx); }

int grd_choose_round_mode(const grd_ctx* ctx) {
  if (policy_no_offload(ctx->params.offload, ctx->last_frontier, ctx->g.V)) return RM_NO_OFFLOAD;
  const bool pull = use_pull(ctx), list = !use_dense(ctx);
  return pull ? (list ? RM_PULL_LIST : RM_PULL_BITVEC) : (list ? RM_PUSH_LIST : RM_PUSH_BITVEC);
}

PolicyArgs grd_policy_args(const grd_ctx* ctx) {
  PolicyArgs a{};
  a.direction = ctx->params.direction;
  a.format = ctx->params.frontier_format;
  a.has_in = pull_available(ctx) ? 1 : 0;
  a.dense_div = ctx->params.dense_div;
  a.pull_div = ctx->params.pull_div;
  a.offload = ctx->params.offload;
  a.edges = ctx->L.E;
  a.round = ctx->stats.rounds;
  return a;
}

const grd_policy_model* grd_policy_model_dev(const grd_ctx* ctx) {
  return (ctx->params.policy == GRD_POLICY_LEARNED && ctx->has_policy) ? ctx->policy_dev : nullptr;
}

// Host loop: the next round's mode, by the same policy kernel the device
// loop runs (so both loops choose identically), read back.
static int host_loop_mode(grd_ctx* ctx, int* mode) {
  const grd_policy_model* m = grd_policy_model_dev(ctx);
  if (!m || policy_no_offload(ctx->params.offload, ctx->last_frontier, ctx->g.V)) {
    *mode = grd_choose_round_mode(ctx);  // k_policy decides the offload the same way
    return GRD_OK;
  }
  const PolicyArgs a = grd_policy_args(ctx);
  if (policy_tiny(ctx->last_frontier, ctx->last_fedges, policy_allowed(a.direction, a.format, a.has_in != 0))) {
    *mode = RM_PUSH_LIST;  // k_policy decides the same without inference
    return GRD_OK;
  }
  k_policy<false><<<1, P_HID, 0, ctx->stream>>>(ctx->g, ctx->st, 0, grd_policy_args(ctx), m);
  CK_LAUNCH();
  CK(cudaMemcpyAsync(ctx->h_seed + 7, ctx->st.counters + C_MODE, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *mode = (int)ctx->h_seed[7];
  ctx->stats.kernel_launches += 1;
  return GRD_OK;
}

int grd_enqueue_fwd(grd_ctx* ctx, bool fused) {
  const uint32_t T = ctx->g.num_tiles;
  k_fwd_bits<false><<<T, 256, 0, ctx->stream>>>(ctx->g, ctx->st);
  if (fused) {
    k_compact<<<T, 256, 0, ctx->stream>>>(ctx->st.FB, nullptr, 0u, ctx->g, ctx->st, OpFwdXfer{}, 2);
  } else {
    k_compact<<<T, 256, 0, ctx->stream>>>(ctx->st.FB, nullptr, 0u, ctx->g, ctx->st, OpFwdPack{}, 2);
    k_compact<<<T, 256, 0, ctx->stream>>>(ctx->st.FB, nullptr, 0u, ctx->g, ctx->st, OpFwdUnpack{}, 0);
  }
  CK_LAUNCH();
  ctx->stats.kernel_launches += fused ? 2 : 3;
  return GRD_OK;
}

// Push rounds in bitvector form: the forward sync also places the degree
// prefix of the active list (both degree passes of the edge-map).
static int enqueue_fwd_push(grd_ctx* ctx) {
  const uint32_t T = ctx->g.num_tiles;
  k_fwd_bits<true><<<T, 256, 0, ctx->stream>>>(ctx->g, ctx->st);
  k_fwd_xfer_deg<<<T, 256, 0, ctx->stream>>>(ctx->g, ctx->st);
  CK_LAUNCH();
  return GRD_OK;
}

// Push + bitvector rounds of the min algorithms aggregate in the dirty diff
// (k_diff_aggregate); PageRank keeps its ordered per-partition aggregate.
static bool diff_aggregates(const grd_ctx* ctx) {
  return ctx->algo == GRD_CC || ctx->algo == GRD_SSSP_HOP || ctx->algo == GRD_SSSP_W;
}

// Kernels of the edge-map of one round in each mode.
uint32_t grd_edge_map_launches(const grd_ctx* ctx, int mode) {
  const bool pr = ctx->algo == GRD_PR_DELTA;
  const uint32_t hub_sums = ctx->pull.num_prd_lists ? 2 : 0;  // delta PageRank's chunked long-list sums
  if (mode == RM_PULL_BITVEC || mode == RM_PULL_LIST)
    return pr ? 1 + hub_sums : 1 + (ctx->pull.num_in_meds ? 1 : 0) + (ctx->pull.num_in_hubs ? 1 : 0);
  // push (NO_OFFLOAD too); PageRank's push adds the fixed-order sums
  return 3 + (ctx->g.num_hubs ? 1 : 0) + (mode == RM_PUSH_BITVEC ? 1 : 0) +
         (pr && (mode == RM_PUSH_BITVEC || mode == RM_PUSH_LIST) ? 1 + hub_sums : 0);
}

// Kernels of a whole round in each mode (edge-map + syncs + update).
uint32_t grd_round_launches(const grd_ctx* ctx, int mode) {
  if (mode == RM_PUSH_TINY || mode == RM_NOOFF_TINY) return 1;
  if (mode == RM_NO_OFFLOAD)  // fwd list fused with the first degree pass, retire, update list
    return 2 + grd_edge_map_launches(ctx, mode);
  const bool list = mode == RM_PUSH_LIST || mode == RM_PULL_LIST;
  const uint32_t groups = ctx->algo == GRD_PR_DELTA ? ctx->L.M : 1;
  // bitvector: fwd bits + compaction; the backward tile counts (pull only:
  // the push map's dirty diff writes them) + one compaction per group (none
  // when the dirty diff aggregates); update
  const uint32_t bwd = mode == RM_PUSH_BITVEC && diff_aggregates(ctx) ? 0u
                                                                      : (mode == RM_PULL_BITVEC ? 1u : 0u) + groups;
  // list: fwd, bwd (PageRank: one per partition), update lists
  const uint32_t sync = list ? 2 + groups : (2 + bwd + 1);
  // push: the forward sync runs the degree passes (bitvector: both, list: the first)
  return sync + grd_edge_map_launches(ctx, mode) - (mode == RM_PUSH_LIST ? 1u : mode == RM_PUSH_BITVEC ? 2u : 0u);
}

// Stage API edge-map (bitvector sync around it): push with dense dirty
// tracking, or pull.
int grd_enqueue_edge_map(grd_ctx* ctx) {
  const int mode = use_pull(ctx) ? RM_PULL_BITVEC : RM_PUSH_BITVEC;
  TRY(grd_enqueue_edge_map_mode(ctx, mode));
  ctx->last_mode = mode;
  if (mode == RM_PULL_BITVEC) {
    ctx->stats.pull_rounds++;
    ctx->pull.edges += ctx->L.E;
  } else {
    ctx->stats.push_rounds++;
  }
  ctx->stats.kernel_launches += grd_edge_map_launches(ctx, mode);
  return GRD_OK;
}

int grd_enqueue_edge_map_mode(grd_ctx* ctx, int mode, int degree_passes_done, bool aggregate) {
  ctx->tile_counts_ready = mode == RM_PUSH_BITVEC && !aggregate;  // k_diff_dirty writes them
  return dispatch(ctx->algo, [&](auto a) -> int {
    constexpr int A = decltype(a)::value;
    const uint32_t pull_hub_grid = std::min<uint32_t>(ctx->pull.num_in_hubs, grid_for(ctx, 8));
    const uint32_t pull_med_grid = std::min<uint32_t>((ctx->pull.num_in_meds + 7) / 8, grid_for(ctx, 8));
    const PullState& PS = ctx->pull;
    const PrHubs ph{PS.prd_lists, PS.hub_coff, PS.chunk_hub, PS.chunk_sum, PS.num_prd_lists, PS.num_hub_chunks};
    const uint32_t hsum_grid = std::max<uint32_t>(1, std::min<uint32_t>((ph.nh + 7) / 8, grid_for(ctx, 8)));
    if (A == A_PR_DELTA && (mode == RM_PULL_BITVEC || mode == RM_PULL_LIST)) {  // the fixed-order sums
      if (mode == RM_PULL_LIST)
        k_pr_delta_pull<true><<<grid_for(ctx, 8), 256, 0, ctx->stream>>>(ctx->g, ctx->st);
      else
        k_pr_delta_pull<false><<<grid_for(ctx, 8), 256, 0, ctx->stream>>>(ctx->g, ctx->st);
      if (ph.nh) {
        k_pr_delta_hub_chunks<0><<<grid_for(ctx, 8), 256, 0, ctx->stream>>>(ctx->g, ctx->st, ph);
        if (mode == RM_PULL_LIST)
          k_pr_delta_hub_sum<0, true><<<hsum_grid, 256, 0, ctx->stream>>>(ctx->g, ctx->st, ph);
        else
          k_pr_delta_hub_sum<0, false><<<hsum_grid, 256, 0, ctx->stream>>>(ctx->g, ctx->st, ph);
      }
      CK_LAUNCH();
      return GRD_OK;
    }
    if constexpr (A != A_PR_DELTA) {  // the generic pull serves CC and SSSP
      if (mode == RM_PULL_BITVEC) {
        k_pull<A, false><<<grid_for(ctx, 8), 256, 0, ctx->stream>>>(ctx->g, ctx->st);
        if (ctx->pull.num_in_meds)
          k_pull_med<A, false><<<pull_med_grid, 256, 0, ctx->stream>>>(ctx->g, ctx->st, ctx->pull.in_meds,
                                                                       ctx->pull.num_in_meds);
        if (ctx->pull.num_in_hubs)
          k_pull_hub<A, false><<<pull_hub_grid, 256, 0, ctx->stream>>>(ctx->g, ctx->st, ctx->pull.in_hubs,
                                                                       ctx->pull.num_in_hubs);
        CK_LAUNCH();
        return GRD_OK;
      }
      if (mode == RM_PULL_LIST) {
        k_pull<A, true><<<grid_for(ctx, 8), 256, 0, ctx->stream>>>(ctx->g, ctx->st);
        if (ctx->pull.num_in_meds)
          k_pull_med<A, true><<<pull_med_grid, 256, 0, ctx->stream>>>(ctx->g, ctx->st, ctx->pull.in_meds,
                                                                      ctx->pull.num_in_meds);
        if (ctx->pull.num_in_hubs)
          k_pull_hub<A, true><<<pull_hub_grid, 256, 0, ctx->stream>>>(ctx->g, ctx->st, ctx->pull.in_hubs,
                                                                      ctx->pull.num_in_hubs);
        CK_LAUNCH();
        return GRD_OK;
      }
    }
    const uint32_t B = lbs_blocks(ctx);
    if (degree_passes_done < 1) k_deg_reduce<<<B, 256, 0, ctx->stream>>>(ctx->g, ctx->st);
    if (degree_passes_done < 2) k_deg_down<<<B, 256, 0, ctx->stream>>>(ctx->g, ctx->st);
    // one block per hub item up to 32 per SM: beside the push, more and
    // shorter blocks fill the SMs the push frees sooner (8 per SM: +1.3 % step)
    const uint32_t hub_grid = std::min<uint32_t>(ctx->g.num_hubs, grid_for(ctx, 32));
    // Hub rows on the side stream, beside the load-balanced push; their
    // blocks take the SMs as the push's blocks finish.  The two kernels only
    // meet in atomics: reductions into mupd (min: the values do not depend
    // on the order), dirty-bit claims and list appends, and the edge count.
    // Profiling times each kernel alone: the hub rows then follow the push.
    const bool hubs = ctx->g.num_hubs != 0;
    const bool fork = hubs && !ctx->profiling;
    cudaStream_t hs = fork ? ctx->side : ctx->stream;
    if (fork) {
      CK(cudaEventRecord(ctx->ev_fork, ctx->stream));
      CK(cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
    }
    grd_prof_mark(ctx, 5);
    if (mode == RM_PUSH_BITVEC) {
      k_push_lbs<A, true><<<resident_grid(ctx, k_push_lbs<A, true>), 256, 0, ctx->stream>>>(ctx->g, ctx->st);
      grd_prof_mark(ctx, 6);
      if (hubs) k_hub_push<A, true><<<hub_grid, 256, 0, hs>>>(ctx->g, ctx->st);
    } else if (mode == RM_NO_OFFLOAD) {  // compute-side push into vertex_updates
      k_push_lbs<A, false, true><<<resident_grid(ctx, k_push_lbs<A, false, true>), 256, 0, ctx->stream>>>(ctx->g,
                                                                                                          ctx->st);
      grd_prof_mark(ctx, 6);
      if (hubs) k_hub_push<A, false, true><<<hub_grid, 256, 0, hs>>>(ctx->g, ctx->st);
    } else {
      k_push_lbs<A, false><<<resident_grid(ctx, k_push_lbs<A, false>), 256, 0, ctx->stream>>>(ctx->g, ctx->st);
      grd_prof_mark(ctx, 6);
      if (hubs) k_hub_push<A, false><<<hub_grid, 256, 0, hs>>>(ctx->g, ctx->st);
    }
    if (fork) {
      CK(cudaEventRecord(ctx->ev_join, ctx->side));
      CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
    }
    if (A == A_PR_DELTA && mode == RM_PUSH_BITVEC) {  // the touched slots get the fixed-order sums
      k_pr_delta_resum_bits<<<grid_for(ctx, 8), 256, 0, ctx->stream>>>(ctx->g, ctx->st);
      if (ph.nh) {
        k_pr_delta_hub_chunks<1><<<grid_for(ctx, 8), 256, 0, ctx->stream>>>(ctx->g, ctx->st, ph);
        k_pr_delta_hub_sum<1, false><<<hsum_grid, 256, 0, ctx->stream>>>(ctx->g, ctx->st, ph);
      }
    }
    if (A == A_PR_DELTA && mode == RM_PUSH_LIST) {
      k_pr_delta_resum_list<<<grid_for(ctx, 8), 256, 0, ctx->stream>>>(ctx->g, ctx->st);
      if (ph.nh) {
        k_pr_delta_hub_chunks<2><<<grid_for(ctx, 8), 256, 0, ctx->stream>>>(ctx->g, ctx->st, ph);
        k_pr_delta_hub_sum<2, false><<<hsum_grid, 256, 0, ctx->stream>>>(ctx->g, ctx->st, ph);
      }
    }
    if (mode == RM_PUSH_BITVEC) {
      if constexpr (A != A_PR_DELTA && A != A_PR_PULL) {
        if (aggregate) {
          k_diff_aggregate<A><<<ctx->g.num_tiles, 256, 0, ctx->stream>>>(ctx->g, ctx->st);
          CK_LAUNCH();
          return GRD_OK;
        }
      }
      k_diff_dirty<A><<<ctx->g.num_tiles, 256, 0, ctx->stream>>>(ctx->g, ctx->st);
    }
    CK_LAUNCH();
    return GRD_OK;
  });
}

// Backward sync; fused = pack and aggregate in one pass per partition group.
int grd_enqueue_bwd(grd_ctx* ctx, bool fused, bool do_pack, bool do_aggregate) {
  const uint32_t T = ctx->g.num_tiles;
  const Layout& L = ctx->L;
  return dispatch(ctx->algo, [&](auto a) -> int {
    constexpr int A = decltype(a)::value;
    constexpr bool kPR = (A == A_PR_DELTA);
    if (do_pack) {
      if (!ctx->tile_counts_ready) {  // the push map's dirty diff already counted them
        k_tile_count<<<T, 256, 0, ctx->stream>>>(ctx->st.MD, ctx->st.tile_cnt, ctx->st.FB);
        ctx->stats.kernel_launches += 1;
      }
      if (!fused) {
        k_compact<<<T, 256, 0, ctx->stream>>>(ctx->st.MD, nullptr, 0u, ctx->g, ctx->st, OpBwdPack<A>{}, 1);
        ctx->stats.kernel_launches += 1;
      }
    }
    if (do_aggregate) {
      // PageRank: one launch per partition in ascending order fixes the
      // per-vertex summation order; min-aggregates run as one launch.
      const uint32_t groups = kPR ? L.M : 1;
      for (uint32_t p = 0; p < groups; ++p) {
        uint32_t t0 = kPR ? L.slot_base[p] / TILE_SLOTS : 0;
        uint32_t t1 = kPR ? ((p + 1 < L.M) ? L.slot_base[p + 1] / TILE_SLOTS : T) : T;
        if (fused)
          k_compact<<<t1 - t0, 256, 0, ctx->stream>>>(ctx->st.MD, ctx->st.MD, t0, ctx->g, ctx->st, OpBwdXfer<A>{},
                                                      1);
        else
          k_compact<<<t1 - t0, 256, 0, ctx->stream>>>(ctx->st.MD, ctx->st.MD, t0, ctx->g, ctx->st,
                                                      OpAggregate<A>{}, 0);
      }
      ctx->stats.kernel_launches += groups;
    }
    CK_LAUNCH();
    return GRD_OK;
  });
}

// The per-round counters and list lengths it rebuilds are cleared by the
// forward sync that starts the round.
int grd_enqueue_update(grd_ctx* ctx) {
  const uint32_t blocks = std::max<uint32_t>(1, std::min<uint32_t>((ctx->g.V + 255) / 256, grid_for(ctx, 8)));
  return dispatch(ctx->algo, [&](auto a) -> int {
    constexpr int A = decltype(a)::value;
    k_update<A><<<blocks, 256, 0, ctx->stream>>>(ctx->g, ctx->st, ctx->params.tolerance, ctx->params.damping);
    CK_LAUNCH();
    ctx->stats.kernel_launches += 1;
    return GRD_OK;
  });
}

// List-round stages (three kernels per round besides the edge-map).
int grd_enqueue_fwd_list(grd_ctx* ctx) {
  k_fwd_list<<<grid_for(ctx, 4), 256, 0, ctx->stream>>>(ctx->g, ctx->st);
  CK_LAUNCH();
  return GRD_OK;
}

// Push rounds in list form: forward list sync + first degree pass.
static int enqueue_fwd_list_deg(grd_ctx* ctx) {
  k_fwd_list_deg<<<lbs_blocks(ctx), 256, 0, ctx->stream>>>(ctx->g, ctx->st);
  CK_LAUNCH();
  return GRD_OK;
}

int grd_enqueue_bwd_update_list(grd_ctx* ctx) {
  return dispatch(ctx->algo, [&](auto a) -> int {
    constexpr int A = decltype(a)::value;
    if (A == A_PR_DELTA)  // partition by partition: each vertex sums its partitions' values in order
      for (uint32_t p = 0; p < ctx->L.M; ++p)
        k_bwd_list<A><<<grid_for(ctx, 4), 256, 0, ctx->stream>>>(ctx->g, ctx->st, p);
    else
      k_bwd_list<A><<<grid_for(ctx, 4), 256, 0, ctx->stream>>>(ctx->g, ctx->st, 0xFFFFFFFFu);
    k_update_list<A><<<grid_for(ctx, 4), 256, 0, ctx->stream>>>(ctx->g, ctx->st, ctx->params.tolerance,
                                                                ctx->params.damping);
    CK_LAUNCH();
    return GRD_OK;
  });
}

// NO_OFFLOAD round after its edge-map: retire the old frontier and count the
// shipped adjacency, then the update over the updated-gid list.
static int enqueue_retire_update_list(grd_ctx* ctx) {
  return dispatch(ctx->algo, [&](auto a) -> int {
    constexpr int A = decltype(a)::value;
    k_retire_list<A><<<grid_for(ctx, 4), 256, 0, ctx->stream>>>(ctx->g, ctx->st);
    grd_prof_mark(ctx, 3);
    k_update_list<A><<<grid_for(ctx, 4), 256, 0, ctx->stream>>>(ctx->g, ctx->st, ctx->params.tolerance,
                                                                ctx->params.damping);
    CK_LAUNCH();
    return GRD_OK;
  });
}

// One whole round in a given mode (host loop and loop-graph branches).
int grd_enqueue_round(grd_ctx* ctx, int mode) {
  if (mode == RM_PUSH_TINY || mode == RM_NOOFF_TINY) {  // the whole round counts as edge-map time
    grd_prof_mark(ctx, 1);
    TRY(dispatch(ctx->algo, [&](auto a) -> int {
      constexpr int A = decltype(a)::value;
      const double tol = ctx->params.tolerance, d = ctx->params.damping;
      if (ctx->capturing_loop) {  // the device-driven loop: small rounds continue in the kernel
        const PolicyArgs pa = grd_policy_args(ctx);
        const grd_policy_model* m = grd_policy_model_dev(ctx);
        const uint32_t cap = ctx->params.max_rounds;
        if (mode == RM_NOOFF_TINY)
          k_round_tiny_loop<A, true><<<1, K_TINY_THREADS, 0, ctx->stream>>>(ctx->g, ctx->st, tol, d, pa, m, cap);
        else
          k_round_tiny_loop<A, false><<<1, K_TINY_THREADS, 0, ctx->stream>>>(ctx->g, ctx->st, tol, d, pa, m, cap);
      } else if (mode == RM_NOOFF_TINY) {
        k_round_tiny<A, true><<<1, K_TINY_THREADS, 0, ctx->stream>>>(ctx->g, ctx->st, tol, d);
      } else {
        k_round_tiny<A><<<1, K_TINY_THREADS, 0, ctx->stream>>>(ctx->g, ctx->st, tol, d);
      }
      CK_LAUNCH();
      return GRD_OK;
    }));
    grd_prof_mark(ctx, 2);
    grd_prof_mark(ctx, 3);
    ctx->stats.kernel_launches += 1;
    return GRD_OK;
  }
  if (mode == RM_NO_OFFLOAD) {
    const uint64_t launches = ctx->stats.kernel_launches;
    TRY(enqueue_fwd_list_deg(ctx));
    grd_prof_mark(ctx, 1);
    TRY(grd_enqueue_edge_map_mode(ctx, mode, 1));
    grd_prof_mark(ctx, 2);
    TRY(enqueue_retire_update_list(ctx));
    ctx->stats.kernel_launches = launches + grd_round_launches(ctx, mode);
    return GRD_OK;
  }
  const bool list = mode == RM_PUSH_LIST || mode == RM_PULL_LIST;
  const uint64_t launches = ctx->stats.kernel_launches;
  const bool push_list = mode == RM_PUSH_LIST;
  if (push_list) {
    TRY(enqueue_fwd_list_deg(ctx));  // timed as the forward sync
  } else if (list) {
    TRY(grd_enqueue_fwd_list(ctx));
  } else if (mode == RM_PUSH_BITVEC) {
    TRY(enqueue_fwd_push(ctx));
  } else {
    TRY(grd_enqueue_fwd(ctx, true));
  }
  grd_prof_mark(ctx, 1);
  const bool aggregate = mode == RM_PUSH_BITVEC && diff_aggregates(ctx);
  TRY(grd_enqueue_edge_map_mode(ctx, mode, push_list ? 1 : mode == RM_PUSH_BITVEC ? 2 : 0, aggregate));
  grd_prof_mark(ctx, 2);
  if (list) {
    TRY(grd_enqueue_bwd_update_list(ctx));
    grd_prof_mark(ctx, 3);
  } else {
    if (!aggregate) TRY(grd_enqueue_bwd(ctx, true, true, true));
    grd_prof_mark(ctx, 3);
    TRY(grd_enqueue_update(ctx));
  }
  ctx->stats.kernel_launches = launches + grd_round_launches(ctx, mode);
  return GRD_OK;
}

// Once per round, after the update: copies the device counters to the host
// (the only host synchronisation of a round) and folds them into the stats.
int grd_read_counters(grd_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->h_counters, ctx->st.counters, sizeof(unsigned long long) * NUM_COUNTERS,
                     cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return grd_fold_counters(ctx);
}

// The counters copied by grd_init, once a host-side decision needs them.
int grd_sync_init_counters(grd_ctx* ctx) {
  if (!ctx->counters_stale) return GRD_OK;
  CK(cudaStreamSynchronize(ctx->stream));
  const grd_stats keep = ctx->stats;  // only the frontier shape is wanted
  const int rc = grd_fold_counters(ctx);
  ctx->stats = keep;
  return rc;
}

// Folds the host copy of the counters into the stats.
int grd_fold_counters(grd_ctx* ctx) {
  ctx->counters_stale = false;
  ctx->stats.edges_scanned = ctx->h_counters[C_EDGES] + ctx->pull.edges;
  ctx->stats.bytes_synced = ctx->h_counters[C_BYTES];
  ctx->stats.reference_bytes_moved = ctx->h_counters[C_REFBYTES];
  ctx->stats.actives_total += ctx->h_counters[C_ACTIVE];
  if (ctx->last_mode >= 0 && !rm_is_pull(ctx->last_mode)) ctx->stats.push_actives += ctx->h_counters[C_ACTIVE];
  ctx->last_mode = -1;
  ctx->last_frontier = ctx->h_counters[C_FRONTIER];
  ctx->last_fedges = ctx->h_counters[C_FEDGES];
  if (ctx->h_counters[C_ERR]) {
    ctx->err = "device-side error code " + std::to_string(ctx->h_counters[C_ERR]);
    return ctx->h_counters[C_ERR] == 1 ? GRD_E_TIMEOUT : GRD_E_CUDA;
  }
  return GRD_OK;
}

// Stage timing: events 0..4 bracket forward sync, edge-map, backward sync and
// update of one round; read after the round's synchronisation.
void grd_prof_mark(grd_ctx* ctx, int i) {
  if (!ctx->profiling) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(ctx->stream, &cs);
  // inside a captured round graph the mark becomes an event-record node
  if (cs == cudaStreamCaptureStatusActive)
    cudaEventRecordWithFlags(ctx->ev[i], ctx->stream, cudaEventRecordExternal);
  else
    cudaEventRecord(ctx->ev[i], ctx->stream);
}

void grd_prof_collect(grd_ctx* ctx, double* out) {
  if (!ctx->profiling) return;
  float ms;
  for (int i = 0; i < 5; ++i) {
    const cudaEvent_t a = ctx->ev[i < 4 ? i : 0], b = ctx->ev[i < 4 ? i + 1 : 4];
    const double v = cudaEventElapsedTime(&ms, a, b) == cudaSuccess ? ms : 0.0;
    ctx->stats.stage_ms[i] += v;
    if (out) out[i] = v;
  }
  (void)cudaGetLastError();
}

void grd_prof_collect(grd_ctx* ctx) { grd_prof_collect(ctx, nullptr); }

// ------------------------------------------------------------------ C ABI --
extern "C" {

const char* grd_version(void) { return "grudon-gb300 0.1 (sm_103a)"; }

int grd_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return n;
}

const char* grd_create_error(void) { return g_create_error.c_str(); }

const char* grd_last_error(const grd_ctx* ctx) { return ctx ? ctx->err.c_str() : "null ctx"; }

int grd_ctx_create(const grd_csr* graph, const uint32_t* mirror_part, uint32_t num_compute, uint32_t num_memory,
                   int device, grd_ctx** out) {
  g_create_error.clear();
  if (!out) {
    g_create_error = "out is NULL";
    return GRD_E_INVALID;
  }
  *out = nullptr;
  if (!graph) {
    g_create_error = "graph is NULL";
    return GRD_E_INVALID;
  }
  if (num_compute != 1) {
    g_create_error = "num_compute must be 1";
    return GRD_E_INVALID;
  }
  int ndev = grd_device_count();
  if (ndev <= 0) {
    g_create_error = "no CUDA device visible";
    return GRD_E_CUDA;
  }
  if (device < 0 || device >= ndev) {
    g_create_error = "device index out of range";
    return GRD_E_INVALID;
  }
  grd_ctx* ctx = new (std::nothrow) grd_ctx();
  if (!ctx) return GRD_E_OOM;
  ctx->device = device;
  std::string why = build_layout(graph->num_vertices, graph->num_edges, graph->row_offsets, graph->col_indices,
                                 graph->weights, mirror_part, num_memory, ctx->L);
  if (!why.empty()) {
    g_create_error = why;
    delete ctx;
    return GRD_E_INVALID;
  }
  int rc = grd_ctx_init_device(ctx);
  if (rc != GRD_OK) {
    g_create_error = ctx->err;
    grd_ctx_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return GRD_OK;
}

int grd_ctx_create_ex(const grd_csr* graph, const uint32_t* mirror_part, uint32_t num_compute, uint32_t num_memory,
                      int device, uint32_t flags, grd_ctx** out) {
  if (!out) return GRD_E_INVALID;
  if (!(flags & GRD_CREATE_DEVICE_LAYOUT))
    return flags ? (g_create_error = "unknown create flags", GRD_E_INVALID)
                 : grd_ctx_create(graph, mirror_part, num_compute, num_memory, device, out);
  if (flags & ~GRD_CREATE_DEVICE_LAYOUT) {
    g_create_error = "unknown create flags";
    return GRD_E_INVALID;
  }
  *out = nullptr;
  g_create_error.clear();
  if (num_compute != 1) {
    g_create_error = "num_compute must be 1";
    return GRD_E_INVALID;
  }
  std::string why;
  if (grd_device_layout_check(graph, num_memory, &why) != GRD_OK) {
    g_create_error = why;
    return GRD_E_INVALID;
  }
  const int ndev = grd_device_count();
  if (ndev <= 0) {
    g_create_error = "no CUDA device visible";
    return GRD_E_CUDA;
  }
  if (device < 0 || device >= ndev) {
    g_create_error = "device index out of range";
    return GRD_E_INVALID;
  }
  grd_ctx* ctx = new (std::nothrow) grd_ctx();
  if (!ctx) return GRD_E_OOM;
  ctx->device = device;
  ctx->device_layout = true;
  ctx->L.V = graph->num_vertices;
  ctx->L.E = graph->num_edges;
  ctx->L.M = num_memory;
  ctx->L.weighted = graph->weights != nullptr;
  int rc = grd_ctx_init_stream(ctx);
  if (rc == GRD_OK) rc = grd_device_layout_build(ctx, graph, mirror_part, true);
  if (rc != GRD_OK) {
    g_create_error = ctx->err;
    grd_ctx_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return GRD_OK;
}

int grd_ingest(grd_ctx* ctx, const grd_csr* graph, const uint32_t* mirror_part, uint64_t* bytes_copied) {
  if (!ctx) return GRD_E_INVALID;
  if (!ctx->device_layout) {
    ctx->err = "grd_ingest needs a ctx created with GRD_CREATE_DEVICE_LAYOUT";
    return GRD_E_INVALID;
  }
  std::string why;
  if (grd_device_layout_check(graph, ctx->L.M, &why) != GRD_OK) {
    ctx->err = why;
    return GRD_E_INVALID;
  }
  CK(cudaSetDevice(ctx->device));
  TRY(grd_wait(ctx, nullptr));
  const int rc = grd_device_layout_build(ctx, graph, mirror_part, false);
  if (bytes_copied) *bytes_copied = ctx->upload_bytes;
  return rc;
}

void grd_ctx_destroy(grd_ctx* ctx) {
  if (!ctx) return;
  if (ctx->stream) {
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
  }
  if (ctx->side) cudaStreamSynchronize(ctx->side);  // joined into `stream` unless a call failed in between
  grd_ctx_release_extras(ctx);
  grd_graph_release(ctx);
  for (void* p : ctx->allocs) cudaFree(p);
  for (auto& t : ctx->pinned_twin) cudaFreeHost(t.second.p);
  for (cudaEvent_t e : ctx->ev)
    if (e) cudaEventDestroy(e);
  if (ctx->h_counters) cudaFreeHost(ctx->h_counters);
  if (ctx->h_small) cudaFreeHost(ctx->h_small);
  if (ctx->ingest_stage) cudaFreeHost(ctx->ingest_stage);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->side) cudaStreamDestroy(ctx->side);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  (void)cudaGetLastError();
  delete ctx;
}

int grd_upload(grd_ctx* ctx, uint64_t* bytes_copied) {
  if (!ctx) return GRD_E_INVALID;
  if (ctx->device_layout) {
    ctx->err = "a device-built layout keeps no host copy: re-ingest the CSR with grd_ingest";
    return GRD_E_INVALID;
  }
  CK(cudaSetDevice(ctx->device));
  int rc = grd_upload_layout(ctx);
  if (bytes_copied) *bytes_copied = ctx->upload_bytes;
  return rc;
}

int grd_set_algo(grd_ctx* ctx, int algo, const grd_params* params) {
  if (!ctx) return GRD_E_INVALID;
  TRY(grd_wait(ctx, nullptr));  // the loop graph of a queued run must finish before it is replaced
  if (algo < GRD_PR_DELTA || algo > GRD_SSSP_W) {
    ctx->err = "unknown algorithm id";
    return GRD_E_INVALID;
  }
  if (algo == GRD_SSSP_W && !ctx->L.weighted) {
    ctx->err = "GRD_SSSP_W needs edge weights";
    return GRD_E_INVALID;
  }
  grd_params p{};
  p.source = 0;
  p.max_rounds = 1000;
  p.damping = 0.85;
  p.tolerance = (algo == GRD_PR_PULL) ? 1e-7 : 1e-6;
  p.direction = GRD_DIR_AUTO;
  p.frontier_format = GRD_FMT_AUTO;
  if (params) p = *params;
  if (p.dense_div == 0) p.dense_div = 8;
  if (p.policy != GRD_POLICY_FIXED && p.policy != GRD_POLICY_LEARNED) {
    ctx->err = "unknown policy";
    return GRD_E_INVALID;
  }
  if (p.pull_div == 0) p.pull_div = 2;
  if (p.offload != GRD_OFFLOAD_NDP && p.offload != GRD_OFFLOAD_ENGINE && p.offload != GRD_OFFLOAD_NONE) {
    ctx->err = "unknown offload setting";
    return GRD_E_INVALID;
  }
  if (algo == GRD_PR_PULL && p.offload != GRD_OFFLOAD_NDP) {
    ctx->err = "PR_PULL runs every round in the memory partitions (offload must be GRD_OFFLOAD_NDP)";
    return GRD_E_INVALID;
  }
  if (p.push_blocks_per_sm > 32) {
    ctx->err = "push_blocks_per_sm must be <= 32";
    return GRD_E_INVALID;
  }
  if ((algo == GRD_SSSP_HOP || algo == GRD_SSSP_W) && p.source >= ctx->L.V) {
    ctx->err = "SSSP source out of range";
    return GRD_E_INVALID;
  }
  if (p.max_rounds == 0) {
    ctx->err = "max_rounds must be > 0";
    return GRD_E_INVALID;
  }
  if (!(p.damping > 0.0 && p.damping < 1.0)) {
    ctx->err = "damping must be in (0,1)";
    return GRD_E_INVALID;
  }
  CK(cudaSetDevice(ctx->device));
  if (algo != GRD_PR_PULL) TRY(grd_ensure_out_edges(ctx));
  if (algo == GRD_PR_PULL || algo == GRD_PR_DELTA /* fixed-order sums */ || p.direction == GRD_DIR_PULL ||
      (p.policy == GRD_POLICY_LEARNED && p.direction == GRD_DIR_AUTO)) {  // the model may pull
    int rc = grd_ensure_in_edges(ctx);
    if (rc != GRD_OK) return rc;
  }
  grd_graph_release(ctx);  // a new algorithm or parameter set needs a new loop graph
  ctx->graph_failed = false;
  ctx->algo = algo;
  ctx->params = p;
  ctx->inited = false;
  return GRD_OK;
}

int grd_init(grd_ctx* ctx) {
  if (!ctx) return GRD_E_INVALID;
  if (!ctx->layout_valid) {
    ctx->err = "the layout was left incomplete by a failed grd_ingest: ingest a matching graph first";
    return GRD_E_INVALID;
  }
  if (ctx->algo < 0) {
    ctx->err = "no algorithm selected (grd_set_algo)";
    return GRD_E_INVALID;
  }
  CK(cudaSetDevice(ctx->device));
  TRY(grd_wait(ctx, nullptr));
  CK(cudaMemsetAsync(ctx->st.counters, 0, sizeof(unsigned long long) * NUM_COUNTERS, ctx->stream));
  CK(cudaMemsetAsync(ctx->st.lc, 0, sizeof(uint32_t) * NUM_LIST_COUNTERS, ctx->stream));
  const uint64_t n = std::max<uint64_t>(ctx->g.S, ctx->g.V);
  const uint32_t blocks = (uint32_t)std::min<uint64_t>((n + 255) / 256, (uint64_t)grid_for(ctx, 16));
  int rc = grd_enqueue_init(ctx, blocks);
  if (rc != GRD_OK) return rc;
  CK_LAUNCH();
  // The initial frontier shape matters only to host-side decisions (the
  // host-driven loop, the per-stage calls): its copy is queued here and read
  // when one of those needs it, so a device-driven run starts without a host
  // round trip.
  CK(cudaMemcpyAsync(ctx->h_counters, ctx->st.counters, sizeof(unsigned long long) * NUM_COUNTERS,
                     cudaMemcpyDeviceToHost, ctx->stream));
  ctx->counters_stale = true;
  ctx->stats = grd_stats{};
  ctx->stats.kernel_launches = 1;
  ctx->pull.edges = 0;
  ctx->round_log.clear();
  ctx->inited = true;
  return GRD_OK;
}

static __global__ void k_seed_sources(DevGraph g, DevState st, const uint32_t* src, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t s = src[i];
    st.prop[s] = 0;
    st.upd[s] = 0;
    atomicOr(&st.F[s >> 5], 1u << (s & 31));
    list_append(st.FL, st.lc + L_FL, s);  // sources are distinct
    const unsigned long long d = g.outdeg[s];
    atomicAdd(&st.counters[C_FEDGES], d);
    atomicAdd(&st.counters[C_UNVISITED], 0ull - d);
    atomicMax(&st.counters[C_FMAXDEG], d);
  }
}

int grd_init_sources(grd_ctx* ctx, const uint32_t* sources, size_t n) {
  if (!ctx) return GRD_E_INVALID;
  if (ctx->algo != GRD_SSSP_HOP && ctx->algo != GRD_SSSP_W) {
    ctx->err = "grd_init_sources applies to SSSP only";
    return GRD_E_INVALID;
  }
  if (!sources || n == 0 || n > 0xFFFFFFFFull) return GRD_E_INVALID;
  std::vector<uint32_t> src(sources, sources + n);
  std::sort(src.begin(), src.end());
  src.erase(std::unique(src.begin(), src.end()), src.end());
  if (src.back() >= ctx->L.V) {
    ctx->err = "source out of range";
    return GRD_E_INVALID;
  }
  const uint32_t saved = ctx->params.source;
  ctx->params.source = 0xFFFFFFFFu;  // init with no source, then seed them all
  const int rc = grd_init(ctx);
  ctx->params.source = saved;
  TRY(rc);
  const size_t m = src.size();
  if (ctx->agg_cap < m) {
    void* p = nullptr;
    TRY(grd_dev_alloc_bytes(ctx, &p, sizeof(uint32_t) * 2 * m));
    ctx->agg_buf = static_cast<uint32_t*>(p);
    ctx->agg_cap = m;
  }
  CK(cudaMemcpyAsync(ctx->agg_buf, src.data(), sizeof(uint32_t) * m, cudaMemcpyHostToDevice, ctx->stream));
  k_seed_sources<<<(uint32_t)std::min<size_t>((m + 255) / 256, grid_for(ctx, 4)), 256, 0, ctx->stream>>>(
      ctx->g, ctx->st, ctx->agg_buf, (uint32_t)m);
  CK_LAUNCH();
  ctx->h_seed[0] = m;
  CK(cudaMemcpyAsync(ctx->st.counters + C_FRONTIER, ctx->h_seed, sizeof(unsigned long long), cudaMemcpyHostToDevice,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->counters_stale = false;
  ctx->last_frontier = m;
  CK(cudaMemcpyAsync(ctx->h_counters, ctx->st.counters, sizeof(unsigned long long) * NUM_COUNTERS,
                     cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->last_fedges = ctx->h_counters[C_FEDGES];
  ctx->stats.kernel_launches += 1;
  return GRD_OK;
}

int grd_sync_fwd(grd_ctx* ctx) {
  TRY(check_ready(ctx));
  TRY(grd_sync_init_counters(ctx));
  if (ctx->algo == GRD_PR_PULL) return grd_pull_stage(ctx, 0);
  return grd_enqueue_fwd(ctx, false);
}

int grd_edge_map(grd_ctx* ctx) {
  TRY(check_ready(ctx));
  TRY(grd_sync_init_counters(ctx));
  if (ctx->algo == GRD_PR_PULL) return grd_pull_stage(ctx, 1);
  return grd_enqueue_edge_map(ctx);
}

int grd_sync_bwd(grd_ctx* ctx) {
  TRY(check_ready(ctx));
  TRY(grd_sync_init_counters(ctx));
  if (ctx->algo == GRD_PR_PULL) return grd_pull_stage(ctx, 2);
  return grd_enqueue_bwd(ctx, false, true, false);
}

int grd_aggregate(grd_ctx* ctx) {
  TRY(check_ready(ctx));
  TRY(grd_sync_init_counters(ctx));
  if (ctx->algo == GRD_PR_PULL) return grd_pull_stage(ctx, 3);
  return grd_enqueue_bwd(ctx, false, false, true);
}

int grd_update(grd_ctx* ctx, uint64_t* frontier_size) {
  TRY(check_ready(ctx));
  TRY(grd_sync_init_counters(ctx));
  uint64_t f;
  ctx->stats.rounds++;
  if (ctx->algo == GRD_PR_PULL) {
    // Every non-dangling vertex stays active; the run is over when the
    // residual drops below the tolerance, reported as an empty frontier.
    TRY(grd_pull_stage(ctx, 4));
    ctx->stats.converged = ctx->stats.last_residual < ctx->params.tolerance;
    f = ctx->stats.converged ? 0 : ctx->h_counters[C_FRONTIER];
  } else {
    TRY(grd_enqueue_update(ctx));
    TRY(grd_read_counters(ctx));
    f = ctx->h_counters[C_FRONTIER];
    ctx->stats.converged = (f == 0);
  }
  if (frontier_size) *frontier_size = f;
  return GRD_OK;
}

int grd_run(grd_ctx* ctx, uint32_t flags, grd_stats* stats) {
  TRY(check_ready(ctx));
  CK(cudaSetDevice(ctx->device));
  TRY(grd_wait(ctx, nullptr));  // a previous asynchronous run first
  bool device_loop = false;
  const bool async = (flags & GRD_RUN_ASYNC) != 0;
  if (!ctx->profiling && !(flags & GRD_RUN_HOST_LOOP) && ctx->stats.rounds < ctx->params.max_rounds) {
    if (ctx->algo == GRD_PR_PULL)
      TRY(grd_pull_graph_run(ctx, &device_loop, async));
    else
      TRY(grd_graph_run(ctx, &device_loop, async));
  }
  ctx->stats.device_loop = device_loop ? 1 : 0;
  if (!device_loop) TRY(grd_sync_init_counters(ctx));  // host-side decisions need the frontier shape
  if (device_loop) {
    // the whole loop ran (or, async, is queued) as one graph launch
    if (ctx->run_pending) {
      ctx->strict_pending = (flags & GRD_RUN_STRICT) != 0;
      if (stats) *stats = ctx->stats;
      return GRD_OK;  // grd_wait completes the statistics
    }
  } else if (ctx->algo == GRD_PR_PULL) {
    TRY(grd_pull_run(ctx));
  } else {
    uint64_t f = 1;
    while (ctx->stats.rounds < ctx->params.max_rounds) {
      const uint64_t f_in = ctx->last_frontier, e_in = ctx->stats.edges_scanned;
      const uint64_t fe_in = ctx->h_counters[C_FEDGES], fm_in = ctx->h_counters[C_FMAXDEG],
                     un_in = ctx->h_counters[C_UNVISITED];
      int mode;
      TRY(host_loop_mode(ctx, &mode));
      const int branch = rm_branch(mode, ctx->last_frontier, ctx->last_fedges);
      grd_prof_mark(ctx, 0);
      if (ctx->profiling)
        TRY(grd_round_graph_launch(ctx, branch));
      else
        TRY(grd_enqueue_round(ctx, branch));
      grd_prof_mark(ctx, 4);
      ctx->last_mode = mode;
      if (rm_is_pull(mode)) {
        ctx->stats.pull_rounds++;
        ctx->pull.edges += ctx->L.E;
      } else {
        ctx->stats.push_rounds++;
        if (mode == RM_NO_OFFLOAD) ctx->stats.no_offload_rounds++;
      }
      TRY(grd_read_counters(ctx));
      f = ctx->h_counters[C_FRONTIER];
      if (ctx->profiling) {
        grd_round_rec rec{};
        rec.round = ctx->stats.rounds;
        rec.mode = mode;
        rec.frontier_in = f_in;
        rec.actives = ctx->h_counters[C_ACTIVE];
        rec.edges = ctx->stats.edges_scanned - e_in;
        rec.frontier_out = f;
        rec.frontier_edges_in = fe_in;
        rec.max_degree_in = fm_in;
        rec.unvisited_in = un_in;
        grd_prof_collect(ctx, rec.ms);
        ctx->round_log.push_back(rec);
        if (branch == RM_PUSH_BITVEC || branch == RM_PUSH_LIST) {  // the push kernel ran this round
          float ms = 0.0f;
          if (cudaEventElapsedTime(&ms, ctx->ev[5], ctx->ev[6]) == cudaSuccess) {
            ctx->stats.lbs_ms += ms;
            ctx->stats.lbs_edges += ctx->h_counters[C_MEDGES];
            ctx->stats.lbs_actives += ctx->h_counters[C_ACTIVE];
            ctx->stats.lbs_launches += 1;
          }
          (void)cudaGetLastError();
        }
      }
      ctx->stats.rounds++;
      if (f == 0) break;
    }
    ctx->stats.converged = (f == 0);
  }
  if (stats) *stats = ctx->stats;
  if ((flags & GRD_RUN_STRICT) && !ctx->stats.converged) {
    ctx->err = "round cap reached with a non-empty frontier";
    return GRD_E_ROUND_CAP;
  }
  return GRD_OK;
}

int grd_wait(grd_ctx* ctx, grd_stats* stats) {
  if (!ctx) return GRD_E_INVALID;
  if (ctx->run_pending) {
    ctx->run_pending = false;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    TRY(grd_fold_counters(ctx));
    TRY(grd_graph_run_finish(ctx));
    if (ctx->strict_pending && !ctx->stats.converged) {
      ctx->err = "round cap reached with a non-empty frontier";
      if (stats) *stats = ctx->stats;
      return GRD_E_ROUND_CAP;
    }
  }
  if (stats) *stats = ctx->stats;
  return GRD_OK;
}

int grd_set_policy(grd_ctx* ctx, const grd_policy_model* model) {
  if (!ctx) return GRD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  TRY(grd_wait(ctx, nullptr));  // a queued run still uses the loop graph
  grd_graph_release(ctx);       // the loop graph holds the model pointer (or none)
  if (!model) {
    ctx->has_policy = false;
    return GRD_OK;
  }
  if (!ctx->policy_dev) {
    void* p = nullptr;
    TRY(grd_dev_alloc_bytes(ctx, &p, sizeof(grd_policy_model)));
    ctx->policy_dev = static_cast<grd_policy_model*>(p);
  }
  CK(cudaMemcpyAsync(ctx->policy_dev, model, sizeof(grd_policy_model), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->has_policy = true;
  return GRD_OK;
}

int grd_aggregate_values(grd_ctx* ctx, const uint32_t* gids, const uint32_t* values, size_t n) {
  TRY(check_ready(ctx));
  TRY(grd_wait(ctx, nullptr));  // a queued run first: the call changes the ctx
  if (n == 0) return GRD_OK;
  if (!gids || !values) return GRD_E_INVALID;
  if (n > 0xFFFFFFFFull) {
    ctx->err = "too many values in one call";
    return GRD_E_INVALID;
  }
  for (size_t i = 0; i < n; ++i)
    if (gids[i] >= ctx->L.V) {
      ctx->err = "gid " + std::to_string(gids[i]) + " out of range";
      return GRD_E_INVALID;
    }
  CK(cudaSetDevice(ctx->device));
  if (ctx->agg_cap < n) {
    void* p = nullptr;
    TRY(grd_dev_alloc_bytes(ctx, &p, sizeof(uint32_t) * 2 * n));
    ctx->agg_buf = static_cast<uint32_t*>(p);
    ctx->agg_cap = n;
  }
  CK(cudaMemcpyAsync(ctx->agg_buf, gids, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->agg_buf + n, values, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, ctx->stream));
  const uint32_t blocks = (uint32_t)std::min<size_t>((n + 255) / 256, grid_for(ctx, 8));
  const int algo = ctx->algo == GRD_PR_PULL ? GRD_PR_DELTA : ctx->algo;
  TRY(dispatch(algo, [&](auto a) -> int {
    constexpr int A = decltype(a)::value;
    k_aggregate_values<A><<<blocks, 256, 0, ctx->stream>>>(ctx->st, ctx->agg_buf, ctx->agg_buf + n, (uint32_t)n);
    CK_LAUNCH();
    return GRD_OK;
  }));
  ctx->stats.kernel_launches += 1;
  CK(cudaStreamSynchronize(ctx->stream));  // caller's buffers may be reused
  return GRD_OK;
}

int grd_get_stats(const grd_ctx* ctx, grd_stats* stats) {
  if (!ctx || !stats) return GRD_E_INVALID;
  *stats = ctx->stats;
  return GRD_OK;
}

int grd_get_round_log(const grd_ctx* ctx, grd_round_rec* out, size_t cap, size_t* n) {
  if (!ctx) return GRD_E_INVALID;
  if (n) *n = ctx->round_log.size();
  if (out) std::memcpy(out, ctx->round_log.data(), sizeof(grd_round_rec) * std::min(cap, ctx->round_log.size()));
  return GRD_OK;
}

int grd_set_profiling(grd_ctx* ctx, int enable) {
  if (!ctx) return GRD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  if (enable && !ctx->ev[0])
    for (cudaEvent_t& e : ctx->ev) CK(cudaEventCreate(&e));
  ctx->profiling = enable != 0;
  return GRD_OK;
}

static int read_dev(grd_ctx* ctx, void* host, const void* dev, size_t bytes, size_t need) {
  if (!ctx || !host) return GRD_E_INVALID;
  if (bytes < need) {
    ctx->err = "host buffer too small: need " + std::to_string(need) + " bytes";
    return GRD_E_INVALID;
  }
  CK(cudaSetDevice(ctx->device));
  CK(cudaMemcpyAsync(host, dev, need, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return GRD_OK;
}

int grd_read_props(grd_ctx* ctx, void* host, size_t bytes) {
  if (!ctx) return GRD_E_INVALID;
  return read_dev(ctx, host, ctx->st.prop, bytes, sizeof(uint32_t) * ctx->L.V);
}

// A queued copy of a resident vertex array (props or ranks): refused while
// the layout is incomplete (a failed grd_ingest may have left it half
// rewritten).
static int read_dev_async(grd_ctx* ctx, void* host, const void* dev, size_t bytes, size_t need) {
  if (!ctx || !host) return GRD_E_INVALID;
  if (!ctx->layout_valid) {
    ctx->err = "the layout was left incomplete by a failed grd_ingest: ingest a matching graph first";
    return GRD_E_INVALID;
  }
  if (bytes < need) {
    ctx->err = "host buffer too small: need " + std::to_string(need) + " bytes";
    return GRD_E_INVALID;
  }
  CK(cudaSetDevice(ctx->device));
  CK(cudaMemcpyAsync(host, dev, need, cudaMemcpyDeviceToHost, ctx->stream));
  return GRD_OK;
}

int grd_read_props_async(grd_ctx* ctx, void* host, size_t bytes) {
  if (!ctx) return GRD_E_INVALID;
  return read_dev_async(ctx, host, ctx->st.prop, bytes, sizeof(uint32_t) * ctx->L.V);
}

int grd_read_ranks_async(grd_ctx* ctx, float* host, size_t count) {
  if (!ctx) return GRD_E_INVALID;
  return read_dev_async(ctx, host, ctx->st.ranks, count * sizeof(float), sizeof(float) * ctx->L.V);
}

int grd_read_ranks(grd_ctx* ctx, float* host, size_t count) {
  if (!ctx) return GRD_E_INVALID;
  return read_dev(ctx, host, ctx->st.ranks, count * sizeof(float), sizeof(float) * ctx->L.V);
}

int grd_read_updates(grd_ctx* ctx, void* host, size_t bytes) {
  if (!ctx) return GRD_E_INVALID;
  return read_dev(ctx, host, ctx->st.upd, bytes, sizeof(uint32_t) * ctx->L.V);
}

int grd_read_frontier(grd_ctx* ctx, uint32_t* host, size_t words) {
  if (!ctx) return GRD_E_INVALID;
  return read_dev(ctx, host, ctx->st.F, words * 4, sizeof(uint32_t) * ((ctx->L.V + 31) / 32));
}

int grd_layout_info(const grd_ctx* ctx, uint32_t part, uint32_t* n_owned, uint32_t* n_proxy, uint64_t* num_edges) {
  if (!ctx || part >= ctx->L.M) return GRD_E_INVALID;
  if (n_owned) *n_owned = ctx->L.n_owned[part];
  if (n_proxy) *n_proxy = ctx->L.n_proxy[part];
  if (num_edges) *num_edges = ctx->L.part_edges[part];
  return GRD_OK;
}

int grd_layout_slots(const grd_ctx* ctx, uint32_t part, uint32_t* host, size_t count) {
  if (!ctx || part >= ctx->L.M || !host) return GRD_E_INVALID;
  const uint32_t T = ctx->L.T(part);
  if (count < T) return GRD_E_INVALID;
  if (ctx->device_layout) {  // resident copy only
    if (cudaSetDevice(ctx->device) != cudaSuccess ||
        cudaMemcpy(host, ctx->g.slot_gid + ctx->L.slot_base[part], sizeof(uint32_t) * T, cudaMemcpyDeviceToHost) !=
            cudaSuccess) {
      (void)cudaGetLastError();
      return GRD_E_CUDA;
    }
    return GRD_OK;
  }
  std::memcpy(host, ctx->L.slot_gid.data() + ctx->L.slot_base[part], sizeof(uint32_t) * T);
  return GRD_OK;
}

int grd_read_layout(grd_ctx* ctx, int which, void* host, size_t cap_bytes, size_t* bytes) {
  if (!ctx || !bytes) return GRD_E_INVALID;
  const Layout& L = ctx->L;
  const void* src = nullptr;
  size_t n = 0;
  const size_t u = sizeof(uint32_t);
  switch (which) {
    case GRD_LAYOUT_SLOT_GID: src = ctx->g.slot_gid, n = u * L.S; break;
    case GRD_LAYOUT_ROW_OFF: src = ctx->g.row_off, n = u * (L.S + 1); break;
    case GRD_LAYOUT_COL: src = ctx->g.col, n = u * L.E; break;
    case GRD_LAYOUT_WGT: src = ctx->g.wgt, n = L.weighted ? u * L.E : 0; break;
    case GRD_LAYOUT_OUTDEG: src = ctx->g.outdeg, n = u * L.V; break;
    case GRD_LAYOUT_OWN_SLOT: src = ctx->st.own_slot, n = u * L.V; break;
    case GRD_LAYOUT_HUBS: src = ctx->g.hubs, n = sizeof(HubChunkD) * ctx->g.num_hubs; break;
    case GRD_LAYOUT_IN_OFF: src = ctx->g.in_off, n = ctx->in_edges_alloc ? u * (L.S + 1) : 0; break;
    case GRD_LAYOUT_IN_SRC: src = ctx->g.in_src, n = ctx->in_edges_alloc ? u * L.E : 0; break;
    case GRD_LAYOUT_IN_WGT: src = ctx->g.in_wgt, n = ctx->in_edges_alloc && L.weighted ? u * L.E : 0; break;
    case GRD_LAYOUT_IN_HUBS: src = ctx->pull.in_hubs, n = sizeof(HubChunkD) * ctx->pull.num_in_hubs; break;
    case GRD_LAYOUT_IN_MEDS: src = ctx->pull.in_meds, n = sizeof(HubChunkD) * ctx->pull.num_in_meds; break;
    default: ctx->err = "unknown layout array"; return GRD_E_INVALID;
  }
  *bytes = n;
  if (!host || n == 0) return GRD_OK;
  if (cap_bytes < n) {
    ctx->err = "buffer too small for the layout array";
    return GRD_E_INVALID;
  }
  CK(cudaSetDevice(ctx->device));
  if (which == GRD_LAYOUT_COL || which == GRD_LAYOUT_WGT || which == GRD_LAYOUT_IN_WGT) TRY(grd_ensure_out_edges(ctx));
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(host, src, n, cudaMemcpyDeviceToHost));
  return GRD_OK;
}

int grd_layout_preview(const grd_csr* graph, const uint32_t* mirror_part, uint32_t num_memory, uint32_t part,
                       uint32_t* slots, size_t cap, uint32_t* n_owned, uint32_t* n_proxy) {
  g_create_error.clear();
  if (!graph || part >= num_memory) return GRD_E_INVALID;
  Layout L;
  std::string why = build_layout(graph->num_vertices, graph->num_edges, graph->row_offsets, graph->col_indices,
                                 graph->weights, mirror_part, num_memory, L);
  if (!why.empty()) {
    g_create_error = why;
    return GRD_E_INVALID;
  }
  if (n_owned) *n_owned = L.n_owned[part];
  if (n_proxy) *n_proxy = L.n_proxy[part];
  if (slots) std::memcpy(slots, L.slot_gid.data() + L.slot_base[part], sizeof(uint32_t) * std::min<size_t>(cap, L.T(part)));
  return GRD_OK;
}

int grd_device_props(grd_ctx* ctx, void** dptr) {
  if (!ctx || !dptr) return GRD_E_INVALID;
  *dptr = ctx->st.prop;
  return GRD_OK;
}

int grd_device_ranks(grd_ctx* ctx, float** dptr) {
  if (!ctx || !dptr) return GRD_E_INVALID;
  *dptr = ctx->st.ranks;
  return GRD_OK;
}

void* grd_stream(grd_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int grd_synchronize(grd_ctx* ctx) {
  if (!ctx) return GRD_E_INVALID;
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  return GRD_OK;
}

}  // extern "C"

// ------------------------------------------------------------ device setup --
int grd_ctx_init_stream(grd_ctx* ctx) {
  CK(cudaSetDevice(ctx->device));
  CK(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device));
  CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
  CK(cudaMallocHost((void**)&ctx->h_counters, sizeof(unsigned long long) * (NUM_COUNTERS + 16)));
  std::memset(ctx->h_counters, 0, sizeof(unsigned long long) * (NUM_COUNTERS + 16));
  ctx->h_seed = ctx->h_counters + NUM_COUNTERS;
  return GRD_OK;
}

int grd_ctx_init_device(grd_ctx* ctx) {
  TRY(grd_ctx_init_stream(ctx));
  TRY(grd_alloc_resident(ctx));
  // Weights that all fit a byte travel as bytes (a quarter of the copy).
  const Layout& L = ctx->L;
  if (L.weighted && L.E > 0 &&
      std::all_of(L.wgt.begin(), L.wgt.begin() + (ptrdiff_t)L.E, [](uint32_t w) { return w < 256u; })) {
    ctx->wgt8_host.assign(L.wgt.begin(), L.wgt.begin() + (ptrdiff_t)L.E);
    void* p = nullptr;
    TRY(grd_dev_alloc_bytes(ctx, &p, L.E));
    ctx->wgt8_dev = static_cast<uint8_t*>(p);
  }
  for (const auto* v : {&ctx->L.col, &ctx->L.row_off, &ctx->L.slot_gid})
    grd_pin_twin(ctx, v->data(), v->size() * sizeof(uint32_t));
  if (ctx->wgt8_host.empty())
    grd_pin_twin(ctx, ctx->L.wgt.data(), ctx->L.wgt.size() * sizeof(uint32_t));
  else
    grd_pin_twin(ctx, ctx->wgt8_host.data(), ctx->wgt8_host.size());
  {  // pinned copy of the small tables: hubs, tile partitions, partition bases, sizes, owned counts
    const size_t nh = sizeof(HubChunk) * L.hubs.size(), nt = sizeof(uint32_t) * L.tile_part.size(),
                 nm = sizeof(uint32_t) * L.M;
    CK(cudaMallocHost((void**)&ctx->h_small, nh + nt + 3 * nm));
    unsigned char* sm = ctx->h_small;
    if (nh) std::memcpy(sm, L.hubs.data(), nh);
    std::memcpy(sm + nh, L.tile_part.data(), nt);
    std::memcpy(sm + nh + nt, L.slot_base.data(), nm);
    uint32_t* T = reinterpret_cast<uint32_t*>(sm + nh + nt + nm);
    for (uint32_t p = 0; p < L.M; ++p) T[p] = L.T(p);
    std::memcpy(sm + nh + nt + 2 * nm, L.n_owned.data(), nm);
  }
  return grd_upload_layout(ctx);
}

// A pinned twin of a large host layout array: one copy into memory the driver
// allocated pinned (cudaHostAlloc), made once, from which every grd_upload
// reads.  Such memory keeps its full host->device rate even when the copy
// comes after the buffer sat idle, where memory pinned in place
// (cudaHostRegister) ran a cold copy at a fraction of it.  The layout arrays
// never change after creation, so the twin stays equal to them; an upload
// still uses a twin only when its size matches the array's.  Without a twin
// (a small array, or pinned memory refused) uploads read the pageable array.
void grd_pin_twin(grd_ctx* ctx, const void* data, size_t bytes) {
  if (bytes < (1u << 20) || ctx->pinned_twin.count(data)) return;
  void* p = nullptr;
  if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
    (void)cudaGetLastError();
    std::fprintf(stderr, "grudon: no pinned twin for %zu B of host layout; uploads read pageable memory\n", bytes);
    return;
  }
  std::memcpy(p, data, bytes);
  ctx->pinned_twin.emplace(data, grd_ctx::PinnedTwin{p, bytes});
}

int grd_enqueue_init(grd_ctx* ctx, uint32_t blocks) {
  const double d = ctx->params.damping;
  const uint32_t src = ctx->params.source;
  switch (ctx->algo) {
    case GRD_PR_DELTA: k_init<A_PR_DELTA><<<blocks, 256, 0, ctx->stream>>>(ctx->g, ctx->st, src, d); break;
    case GRD_PR_PULL: k_init<A_PR_PULL><<<blocks, 256, 0, ctx->stream>>>(ctx->g, ctx->st, src, d); break;
    case GRD_CC: k_init<A_CC><<<blocks, 256, 0, ctx->stream>>>(ctx->g, ctx->st, src, d); break;
    case GRD_SSSP_HOP: k_init<A_SSSP_HOP><<<blocks, 256, 0, ctx->stream>>>(ctx->g, ctx->st, src, d); break;
    case GRD_SSSP_W: k_init<A_SSSP_W><<<blocks, 256, 0, ctx->stream>>>(ctx->g, ctx->st, src, d); break;
    default: return GRD_E_INVALID;
  }
  CK_LAUNCH();
  if (ctx->algo == GRD_PR_PULL) return grd_pull_stage(ctx, -1);  // pull-specific init
  if (ctx->algo == GRD_PR_DELTA) return grd_pr_delta_hubs(ctx);
  return GRD_OK;
}
