// GRD_PR_PULL: Jacobi PageRank through the partitioned round structure.
//
// Fixed point (the one the reference's delta-push PageRank converges to,
// src/graph_algorithms/pr.cpp:20-88):
//   pr[v] = (1-d)*[outdeg(v) > 0] + sum_{u->v} d * pr[u] / outdeg(u)
// Each iteration is one round: the compute partition sends the contribution
// c[u] = d*pr[u]/outdeg(u) of every non-dangling vertex to its mirror
// partition (bitvector + packed values), every memory partition pulls, for
// each destination slot, the Kahan-compensated FP32 sum of its in-edges'
// contributions in ascending source-slot order, sends the partial sums back,
// and the compute side merges the partials (Kahan, partition order), forms the
// new ranks in FP32 and reduces the L1 residual in FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "ctx.hpp"
#include "kernels.cuh"

using namespace grd;

namespace {

// Kahan merge of one partition's partial sum into the compute-side
// accumulator (upd = running sum, comp = compensation).
struct OpPullXfer {
  uint32_t* comp;
  bool pack, merge;
  __device__ __forceinline__ Payload gather(const DevGraph& g, const DevState& st, uint32_t p, uint32_t slot,
                                            uint32_t j) const {
    const uint32_t gid = __ldg(&g.slot_gid[slot]);
    const uint32_t v = pack ? st.mupd[slot] : st.BV[g.part_base[p] + j];
    return Payload{v, gid, merge ? st.upd[gid] : 0u, merge ? comp[gid] : 0u};
  }
  __device__ __forceinline__ void scatter(const DevGraph& g, const DevState& st, uint32_t p, uint32_t, uint32_t j,
                                          uint32_t, const Payload& v) const {
    if (pack && !merge) st.BV[g.part_base[p] + j] = v.v;  // the wire buffer feeds a separate merge only
    if (merge) {
      float s = __uint_as_float(v.cur), c = __uint_as_float(v.cmp);
      kahan_add(s, c, __uint_as_float(v.v));
      st.upd[v.gid] = __float_as_uint(s);
      comp[v.gid] = __float_as_uint(c);
    }
  }
};

// New ranks, contributions and the FP64 L1 residual; resets the accumulators.
__global__ void __launch_bounds__(256) k_update_pull(DevGraph g, DevState st, uint32_t* comp, double* residual,
                                                     float damping_f, float base_f) {
  __shared__ double s_red[8];
  double r = 0.0;
  uint32_t cnt = 0;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += gridDim.x * blockDim.x) {
    const uint32_t deg = g.outdeg[v];
    const float total = __fsub_rn(__uint_as_float(st.upd[v]), __uint_as_float(comp[v]));
    const float nv = __fadd_rn(deg ? base_f : 0.0f, total);
    const float ov = st.ranks[v];
    r += fabs((double)nv - (double)ov);
    st.ranks[v] = nv;
    st.prop[v] = __float_as_uint(deg ? __fdiv_rn(__fmul_rn(damping_f, nv), (float)deg) : 0.0f);
    st.upd[v] = 0;
    comp[v] = 0;
    cnt += deg ? 1u : 0u;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) r += __shfl_xor_sync(FULL, r, o);
  if (lane_id() == 0) s_red[threadIdx.x >> 5] = r;
  cnt = block_sum(cnt);
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < 8; ++i) t += s_red[i];
    atomicAdd(residual, t);
    if (cnt) atomicAdd(&st.counters[C_FRONTIER], (unsigned long long)cnt);
  }
}

__global__ void k_zero_u32(uint32_t* p, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    p[i] = 0;
}

int ensure_pull_state(grd_ctx* ctx) {
  PullState& ps = ctx->pull;
  if (ps.comp) return GRD_OK;
  TRY(grd_dev_alloc_bytes(ctx, (void**)&ps.comp, sizeof(uint32_t) * ctx->L.V));
  TRY(grd_dev_alloc_bytes(ctx, (void**)&ps.residual, sizeof(double)));
  CK(cudaMallocHost((void**)&ps.h_residual, sizeof(double)));
  return GRD_OK;
}

uint32_t sms(const grd_ctx* ctx, uint32_t per_sm) { return (uint32_t)ctx->num_sms * per_sm; }

int enqueue_pull_edge_map(grd_ctx* ctx) {
  k_pull<A_PR_PULL><<<sms(ctx, 8), 256, 0, ctx->stream>>>(ctx->g, ctx->st);
  if (ctx->pull.num_in_meds)
    k_pull_med<A_PR_PULL><<<std::min<uint32_t>((ctx->pull.num_in_meds + 7) / 8, sms(ctx, 8)), 256, 0,
                            ctx->stream>>>(ctx->g, ctx->st, ctx->pull.in_meds, ctx->pull.num_in_meds);
  if (ctx->pull.num_in_hubs)
    k_pull_hub<A_PR_PULL><<<std::min<uint32_t>(ctx->pull.num_in_hubs, sms(ctx, 8)), 256, 0, ctx->stream>>>(
        ctx->g, ctx->st, ctx->pull.in_hubs, ctx->pull.num_in_hubs);
  CK_LAUNCH();
  ctx->stats.kernel_launches += 1 + (ctx->pull.num_in_meds ? 1 : 0) + (ctx->pull.num_in_hubs ? 1 : 0);
  ctx->stats.pull_rounds++;
  ctx->pull.edges += ctx->L.E;  // every in-edge is read once per iteration
  return GRD_OK;
}

// Backward sync of the partial sums: per-tile counts, scan, then one ordered
// launch per partition so the compute-side merge order is 0, 1, ..., M-1.
int enqueue_pull_bwd(grd_ctx* ctx, bool pack, bool merge) {
  const uint32_t T = ctx->g.num_tiles;
  const Layout& L = ctx->L;
  if (pack) {
    k_tile_count<<<T, 256, 0, ctx->stream>>>(ctx->st.MD, ctx->st.tile_cnt);
    ctx->stats.kernel_launches += 1;
  }
  for (uint32_t p = 0; p < L.M; ++p) {
    const uint32_t t0 = L.slot_base[p] / TILE_SLOTS;
    const uint32_t t1 = (p + 1 < L.M) ? L.slot_base[p + 1] / TILE_SLOTS : T;
    OpPullXfer op{ctx->pull.comp, pack, merge};
    k_compact<<<t1 - t0, 256, 0, ctx->stream>>>(ctx->st.MD, merge ? ctx->st.MD : nullptr, t0, ctx->g, ctx->st, op,
                                                pack ? 1 : 0);
    ctx->stats.kernel_launches += 1;
  }
  CK_LAUNCH();
  return GRD_OK;
}

int enqueue_pull_update(grd_ctx* ctx) {
  CK(cudaMemsetAsync(ctx->st.counters + C_FRONTIER, 0, sizeof(unsigned long long), ctx->stream));
  CK(cudaMemsetAsync(ctx->pull.residual, 0, sizeof(double), ctx->stream));
  const uint32_t blocks = std::max<uint32_t>(1, std::min<uint32_t>((ctx->g.V + 255) / 256, sms(ctx, 8)));
  const double d = ctx->params.damping;
  k_update_pull<<<blocks, 256, 0, ctx->stream>>>(ctx->g, ctx->st, ctx->pull.comp, ctx->pull.residual, (float)d,
                                                 (float)(1.0 - d));
  CK_LAUNCH();
  ctx->stats.kernel_launches += 1;
  return GRD_OK;
}

int read_residual(grd_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->pull.h_residual, ctx->pull.residual, sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream));
  TRY(grd_read_counters(ctx));  // synchronises the stream
  ctx->stats.last_residual = *ctx->pull.h_residual / (double)ctx->L.V;
  return GRD_OK;
}

}  // namespace

void grd_ctx_release_extras(grd_ctx* ctx) {
  if (ctx->pull.h_residual) cudaFreeHost(ctx->pull.h_residual);
  ctx->pull.h_residual = nullptr;
}

int grd_pull_stage(grd_ctx* ctx, int stage) {
  switch (stage) {
    case -1: {  // init: accumulators and compensation start at zero
      TRY(ensure_pull_state(ctx));
      k_zero_u32<<<sms(ctx, 4), 256, 0, ctx->stream>>>(ctx->pull.comp, ctx->L.V);
      CK_LAUNCH();
      return GRD_OK;
    }
    case 0: return grd_enqueue_fwd(ctx, false);
    case 1: return enqueue_pull_edge_map(ctx);
    case 2: return enqueue_pull_bwd(ctx, true, false);
    case 3: return enqueue_pull_bwd(ctx, false, true);
    case 4: {
      TRY(enqueue_pull_update(ctx));
      return read_residual(ctx);
    }
    default: return GRD_E_INVALID;
  }
}

int grd_pull_run(grd_ctx* ctx) {
  const double tol = ctx->params.tolerance;
  ctx->stats.converged = 0;
  while (ctx->stats.rounds < ctx->params.max_rounds) {
    grd_prof_mark(ctx, 0);
    TRY(grd_enqueue_fwd(ctx, true));
    grd_prof_mark(ctx, 1);
    TRY(enqueue_pull_edge_map(ctx));
    grd_prof_mark(ctx, 2);
    TRY(enqueue_pull_bwd(ctx, true, true));
    grd_prof_mark(ctx, 3);
    TRY(enqueue_pull_update(ctx));
    grd_prof_mark(ctx, 4);
    TRY(read_residual(ctx));
    grd_prof_collect(ctx);
    ctx->stats.rounds++;
    if (ctx->stats.last_residual < tol) {
      ctx->stats.converged = 1;
      break;
    }
  }
  return GRD_OK;
}
