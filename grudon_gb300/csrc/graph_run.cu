// Device-driven round loop: one CUDA graph per (ctx, algorithm, parameters).
//
// Top level: a conditional WHILE node whose body is one round of
// GraphAlgorithm::run (src/GraphAlgorithm.cpp:177-690):
//   k_policy -> SWITCH {push+bitvector, push+list, pull+bitvector, pull+list,
//                       push+list in one CTA, NO_OFFLOAD, NO_OFFLOAD in one
//                       CTA} -> k_round_end
// where every branch is a whole round (forward sync, edge-map, backward sync
// + aggregate, update) in that mode.  k_policy applies the offload decision
// and the direction / frontier-format rule on the device (the frontier size
// of the previous update is already there) and selects the branch;
// k_round_end counts the round and keeps the loop going while the frontier
// is non-empty and the round cap is not reached, so the loop is always
// bounded.  One graph launch
// runs the whole algorithm with no host round trip; the host reads the
// counters once at the end.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "ctx.hpp"
#include "kernels.cuh"
#include "policy.cuh"

using namespace grd;

namespace {

// Carries the host-side round statistics into the device counters.  A
// kernel, not a copy: a host-to-device copy would queue behind any large
// upload another stream has on the copy engine.
struct LoopSeed {
  unsigned long long rounds, push_rounds, pull_rounds, actives_total, push_actives, no_offload_rounds;
};

__global__ void k_seed_loop(DevState st, LoopSeed s) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  st.counters[C_ROUNDS] = s.rounds;
  st.counters[C_PUSH_ROUNDS] = s.push_rounds;
  st.counters[C_PULL_ROUNDS] = s.pull_rounds;
  st.counters[C_ACTIVE_TOTAL] = s.actives_total;
  st.counters[C_MODE] = 0;
  st.counters[C_LAUNCHES] = 0;
  st.counters[C_PUSH_ACTIVES] = s.push_actives;
  st.counters[C_NOOFF_ROUNDS] = s.no_offload_rounds;
}

__global__ void k_round_end(DevState st, cudaGraphConditionalHandle wh, uint32_t max_rounds) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const unsigned long long r = st.counters[C_ROUNDS] + 1;
  st.counters[C_ROUNDS] = r;
  st.counters[C_ACTIVE_TOTAL] += st.counters[C_ACTIVE];
  if (!rm_is_pull((int)st.counters[C_MODE])) st.counters[C_PUSH_ACTIVES] += st.counters[C_ACTIVE];
  cudaGraphSetConditional(wh, (st.counters[C_FRONTIER] > 0 && r < max_rounds) ? 1u : 0u);
}

// Appends a conditional node to the graph being captured on `s` and returns
// its body graphs; the capture continues after the node.
int add_conditional(grd_ctx* ctx, cudaStream_t s, cudaGraphConditionalHandle h, cudaGraphConditionalNodeType type,
                    unsigned size, cudaGraph_t* bodies) {
  cudaStreamCaptureStatus status;
  cudaGraph_t graph;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  CK(cudaStreamGetCaptureInfo(s, &status, nullptr, &graph, &deps, nullptr, &ndeps));
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = type;
  p.conditional.size = size;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &p));
  for (unsigned i = 0; i < size; ++i) bodies[i] = p.conditional.phGraph_out[i];
  CK(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return GRD_OK;
}

int capture_into(grd_ctx* ctx, cudaGraph_t body) {
  CK(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  return GRD_OK;
}

int end_capture(grd_ctx* ctx, cudaGraph_t body) {
  cudaGraph_t out = nullptr;
  CK(cudaStreamEndCapture(ctx->stream, &out));
  if (out != body) {
    ctx->err = "capture returned an unexpected graph";
    return GRD_E_CUDA;
  }
  return GRD_OK;
}

// Builds the graph; on any error the capture is ended and the error kept.
int build(grd_ctx* ctx) {
  const grd_stats saved = ctx->stats;  // enqueue helpers count host-side launches
  cudaGraph_t top = nullptr;
  CK(cudaGraphCreate(&top, 0));
  ctx->run_graph = top;
  cudaGraphConditionalHandle wh, sw;
  CK(cudaGraphConditionalHandleCreate(&wh, top, 1, cudaGraphCondAssignDefault));
  cudaGraph_t loop_body;
  {
    // The while node is the only node of the top-level graph.
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = wh;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, top, nullptr, nullptr, 0, &p));
    loop_body = p.conditional.phGraph_out[0];
  }
  CK(cudaGraphConditionalHandleCreate(&sw, loop_body, 0, 0));
  PolicyArgs pa = grd_policy_args(ctx);
  for (int m = 0; m < NUM_BRANCHES; ++m) pa.launches[m] = 2 /*policy, round end*/ + grd_round_launches(ctx, m);

  int rc = capture_into(ctx, loop_body);
  if (rc != GRD_OK) return rc;
  cudaGraph_t branches[NUM_BRANCHES] = {};
  k_policy<true><<<1, P_HID, 0, ctx->stream>>>(ctx->g, ctx->st, sw, pa, grd_policy_model_dev(ctx));
  rc = add_conditional(ctx, ctx->stream, sw, cudaGraphCondTypeSwitch, NUM_BRANCHES, branches);
  if (rc == GRD_OK) k_round_end<<<1, 32, 0, ctx->stream>>>(ctx->st, wh, ctx->params.max_rounds);
  const int rc_end = end_capture(ctx, loop_body);
  if (rc != GRD_OK) return rc;
  if (rc_end != GRD_OK) return rc_end;
  const int offload = ctx->params.offload;
  for (int m = 0; m < NUM_BRANCHES; ++m) {
    // never selected: empty branch
    if (rm_is_pull(m) && !ctx->in_edges_alloc) continue;
    const bool nooff = m == RM_NO_OFFLOAD || m == RM_NOOFF_TINY;
    if (nooff ? offload == GRD_OFFLOAD_NDP : offload == GRD_OFFLOAD_NONE) continue;
    TRY(capture_into(ctx, branches[m]));
    ctx->capturing_loop = true;
    rc = grd_enqueue_round(ctx, m);
    ctx->capturing_loop = false;
    const int e = end_capture(ctx, branches[m]);
    if (rc != GRD_OK) return rc;
    if (e != GRD_OK) return e;
  }
  CK(cudaGraphInstantiate(&ctx->run_exec, top, 0));
  ctx->stats = saved;
  return GRD_OK;
}

}  // namespace

void grd_graph_release(grd_ctx* ctx) {
  grd_pull_graph_release(ctx);
  if (ctx->run_exec) cudaGraphExecDestroy(ctx->run_exec);
  if (ctx->run_graph) cudaGraphDestroy(ctx->run_graph);
  ctx->run_exec = nullptr;
  ctx->run_graph = nullptr;
  for (auto& e : ctx->round_exec) {
    if (e) cudaGraphExecDestroy(e);
    e = nullptr;
  }
}

// Profiled host-loop rounds run as one graph launch each, so their timings
// carry the device loop's launch costs (the learned policy trains on them).
int grd_round_graph_launch(grd_ctx* ctx, int mode) {
  if (!ctx->round_exec[mode]) {
    const grd_stats saved = ctx->stats;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = grd_enqueue_round(ctx, mode);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    ctx->stats = saved;
    if (rc != GRD_OK || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      (void)cudaGetLastError();
      if (rc != GRD_OK) return rc;
      CK(e);
    }
    const cudaError_t ie = cudaGraphInstantiate(&ctx->round_exec[mode], g, 0);
    cudaGraphDestroy(g);
    CK(ie);
  }
  CK(cudaGraphLaunch(ctx->round_exec[mode], ctx->stream));
  ctx->stats.kernel_launches += grd_round_launches(ctx, mode);
  return GRD_OK;
}

// Runs the rest of the algorithm as one graph launch.  Returns GRD_OK with
// *used = false when the graph cannot be built here (the caller then runs the
// host-driven loop); the reason is kept in ctx->graph_error.
int grd_graph_run(grd_ctx* ctx, bool* used, bool async) {
  *used = false;
  if (ctx->graph_failed) return GRD_OK;
  if (!ctx->run_exec) {
    CK(cudaStreamSynchronize(ctx->stream));  // capture starts on an idle stream
    const int rc = build(ctx);
    if (rc != GRD_OK) {
      ctx->graph_failed = true;
      ctx->graph_error = ctx->err;
      ctx->err.clear();
      grd_graph_release(ctx);
      cudaStreamCaptureStatus st;
      if (cudaStreamIsCapturing(ctx->stream, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(ctx->stream, &g);
        if (g) cudaGraphDestroy(g);
      }
      (void)cudaGetLastError();
      return GRD_OK;
    }
  }
  const LoopSeed seed{ctx->stats.rounds,        ctx->stats.push_rounds,  ctx->stats.pull_rounds,
                      ctx->stats.actives_total, ctx->stats.push_actives, ctx->stats.no_offload_rounds};
  k_seed_loop<<<1, 32, 0, ctx->stream>>>(ctx->st, seed);
  CK_LAUNCH();
  CK(cudaGraphLaunch(ctx->run_exec, ctx->stream));
  *used = true;
  if (async) {
    CK(cudaMemcpyAsync(ctx->h_counters, ctx->st.counters, sizeof(unsigned long long) * NUM_COUNTERS,
                       cudaMemcpyDeviceToHost, ctx->stream));
    ctx->run_pending = true;
    return GRD_OK;
  }
  TRY(grd_read_counters(ctx));
  return grd_graph_run_finish(ctx);
}

// Statistics of a finished loop launch (its counters already on the host).
int grd_graph_run_finish(grd_ctx* ctx) {
  if (ctx->algo == GRD_PR_PULL) return grd_pull_run_finish(ctx);
  if (!ctx->run_exec) return GRD_OK;
  const unsigned long long* c = ctx->h_counters;
  ctx->stats.rounds = (uint32_t)c[C_ROUNDS];
  ctx->stats.push_rounds = (uint32_t)c[C_PUSH_ROUNDS];
  ctx->stats.pull_rounds = (uint32_t)c[C_PULL_ROUNDS];
  ctx->stats.actives_total = c[C_ACTIVE_TOTAL];
  ctx->stats.push_actives = c[C_PUSH_ACTIVES];
  ctx->stats.no_offload_rounds = (uint32_t)c[C_NOOFF_ROUNDS];
  ctx->stats.kernel_launches += c[C_LAUNCHES];
  ctx->stats.converged = c[C_FRONTIER] == 0;
  return GRD_OK;
}
