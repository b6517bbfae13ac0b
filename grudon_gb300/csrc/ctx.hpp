// grd_ctx: everything one partitioned graph owns on the host and device.
#pragma once
#include <cuda_runtime.h>

#include <initializer_list>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/grudon_gpu.h"
#include "kernels.cuh"
#include "layout.hpp"
#include "policy.cuh"

// PageRank Jacobi (GRD_PR_PULL) arrays derived from the resident layout
// (pr_pull.cu): rebuilt whenever the layout changes.
struct PrPullState {
  uint64_t layout_gen = ~0ull;  // layout generation the arrays below describe
  uint64_t E = 0, S_nz = 0, T = 0;  // in-edges, non-empty in-lists, 512-edge tiles
  uint32_t H = 0;                // hot sources (staged in shared memory by the pull)
  uint32_t hot_deg = 0;          // out-degree threshold of the hot set
  uint64_t nondangling = 0;      // vertices with out-edges
  uint64_t cap_E = 0, cap_S = 0, cap_V = 0, cap_T = 0;  // allocated sizes
  uint32_t* src = nullptr;       // [E] in-edges, lists vertex-major: hot rank | 0x80000000, or the source slot
  uint32_t* start_bits = nullptr;  // [E/32 + 2] bit e: edge e opens a non-empty in-list
  uint32_t* tile_nz = nullptr;   // [T + 1] non-empty in-lists opened before tile t
  uint4* piece = nullptr;        // [T] (head, tail sum, tail compensation, tail list)
  uint32_t* piece_flags = nullptr;  // [T]
  float* part = nullptr;         // [S_nz] partial sum of each non-empty in-list, vertex-major
  uint32_t* vmap_off = nullptr;  // [V + 1] per vertex: its in-lists' range in part
  uint32_t* hot_base = nullptr;  // [V/32 + 1] hot rank of each 32-vertex word's first hot vertex
  float* hot_val = nullptr;      // [H] contributions of the hot sources
  double* resid_part = nullptr;  // [update blocks] residual partial sums
  uint32_t update_blocks = 0;
  char* scratch = nullptr;       // set-up scratch, kept between set-ups
  size_t scratch_cap = 0;
};

struct PullState {
  grd::HubChunkD* in_hubs = nullptr;  // destination slots with long in-lists
  uint32_t num_in_hubs = 0;
  grd::HubChunkD* in_meds = nullptr;  // destination slots with medium in-lists
  uint32_t num_in_meds = 0;
  uint64_t edges = 0;                 // in-edges read since init
  // Delta PageRank's sums of lists of more than 32 in-edges (32-edge chunks
  // summed grid-wide): the lists (slot, first edge, end), the first chunk of
  // each, the list of each chunk, the chunk sums.
  grd::HubChunkD* prd_lists = nullptr;
  uint32_t num_prd_lists = 0, prd_list_cap = 0;
  uint32_t* hub_coff = nullptr;
  uint32_t* chunk_hub = nullptr;
  float* chunk_sum = nullptr;
  uint32_t num_hub_chunks = 0, hub_chunk_cap = 0;
  uint64_t hub_gen = ~0ull;  // layout generation the tables describe
};

struct grd_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  // The push edge-map runs the hub rows (k_hub_push) on `side`, beside the
  // load-balanced push: fork and join are events on the two streams, also
  // inside a graph capture (two parallel kernel nodes).
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int num_sms = 0;
  grd::Layout L;
  grd::DevGraph g{};
  grd::DevState st{};
  std::vector<void*> allocs;
  int algo = -1;
  grd_params params{};
  bool inited = false;
  grd_stats stats{};
  std::string err;
  unsigned long long* h_counters = nullptr;  // pinned, NUM_COUNTERS + 16 entries
  unsigned long long* h_seed = nullptr;      // = h_counters + NUM_COUNTERS
  uint64_t upload_bytes = 0;
  bool in_edges_alloc = false;
  // Host layout: the out-edge columns and the weights of both views were left
  // out of the last upload (a PR_PULL ctx reads neither); uploaded again
  // before anything reads them.
  bool out_edges_stale = false;
  uint64_t layout_gen = 0;     // bumped whenever a layout array is rewritten
  PullState pull;
  PrPullState pr;
  uint64_t last_frontier = 0;  // |frontier| entering the next round
  uint64_t last_fedges = 0;    // its out-edges
  std::vector<grd_round_rec> round_log;  // profiled host-loop rounds
  int last_mode = -1;          // edge-map mode of the round in flight (host loop)
  cudaGraph_t run_graph = nullptr;     // device-driven round loop (graph_run.cu)
  cudaGraphExec_t run_exec = nullptr;
  cudaGraphExec_t round_exec[7] = {};  // one round per branch (profiled host loop)
  cudaGraph_t pr_graph = nullptr;      // PR_PULL device-driven loop (pr_pull.cu)
  cudaGraphExec_t pr_exec = nullptr;
  bool graph_failed = false;           // building it failed here: host loop
  std::string graph_error;
  uint32_t* agg_buf = nullptr; // staging of grd_aggregate_values (gids, values)
  size_t agg_cap = 0;
  bool profiling = false;
  // profiling events: [0..4] bracket the stages of a round, [5..6] the
  // load-balanced push kernel
  cudaEvent_t ev[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  // Pinned twins of the large host layout arrays (cudaHostAlloc, filled once
  // at creation), keyed by the array's data pointer: uploads read the twin.
  struct PinnedTwin {
    void* p;
    size_t bytes;
  };
  std::unordered_map<const void*, PinnedTwin> pinned_twin;
  std::vector<uint8_t> wgt8_host;  // weights as bytes when all are < 256 (uploaded instead of L.wgt)
  uint8_t* wgt8_dev = nullptr;     // their device staging copy
  unsigned char* h_small = nullptr;  // pinned small tables of the upload (hubs, tiles, partitions)
  // Pinned staging copy of a caller's CSR for grd_ingest (grown on demand):
  // host threads copy the caller's arrays in, the copy engine reads them out.
  unsigned char* ingest_stage = nullptr;
  size_t ingest_stage_bytes = 0;
  grd_policy_model* policy_dev = nullptr;  // learned round policy (device copy)
  // grd_sssp_multi (msssp.cu): 64 distance lanes per vertex, the lane masks,
  // the active list with its degree prefix, the source-major output copy
  uint32_t* ms_dist = nullptr;
  unsigned long long* ms_mask = nullptr;
  uint32_t* ms_list = nullptr;
  uint32_t* ms_out = nullptr;
  size_t ms_out_cap = 0;
  unsigned long long* verify_buf = nullptr;  // grd_verify per-block top ranks
  size_t verify_cap = 0;
  bool has_policy = false;
  bool device_layout = false;  // layout built on the device (no host copy of its arrays)
  bool tile_counts_ready = false;  // the last edge-map wrote the backward tile counts
  bool capturing_loop = false;     // the device-driven loop graph's branches are being captured
  bool counters_stale = false;     // h_counters holds grd_init's queued copy, not yet read
  bool layout_valid = true;    // false while (or after a failed) grd_ingest rewrites the layout
  bool run_pending = false;    // a GRD_RUN_ASYNC loop launch not yet waited for
  bool strict_pending = false; // ... run with GRD_RUN_STRICT
};

// Error plumbing shared by the host translation units (expects a `ctx`).
#define CK(call)                                                                       \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                   \
      return GRD_E_CUDA;                                                               \
    }                                                                                  \
  } while (0)

#define CK_LAUNCH()                                                                    \
  do {                                                                                 \
    cudaError_t e_ = cudaGetLastError();                                               \
    if (e_ != cudaSuccess) {                                                           \
      ctx->err = std::string("kernel launch: ") + cudaGetErrorString(e_);              \
      return GRD_E_CUDA;                                                               \
    }                                                                                  \
  } while (0)

#define TRY(x)                   \
  do {                           \
    int r_ = (x);                \
    if (r_ != GRD_OK) return r_; \
  } while (0)

int grd_ctx_init_stream(grd_ctx* ctx);
// GRD_OK when the ctx can run stages: a complete layout, an algorithm, init done.
int grd_check_ready(grd_ctx* ctx);
int grd_ctx_init_device(grd_ctx* ctx);
int grd_alloc_resident(grd_ctx* ctx);
// On-device layout build (layout_dev.cu).
int grd_device_layout_check(const grd_csr* graph, uint32_t M, std::string* why);
int grd_device_layout_build(grd_ctx* ctx, const grd_csr* graph, const uint32_t* mirror_part, bool first);
int grd_device_in_edges(grd_ctx* ctx);
void grd_pin_twin(grd_ctx* ctx, const void* data, size_t bytes);
int grd_dev_alloc_bytes(grd_ctx* ctx, void** p, size_t bytes);
void grd_prof_mark(grd_ctx* ctx, int i);
void grd_prof_collect(grd_ctx* ctx);
void grd_ctx_release_extras(grd_ctx* ctx);
int grd_enqueue_init(grd_ctx* ctx, uint32_t blocks);
// Delta PageRank's chunked long-list tables for the resident layout (abi.cu).
int grd_pr_delta_hubs(grd_ctx* ctx);
int grd_upload_layout(grd_ctx* ctx);
int grd_ensure_in_edges(grd_ctx* ctx);
int grd_ensure_out_edges(grd_ctx* ctx);
int grd_read_counters(grd_ctx* ctx);
int grd_fold_counters(grd_ctx* ctx);
int grd_sync_init_counters(grd_ctx* ctx);
int grd_enqueue_fwd(grd_ctx* ctx, bool fused);
int grd_enqueue_edge_map(grd_ctx* ctx);
// Round modes: direction x sync format.  Values are the SWITCH branch indices
// of the loop graph and the `mode` field of grd_round_rec.
enum RoundMode {
  RM_PUSH_BITVEC = GRD_ROUND_PUSH_BITVEC,
  RM_PUSH_LIST = GRD_ROUND_PUSH_LIST,
  RM_PULL_BITVEC = GRD_ROUND_PULL_BITVEC,
  RM_PULL_LIST = GRD_ROUND_PULL_LIST,
  NUM_ROUND_MODES = 4,
  // push + list for a frontier small enough for one CTA (k_round_tiny); an
  // implementation of RM_PUSH_LIST, chosen by size, not by the policy
  RM_PUSH_TINY = grd::P_BRANCH_TINY,
  // NO_OFFLOAD round (compute-side push over the shipped adjacency), and its
  // one-CTA form for the same small frontiers
  RM_NO_OFFLOAD = GRD_ROUND_NO_OFFLOAD,
  RM_NOOFF_TINY = grd::P_BRANCH_NOOFF_TINY,
  NUM_BRANCHES = 7
};
static_assert(RM_NO_OFFLOAD == 5, "branch index of the NO_OFFLOAD round");
static_assert(sizeof(grd_ctx::round_exec) / sizeof(cudaGraphExec_t) == NUM_BRANCHES, "one graph per branch");
// The branch that runs a round the policy gave `mode`.
__host__ __device__ inline int rm_branch(int mode, unsigned long long frontier, unsigned long long fedges) {
  return grd::policy_branch(mode, frontier, fedges);
}
__host__ __device__ inline bool rm_is_pull(int m) { return m == RM_PULL_BITVEC || m == RM_PULL_LIST; }
int grd_choose_round_mode(const grd_ctx* ctx);
// degree_passes_done: 1 = the first degree pass already ran (k_fwd_list_deg),
// 2 = both (k_fwd_xfer_deg).  aggregate (push + bitvector, min algorithms):
// the dirty diff also runs the backward transfer and the aggregate.
int grd_enqueue_edge_map_mode(grd_ctx* ctx, int mode, int degree_passes_done = 0, bool aggregate = false);
uint32_t grd_edge_map_launches(const grd_ctx* ctx, int mode);
uint32_t grd_round_launches(const grd_ctx* ctx, int mode);
int grd_enqueue_fwd_list(grd_ctx* ctx);
int grd_enqueue_bwd_update_list(grd_ctx* ctx);
int grd_enqueue_round(grd_ctx* ctx, int mode);
// Policy inputs of this ctx, and the model the device loop uses (nullptr:
// the fixed rule).
grd::PolicyArgs grd_policy_args(const grd_ctx* ctx);
const grd_policy_model* grd_policy_model_dev(const grd_ctx* ctx);
// Device-driven loop (graph_run.cu).  async: queue the launch and the
// counter read-back only (ctx->run_pending); grd_graph_run_finish folds them
// once the stream has drained.
int grd_graph_run(grd_ctx* ctx, bool* used, bool async = false);
int grd_graph_run_finish(grd_ctx* ctx);
// One round in `mode` as one graph launch (built on first use).
int grd_round_graph_launch(grd_ctx* ctx, int mode);
void grd_graph_release(grd_ctx* ctx);
int grd_enqueue_bwd(grd_ctx* ctx, bool fused, bool do_pack, bool do_aggregate);
int grd_enqueue_update(grd_ctx* ctx);
// PR_PULL (pr_pull.cu): stage -1 init, 0 fwd, 1 pull edge-map, 2 bwd, 3
// aggregate, 4 update; the host-driven loop; the device-driven loop (one
// graph launch, *used = false when it cannot be built here).
int grd_pull_stage(grd_ctx* ctx, int stage);
int grd_pull_run(grd_ctx* ctx);
int grd_pull_graph_run(grd_ctx* ctx, bool* used, bool async);
void grd_pull_graph_release(grd_ctx* ctx);
int grd_pull_run_finish(grd_ctx* ctx);
// Exclusive add-scan of n u32 (out may alias in); with total_at_n, out[n]
// also receives the total (layout_dev.cu).
int grd_scan_add_u32(grd_ctx* ctx, const uint32_t* in, uint32_t* out, uint64_t n, bool total_at_n);
int grd_scan_u32(grd_ctx* ctx, const uint32_t* in, uint32_t* out, uint64_t n, bool inclusive, bool total_at_n);
