/*
 * grudon_gpu.h — C ABI of the GB300 (sm_103a) per-round graph operator.
 *
 * One opaque grd_ctx owns every device buffer of one partitioned graph: the
 * compute partition (master copies, gid-indexed) and the M memory partitions
 * (out-edge CSR over owned vertices plus proxy slots), all resident in one
 * GPU's HBM.  Every call is stream-ordered on the ctx's own CUDA stream; a ctx
 * is single-threaded, distinct ctxs may be used concurrently.
 *
 * Reference interfaces replaced (paths relative to the Grudon project):
 *   grd_ctx_create      DistributedGraph ctor, src/DistributedGraph.cpp:13-785
 *                       (layout, proxies, translation tables, bitCommVector)
 *   grd_set_algo        choice of plugin class, src/main.cpp:133-134
 *   grd_init            GraphAlgorithm::init overrides: pr.cpp:20-61,
 *                       cc.cpp:18-40, sssp.cpp:18-47
 *   grd_sync_fwd        compute->memory frontier pack + unpack,
 *                       src/GraphAlgorithm.cpp:199-343
 *   grd_edge_map        TraverseWorker::traverse -> gen_updates,
 *                       src/Workers.cpp:109-113, pr.cpp:91-121, cc.cpp:54-84,
 *                       sssp.cpp:61-90
 *   grd_sync_bwd        memory->compute dirty pack, src/GraphAlgorithm.cpp:356-424
 *   grd_aggregate       compute-side aggregate, src/GraphAlgorithm.cpp:478-581
 *                       + pr.cpp:149-153, cc.cpp:109-113, sssp.cpp:115-119
 *   grd_update          UpdateWorker::update (update_frontier + apply_updates)
 *                       + termination_check, src/GraphAlgorithm.cpp:643-662
 *   grd_run             GraphAlgorithm::run, src/GraphAlgorithm.cpp:145-701
 *                       (offload choice per round: NDPEngine,
 *                       include/offload_engine/NDPEngine.hpp:10-51; NO_OFFLOAD
 *                       rounds: src/GraphAlgorithm.cpp:426-474, 582-637)
 *   grd_read_*          PageRank/CC/SSSP::printState output, pr.cpp:162-176
 *
 * Status convention: every int-returning call returns GRD_OK (0) or a negative
 * GRD_E_* code; grd_last_error(ctx) gives a one-line reason.
 */
#ifndef GRUDON_GPU_H
#define GRUDON_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GRD_OK            0
#define GRD_E_INVALID   (-1) /* bad argument, size or state                   */
#define GRD_E_OOM       (-2) /* device or host allocation failed              */
#define GRD_E_CUDA      (-3) /* CUDA runtime error (incl. no device)          */
#define GRD_E_TIMEOUT   (-4) /* a bounded device wait gave up                 */
#define GRD_E_ROUND_CAP (-5) /* grd_run hit max_rounds with a live frontier
                                and GRD_RUN_STRICT was requested              */
#define GRD_E_IO        (-6) /* file could not be read/written or is corrupt  */

/* ---- algorithms (GraphAlgorithm plugins) -------------------------------- */
#define GRD_PR_DELTA  0 /* reference delta-push PageRank, float, TOL 1e-6    */
#define GRD_PR_PULL   1 /* Jacobi PageRank, FP32 Kahan sums, FP64 residual   */
#define GRD_CC        2 /* min-label propagation along out-edges, uint32     */
#define GRD_SSSP_HOP  3 /* reference unit-weight SSSP (hop count), uint32    */
#define GRD_SSSP_W    4 /* weighted SSSP: prop[u] + w(u,v), uint32 weights   */

/* ---- traversal direction / frontier format (per-round policy) ----------- */
#define GRD_DIR_AUTO  0
#define GRD_DIR_PUSH  1
#define GRD_DIR_PULL  2
#define GRD_FMT_AUTO    0
#define GRD_FMT_BITVEC  1
#define GRD_FMT_LIST    2

/* ---- offload decision per round (grd_params.offload) -------------------- */
/* NDP_OFFLOAD rounds run the edge-map in the memory partitions and sync the
 * dirty updates back (the reference's only live path: run() hard-codes
 * NDP_OFFLOAD, src/GraphAlgorithm.cpp:189).  NO_OFFLOAD rounds ship the
 * frontier's adjacency to the compute partition, which applies the
 * algorithm's own update to its vertex_updates directly: no memory-side
 * dirty tracking, backward sync or aggregate (src/GraphAlgorithm.cpp:426-474,
 * 582-637).  Results are identical either way (PageRank: up to float
 * summation order). */
#define GRD_OFFLOAD_NDP     0 /* every round NDP_OFFLOAD (the reference)     */
#define GRD_OFFLOAD_ENGINE  1 /* NDPEngine rule per round: NO_OFFLOAD when
                                 0 < |frontier| <= V/20 and the coverage and
                                 imbalance tests pass (NDPEngine.hpp:17-50)  */
#define GRD_OFFLOAD_NONE    2 /* every round NO_OFFLOAD                      */
/* grd_run applies the setting; the per-stage calls (grd_sync_fwd ...
 * grd_update) always run an NDP_OFFLOAD round. */

#define GRD_RUN_STRICT  1u /* flag: return GRD_E_ROUND_CAP at the round cap */
#define GRD_RUN_HOST_LOOP 2u /* flag: drive rounds from the host (one
                                synchronisation per round) instead of the
                                device-driven CUDA-graph loop */
#define GRD_RUN_ASYNC 4u     /* flag: queue the device-driven loop and return
                                at once; grd_wait completes the run and its
                                statistics (runs that cannot use the device
                                loop still return finished) */

/* Host CSR as handed to the library: row_offsets has num_vertices+1 entries
 * (u64, like the reference's LC_CSR_Graph row ends), col_indices num_edges
 * u32 global ids, weights num_edges u32 or NULL. */
typedef struct grd_csr {
  uint32_t num_vertices;
  uint64_t num_edges;
  const uint64_t* row_offsets;
  const uint32_t* col_indices;
  const uint32_t* weights;
} grd_csr;

typedef struct grd_params {
  uint32_t source;      /* SSSP source gid (reference: gid 0)                */
  uint32_t max_rounds;  /* round cap (reference MAX_ITERATIONS = 1000)       */
  double damping;       /* PageRank damping (reference 0.85)                 */
  double tolerance;     /* PR_DELTA: activation threshold (reference 1e-6);
                           PR_PULL: stop when L1 residual / V < tolerance    */
  int direction;        /* GRD_DIR_*                                          */
  int frontier_format;  /* GRD_FMT_*                                          */
  /* Schedule knobs (0 = built-in default); results never depend on them.   */
  uint32_t dense_div;   /* bitvector round when |F| >= S/dense_div or its
                           out-edges >= E/dense_div (default 8)           */
  uint32_t pull_div;    /* AUTO pulls when |F| >= V / pull_div (2); needs the
                           in-edge view                                       */
  uint32_t push_blocks_per_sm; /* push grid; 0 = occupancy limit            */
  int policy;           /* GRD_POLICY_FIXED (threshold rule above) or
                           GRD_POLICY_LEARNED (model set by grd_set_policy;
                           the fixed rule when none is set)               */
  int offload;          /* GRD_OFFLOAD_* (default NDP).  The direction,
                           format and policy settings apply to NDP_OFFLOAD
                           rounds; NO_OFFLOAD rounds push from the compute
                           partition with list syncs.  Not for PR_PULL.   */
} grd_params;

#define GRD_POLICY_FIXED   0
#define GRD_POLICY_LEARNED 1

typedef struct grd_stats {
  uint32_t rounds;            /* reference "Iterations" statistic          */
  uint32_t converged;         /* 1 if the frontier emptied before the cap  */
  uint64_t edges_scanned;     /* out-edges (push) / in-edges (pull) read   */
  uint64_t bytes_synced;      /* bitvector words + packed values, both
                                 directions, all partitions (true size);
                                 NO_OFFLOAD rounds: forward sync plus the
                                 shipped adjacency, 4 B per frontier vertex
                                 and per edge (x2 with weights)            */
  uint64_t reference_bytes_moved; /* the reference's TotalBytesMoved
                                 formula (bitvector count inflated x8,
                                 src/GraphAlgorithm.cpp:251-265; MPI send
                                 and recv of the shipped adjacency both
                                 counted, include/MPI.hpp:40-54)           */
  double last_residual;       /* PR_PULL: last L1 residual / V (FP64)      */
  uint32_t push_rounds;       /* rounds that ran the push edge-map         */
  uint32_t pull_rounds;       /* rounds that ran the pull edge-map         */
  uint64_t actives_total;     /* sum over rounds of unpacked active slots  */
  uint64_t kernel_launches;   /* kernels this ctx launched since grd_init  */
  /* With grd_set_profiling(ctx,1): CUDA-event milliseconds per stage, summed
   * over rounds: [0] forward sync, [1] edge-map, [2] backward sync +
   * aggregate, [3] update, [4] whole rounds. */
  double stage_ms[5];
  uint32_t device_loop;       /* 1 if the last grd_run ran as one graph
                                 launch (device-driven loop), 0 if the host
                                 drove the rounds                          */
  uint64_t push_actives;      /* actives_total restricted to push rounds   */
  /* With profiling, host-driven rounds: the load-balanced push kernel alone
   * (CUDA events around each launch), the edges of non-hub rows it ran and
   * the actives of its rounds. */
  double lbs_ms;
  uint64_t lbs_edges, lbs_actives, lbs_launches;
  uint32_t no_offload_rounds; /* rounds run NO_OFFLOAD (counted in
                                 push_rounds too)                          */
  /* With profiling, host-driven PR_PULL iterations: the edge-balanced pull
   * kernel alone (CUDA events around each launch) and its launches. */
  double pull_ms;
  uint64_t pull_launches;
} grd_stats;

typedef struct grd_ctx grd_ctx;

/* Library / device info ----------------------------------------------------*/
const char* grd_version(void);
/* Returns number of CUDA devices visible (0 when none); never faults. */
int grd_device_count(void);

/* Context lifetime ---------------------------------------------------------*/
/* Builds the 1-compute + num_memory-partition layout from a host CSR and a
 * mirror (memory) partition id per vertex (NULL => gid % num_memory, the
 * reference's NaivePartitioner), and uploads it to device `device`.
 * num_compute must be 1 (every configuration of this operator uses one). */
int grd_ctx_create(const grd_csr* graph, const uint32_t* mirror_part,
                   uint32_t num_compute, uint32_t num_memory, int device,
                   grd_ctx** out);
void grd_ctx_destroy(grd_ctx* ctx);

/* grd_ctx_create with flags.  GRD_CREATE_DEVICE_LAYOUT uploads the CSR (and
 * mirror_part) as given and builds the partition layout on the device —
 * proxy discovery, translation slots, relabelled out-edges, hub work items
 * and, when pull needs it, the in-edge view — instead of on the host
 * (the DistributedGraph ctor, src/DistributedGraph.cpp:285-785).  Every
 * resident array equals the host build's, so runs give identical results.
 * Takes 1..64 memory partitions.  The ctx keeps no host copy of the layout:
 * grd_upload is refused and grd_ingest re-uploads a CSR instead.  flags = 0
 * is grd_ctx_create. */
#define GRD_CREATE_DEVICE_LAYOUT 1u
int grd_ctx_create_ex(const grd_csr* graph, const uint32_t* mirror_part,
                      uint32_t num_compute, uint32_t num_memory, int device,
                      uint32_t flags, grd_ctx** out);
/* Re-uploads a CSR of the same shape (V, E, weights, and the same partition,
 * proxy and hub counts) into a GRD_CREATE_DEVICE_LAYOUT ctx and rebuilds
 * its layout on the device; *bytes_copied = host->device bytes.  Blocks
 * until the layout is built. */
int grd_ingest(grd_ctx* ctx, const grd_csr* graph, const uint32_t* mirror_part,
               uint64_t* bytes_copied);
const char* grd_last_error(const grd_ctx* ctx);
/* Error text of the most recent failed grd_ctx_create on this thread. */
const char* grd_create_error(void);

/* Re-uploads the layout arrays from the host copy kept at create time
 * (timed host->device traffic for end-to-end runs). Returns bytes copied.
 * The copies are queued on the ctx stream from pinned copies of the layout
 * made at create time, and the call returns at once; every later call on the
 * ctx sees the new data.  A ctx whose algorithm is GRD_PR_PULL copies what
 * that algorithm reads (slot map, row offsets, the in-edge view's offsets
 * and sources); the out-edge columns and the weights follow before another
 * algorithm or grd_read_layout needs them. */
int grd_upload(grd_ctx* ctx, uint64_t* bytes_copied);

/* Algorithm selection and per-stage round API -----------------------------*/
int grd_set_algo(grd_ctx* ctx, int algo, const grd_params* params);
int grd_init(grd_ctx* ctx);
/* SSSP init with several sources at distance 0 (e.g. one per copy of a
 * disjoint-union batch); other algorithms: GRD_E_INVALID. */
int grd_init_sources(grd_ctx* ctx, const uint32_t* sources, size_t n);
int grd_sync_fwd(grd_ctx* ctx);
int grd_edge_map(grd_ctx* ctx);
int grd_sync_bwd(grd_ctx* ctx);
int grd_aggregate(grd_ctx* ctx);
/* Applies update_frontier + apply_updates; *frontier_size = |frontier|. */
int grd_update(grd_ctx* ctx, uint64_t* frontier_size);
/* Aggregates n caller-supplied (gid, value) pairs into the compute-side
 * vertex_updates with the algorithm's aggregate operator (PR add, CC/SSSP
 * min), marking them dirty for the next grd_update — the batch form of the
 * plugin's aggregate(lid, value) (pr.cpp:149-153, cc.cpp:109-113,
 * sssp.cpp:115-119).  Values are 32-bit (float bits for PageRank). */
int grd_aggregate_values(grd_ctx* ctx, const uint32_t* gids,
                         const uint32_t* values, size_t n);

/* grd_aggregate_values for callers that cannot allocate device memory — a
 * serving process whose memory is already reserved for its own pool, or a
 * latency-bound caller that must not take the allocator's device
 * synchronisation.  No counterpart in the reference.  Same arguments and result as
 * grd_aggregate_values, but the pairs are staged in a fixed device array
 * inside the library (2 MiB, held by every GPU that loads the library until
 * exit) instead of an allocated buffer, so at most GRD_NOALLOC_MAX_VALUES
 * pairs per call (larger n returns GRD_E_INVALID).  The first call on a
 * device looks the array's address up for that device: make it before any
 * stream capture.  All calls share the one array: calls whose work overlaps on
 * the GPU (several ctxs on different streams) race; each call waits for its
 * own work before returning. */
#define GRD_NOALLOC_MAX_VALUES (1u << 18)
int grd_aggregate_values_noalloc(grd_ctx* ctx, const uint32_t* gids,
                                 const uint32_t* values, size_t n);

/* SSSP from up to GRD_MS_MAX_SOURCES sources at once over the ctx's resident
 * graph (the batched-sources workload): 64 distance lanes per vertex, and each
 * round relaxes every edge once for all of its source's changed lanes, so
 * the CSR is held and read once however many sources run.  Per lane this is
 * the reference's SSSP (src/graph_algorithms/sssp.cpp:61-113, seeded at
 * :40-46 with one source; here n) and the distances equal n single-source
 * runs.  The ctx's algorithm (grd_set_algo) must be GRD_SSSP_HOP or
 * GRD_SSSP_W, and grd_init must have run; sources may repeat.  dist_out
 * receives n * V uint32 distances, source-major (UINT32_MAX: unreachable).
 * Runs to convergence or params.max_rounds rounds; stats (may be null) gets
 * rounds, converged and edges scanned.  Allocates its device arrays on the
 * first call (about 280 B per vertex). */
#define GRD_MS_MAX_SOURCES 64
int grd_sssp_multi(grd_ctx* ctx, const uint32_t* sources, uint32_t n,
                   uint32_t* dist_out, grd_stats* stats);

/* Full run: init() already called; loops rounds until the frontier is empty
 * or params.max_rounds.  flags: GRD_RUN_STRICT. */
int grd_run(grd_ctx* ctx, uint32_t flags, grd_stats* stats);
/* Completes a GRD_RUN_ASYNC run (no-op otherwise) and copies the stats.
 * Every call that changes the ctx's algorithm, init state or layout waits
 * first; the result reads are stream-ordered behind the run. */
int grd_wait(grd_ctx* ctx, grd_stats* stats);
int grd_get_stats(const grd_ctx* ctx, grd_stats* stats);
/* Per-stage CUDA-event timing inside grd_run (off by default).  While it is
 * on, grd_run drives the rounds from the host and records one grd_round_rec
 * per round (cleared by grd_init). */
int grd_set_profiling(grd_ctx* ctx, int enable);

/* Round modes: direction x sync format.  Bitvector rounds sync through one
 * bitvector per memory partition and track dirty slots densely; list rounds
 * sync through (slot, value) lists of the frontier and of the dirty slots. */
#define GRD_ROUND_PUSH_BITVEC 0
#define GRD_ROUND_PUSH_LIST   1
#define GRD_ROUND_PULL_BITVEC 2
#define GRD_ROUND_PULL_LIST   3
/* NO_OFFLOAD round: frontier values forward (list form, as the reference
 * still sends them), adjacency to the compute partition, compute-side push
 * into vertex_updates, update.  Never predicted by the learned model. */
#define GRD_ROUND_NO_OFFLOAD  5

typedef struct grd_round_rec {
  uint32_t round;         /* 0-based round index                          */
  int32_t mode;           /* GRD_ROUND_* (direction x sync format, or
                             GRD_ROUND_NO_OFFLOAD)                        */
  uint64_t frontier_in;   /* |frontier| entering the round                */
  uint64_t actives;       /* actives unpacked by the forward sync         */
  uint64_t edges;         /* edges the edge-map read this round           */
  uint64_t frontier_out;  /* |frontier| after the update                  */
  double ms[5];           /* fwd, edge-map, bwd+aggregate, update, round  */
  uint64_t frontier_edges_in; /* out-edges of the entering frontier       */
  uint64_t max_degree_in;     /* largest out-degree in it                 */
  uint64_t unvisited_in;      /* SSSP: out-edges of unreached vertices    */
} grd_round_rec;
/* Copies up to cap records; *n = number recorded. */
int grd_get_round_log(const grd_ctx* ctx, grd_round_rec* out, size_t cap,
                      size_t* n);

/* Results (blocking device->host copies) -----------------------------------*/
/* Compute-side vertex_properties, gid order (uint32 for CC/SSSP, float for PR
 * contributions). */
int grd_read_props(grd_ctx* ctx, void* host, size_t bytes);
/* The same copy queued on the ctx stream after the work queued so far, without
 * waiting: `host` holds the values once grd_synchronize returns, or grd_wait
 * for an asynchronous run queued before the copy (pinned memory; a pageable
 * buffer makes the copy synchronous).  Lets a
 * caller chain upload, run and read of several contexts with no host round
 * trip in between.  No counterpart in the reference, whose results stay in
 * host memory. */
int grd_read_props_async(grd_ctx* ctx, void* host, size_t bytes);
/* PageRank values (pr_vals for PR_DELTA, ranks for PR_PULL), float[V]. */
int grd_read_ranks(grd_ctx* ctx, float* host, size_t count);
/* The ranks copy queued like grd_read_props_async (same rules). */
int grd_read_ranks_async(grd_ctx* ctx, float* host, size_t count);
/* Compute-side vertex_updates, gid order. */
int grd_read_updates(grd_ctx* ctx, void* host, size_t bytes);
/* Current compute frontier bitmap, ceil(V/32) uint32 words. */
int grd_read_frontier(grd_ctx* ctx, uint32_t* host, size_t words);

/* Layout introspection (translation-slot index space, reference
 * src/DistributedGraph.cpp:630-775) ---------------------------------------*/
int grd_layout_info(const grd_ctx* ctx, uint32_t part, uint32_t* n_owned,
                    uint32_t* n_proxy, uint64_t* num_edges);
/* slot -> gid of memory partition `part` (owned slots, then proxy slots). */
int grd_layout_slots(const grd_ctx* ctx, uint32_t part, uint32_t* host,
                     size_t count);

/* Copies one resident layout array to the host (either build).  *bytes gets
 * its size; host == NULL only queries it.  The in-edge arrays exist once
 * pull has been set up (GRD_PR_PULL, GRD_DIR_PULL or the learned policy).
 * Hub entries are (slot, e0, e1) u32 triples. */
#define GRD_LAYOUT_SLOT_GID 0 /* [S] gid of each slot, 0xFFFFFFFF padding  */
#define GRD_LAYOUT_ROW_OFF  1 /* [S+1] out-edge offsets                    */
#define GRD_LAYOUT_COL      2 /* [E] destination slot of each out-edge     */
#define GRD_LAYOUT_WGT      3 /* [E] its weight (weighted graphs)          */
#define GRD_LAYOUT_OUTDEG   4 /* [V] out-degree of each gid                */
#define GRD_LAYOUT_OWN_SLOT 5 /* [V] owned slot of each gid                */
#define GRD_LAYOUT_HUBS     6 /* hub work items of the push map            */
#define GRD_LAYOUT_IN_OFF   7 /* [S+1] in-edge offsets                     */
#define GRD_LAYOUT_IN_SRC   8 /* [E] source slot of each in-edge           */
#define GRD_LAYOUT_IN_WGT   9 /* [E] its weight                            */
#define GRD_LAYOUT_IN_HUBS 10 /* destinations pulled per block             */
#define GRD_LAYOUT_IN_MEDS 11 /* destinations pulled per warp              */
int grd_read_layout(grd_ctx* ctx, int which, void* host, size_t cap_bytes,
                    size_t* bytes);

/* Host-only preview of the same slot space without a device: writes the
 * slot -> gid order of partition `part` (up to cap entries) and its sizes. */
int grd_layout_preview(const grd_csr* graph, const uint32_t* mirror_part,
                       uint32_t num_memory, uint32_t part, uint32_t* slots,
                       size_t cap, uint32_t* n_owned, uint32_t* n_proxy);

/* Device pointers of the compute-side arrays (for zero-copy callers). */
int grd_device_props(grd_ctx* ctx, void** dptr);
int grd_device_ranks(grd_ctx* ctx, float** dptr);
/* CUDA stream the ctx launches on (cudaStream_t as void*). */
void* grd_stream(grd_ctx* ctx);
/* Blocks until all work on the ctx stream is done. */
int grd_synchronize(grd_ctx* ctx);

/* ---- host graph tools (seeded generators, formats, partition files) ----- */
typedef struct grd_host_graph {
  uint32_t num_vertices;
  uint64_t num_edges;
  uint64_t* row_offsets; /* V+1 */
  uint32_t* col_indices; /* E, ascending within each row, no dups/loops */
  uint32_t* weights;     /* E or NULL */
  uint64_t seed;
} grd_host_graph;

/* RMAT: 2^scale vertices, edge_factor*2^scale draws, quadrant probabilities
 * a,b,c (d = 1-a-b-c); self-loops and duplicates removed; no relabelling.
 * symmetrize: add reverse edges before dedupe.  weighted: u32 weights in
 * [1,255] keyed by the final sorted edge index.  threads<=0: all cores. */
int grd_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b,
                 double c, uint64_t seed, int symmetrize, int weighted,
                 int threads, grd_host_graph** out);
/* Erdos-Renyi G(n, m = edge_factor*n) uniform pairs, deduped. */
int grd_gen_er(uint32_t num_vertices, uint32_t edge_factor, uint64_t seed,
               int symmetrize, int weighted, int threads,
               grd_host_graph** out);
/* k x k 4-neighbour grid, both directions, weights in [1,255]. */
int grd_gen_grid(uint32_t k, uint64_t seed, int weighted, int threads,
                 grd_host_graph** out);
/* Host graph from caller arrays (copied). */
int grd_graph_from_csr(const grd_csr* csr, grd_host_graph** out);
void grd_graph_free(grd_host_graph* g);
/* Default seed of the RMAT workloads: 0x6772756E ^ (scale<<8) ^ ef. */
uint64_t grd_rmat_seed(uint32_t scale, uint32_t edge_factor);

/* Galois binary .gr (version 1) and MatrixMarket .mtx I/O. */
int grd_write_gr(const grd_host_graph* g, const char* path);
int grd_read_gr(const char* path, grd_host_graph** out);
int grd_write_mtx(const grd_host_graph* g, const char* path);
int grd_read_mtx(const char* path, grd_host_graph** out);

/* Edge-balanced contiguous mirror partitioning (one id per vertex). */
int grd_partition_edge_balanced(const grd_host_graph* g, uint32_t num_memory,
                                uint32_t* mirror_part);
/* Partition file: one integer per line (include/partitioning_engine/
 * Partitioner.hpp:98-102 format). */
int grd_write_partition_file(const uint32_t* part, uint32_t n, const char* path);
int grd_read_partition_file(const char* path, uint32_t n, uint32_t num_memory,
                            uint32_t* part);

/* Validators ----------------------------------------------------------------
 * The reference's verify() checks (cc.cpp:139-177, sssp.cpp:145-189,
 * pr.cpp:179-205) as device kernels over the resident graph, for the
 * algorithm last run on the ctx:
 *   CC    errors = edges whose endpoints hold different labels;
 *         count = components (vertices that are their own label);
 *   SSSP  errors = edges (u,v) with u reached and dist[v] > dist[u] + w
 *         (w = 1 for the hop count); count = reached vertices ("Total
 *         Visited Dist"); max_value = largest distance ("Max Dist");
 *   PR    the GRD_VERIFY_TOPK largest pr_vals, descending (ties: lower gid
 *         first). */
#define GRD_VERIFY_TOPK 20
typedef struct grd_verify_result {
  uint64_t errors;
  uint64_t edges_checked;
  uint64_t count;
  uint64_t max_value;
  uint32_t num_top;
  uint32_t top_ids[GRD_VERIFY_TOPK];
  float top_values[GRD_VERIFY_TOPK];
} grd_verify_result;
int grd_verify(grd_ctx* ctx, grd_verify_result* out);

/* Learned round policy ----------------------------------------------------
 * No reference counterpart: the reference's only per-round decision engine
 * is the disabled NDP/INC offload rule (include/offload_engine/
 * NDPEngine.hpp:17-50).  An MLP 8 -> 64 -> 64 -> 4 (ReLU) predicts the
 * log2 round time of each round mode (GRD_ROUND_*), relative to their mean,
 * from the shape of the frontier entering the round; the round runs in the
 * allowed mode with the smallest prediction when it beats the plain
 * method's choice (the fixed rule, push only) by more than 0.1 in log2
 * units, else the plain choice (a frontier of at most 2048 vertices and
 * 16384 edges always runs push + list in one CTA, without inference).
 * Weights are IEEE fp16 (bit patterns), biases and accumulation fp32.
 * Inputs, each then mapped x = (clamp(f, lo, hi) - mean) * scale:
 *   f0 log2(1+|F|) - log2 V            f1 log2(1+out-edges of F) - log2(1+E)
 *   f2 log2(1+unvisited out-edges) - log2(1+E)   (SSSP; 0 edges otherwise)
 *   f3 log2(1+mean degree in F)        f4 log2(1+max degree in F) - log2 V
 *   f5 log2(1+round index)             f6 log2 V     f7 log2(1+E/V)
 * The choice never changes CC/SSSP results (min fixed points; every mode
 * computes the same values, dirty sets and round counts). */
#define GRD_POLICY_IN  8
#define GRD_POLICY_HID 64
#define GRD_POLICY_OUT 4
#define GRD_POLICY_NPARAM (GRD_POLICY_HID * GRD_POLICY_IN + GRD_POLICY_HID + \
                           GRD_POLICY_HID * GRD_POLICY_HID + GRD_POLICY_HID + \
                           GRD_POLICY_OUT * GRD_POLICY_HID + GRD_POLICY_OUT)

typedef struct grd_policy_model {
  float mean[GRD_POLICY_IN], scale[GRD_POLICY_IN];
  uint16_t w1[GRD_POLICY_HID * GRD_POLICY_IN];   /* [out][in], fp16 */
  float b1[GRD_POLICY_HID];
  uint16_t w2[GRD_POLICY_HID * GRD_POLICY_HID];  /* [out][in], fp16 */
  float b2[GRD_POLICY_HID];
  uint16_t w3[GRD_POLICY_OUT * GRD_POLICY_HID];  /* [out][in], fp16 */
  float b3[GRD_POLICY_OUT];
  /* Raw features are clamped to [lo, hi] (the training range) before the
   * mapping, so graphs beyond the training scales are seen as the nearest
   * trained ones rather than extrapolated. */
  float lo[GRD_POLICY_IN], hi[GRD_POLICY_IN];
} grd_policy_model;

/* Uploads a model for GRD_POLICY_LEARNED runs (NULL clears it). */
int grd_set_policy(grd_ctx* ctx, const grd_policy_model* model);

/* Raw features f0..f7 of n rounds from their frontier shape (host helper,
 * same formulas as the device). */
int grd_policy_features(const uint64_t* frontier, const uint64_t* frontier_edges,
                        const uint64_t* unvisited, const uint64_t* max_degree,
                        const uint32_t* round, uint32_t num_vertices,
                        uint64_t num_edges, size_t n, float* features);

typedef struct grd_policy_train_cfg {
  uint32_t steps;       /* full-batch Adam steps                            */
  float lr;             /* Adam step size                                   */
  float weight_decay;   /* L2 on weights (not biases)                       */
  uint64_t seed;        /* initialisation                                   */
  int device;
} grd_policy_train_cfg;

/* Trains on the GPU (own forward/backward kernels, Adam, fp32 master
 * weights rounded to fp16 for every forward pass).  x: n x 8 raw features;
 * y: n x 4 log2(round ms) targets; mask: n x 4 (1 = target measured).
 * mean/scale/lo/hi of `model` are computed from x.  loss_curve (optional, `steps`
 * entries) receives the masked MSE before each step. */
int grd_policy_train(const float* x, const float* y, const uint8_t* mask,
                     size_t n, const grd_policy_train_cfg* cfg,
                     grd_policy_model* model, float* loss_curve);

/* One forward + backward pass on the GPU: masked MSE and its gradient with
 * respect to every parameter, in the order w1, b1, w2, b2, w3, b3
 * (GRD_POLICY_NPARAM floats; fp16 weights are differentiated as values). */
int grd_policy_grad(const grd_policy_model* model, const float* x,
                    const float* y, const uint8_t* mask, size_t n, int device,
                    float* loss, float* grad);

/* GPU inference: out = n x 4 predictions, choice = argmin over the modes
 * whose bit is set in allowed_mask (bit m = mode m). */
int grd_policy_predict(const grd_policy_model* model, const float* x, size_t n,
                       uint32_t allowed_mask, int device, float* out,
                       int32_t* choice);
/* Error text of the most recent failed grd_policy_* call on this thread. */
const char* grd_policy_error(void);
/* Model files (the JSON layout grudon_gb300/policy_model.json uses): load
 * returns GRD_E_IO for a missing file or a missing / short field. */
int grd_policy_load(const char* path, grd_policy_model* out);
int grd_policy_save(const char* path, const grd_policy_model* model);

#ifdef __cplusplus
}
#endif
#endif /* GRUDON_GPU_H */
