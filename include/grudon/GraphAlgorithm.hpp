// grudon/GraphAlgorithm.hpp — the reference's plugin API on one GB300.
//
// Mirrors include/GraphAlgorithm.hpp, include/Workers.hpp and
// include/DistributedGraph.hpp of the Grudon project: the same class names,
// constructor arguments (MPICore replaced by GpuCore), pure virtuals and
// run() round structure, so an algorithm written against the reference's
// GraphAlgorithm<V> ports by changing its includes.  All 1 + M partitions live
// in one grd_ctx on the GPU; the per-round stages the reference runs as MPI
// ranks (C2-C9 of GraphAlgorithm::run, src/GraphAlgorithm.cpp:145-701) become
// stream-ordered kernel stages of the C ABI (grudon_gpu.h).
//
// Differences a caller can see (all deliberate):
//  * one process drives every partition: node_type is COMPUTE_NODE and
//    node_id 0 (anything else is rejected); memory partitions have no host
//    object;
//  * num_compute must be 1 (every configuration of the operator uses one);
//  * the default partitioner for num_memory > 1 without a file is gid % M
//    (the reference silently puts every vertex in partition 0,
//    include/partitioning_engine/Partitioner.hpp:87);
//  * errors throw grudon::GpuError (the reference logs and continues).
#pragma once

#include <cstdint>
#include <cstdio>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../grudon_gpu.h"

#define MAX_ITERATIONS 1000

namespace grudon {

using GNode = uint32_t;

enum NODE_TYPE { COMPUTE_NODE, MEMORY_NODE, SWITCH_NODE };       // include/Graph.hpp:12-17
enum OFFLOAD_DECISION { NDP_OFFLOAD, NO_OFFLOAD, INC_OFFLOAD };  // include/Graph.hpp:19-24

class GpuError : public std::runtime_error {
 public:
  GpuError(int code, const std::string& what) : std::runtime_error(what), code(code) {}
  int code;
};

inline void check(int rc, grd_ctx* ctx, const char* what) {
  if (rc != GRD_OK)
    throw GpuError(rc, std::string(what) + ": " + (ctx ? grd_last_error(ctx) : grd_create_error()));
}

// Stands in for MPICore: the device the ctx lives on and the bytes-moved
// counter the reference keeps (include/MPI.hpp:41-61).
class GpuCore {
 public:
  explicit GpuCore(int device = 0) : device_(device) {}
  int getRank() const { return 0; }
  int getNumProcs() const { return 1; }
  int device() const { return device_; }
  uint64_t& getBytesMoved() { return bytes_moved_; }

 private:
  int device_;
  uint64_t bytes_moved_ = 0;
};

// Graph file + partitioning + device layout (src/DistributedGraph.cpp:13-785).
class DistributedGraph {
 public:
  DistributedGraph(const std::string& graph_path, size_t num_compute, size_t num_memory,
                   const std::string& partitioning_scheme_file, int device) {
    if (num_compute != 1) throw GpuError(GRD_E_INVALID, "num_compute must be 1");
    grd_host_graph* h = nullptr;
    const bool mtx = graph_path.size() > 4 && graph_path.compare(graph_path.size() - 4, 4, ".mtx") == 0;
    check(mtx ? grd_read_mtx(graph_path.c_str(), &h) : grd_read_gr(graph_path.c_str(), &h), nullptr,
          "reading the graph");
    host_.reset(h);
    init(num_memory, partitioning_scheme_file, device);
  }
  // Takes ownership of a host graph (generators, tests).
  DistributedGraph(grd_host_graph* g, size_t num_memory, const std::string& partitioning_scheme_file, int device) {
    host_.reset(g);
    init(num_memory, partitioning_scheme_file, device);
  }
  ~DistributedGraph() {
    if (ctx_) grd_ctx_destroy(ctx_);
  }
  DistributedGraph(const DistributedGraph&) = delete;
  DistributedGraph& operator=(const DistributedGraph&) = delete;

  // With one compute partition the compute-side lid equals the gid.
  GNode getLocalNode(const GNode& gid) const { return gid; }
  GNode getGlobalNode(const GNode& lid) const { return lid; }
  uint64_t getOutDegree(const GNode& lid) const {
    return host_->row_offsets[lid + 1] - host_->row_offsets[lid];
  }
  uint64_t getMirrorPartition(const GNode& lid) const { return mirror_[lid]; }
  uint64_t getMasterPartition(const GNode&) const { return 0; }
  uint64_t getNumVertices() const { return host_->num_vertices; }
  uint64_t getNumEdges() const { return host_->num_edges; }
  const grd_host_graph& host() const { return *host_; }
  grd_ctx* ctx() const { return ctx_; }

 private:
  struct Free {
    void operator()(grd_host_graph* g) const { grd_graph_free(g); }
  };
  void init(size_t num_memory, const std::string& file, int device) {
    const uint32_t V = host_->num_vertices;
    mirror_.assign(V, 0);
    if (!file.empty()) {
      check(grd_read_partition_file(file.c_str(), V, (uint32_t)num_memory, mirror_.data()), nullptr,
            "reading the partition file");
    } else {
      for (uint32_t v = 0; v < V; ++v) mirror_[v] = v % (uint32_t)num_memory;
    }
    grd_csr csr{host_->num_vertices, host_->num_edges, host_->row_offsets, host_->col_indices, host_->weights};
    check(grd_ctx_create(&csr, mirror_.data(), 1, (uint32_t)num_memory, device, &ctx_), nullptr, "grd_ctx_create");
  }
  std::unique_ptr<grd_host_graph, Free> host_;
  std::vector<uint32_t> mirror_;
  grd_ctx* ctx_ = nullptr;
};

template <typename VertexProperty>
class GraphAlgorithm;

// Worker roles (include/Workers.hpp:12-115).  On one GPU the update role
// runs on the compute partition's arrays and the traverse role on all
// memory partitions at once; both only forward to the plugin's virtuals.
template <typename T>
class Worker {
 public:
  virtual ~Worker() = default;
  virtual void update(GraphAlgorithm<T>& algorithm) = 0;
  virtual void traverse(GraphAlgorithm<T>& algorithm) = 0;
  virtual void aggregate(GraphAlgorithm<T>& algorithm, GNode& lid, const T& buffer_val) = 0;
};

template <typename T>
class UpdateWorker : public Worker<T> {  // src/Workers.cpp:71-82
 public:
  void update(GraphAlgorithm<T>& a) override {
    a.update_frontier();
    a.apply_updates();
  }
  void traverse(GraphAlgorithm<T>&) override {}
  void aggregate(GraphAlgorithm<T>& a, GNode& lid, const T& v) override { a.aggregate(lid, v); }
};

template <typename T>
class TraverseWorker : public Worker<T> {  // src/Workers.cpp:109-113
 public:
  void update(GraphAlgorithm<T>&) override {}
  void traverse(GraphAlgorithm<T>& a) override { a.gen_updates(); }
  void aggregate(GraphAlgorithm<T>&, GNode&, const T&) override {}
};

template <typename VertexProperty>
class GraphAlgorithm {
 public:
  // Same argument list as include/GraphAlgorithm.hpp:28-36 with GpuCore in
  // place of MPICore.
  GraphAlgorithm(NODE_TYPE node_type, std::string algorithm_name, std::string graph_path, size_t num_compute,
                 size_t num_memory, uint32_t node_id, GpuCore& net, std::string& partitioning_scheme_file)
      : algorithm_name(std::move(algorithm_name)), graph_path(graph_path), node_type(node_type), net(net),
        num_compute((uint32_t)num_compute), num_memory((uint32_t)num_memory) {
    if (node_type != COMPUTE_NODE || node_id != 0)
      throw GpuError(GRD_E_INVALID, "one process drives every partition: use COMPUTE_NODE, node_id 0");
    graph = std::make_unique<DistributedGraph>(graph_path, num_compute, num_memory, partitioning_scheme_file,
                                               net.device());
  }
  GraphAlgorithm(std::unique_ptr<DistributedGraph> g, std::string algorithm_name, GpuCore& net)
      : algorithm_name(std::move(algorithm_name)), node_type(COMPUTE_NODE), net(net), num_compute(1) {
    graph = std::move(g);
    num_memory = 0;
  }
  virtual ~GraphAlgorithm() = default;

  virtual void init() = 0;
  virtual void apply_updates() = 0;
  virtual void gen_updates() = 0;
  virtual void update_frontier() = 0;
  virtual void aggregate(GNode& lid, const VertexProperty& buffer_val) = 0;
  virtual bool termination_check() = 0;
  virtual void printState() = 0;
  virtual void verify() = 0;

  // The BSP round loop of src/GraphAlgorithm.cpp:177-690: forward sync (C2,
  // C3), traverse (C4), backward sync + aggregate (C5, C6), update and
  // termination (C7), until the frontier is empty or MAX_ITERATIONS rounds.
  void run() {
    grd_ctx* c = graph->ctx();
    if (fused) {  // the whole loop as one device-driven launch (grd_run)
      grd_stats st{};
      check(grd_run(c, 0, &st), c, "grd_run");
      net.getBytesMoved() = st.reference_bytes_moved;
      iterations = st.rounds;
      std::printf("STAT %s Iterations %u\nSTAT %s TotalBytesMoved %llu\n", algorithm_name.c_str(), st.rounds,
                  algorithm_name.c_str(), (unsigned long long)st.reference_bytes_moved);
      return;
    }
    uint32_t iteration = 0;
    bool done = false;
    while (!done && iteration < max_rounds) {
      check(grd_sync_fwd(c), c, "grd_sync_fwd");
      traverse_worker.traverse(*this);
      check(grd_sync_bwd(c), c, "grd_sync_bwd");
      check(grd_aggregate(c), c, "grd_aggregate");
      update_worker.update(*this);
      done = termination_check();
      ++iteration;
    }
    grd_stats st{};
    check(grd_get_stats(c, &st), c, "grd_get_stats");
    net.getBytesMoved() = st.reference_bytes_moved;
    iterations = iteration;
    std::printf("STAT %s Iterations %u\nSTAT %s TotalBytesMoved %llu\n", algorithm_name.c_str(), iteration,
                algorithm_name.c_str(), (unsigned long long)st.reference_bytes_moved);
  }

  // Per-round schedule (results never depend on it): GRD_DIR_*, GRD_FMT_*,
  // GRD_POLICY_* and the learned model (copied; NULL: none).  With a schedule
  // set, run() drives the rounds as one device-side loop (grd_run) instead
  // of stage by stage, and prints the same statistics.
  void setSchedule(int direction, int frontier_format, int policy, const grd_policy_model* model) {
    sched_direction = direction;
    sched_format = frontier_format;
    sched_policy = policy;
    has_model = model != nullptr;
    if (model) sched_model = *model;
    fused = true;
  }

  // Offload decision per round (GRD_OFFLOAD_*), the reference's NDPEngine
  // choice (include/offload_engine/NDPEngine.hpp:10-51) that its run()
  // leaves at NDP_OFFLOAD.  Anything but GRD_OFFLOAD_NDP runs the rounds as
  // one device-side loop (grd_run), like a schedule.
  void setOffload(int offload) {
    sched_offload = offload;
    if (offload != GRD_OFFLOAD_NDP) fused = true;
  }

  uint32_t getIterations() const { return iterations; }
  DistributedGraph& distributedGraph() { return *graph; }
  void setMaxRounds(uint32_t r) { max_rounds = r; }

 protected:
  std::string algorithm_name;
  std::string graph_path;
  NODE_TYPE node_type;
  GpuCore& net;
  uint32_t num_compute, num_memory;
  std::unique_ptr<DistributedGraph> graph;
  UpdateWorker<VertexProperty> update_worker;
  TraverseWorker<VertexProperty> traverse_worker;
  uint64_t last_frontier = 0;
  uint32_t iterations = 0;
  uint32_t max_rounds = MAX_ITERATIONS;
  bool clear_updates = false;
  bool fused = false;
  int sched_direction = GRD_DIR_AUTO, sched_format = GRD_FMT_AUTO, sched_policy = GRD_POLICY_FIXED;
  int sched_offload = GRD_OFFLOAD_NDP;
  bool has_model = false;
  grd_policy_model sched_model{};

  grd_ctx* ctx() const { return graph->ctx(); }
  uint32_t V() const { return (uint32_t)graph->getNumVertices(); }

  // Shared plumbing of the GPU plugins below.
  void gpu_init(int algo, grd_params p) {
    p.direction = sched_direction;
    p.frontier_format = sched_format;
    p.policy = sched_policy;
    p.offload = sched_offload;
    check(grd_set_algo(ctx(), algo, &p), ctx(), "grd_set_algo");
    check(grd_set_policy(ctx(), has_model ? &sched_model : nullptr), ctx(), "grd_set_policy");
    check(grd_init(ctx()), ctx(), "grd_init");
    last_frontier = 1;
  }
  void gpu_update() { check(grd_update(ctx(), &last_frontier), ctx(), "grd_update"); }
  void gpu_aggregate_one(GNode lid, uint32_t bits) {
    check(grd_aggregate_values(ctx(), &lid, &bits, 1), ctx(), "grd_aggregate_values");
  }
  template <class T>
  std::vector<T> read_props() {
    std::vector<T> out(V());
    check(grd_read_props(ctx(), out.data(), out.size() * sizeof(T)), ctx(), "grd_read_props");
    return out;
  }
};

}  // namespace grudon
