// grudon/graph_algorithms.hpp — PageRank, CC and SSSP plugins on one GB300.
//
// Same class names and virtuals as the reference's
// include/graph_algorithms/{pr,cc,sssp}.hpp; each virtual calls the C ABI
// stage that replaces the reference's loop:
//   init()            -> grd_set_algo + grd_init     (pr.cpp:20-61, cc.cpp:18-40, sssp.cpp:18-47)
//   gen_updates()     -> grd_edge_map                (pr.cpp:91-121, cc.cpp:54-84, sssp.cpp:61-90)
//   update_frontier() -> grd_update, which also applies the updates in the same
//                        kernel, so apply_updates() has nothing left to do
//                        (pr.cpp:63-147, cc.cpp:86-107, sssp.cpp:92-113)
//   aggregate()       -> grd_aggregate_values        (pr.cpp:149-153, cc.cpp:109-113, sssp.cpp:115-119)
//   verify()          -> the reference's invariants, checked on the device by
//                        grd_verify (cc.cpp:139-177, sssp.cpp:145-189,
//                        pr.cpp:179-205)
// Supported value types are the ones the GPU computes in: PageRank<float>,
// CC<uint32_t>, SSSP<uint32_t>.
#pragma once

#include <algorithm>
#include <cstring>
#include <type_traits>

#include "GraphAlgorithm.hpp"

#define DAMPING_FACTOR 0.85
#define TOLERANCE 1e-6

namespace grudon {

inline grd_params default_params() {
  grd_params p{};
  p.source = 0;
  p.max_rounds = MAX_ITERATIONS;
  p.damping = DAMPING_FACTOR;
  p.tolerance = TOLERANCE;
  p.direction = GRD_DIR_AUTO;
  p.frontier_format = GRD_FMT_AUTO;
  return p;
}

template <typename VertexProperty>
class PageRank : public GraphAlgorithm<VertexProperty> {
  static_assert(std::is_same<VertexProperty, float>::value, "the GPU PageRank computes in float");

 public:
  PageRank(NODE_TYPE node_type, std::string algorithm_name, std::string graph_path, size_t num_compute,
           size_t num_memory, uint32_t node_id, GpuCore& net, std::string partitioning_scheme_file = "")
      : GraphAlgorithm<VertexProperty>(node_type, algorithm_name, graph_path, num_compute, num_memory, node_id, net,
                                       partitioning_scheme_file) {
    this->algorithm_name = "PageRank";
  }
  PageRank(std::unique_ptr<DistributedGraph> g, GpuCore& net)
      : GraphAlgorithm<VertexProperty>(std::move(g), "PageRank", net) {}

  void init() override {
    grd_params p = default_params();
    p.max_rounds = this->max_rounds;
    this->gpu_init(GRD_PR_DELTA, p);
    this->clear_updates = true;
  }
  void apply_updates() override {}
  void gen_updates() override { check(grd_edge_map(this->ctx()), this->ctx(), "grd_edge_map"); }
  void update_frontier() override { this->gpu_update(); }
  void aggregate(GNode& lid, const VertexProperty& v) override {
    uint32_t bits;
    std::memcpy(&bits, &v, 4);
    this->gpu_aggregate_one(lid, bits);
  }
  bool termination_check() override { return this->last_frontier == 0; }
  std::vector<float> ranks() {
    std::vector<float> r(this->V());
    check(grd_read_ranks(this->ctx(), r.data(), r.size()), this->ctx(), "grd_read_ranks");
    return r;
  }
  void printState() override {
    std::vector<float> r = ranks();
    for (uint32_t n = 0; n < r.size(); ++n) std::printf("Vertex/PR: %u/%g\n", n, r[n]);
  }
  // Top 20 PageRank values.
  void verify() override {
    grd_verify_result r{};
    check(grd_verify(this->ctx(), &r), this->ctx(), "grd_verify");
    std::printf("Top 20 PageRank Values:\n");
    for (uint32_t i = 0; i < r.num_top; ++i) std::printf("Node: %u, PR: %g\n", r.top_ids[i], r.top_values[i]);
  }
};

template <typename VertexProperty>
class CC : public GraphAlgorithm<VertexProperty> {
  static_assert(std::is_same<VertexProperty, uint32_t>::value, "the GPU CC computes in uint32_t");

 public:
  CC(NODE_TYPE node_type, std::string algorithm_name, std::string graph_path, size_t num_compute, size_t num_memory,
     uint32_t node_id, GpuCore& net, std::string partitioning_scheme_file = "")
      : GraphAlgorithm<VertexProperty>(node_type, algorithm_name, graph_path, num_compute, num_memory, node_id, net,
                                       partitioning_scheme_file) {
    this->algorithm_name = "CC";
  }
  CC(std::unique_ptr<DistributedGraph> g, GpuCore& net) : GraphAlgorithm<VertexProperty>(std::move(g), "CC", net) {}

  void init() override {
    grd_params p = default_params();
    p.max_rounds = this->max_rounds;
    this->gpu_init(GRD_CC, p);
  }
  void apply_updates() override {}
  void gen_updates() override { check(grd_edge_map(this->ctx()), this->ctx(), "grd_edge_map"); }
  void update_frontier() override { this->gpu_update(); }
  void aggregate(GNode& lid, const VertexProperty& v) override { this->gpu_aggregate_one(lid, v); }
  bool termination_check() override { return this->last_frontier == 0; }
  std::vector<uint32_t> labels() { return this->template read_props<uint32_t>(); }
  void printState() override {
    std::vector<uint32_t> l = labels();
    for (uint32_t n = 0; n < l.size(); ++n) std::printf("Vertex/Dist: %u/%u\n", n, l[n]);
  }
  // Every edge's endpoints carry the same label; returns via the count.
  // Edges whose endpoints hold different labels, counted on the device.
  void verify() override {
    grd_verify_result r{};
    check(grd_verify(this->ctx(), &r), this->ctx(), "grd_verify");
    errors = r.errors;
    components = r.count;
  }
  uint64_t errors = 0, components = 0;
};

template <typename VertexProperty>
class SSSP : public GraphAlgorithm<VertexProperty> {
  static_assert(std::is_same<VertexProperty, uint32_t>::value, "the GPU SSSP computes in uint32_t");

 public:
  SSSP(NODE_TYPE node_type, std::string algorithm_name, std::string graph_path, size_t num_compute,
       size_t num_memory, uint32_t node_id, GpuCore& net, std::string partitioning_scheme_file = "",
       bool weighted = false)
      : GraphAlgorithm<VertexProperty>(node_type, algorithm_name, graph_path, num_compute, num_memory, node_id, net,
                                       partitioning_scheme_file),
        weighted(weighted) {
    this->algorithm_name = "SSSP";
  }
  SSSP(std::unique_ptr<DistributedGraph> g, GpuCore& net, bool weighted = false)
      : GraphAlgorithm<VertexProperty>(std::move(g), "SSSP", net), weighted(weighted) {}

  void init() override {
    grd_params p = default_params();
    p.max_rounds = this->max_rounds;
    p.source = source;
    this->gpu_init(weighted ? GRD_SSSP_W : GRD_SSSP_HOP, p);
  }
  void apply_updates() override {}
  void gen_updates() override { check(grd_edge_map(this->ctx()), this->ctx(), "grd_edge_map"); }
  void update_frontier() override { this->gpu_update(); }
  void aggregate(GNode& lid, const VertexProperty& v) override { this->gpu_aggregate_one(lid, v); }
  bool termination_check() override { return this->last_frontier == 0; }
  std::vector<uint32_t> distances() { return this->template read_props<uint32_t>(); }
  void printState() override {
    std::vector<uint32_t> d = distances();
    for (uint32_t n = 0; n < d.size(); ++n) std::printf("Vertex/Dist: %u/%u\n", n, d[n]);
  }
  // dist[dst] <= dist[src] + w(src,dst) for every reached src; also the
  // reference's max distance and visited count.
  // Edge relaxation invariant, reached count and largest distance, on the
  // device.
  void verify() override {
    grd_verify_result r{};
    check(grd_verify(this->ctx(), &r), this->ctx(), "grd_verify");
    errors = r.errors;
    visited = r.count;
    max_dist = (uint32_t)r.max_value;
    std::printf("Max Dist: %u\nTotal Visited Dist: %llu\n", max_dist, (unsigned long long)visited);
  }
  bool weighted;
  uint32_t source = 0;
  uint64_t errors = 0, visited = 0;
  uint32_t max_dist = 0;
};

}  // namespace grudon
