// grudon — command-line driver with the reference's flags (src/main.cpp:21-26)
// plus the algorithm choice the reference hard-codes (src/main.cpp:133-134):
//   -g graph (.gr or .mtx)   -c num compute (1)   -m num memory
//   -t threads (host tools)  -p partition file    -a pr|cc|sssp|sssp_w
//   --max-rounds N  --verify  --print
//   --policy fixed|learned [--policy-model FILE]  --frontier auto|bitvec|list
//   --direction auto|push|pull   (any of these: the rounds run as one
//   device-driven loop with that per-round schedule)
//   --offload ndp|engine|none    per-round offload decision (default ndp,
//   the reference's; engine = its NDPEngine rule)
// Runs one algorithm through the GraphAlgorithm plugin API on GPU 0 and
// prints the reference's statistics (Iterations, TotalBytesMoved).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/grudon/graph_algorithms.hpp"

using namespace grudon;

static void usage() {
  std::printf(
      "usage: grudon -g GRAPH -c 1 -m M [-p PARTFILE] [-a pr|cc|sssp|sssp_w] [--max-rounds N] [--verify] [--print]\n"
      "              [--policy fixed|learned] [--policy-model FILE] [--frontier auto|bitvec|list]\n"
      "              [--direction auto|push|pull] [--offload ndp|engine|none]\n");
}

int main(int argc, char** argv) {
  std::string graph_path, part_file, algo = "pr";
  size_t num_compute = 0, num_memory = 0;
  uint32_t max_rounds = MAX_ITERATIONS;
  bool do_verify = false, do_print = false, scheduled = false;
  int direction = GRD_DIR_AUTO, format = GRD_FMT_AUTO, policy = GRD_POLICY_FIXED, offload = GRD_OFFLOAD_NDP;
  std::string model_path;
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) {
        usage();
        std::exit(1);
      }
      return argv[++i];
    };
    if (a == "-g" || a == "--graph-path") graph_path = next();
    else if (a == "-c" || a == "--num-compute") num_compute = std::strtoul(next().c_str(), nullptr, 10);
    else if (a == "-m" || a == "--num-memory") num_memory = std::strtoul(next().c_str(), nullptr, 10);
    else if (a == "-t" || a == "--threads") next();
    else if (a == "-p" || a == "--partitioning-scheme") part_file = next();
    else if (a == "-a" || a == "--algorithm") algo = next();
    else if (a == "--max-rounds") max_rounds = (uint32_t)std::strtoul(next().c_str(), nullptr, 10);
    else if (a == "--policy" || a == "--frontier" || a == "--direction") {
      const std::string v = next();
      scheduled = true;
      bool ok = true;
      if (a == "--policy") ok = (v == "fixed" || v == "learned"), policy = v == "learned" ? GRD_POLICY_LEARNED : policy;
      if (a == "--frontier")
        ok = (v == "auto" || v == "bitvec" || v == "list"),
        format = v == "bitvec" ? GRD_FMT_BITVEC : v == "list" ? GRD_FMT_LIST : GRD_FMT_AUTO;
      if (a == "--direction")
        ok = (v == "auto" || v == "push" || v == "pull"),
        direction = v == "push" ? GRD_DIR_PUSH : v == "pull" ? GRD_DIR_PULL : GRD_DIR_AUTO;
      if (!ok) {
        usage();
        return 1;
      }
    } else if (a == "--offload") {
      const std::string v = next();
      if (v != "ndp" && v != "engine" && v != "none") {
        usage();
        return 1;
      }
      offload = v == "engine" ? GRD_OFFLOAD_ENGINE : v == "none" ? GRD_OFFLOAD_NONE : GRD_OFFLOAD_NDP;
    } else if (a == "--policy-model") model_path = next();
    else if (a == "--verify") do_verify = true;
    else if (a == "--print") do_print = true;
    else if (a == "-h" || a == "--help") {
      usage();
      return 0;
    } else {
      usage();
      return 1;
    }
  }
  if (graph_path.empty()) {
    std::fprintf(stderr, "Please provide a graph path\n");
    return 1;
  }
  if (num_compute == 0) {
    std::fprintf(stderr, "Please provide the number of master nodes\n");
    return 1;
  }
  if (num_memory == 0) {
    std::fprintf(stderr, "Please provide the number of mirror nodes\n");
    return 1;
  }
  grd_policy_model model{};
  const bool has_model = !model_path.empty();
  if (has_model && grd_policy_load(model_path.c_str(), &model) != GRD_OK) {
    std::fprintf(stderr, "error: cannot read policy model %s\n", model_path.c_str());
    return 2;
  }
  if (policy == GRD_POLICY_LEARNED && !has_model) {
    std::fprintf(stderr, "error: --policy learned needs --policy-model\n");
    return 1;
  }
  auto schedule = [&](auto& alg) {
    if (scheduled) alg.setSchedule(direction, format, policy, has_model ? &model : nullptr);
    alg.setOffload(offload);
  };
  try {
    GpuCore net(0);
    if (algo == "pr") {
      PageRank<float> pr(COMPUTE_NODE, "", graph_path, num_compute, num_memory, 0, net, part_file);
      pr.setMaxRounds(max_rounds);
      schedule(pr);
      pr.init();
      pr.run();
      if (do_print) pr.printState();
      if (do_verify) pr.verify();
      double sum = 0;
      for (float x : pr.ranks()) sum += x;
      std::printf("CHECKSUM %.6f\n", sum);
    } else if (algo == "cc") {
      CC<uint32_t> cc(COMPUTE_NODE, "", graph_path, num_compute, num_memory, 0, net, part_file);
      cc.setMaxRounds(max_rounds);
      schedule(cc);
      cc.init();
      cc.run();
      if (do_print) cc.printState();
      if (do_verify) {
        cc.verify();
        std::printf("VERIFY_ERRORS %llu\n", (unsigned long long)cc.errors);
      }
      unsigned long long sum = 0;
      for (uint32_t x : cc.labels()) sum += x;
      std::printf("CHECKSUM %llu\n", sum);
    } else if (algo == "sssp" || algo == "sssp_w") {
      SSSP<uint32_t> s(COMPUTE_NODE, "", graph_path, num_compute, num_memory, 0, net, part_file, algo == "sssp_w");
      s.setMaxRounds(max_rounds);
      schedule(s);
      s.init();
      s.run();
      if (do_print) s.printState();
      if (do_verify) {
        s.verify();
        std::printf("VERIFY_ERRORS %llu\n", (unsigned long long)s.errors);
      }
      unsigned long long sum = 0;
      for (uint32_t x : s.distances())
        if (x != 0xFFFFFFFFu) sum += x;
      std::printf("CHECKSUM %llu\n", sum);
    } else {
      usage();
      return 1;
    }
  } catch (const GpuError& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 2;
  }
  return 0;
}
