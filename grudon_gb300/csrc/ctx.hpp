// grd_ctx: everything one partitioned graph owns on the host and device.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/grudon_gpu.h"
#include "kernels.cuh"
#include "layout.hpp"

struct PullState {
  uint32_t* comp = nullptr;       // [V] Kahan compensation of the aggregate
  double* residual = nullptr;     // [1] FP64 L1 residual of the last iteration
  double* h_residual = nullptr;   // pinned mirror
  grd::HubChunkD* in_hubs = nullptr;  // destination slots with long in-lists
  uint32_t num_in_hubs = 0;
};

struct grd_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
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
  unsigned long long* h_counters = nullptr;  // pinned
  uint64_t upload_bytes = 0;
  bool in_edges_alloc = false;
  PullState pull;
  bool profiling = false;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  std::vector<void*> host_registered;  // layout arrays pinned for H2D uploads
};

int grd_ctx_init_device(grd_ctx* ctx);
void grd_ctx_release_extras(grd_ctx* ctx);
int grd_enqueue_init(grd_ctx* ctx, uint32_t blocks);
int grd_upload_layout(grd_ctx* ctx);
int grd_ensure_in_edges(grd_ctx* ctx);
int grd_read_counters(grd_ctx* ctx);
int grd_enqueue_fwd(grd_ctx* ctx, bool fused);
int grd_enqueue_edge_map(grd_ctx* ctx);
int grd_enqueue_bwd(grd_ctx* ctx, bool fused, bool do_pack, bool do_aggregate);
int grd_enqueue_update(grd_ctx* ctx);
// PR_PULL: stage 0 fwd, 1 pull edge-map, 2 bwd pack, 3 aggregate, 4 update.
int grd_pull_stage(grd_ctx* ctx, int stage);
int grd_pull_run(grd_ctx* ctx);
