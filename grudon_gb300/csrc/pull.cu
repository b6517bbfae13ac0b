// PR_PULL: Jacobi PageRank through the partitioned structure (placeholder
// until the pull kernels land).
#include "ctx.hpp"

void grd_ctx_release_extras(grd_ctx* ctx) { (void)ctx; }

int grd_pull_stage(grd_ctx* ctx, int stage) {
  (void)stage;
  ctx->err = "GRD_PR_PULL is not available in this build";
  return GRD_E_INVALID;
}

int grd_pull_run(grd_ctx* ctx) { return grd_pull_stage(ctx, 0); }
