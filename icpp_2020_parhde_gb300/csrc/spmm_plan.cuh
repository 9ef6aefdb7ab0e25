// spmm_plan.cuh -- heavy-row chunk plan shared by the FP64 and mixed-precision Laplacian SpMM.
// Rows of degree <= SPMM_HEAVY are done by one warp; heavier rows (R-MAT hubs) are cut into chunks of
// SPMM_CHUNK neighbours whose partial sums are added back in chunk order.
#pragma once
#include "ctx.h"

constexpr int SPMM_HEAVY = 512, SPMM_CHUNK = 512;

struct HeavyRow {
  int64_t row;
  int64_t first_chunk;
  int64_t nchunks;
};
struct Chunk {
  int64_t e0, e1;
};

// Build (once per uploaded graph) or fetch the plan.
int phde_spmm_plan(phde_ctx *ctx, HeavyRow **heavy, Chunk **chunks, int64_t *nheavy, int64_t *nchunks);
