// ctx.h -- the library context (one CUDA stream, the uploaded graph, grow-only device workspace).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "common.cuh"
#include "parhde.h"

struct phde_ctx {
  int device = 0;
  int nsm = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  long long launches = 0;
  uint64_t timeout_ns = 5000000000ull;  // bounded device waits: 5 s per wait
  bool column_cgs2 = false;  // mixed path: column-at-a-time CGS2 (PHDE_CGS2=column) instead of blocked
  // mixed path: S^T (L S) on the tensor cores (PHDE_TC_GRAM=0: FP32 CUDA cores); the CGS2 Grams on them too
  // with PHDE_TC_GRAM=all (slower there: those Grams are 32 columns wide and stream at the memory roofline
  // on the CUDA cores)
  bool tc_gram = true;
  bool tc_gram_cgs2 = false;
  // uploaded batch (phde_batch_upload): the device CSR is the disjoint union of batch_B graphs
  int batch_B = 0;
  int64_t off_cap = 0, adj_cap = 0, gid_cap = 0;   // allocated entries of d_off, d_adj (and d_w), d_gid
  std::vector<int64_t> batch_vbase, batch_ebase;  // host copies, batch_B + 1 entries
  int64_t *d_vbase = nullptr;                      // [batch_B + 1]
  int32_t *d_gid = nullptr;                        // [n]: graph of each vertex
  int32_t *d_order = nullptr;                      // [batch_B]: graphs, largest first
  bool batch_blocks = false;                       // Kcenters with one CTA per graph
  int64_t batch_tuned_shape = -1;                  // autotuned segment length for this batch shape and k
  int batch_tuned_k = 0;
  int64_t batch_seg_rows = 8192;
  float batch_tune_ms = 0;
  cudaGraphExec_t batch_graph = nullptr;           // the captured batched pipeline
  int64_t batch_graph_epoch = -1;
  int batch_graph_c = 0;
  int batch_warm_key = -1;                         // the sequence last run uncaptured (c, strategy)
  int batch_last_c = 0;                            // coordinates of the last batched layout
  int64_t batch_graph_ws = -1;
  int64_t batch_graph_launches = 0;
  bool batch_no_graph = false;                     // capture failed once: launch directly
  int64_t ws_epoch = 0;                            // bumped whenever a workspace buffer is (re)allocated
  // SSSP band width: the mean edge weight of the uploaded graph (sssp.cu)
  double w_mean = 1.0;
  long long w_mean_epoch = -1;
  // drawing (draw.cu): the entry-row array's graph, and the size of the last image drawn
  long long draw_rows_epoch = -1;
  void *draw_rows_buf = nullptr;
  unsigned draw_W = 0, draw_H = 0;
  long long draw_epoch = -1;

  // uploaded graph (offsets widened to int64)
  int64_t n = 0, nnz = 0;
  bool weighted = false;
  int64_t *d_off = nullptr;
  uint32_t *d_adj = nullptr;
  int32_t *d_w = nullptr;
  long long graph_epoch = 0;  // bumped by every upload; caches keyed on it (the SpMM chunk plan)
  long long spmm_plan_epoch = -1;
  long long w64_epoch = -1;  // FP64 copy of the edge weights for the Laplacian SpMM
  void *w64_buf = nullptr;
  int64_t spmm_nheavy = 0, spmm_nchunks = 0;
  std::vector<float> pivot_model;  // MLP weights of the learned pivot strategy
  int pivot_check_rule = PHDE_CHECK_SUM;  // PHDE_STRAT_LEARNED_CHECKED's acceptance rule and tolerance
  double pivot_check_tol = 0.02;
  bool want_rq = false;            // compute the Rayleigh quotients of every layout (the checked strategy's reference)
  long long ms_plan_epoch = -1;  // multi-source BFS heavy-row plan
  int64_t ms_nheavy = 0, ms_nchunks = 0;
  bool ms_local = false;  // index-local numbering: the multi-source BFS stages frontier windows

  // device control block for persistent kernels: barrier + error word
  GridSync *d_sync = nullptr;
  int *d_err = nullptr;

  std::map<std::string, std::pair<void *, size_t>> ws;
  cudaEvent_t ev[8] = {};
  // events bracketing each distance-kernel launch; kev_pending says a pair was recorded
  cudaEvent_t kev[2] = {};
  cudaEvent_t lev[2] = {};  // around the exact path's Laplacian Gram kernel; lev_pending says they were recorded
  // PHDE_LAYOUT_TRACE=1: events at the learned pivot path's steps, printed after each layout
  cudaEvent_t tev[8] = {};
  int ntev = 0;
  bool lev_pending = false;
  bool kev_pending = false;
  double kernel_ms = 0;  // accumulated by phde_collect_kernel_time()
  double msbfs_ms = 0;   // of which multi-source BFS sweeps
  int msbfs_levels = 0;
  int kernel_launches = 0;
};

// Add the elapsed time of the last bracketed distance-kernel launch (the stream must have drained).
void phde_collect_kernel_time(phde_ctx *ctx);

// Set the context error message and return `status`.
int phde_fail(phde_ctx *ctx, int status, const std::string &msg);

// Grow-only named device buffer; returns nullptr on allocation failure (ctx->err set).
void *phde_buf(phde_ctx *ctx, const char *name, size_t bytes);

#define PHDE_CK(ctx, call)                                                                      \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      return phde_fail((ctx), e_ == cudaErrorMemoryAllocation ? PHDE_ERR_OOM : PHDE_ERR_CUDA, \
                       std::string(#call) + ": " + cudaGetErrorString(e_));                    \
  } while (0)

// After a launch: count it and surface launch-configuration errors.
#define PHDE_LAUNCHED(ctx)                                                                                  \
  do {                                                                                                      \
    (ctx)->launches++;                                                                                      \
    cudaError_t e_ = cudaGetLastError();                                                                    \
    if (e_ != cudaSuccess)                                                                                  \
      return phde_fail((ctx), PHDE_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e_)); \
  } while (0)

// Reset the device error word and barrier before a persistent kernel.
int phde_reset_sync(phde_ctx *ctx);
// Read the device error word after the stream drained; returns PHDE_OK or the recorded status.
int phde_check_device_err(phde_ctx *ctx, const char *what);

// ---- tensor-core Gram products (tcgram.cu) ----
// FP64 partials [nsplit][acols x bcols] of A^T diag(w) B (w may be null).
int phde_tc_gram64(phde_ctx *ctx, const float *A, int lda, int acols, const float *B, int ldb, int bcols,
                   const double *w, int64_t n, int nsplit, double *out64);
// FP32 partials in the blocked-CGS2 layout (bcgs.cu): self == 0 projection [S u0]^T D X over nqc chunks of 64
// Gram rows, self == 1 block Grams (X^T D X, X^T X).
int phde_tc_gram32(phde_ctx *ctx, const float *A, int lda, int nq, int ones, const float *X, const double *w,
                   int64_t n, int ncta, int nqc, int self, float *part);

// ---- exact-Gram dense stages (exact.cu, PHDE_PREC_EXACT) ----
// Where the candidate distance columns live: Z column t (1 <= t <= P) is int32 column t - 1 of D (column-major,
// n rows) for t <= P0, else column rmap[t - 1 - P0] of the multi-source BFS record R (row-major n x RW uint16,
// level + 1).  Kcenters and random pivots have every column in D (P0 = P).
struct ZSrc {
  const int32_t *D = nullptr;
  int P0 = 0;
  const uint16_t *R = nullptr;
  int RW = 0;
  const int *rmap = nullptr;  // device array
  // level mode instead of R (lvl non-null): record column c is the distance from source c, read from the
  // sweep's per-level frontier arrays (MsLevels)
  const unsigned long long *lvl = nullptr;
  int nlev = 0, W = 0;
};
// The accepted basis as coefficients over the integer columns Z = [1, D columns]: S_q = Z A[q][*].
struct ExactBasis {
  double *A = nullptr;   // [k][ld]
  const ull *GI = nullptr;  // [ld][ld] Z^T Z (upper triangle)
  const ull *GD = nullptr;  // [ld][ld] Z^T D Z (upper triangle)
  int *acc_idx = nullptr;  // [k] Z index of each accepted column (D column + 1)
  int ld = 0;
  unsigned maxz = 0, maxdeg = 0;
  void *Z = nullptr;     // accepted columns, row-major n x kp, uint8 (maxz <= 255) or uint16
  bool z16 = false;
  int kp = 0;
  const uint32_t *Zq = nullptr;  // byte path: the candidate columns in the quad layout (row stride ld words)
};
int phde_exact_orth(phde_ctx *ctx, const ZSrc &src, int P, int k, ExactBasis *eb, int *h_state, double *h_dlog);
int phde_exact_lap(phde_ctx *ctx, const ZSrc &src, int k, ExactBasis *eb, double *M);
int phde_exact_coords(phde_ctx *ctx, const double *M, const double *Y, int k, int c, ExactBasis *eb, double *X,
                      double *rq);
// Rayleigh quotients of the first min(c, PHDE_RQ_MAX) coordinates X = S Y: y^T M y / ||S y||^2 (device arrays),
// into rq (device).
int phde_rayleigh(phde_ctx *ctx, const double *M, const double *Y, int k, int c, const double *norm2, double *rq);
int phde_exact_basis(phde_ctx *ctx, const ZSrc &src, int k, const ExactBasis *eb, double *S);

// ---- drawing (draw.cu) ----
// The last drawn image's 4-bit palette scanlines (H rows of 1 + ceil(W / 2) bytes) copied to the host.
int phde_draw_scanlines(phde_ctx *ctx, std::vector<uint8_t> &out, unsigned &W, unsigned &H);

// ---- kernels (kcenters.cu) ----
// Kcenters / fixed-source BFS passes into D (n * P int32, column-major).  variant: 0 ParHDE history
// rule, 1 fixed sources (no selection; unreached vertices allowed), 2 DrawingBase history rule.
// require_all: an unreached vertex is an error (PHDE_ERR_DISCONNECTED); otherwise it keeps distance -1.
int phde_run_bfs_passes(phde_ctx *ctx, int P, int variant, const int64_t *d_fixed_src, int32_t *d_D,
                        int64_t *d_sources, unsigned long long *d_sumsq, unsigned long long *d_edges, int require_all);

// ---- kernels (msbfs.cu) ----
// The frontier words of every level of a level-mode sweep: bit b of word w of vertex v is set in level L's
// array, lvl[(L * n + v) * W + w], exactly when source 64 w + b reaches v first at level L; levels 0 .. nlev - 1.
constexpr int64_t PHDE_LEVEL_MODE_BYTES = 16ll << 30;  // largest frontier-array set a level-mode sweep keeps
struct MsLevels {
  const ull *lvl = nullptr;
  int nlev = 0;
  int W = 0;
};
int phde_msbfs_levels(phde_ctx *ctx, const int64_t *d_src, int nsrc, int lvl_cap, MsLevels *lv);
int phde_level_columns(phde_ctx *ctx, const MsLevels *lv, const int *h_cols, int ncols, int32_t *D,
                       unsigned long long *sumsq, int *h_unreached);
// Distance columns for nsrc given sources (device array) into D (n * nsrc int32, -1 unreached), up to 256
// sources per sweep.  With sumsq: exact per-column sums of squares and *h_unreached (synchronises).
int phde_msbfs(phde_ctx *ctx, const int64_t *d_src, int nsrc, int32_t *D, unsigned long long *sumsq,
               int *h_unreached);
// The same search, leaving the row-major uint16 record (level + 1, 0 = unreached; RW = nsrc rounded up to
// 64) in the context, and a gather of chosen columns of it into int32 column-major D.
int phde_msbfs_record(phde_ctx *ctx, const int64_t *d_src, int nsrc, uint16_t **R_out, int *RW_out);
int phde_heavy_chunks(phde_ctx *ctx, const int64_t **chunk_row, const int64_t **chunk_e0, int64_t *nchunks,
                      int64_t *chunk);
int phde_record_columns(phde_ctx *ctx, const uint16_t *R, int RW, const int *h_cols, int ncols, int32_t *D,
                        unsigned long long *sumsq, int *h_unreached);

// ---- kernels (sssp.cu) ----
// One exact SSSP pass from *d_src into d_col (int32, INF = INT32_MAX/2 for unreachable).
int phde_run_sssp(phde_ctx *ctx, const int64_t *d_src, int32_t *d_col, int32_t delta, unsigned long long *d_edges);
// Kcenters selection for one WParHDE pass (WParHDE.cpp:117-153): fold d_col into d_min, choose the
// next source into *d_next_src, append the raw argmax to the history, add sum(d^2) into *d_sumsq.
int phde_run_select(phde_ctx *ctx, const int32_t *d_col, int32_t *d_min, int pass, int check_fix, int64_t *d_hist,
                    int64_t *d_next_src, unsigned long long *d_sumsq);
