// api.cu -- C ABI entry points (include/parhde.h) and the host orchestration of the layout pipelines.
//
// phde_layout reproduces the control flow of the reference variants' run() methods (ParHDE.cpp:45-352,
// WParHDE.cpp:40-292, PivotMDS.cpp:68-147, PHDE.cpp:50-136) and of getCoordinates()
// (DrawingBase.cpp:196-205); every numeric stage runs on the GPU.  The host only sequences launches,
// reads a handful of status words and copies the n x c coordinates back.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ctx.h"

int phde_fill_i32(phde_ctx *ctx, int32_t *p, int64_t n, int32_t v);
int phde_degrees(phde_ctx *ctx, double *deg);
int phde_cgs(phde_ctx *ctx, const int32_t *D, int P, const ull *sumsq, const double *deg, double *S, int k,
             int *h_state, double *h_dlog);
int phde_mgs_pass(phde_ctx *ctx, const int32_t *col, const ull *sumsq, double *U, int j, int g, int k,
                  const double *deg, double *h_nrm2);
int phde_const_col(phde_ctx *ctx, double *U);
int phde_accept_col(phde_ctx *ctx, double *U, int xcol, double scale);
int phde_basis_rows(phde_ctx *ctx, const double *U, int k, double *S);
int phde_lap_spmm(phde_ctx *ctx, const double *deg, const double *S, double *LS, int k);
int phde_gram(phde_ctx *ctx, const double *A, const double *B, int k, double *M);
int phde_centre(phde_ctx *ctx, const int32_t *D, int k, int pivotmds, double *C);
int phde_coords(phde_ctx *ctx, const double *M, const double *Y, int k, int c, double *X, int seq,
                double *norm2 = nullptr);
int phde_gram_seq(phde_ctx *ctx, const double *C, int k, double *M);
int phde_cgs2_mixed(phde_ctx *ctx, const int32_t *D, int P, const ull *sumsq, const double *deg, float *S, int k,
                    int *h_state, double *h_dlog);
int phde_bcgs2_mixed(phde_ctx *ctx, const int32_t *D, int P, const ull *sumsq, const double *deg, float *S, int k,
                     int *h_state, double *h_dlog);
int phde_lap_spmm_mixed(phde_ctx *ctx, const double *deg, const float *S, float *LS, int k);
int phde_gram_mixed(phde_ctx *ctx, const float *A, const float *B, int k, double *M);
int phde_coords_mixed(phde_ctx *ctx, const float *S, const double *Y, int k, int c, double *X, double *norm2);
int phde_default_pivot_model(const float **w, int *count);
int phde_pivot_candidates(phde_ctx *ctx, const float *h_weights, int M, const int32_t *d_d0,
                          std::vector<int64_t> &h_cand, std::vector<float> &h_score);
int phde_cand_distances(phde_ctx *ctx, const int32_t *D, int P0, const uint16_t *R, int RW, const int64_t *d_cand,
                        int M, std::vector<int32_t> &h_sub, std::vector<int32_t> &h_csub,
                        const MsLevels *lv = nullptr);
int phde_eigensolve(phde_ctx *ctx, const double *d_M, int N, int c, int largest, int eig, double *d_K,
                    double *d_evals, double *d_Y, int *h_iters, int seq);

namespace {

__global__ void widen_offsets_kernel(const uint32_t *in, int64_t *out, int64_t count) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int64_t)in[i];
}

// Device-side CSR validation: offsets start at 0, never decrease, end at nnz; neighbours < n.
__global__ void validate_csr_kernel(const int64_t *off, const uint32_t *adj, int64_t n, int64_t nnz, int *bad) {
  int b = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    if (off[i + 1] < off[i]) b = 1;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += stride)
    if ((int64_t)adj[e] >= n) b = 1;
  if (blockIdx.x == 0 && threadIdx.x == 0 && (off[0] != 0 || off[n] != nnz)) b = 1;
  if (b) atomicExch(bad, 1);
}

// A barrier that waits for one more block than is launched: the bounded wait must give up.
__global__ void barrier_timeout_kernel(GridSync *gs, int *err, uint64_t timeout_ns) {
  grid_barrier(gs, err, timeout_ns, gridDim.x + 1);
}

// Published glibc TYPE_3 rand() stream (see eigen.cu); the reference draws random pivots with rand() % n.
void glibc_rand_host(uint32_t seed, int count, std::vector<int32_t> &out) {
  std::vector<int32_t> r((size_t)count + 344);
  if (seed == 0) seed = 1;
  r[0] = (int32_t)seed;
  for (int i = 1; i < 31; i++) {
    int32_t hi = r[i - 1] / 127773, lo = r[i - 1] % 127773;
    int32_t word = 16807 * lo - 2836 * hi;
    if (word < 0) word += 2147483647;
    r[i] = word;
  }
  for (int i = 31; i < 34; i++) r[i] = r[i - 31];
  for (int i = 34; i < count + 344; i++) r[i] = (int32_t)((uint32_t)r[i - 31] + (uint32_t)r[i - 3]);
  out.resize(count);
  for (int i = 0; i < count; i++) out[i] = (int32_t)(((uint32_t)r[i + 344]) >> 1);
}

struct Timer {
  phde_ctx *ctx;
  explicit Timer(phde_ctx *c) : ctx(c) {}
  void mark(int i) { cudaEventRecord(ctx->ev[i], ctx->stream); }
  double ms(int a, int b) {
    float t = 0;
    cudaEventElapsedTime(&t, ctx->ev[a], ctx->ev[b]);
    return t;
  }
};

}  // namespace

// ------------------------------------------------------------------------------------------------
int phde_fail(phde_ctx *ctx, int status, const std::string &msg) {
  if (ctx) ctx->err = msg;
  return status;
}

void *phde_buf(phde_ctx *ctx, const char *name, size_t bytes) {
  auto it = ctx->ws.find(name);
  if (it != ctx->ws.end() && it->second.second >= bytes) return it->second.first;
  if (it != ctx->ws.end()) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(it->second.first);
    ctx->ws.erase(it);
  }
  void *p = nullptr;
  ctx->ws_epoch++;
  if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) {
    cudaGetLastError();
    ctx->err = std::string("device allocation of ") + std::to_string(bytes) + " bytes for " + name + " failed";
    return nullptr;
  }
  ctx->ws[name] = {p, bytes};
  return p;
}

int phde_reset_sync(phde_ctx *ctx) {
  PHDE_CK(ctx, cudaMemsetAsync(ctx->d_sync, 0, sizeof(GridSync), ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
  return PHDE_OK;
}

void phde_collect_kernel_time(phde_ctx *ctx) {
  if (!ctx->kev_pending) return;
  float t = 0;
  if (cudaEventElapsedTime(&t, ctx->kev[0], ctx->kev[1]) == cudaSuccess) {
    ctx->kernel_ms += t;
    ctx->kernel_launches++;
  }
  cudaGetLastError();
  ctx->kev_pending = false;
}

int phde_check_device_err(phde_ctx *ctx, const char *what) {
  int e = 0;
  PHDE_CK(ctx, cudaMemcpyAsync(&e, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  phde_collect_kernel_time(ctx);
  if (e == PHDE_ERR_DISCONNECTED) return phde_fail(ctx, e, std::string(what) + ": the graph is not connected");
  if (e == PHDE_ERR_TIMEOUT) return phde_fail(ctx, e, std::string(what) + ": a bounded device wait gave up");
  if (e) return phde_fail(ctx, e, std::string(what) + ": device error " + std::to_string(e));
  return PHDE_OK;
}

extern "C" {

int phde_version(void) { return 10000; }

const char *phde_status_string(int s) {
  switch (s) {
    case PHDE_OK: return "ok";
    case PHDE_ERR_INVALID: return "invalid argument";
    case PHDE_ERR_CSR: return "malformed CSR";
    case PHDE_ERR_DISCONNECTED: return "graph is not connected";
    case PHDE_ERR_K_RANGE: return "k or c out of range";
    case PHDE_ERR_TOO_FEW_PIVOTS: return "too few pivots survived D-orthogonalisation";
    case PHDE_ERR_OOM: return "out of device memory";
    case PHDE_ERR_NOCONVERGE: return "eigensolver did not converge";
    case PHDE_ERR_TIMEOUT: return "bounded device wait timed out";
    case PHDE_ERR_CUDA: return "CUDA error";
    case PHDE_ERR_WEIGHTS: return "weights missing or unexpected";
    case PHDE_ERR_NO_GRAPH: return "no graph uploaded";
    default: return "unknown status";
  }
}

int phde_create(phde_ctx **out, int device) {
  if (!out) return PHDE_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return PHDE_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) return PHDE_ERR_INVALID;
  phde_ctx *c = new phde_ctx();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaMalloc(&c->d_sync, sizeof(GridSync)) != cudaSuccess || cudaMalloc(&c->d_err, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return PHDE_ERR_CUDA;
  }
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  if (!coop) {
    delete c;
    return PHDE_ERR_CUDA;
  }
  for (auto &e : c->ev) cudaEventCreate(&e);
  for (auto &e : c->kev) cudaEventCreate(&e);
  for (auto &e : c->lev) cudaEventCreate(&e);
  for (auto &e : c->tev) cudaEventCreate(&e);
  if (const char *t = getenv("PHDE_WAIT_LIMIT_MS")) c->timeout_ns = (uint64_t)atoll(t) * 1000000ull;
  if (const char *t = getenv("PHDE_CGS2")) c->column_cgs2 = std::string(t) == "column";
  if (const char *t = getenv("PHDE_TC_GRAM")) {
    c->tc_gram = std::string(t) != "0";
    c->tc_gram_cgs2 = std::string(t) == "all";
  }
  *out = c;
  return PHDE_OK;
}

void phde_destroy(phde_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto &kv : c->ws) cudaFree(kv.second.first);
  cudaFree(c->d_off);
  cudaFree(c->d_adj);
  cudaFree(c->d_w);
  cudaFree(c->d_sync);
  cudaFree(c->d_err);
  cudaFree(c->d_vbase);
  cudaFree(c->d_gid);
  cudaFree(c->d_order);
  if (c->batch_graph) cudaGraphExecDestroy(c->batch_graph);
  for (auto &e : c->ev) cudaEventDestroy(e);
  for (auto &e : c->kev) cudaEventDestroy(e);
  for (auto &e : c->lev) cudaEventDestroy(e);
  cudaStreamDestroy(c->stream);
  delete c;
}

const char *phde_last_error(const phde_ctx *c) { return c ? c->err.c_str() : "no context"; }
int64_t phde_graph_n(const phde_ctx *c) { return c ? c->n : 0; }
int64_t phde_graph_nnz(const phde_ctx *c) { return c ? c->nnz : 0; }
int64_t phde_launch_count(const phde_ctx *c) { return c ? c->launches : 0; }

int phde_graph_upload(phde_ctx *ctx, const void *offsets, int offset_bytes, const uint32_t *adj,
                      const int32_t *weights, int64_t n, int64_t nnz) {
  if (!ctx) return PHDE_ERR_INVALID;
  if (!offsets || (!adj && nnz > 0) || n <= 0 || nnz < 0 || (offset_bytes != 4 && offset_bytes != 8))
    return phde_fail(ctx, PHDE_ERR_INVALID, "phde_graph_upload: bad arguments");
  if (n >= 0xffffffffll || nnz >= 0xffffffffll)
    return phde_fail(ctx, PHDE_ERR_INVALID, "phde_graph_upload: n and nnz must be below 2^32");
  PHDE_CK(ctx, cudaSetDevice(ctx->device));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (n + 1 > ctx->off_cap || !ctx->d_off) {
    cudaFree(ctx->d_off);
    ctx->d_off = nullptr;
    ctx->off_cap = 0;
    PHDE_CK(ctx, cudaMalloc(&ctx->d_off, sizeof(int64_t) * (n + 1)));
    ctx->off_cap = n + 1;
  }
  if (nnz > ctx->adj_cap || !ctx->d_adj) {
    cudaFree(ctx->d_adj);
    ctx->d_adj = nullptr;
    ctx->adj_cap = 0;
    PHDE_CK(ctx, cudaMalloc(&ctx->d_adj, sizeof(uint32_t) * std::max<int64_t>(nnz, 1)));
    ctx->adj_cap = std::max<int64_t>(nnz, 1);
    cudaFree(ctx->d_w);
    ctx->d_w = nullptr;
  }
  ctx->n = n;
  ctx->nnz = nnz;
  ctx->graph_epoch++;
  ctx->batch_B = 0;
  if (offset_bytes == 8) {
    PHDE_CK(ctx, cudaMemcpyAsync(ctx->d_off, offsets, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
  } else {
    uint32_t *stage = (uint32_t *)phde_buf(ctx, "upload.off32", sizeof(uint32_t) * (n + 1));
    if (!stage) return PHDE_ERR_OOM;
    PHDE_CK(ctx, cudaMemcpyAsync(stage, offsets, sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
    widen_offsets_kernel<<<(int)std::min<int64_t>((n + 256) / 256, ctx->nsm * 8), 256, 0, ctx->stream>>>(stage, ctx->d_off,
                                                                                                       n + 1);
    PHDE_LAUNCHED(ctx);
  }
  if (nnz > 0)
    PHDE_CK(ctx, cudaMemcpyAsync(ctx->d_adj, adj, sizeof(uint32_t) * nnz, cudaMemcpyHostToDevice, ctx->stream));
  ctx->weighted = weights != nullptr;
  if (weights) {
    if (!ctx->d_w) PHDE_CK(ctx, cudaMalloc(&ctx->d_w, sizeof(int32_t) * ctx->adj_cap));
    if (nnz > 0)
      PHDE_CK(ctx, cudaMemcpyAsync(ctx->d_w, weights, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, ctx->stream));
  }
  int *bad = (int *)phde_buf(ctx, "upload.bad", sizeof(int));
  if (!bad) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
  validate_csr_kernel<<<(int)std::max<int64_t>(1, std::min<int64_t>((std::max(n, nnz) + 255) / 256, ctx->nsm * 8)), 256, 0,
                        ctx->stream>>>(ctx->d_off, ctx->d_adj, n, nnz, bad);
  PHDE_LAUNCHED(ctx);
  int h = 0;
  PHDE_CK(ctx, cudaMemcpyAsync(&h, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (h) {
    ctx->n = ctx->nnz = 0;
    return phde_fail(ctx, PHDE_ERR_CSR, "phde_graph_upload: offsets must start at 0, never decrease and end at nnz; "
                                        "neighbours must be < n");
  }
  return PHDE_OK;
}

// ------------------------------------------------------------------------------------------------
static int layout_impl(phde_ctx *ctx, const phde_layout_opts *o, double *coords_out, int64_t *sources_out,
                       phde_layout_extra *extra, phde_layout_stats *st) {
  const int64_t n = ctx->n;
  const int k = o->k, c = o->c;
  const int algo = o->algo;
  const bool hde = algo == PHDE_ALGO_PARHDE || algo == PHDE_ALGO_WPARHDE;
  Timer tm(ctx);
  const long long launches0 = ctx->launches;
  ctx->kernel_ms = 0;
  ctx->kernel_launches = 0;
  ctx->msbfs_ms = 0;
  ctx->msbfs_levels = 0;
  ctx->kev_pending = false;
  ctx->lev_pending = false;
  tm.mark(0);
  double *deg = (double *)phde_buf(ctx, "deg", sizeof(double) * n);
  ull *edges = (ull *)phde_buf(ctx, "edges", 2 * sizeof(ull));  // [0] edges examined, [1] SSSP rounds
  if (!deg || !edges) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(edges, 0, 2 * sizeof(ull), ctx->stream));
  int rc = phde_degrees(ctx, deg);
  if (rc) return rc;

  const int P = hde ? 3 * k : k;
  int64_t *d_src = (int64_t *)phde_buf(ctx, "layout.src", sizeof(int64_t) * (P + 2));
  ull *sumsq = (ull *)phde_buf(ctx, "layout.sumsq", sizeof(ull) * P);
  double *Sbuf = (double *)phde_buf(ctx, "layout.S", sizeof(double) * n * k);  // S (HDE) or C (MDS), row-major
  double *M = (double *)phde_buf(ctx, "layout.M", sizeof(double) * k * k);
  double *K = (double *)phde_buf(ctx, "layout.K", sizeof(double) * k * k);
  double *ev = (double *)phde_buf(ctx, "layout.ev", sizeof(double) * k);
  double *Y = (double *)phde_buf(ctx, "layout.Y", sizeof(double) * k * c);
  if (!d_src || !sumsq || !Sbuf || !M || !K || !ev || !Y) return PHDE_ERR_OOM;
  const bool mixed = o->precision == PHDE_PREC_MIXED;
  bool exact = o->precision == PHDE_PREC_EXACT;  // cleared when the inputs are out of the exact path's range
  ExactBasis eb;
  ZSrc zsrc;                   // where the exact path reads the candidate columns
  MsLevels lvl_sweep;          // learned pivots, exact path: the multi-source sweep's per-level frontier arrays
  std::vector<int> rec_order;  // learned pivots: the record columns of candidates P0.. (exact path)
  float *S32 = nullptr;
  if (mixed) {
    S32 = (float *)phde_buf(ctx, "layout.S32", sizeof(float) * n * k);
    if (!S32) return PHDE_ERR_OOM;
  }
  int npasses = 0, naccepted = 0, ndiscarded = 0;
  int P_used = P;  // distance columns handed to the D-orthogonalisation
  double ms_dist = 0, ms_orth = 0;
  const bool random = algo != PHDE_ALGO_WPARHDE && (o->strategy == PHDE_STRAT_RANDFINE ||
                                                    o->strategy == PHDE_STRAT_RANDCOARSE);

  if (algo == PHDE_ALGO_WPARHDE) {
    // ---- coupled SSSP + MGS loop (WParHDE.cpp:113-224) ----
    double *U = (double *)phde_buf(ctx, "wp.U", sizeof(double) * n * (k + 1));
    int32_t *col = (int32_t *)phde_buf(ctx, "wp.col", sizeof(int32_t) * n);
    int32_t *min_d = (int32_t *)phde_buf(ctx, "wp.min_d", sizeof(int32_t) * n);
    int64_t *hist = (int64_t *)phde_buf(ctx, "wp.hist", sizeof(int64_t) * P);
    int64_t *cur = (int64_t *)phde_buf(ctx, "wp.cur", sizeof(int64_t) * 2);
    if (!U || !col || !min_d || !hist || !cur) return PHDE_ERR_OOM;
    if ((rc = phde_const_col(ctx, U))) return rc;
    if ((rc = phde_fill_i32(ctx, min_d, n, 0x7fffffff))) return rc;
    PHDE_CK(ctx, cudaMemsetAsync(cur, 0, sizeof(int64_t) * 2, ctx->stream));
    PHDE_CK(ctx, cudaMemsetAsync(sumsq, 0, sizeof(ull) * P, ctx->stream));
    int correct = 1, gram_cols = 0;  // columns of U whose D-Gram entries the MGS kernels hold
    for (int r = 0; r < P; r++) {
      if (correct > k) break;
      tm.mark(6);
      PHDE_CK(ctx, cudaMemcpyAsync(d_src + r, cur, sizeof(int64_t), cudaMemcpyDeviceToDevice, ctx->stream));
      if ((rc = phde_reset_sync(ctx))) return rc;
      if ((rc = phde_run_sssp(ctx, cur, col, 10000, edges))) return rc;  // delta: WParHDE.cpp:104
      if ((rc = phde_run_select(ctx, col, min_d, r, correct != 1, hist, cur + 1, sumsq + r))) return rc;
      PHDE_CK(ctx, cudaMemcpyAsync(cur, cur + 1, sizeof(int64_t), cudaMemcpyDeviceToDevice, ctx->stream));
      tm.mark(7);
      double nrm2 = 0;
      const int g = gram_cols < correct ? correct - 1 : -1;
      if ((rc = phde_mgs_pass(ctx, col, sumsq + r, U, correct, g, k, deg, &nrm2))) return rc;
      gram_cols = correct;
      if ((rc = phde_check_device_err(ctx, "WParHDE distance pass"))) return rc;
      npasses++;
      ms_dist += tm.ms(6, 7);
      const double nrm = std::sqrt(nrm2);
      if (nrm < 0.001) {
        ndiscarded++;
        if (o->verbose) printf("discarding vec %d, normdist %g\n", correct, nrm);
      } else {
        if ((rc = phde_accept_col(ctx, U, correct, 1.0 / nrm))) return rc;
        correct++;
      }
      tm.mark(6);
      PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
      ms_orth += tm.ms(7, 6);
    }
    naccepted = correct - 1;
    if (naccepted < k)
      return phde_fail(ctx, PHDE_ERR_TOO_FEW_PIVOTS,
                       "Number of Pivots obtained: " + std::to_string(naccepted) + " inadequate, increase the Pivots Limits: " +
                           std::to_string(P));
    tm.mark(7);
    if ((rc = phde_basis_rows(ctx, U, k, Sbuf))) return rc;  // U's accepted columns -> row-major S
    tm.mark(2);
    PHDE_CK(ctx, cudaEventSynchronize(ctx->ev[2]));
    ms_orth += tm.ms(7, 2);
  } else {
    // ---- distance phase: Kcenters (or random) BFS passes into D ----
    int32_t *D = (int32_t *)phde_buf(ctx, "layout.D", sizeof(int32_t) * n * P);
    if (!D) return PHDE_ERR_OOM;
    if (o->strategy == PHDE_STRAT_LEARNED) {
      // ---- learned pivots: Kcenters warm start, MLP candidates, one multi-source BFS, farthest-point ----
      const int P0 = std::min(P, PHDE_LEARNED_WARM);  // exact Kcenters passes (serial, few)
      const int M = (int)std::min<int64_t>(PHDE_LEARNED_CANDIDATES, n);
      int64_t *dc = (int64_t *)phde_buf(ctx, "lp.dcand", sizeof(int64_t) * M);
      if (!dc) return PHDE_ERR_OOM;
      if (ctx->pivot_model.empty()) {
        const float *w0;
        int cnt;
        if ((rc = phde_default_pivot_model(&w0, &cnt))) return phde_fail(ctx, rc, "built-in pivot model has the wrong size");
        ctx->pivot_model.assign(w0, w0 + cnt);
      }
      const bool ltrace = getenv("PHDE_LAYOUT_TRACE") != nullptr;
      auto tmark = [&]() {
        if (ltrace && ctx->ntev < 8) cudaEventRecord(ctx->tev[ctx->ntev++], ctx->stream);
      };
      ctx->ntev = 0;
      tmark();
      if ((rc = phde_run_bfs_passes(ctx, P0, 0, nullptr, D, d_src, sumsq, edges, 1))) return rc;
      tmark();
      // the first warm-start pass's Kcenters key (its eccentricity in the high word), read with the error word
      unsigned long long key0 = 0;
      {
        const ull *keys = (const ull *)phde_buf(ctx, "kc.keys", 0);
        if (!keys) return PHDE_ERR_OOM;
        PHDE_CK(ctx, cudaMemcpyAsync(&key0, keys, sizeof(key0), cudaMemcpyDeviceToHost, ctx->stream));
      }
      if ((rc = phde_check_device_err(ctx, "learned pivots: warm start"))) return rc;
      std::vector<int64_t> cand, warm(P0);
      std::vector<float> cscore;
      // the candidates are scored on the warm start's running minimum distance (Kcenters' own criterion)
      const int32_t *mind0 = (const int32_t *)phde_buf(ctx, "kc.min_d", sizeof(int32_t) * n);
      if (!mind0) return PHDE_ERR_OOM;
      if ((rc = phde_pivot_candidates(ctx, ctx->pivot_model.data(), M, mind0, cand, cscore))) return rc;
      tmark();
      const int Mc = (int)cand.size();
      PHDE_CK(ctx, cudaMemcpyAsync(dc, cand.data(), sizeof(int64_t) * Mc, cudaMemcpyHostToDevice, ctx->stream));
      uint16_t *R = nullptr;
      int RW = 0;
      // the candidates' distances are read straight from the sweep's per-level frontier arrays (no record) when
      // their number fits: the sweep has at most diameter + 1 <= 2 ecc + 1 levels, ecc the first warm-start
      // source's eccentricity (the Kcenters key of pass 0), and the exact path's byte layout needs distances < 255
      bool level_mode = false;
      {
        const int64_t cap = 2 * (int64_t)(key0 >> 32) + 1;
        const int64_t bytes = (cap + 1) * n * ((Mc + 63) / 64) * (int64_t)sizeof(ull);
        if (cap <= 254 && bytes <= PHDE_LEVEL_MODE_BYTES) {
          rc = phde_msbfs_levels(ctx, dc, Mc, (int)cap, &lvl_sweep);
          if (rc == PHDE_OK) level_mode = true;
          else if (rc != PHDE_ERR_TOO_LARGE) return rc;
        }
      }
      if (!level_mode && (rc = phde_msbfs_record(ctx, dc, Mc, &R, &RW))) return rc;
      tmark();
      std::vector<int32_t> sub, csub;
      if ((rc = phde_cand_distances(ctx, D, P0, R, RW, dc, Mc, sub, csub, level_mode ? &lvl_sweep : nullptr)))
        return rc;
      // farthest-point selection over the candidates: distance to the pivots chosen so far (warm start
      // included), best score first on ties
      const int Pl = std::min(P, P0 + Mc);
      std::vector<int32_t> mind(Mc, INT32_MAX);
      for (int i = 0; i < Mc; i++)
        for (int j = 0; j < P0; j++) mind[i] = std::min(mind[i], sub[(size_t)i * P0 + j]);
      std::vector<char> used(Mc, 0);
      std::vector<int> order;
      for (int p = P0; p < Pl; p++) {
        int best = -1;
        for (int i = 0; i < Mc; i++)
          if (!used[i] && (best < 0 || mind[i] > mind[best])) best = i;
        if (best < 0) break;
        used[best] = 1;
        order.push_back(best);
        for (int i = 0; i < Mc; i++) mind[i] = std::min(mind[i], csub[(size_t)i * Mc + best]);
      }
      const int Pn = (int)order.size();
      if (exact && hde) {
        // the exact path reads the candidates' columns from the record where they are (no gather); the warm
        // start's first pass already required every vertex to be reached
        int *rmap = (int *)phde_buf(ctx, "lp.rmap", sizeof(int) * std::max(Pn, 1));
        if (!rmap) return PHDE_ERR_OOM;
        if (Pn > 0)
          PHDE_CK(ctx, cudaMemcpyAsync(rmap, order.data(), sizeof(int) * Pn, cudaMemcpyHostToDevice, ctx->stream));
        zsrc.D = D;
        zsrc.P0 = P0;
        zsrc.R = R;
        zsrc.RW = RW;
        zsrc.rmap = rmap;
        if (level_mode) {
          zsrc.lvl = lvl_sweep.lvl;
          zsrc.nlev = lvl_sweep.nlev;
          zsrc.W = lvl_sweep.W;
        }
        rec_order = order;
      } else {
        int unreached = 0;
        rc = level_mode
                 ? phde_level_columns(ctx, &lvl_sweep, order.data(), Pn, D + (int64_t)P0 * n, sumsq + P0, &unreached)
                 : phde_record_columns(ctx, R, RW, order.data(), Pn, D + (int64_t)P0 * n, sumsq + P0, &unreached);
        if (rc) return rc;
        if (unreached) return phde_fail(ctx, PHDE_ERR_DISCONNECTED, "distance passes: the graph is not connected");
      }
      std::vector<int64_t> srcs(Pn);
      for (int p = 0; p < Pn; p++) srcs[p] = cand[order[p]];
      if (Pn > 0)
        PHDE_CK(ctx, cudaMemcpyAsync(d_src + P0, srcs.data(), sizeof(int64_t) * Pn, cudaMemcpyHostToDevice, ctx->stream));
      P_used = P0 + Pn;
      tmark();
      if (ltrace) {
        PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
        static const char *names[] = {"warm start", "features, scores, candidates", "multi-source BFS",
                                      "candidate distances, order, columns"};
        for (int i = 1; i < ctx->ntev; i++) {
          float t = 0;
          cudaEventElapsedTime(&t, ctx->tev[i - 1], ctx->tev[i]);
          fprintf(stderr, "learned pivots: %s %.3f ms\n", i <= 4 ? names[i - 1] : "?", t);
        }
      }
    } else if (random) {
      std::vector<int32_t> r;
      glibc_rand_host((uint32_t)o->seed, P, r);
      std::vector<int64_t> s(P);
      for (int i = 0; i < P; i++) s[i] = (int64_t)r[i] % n;
      PHDE_CK(ctx, cudaMemcpyAsync(d_src, s.data(), sizeof(int64_t) * P, cudaMemcpyHostToDevice, ctx->stream));
      int64_t *d_src2 = (int64_t *)phde_buf(ctx, "layout.src2", sizeof(int64_t) * P);
      if (!d_src2) return PHDE_ERR_OOM;
      // all sources are known up front: one multi-source sweep per 256 sources
      int unreached = 0;
      (void)d_src2;
      if ((rc = phde_msbfs(ctx, d_src, P, D, sumsq, &unreached))) return rc;
      if (unreached) return phde_fail(ctx, PHDE_ERR_DISCONNECTED, "distance passes: the graph is not connected");
    } else {
      if ((rc = phde_run_bfs_passes(ctx, P, hde ? 0 : 2, nullptr, D, d_src, sumsq, edges, 1))) return rc;
    }
    if ((rc = phde_check_device_err(ctx, "distance passes"))) return rc;
    npasses = P_used;
    tm.mark(1);
    if (hde) {
      int state[4] = {0, 0, 0, 0};
      std::vector<double> dlog(P);
      if (exact) {
        if (!zsrc.R && !zsrc.lvl) {
          zsrc.D = D;
          zsrc.P0 = P_used;
        }
        rc = phde_exact_orth(ctx, zsrc, P_used, k, &eb, state, dlog.data());
        if (rc == PHDE_ERR_TOO_LARGE) {  // distances or degrees beyond the exact sums: the FP64 vector kernels
          exact = false;
          if (zsrc.R || zsrc.lvl) {  // they need the learned candidates' columns in D, with their sums of squares
            int unreached = 0;
            const int P0 = zsrc.P0, Pn = (int)rec_order.size();
            if (zsrc.lvl)
              rc = phde_level_columns(ctx, &lvl_sweep, rec_order.data(), Pn, D + (int64_t)P0 * n, sumsq + P0,
                                      &unreached);
            else
              rc = phde_record_columns(ctx, zsrc.R, zsrc.RW, rec_order.data(), Pn, D + (int64_t)P0 * n, sumsq + P0,
                                       &unreached);
            if (rc) return rc;
          }
          rc = phde_cgs(ctx, D, P_used, sumsq, deg, Sbuf, k, state, dlog.data());
        }
      } else if (mixed && !ctx->column_cgs2)
        rc = phde_bcgs2_mixed(ctx, D, P_used, sumsq, deg, S32, k, state, dlog.data());
      else if (mixed)
        rc = phde_cgs2_mixed(ctx, D, P_used, sumsq, deg, S32, k, state, dlog.data());
      else
        rc = phde_cgs(ctx, D, P_used, sumsq, deg, Sbuf, k, state, dlog.data());
      if (rc) return rc;
      if ((rc = phde_check_device_err(ctx, "D-orthogonalisation"))) return rc;
      naccepted = state[0];
      ndiscarded = state[1];
      if (o->verbose) {
        int j = 1;
        for (int r = 0; r < state[2]; r++) {
          if (std::isnan(dlog[r]))
            j++;
          else
            printf("discarding vec %d, normdist %g\n", j, dlog[r]);
        }
      }
      if (naccepted < k)
        return phde_fail(ctx, PHDE_ERR_TOO_FEW_PIVOTS,
                         "Number of Pivots obtained: " + std::to_string(naccepted) +
                             " inadequate, increase the Pivots Limits: " + std::to_string(P));
    } else {
      if ((rc = phde_centre(ctx, D, k, algo == PHDE_ALGO_PIVOTMDS, Sbuf))) return rc;
      naccepted = k;
    }
    tm.mark(2);
    PHDE_CK(ctx, cudaEventSynchronize(ctx->ev[2]));
    ms_dist = tm.ms(0, 1);
    ms_orth = tm.ms(1, 2);
  }

  // ---- Laplacian SpMM + Gram (HDE) or C^T C (MDS) ----
  if (hde && exact) {
    if ((rc = phde_exact_lap(ctx, zsrc, k, &eb, M))) return rc;
  } else if (hde && mixed) {
    float *LS32 = (float *)phde_buf(ctx, "layout.LS32", sizeof(float) * n * k);
    if (!LS32) return PHDE_ERR_OOM;
    if ((rc = phde_lap_spmm_mixed(ctx, deg, S32, LS32, k))) return rc;
    if ((rc = phde_gram_mixed(ctx, S32, LS32, k, M))) return rc;
  } else if (hde) {
    double *LS = (double *)phde_buf(ctx, "layout.LS", sizeof(double) * n * k);
    if (!LS) return PHDE_ERR_OOM;
    if ((rc = phde_lap_spmm(ctx, deg, Sbuf, LS, k))) return rc;
    if ((rc = phde_gram(ctx, Sbuf, LS, k, M))) return rc;
  } else {
    if ((rc = phde_gram_seq(ctx, Sbuf, k, M))) return rc;  // reference summation order: bit-exact C^T C
  }
  tm.mark(3);
  if (extra && extra->gram)
    PHDE_CK(ctx, cudaMemcpyAsync(extra->gram, M, sizeof(double) * k * k, cudaMemcpyDeviceToHost, ctx->stream));
  int iters = 0;
  if ((rc = phde_eigensolve(ctx, M, k, c, hde ? 0 : 1, o->eig, K, ev, Y, &iters, !hde))) return rc;
  tm.mark(4);
  double *X = (double *)phde_buf(ctx, "layout.X", sizeof(double) * n * c);
  if (!X) return PHDE_ERR_OOM;
  double *rqd = (double *)phde_buf(ctx, "layout.rq", sizeof(double) * PHDE_RQ_MAX);
  double *norm2 = (double *)phde_buf(ctx, "layout.norm2", sizeof(double) * PHDE_MAX_K);
  if (!rqd || !norm2) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(rqd, 0, sizeof(double) * PHDE_RQ_MAX, ctx->stream));
  const bool want_rq = ctx->want_rq || o->strategy == PHDE_STRAT_LEARNED;
  if (exact)
    rc = phde_exact_coords(ctx, M, Y, k, c, &eb, X, rqd);  // the quotients come with it, from k x k products
  else if (mixed)
    rc = phde_coords_mixed(ctx, S32, Y, k, c, X, want_rq ? norm2 : nullptr);
  else
    rc = phde_coords(ctx, Sbuf, Y, k, c, X, !hde, want_rq ? norm2 : nullptr);
  if (rc) return rc;
  if (want_rq && !exact && hde && (rc = phde_rayleigh(ctx, M, Y, k, c, norm2, rqd))) return rc;
  PHDE_CK(ctx, cudaMemcpyAsync(coords_out, X, sizeof(double) * n * c, cudaMemcpyDeviceToHost, ctx->stream));
  tm.mark(5);
  if (sources_out && npasses > 0)
    PHDE_CK(ctx, cudaMemcpyAsync(sources_out, d_src, sizeof(int64_t) * npasses, cudaMemcpyDeviceToHost, ctx->stream));
  ull h_edges[2] = {0, 0};
  PHDE_CK(ctx, cudaMemcpyAsync(h_edges, edges, 2 * sizeof(ull), cudaMemcpyDeviceToHost, ctx->stream));
  double h_rq[PHDE_RQ_MAX];
  PHDE_CK(ctx, cudaMemcpyAsync(h_rq, rqd, sizeof(h_rq), cudaMemcpyDeviceToHost, ctx->stream));
  if (extra && extra->evecs)
    PHDE_CK(ctx, cudaMemcpyAsync(extra->evecs, K, sizeof(double) * k * k, cudaMemcpyDeviceToHost, ctx->stream));
  if (extra && extra->evals)
    PHDE_CK(ctx, cudaMemcpyAsync(extra->evals, ev, sizeof(double) * k, cudaMemcpyDeviceToHost, ctx->stream));
  std::vector<double> Srow;
  std::vector<float> Srow32;
  if (extra && extra->basis) {
    if (exact && (rc = phde_exact_basis(ctx, zsrc, k, &eb, Sbuf))) return rc;
    if (mixed) {
      Srow32.resize((size_t)n * k);
      PHDE_CK(ctx, cudaMemcpyAsync(Srow32.data(), S32, sizeof(float) * n * k, cudaMemcpyDeviceToHost, ctx->stream));
    } else {
      Srow.resize((size_t)n * k);
      PHDE_CK(ctx, cudaMemcpyAsync(Srow.data(), Sbuf, sizeof(double) * n * k, cudaMemcpyDeviceToHost, ctx->stream));
    }
  }
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (extra && extra->basis)
    for (int64_t i = 0; i < n; i++)
      for (int q = 0; q < k; q++)
        extra->basis[i + (int64_t)q * n] = mixed ? (double)Srow32[(size_t)i * k + q] : Srow[(size_t)i * k + q];
  if (st) {
    st->npasses = npasses;
    st->naccepted = naccepted;
    st->ndiscarded = ndiscarded;
    st->eig_iters = iters;
    st->ms_dist = ms_dist;
    st->ms_orth = ms_orth;
    st->ms_mmult = tm.ms(2, 3);
    st->ms_eig = tm.ms(3, 4);
    st->ms_coords = tm.ms(4, 5);
    st->ms_total = tm.ms(0, 5);
    st->edges_examined = (int64_t)h_edges[0];
    st->sssp_rounds = (int64_t)h_edges[1];
    st->gpu_launches = (int)(ctx->launches - launches0);
    st->ms_dist_kernel = ctx->kernel_ms;
    st->dist_kernel_launches = ctx->kernel_launches;
    st->ms_msbfs_kernel = ctx->msbfs_ms;
    st->msbfs_levels = ctx->msbfs_levels;
    if (exact || (want_rq && hde))
      for (int j = 0; j < PHDE_RQ_MAX; j++) st->rayleigh[j] = j < c ? h_rq[j] : 0.0;
    if (ctx->lev_pending) {
      float t = 0;
      if (cudaEventElapsedTime(&t, ctx->lev[0], ctx->lev[1]) == cudaSuccess) st->ms_lap_kernel = t;
      cudaGetLastError();
    }
  }
  return PHDE_OK;
}

// The learned strategies: PHDE_STRAT_LEARNED falls back to Kcenters when the proposal gives no layout;
// PHDE_STRAT_LEARNED_CHECKED also lays the graph out with Kcenters and returns the learned layout only when its
// Rayleigh quotients pass the acceptance rule against Kcenters'.
static bool pivots_accepted(const phde_ctx *ctx, const double *rl, const double *rk, int c) {
  const int cc = std::min(c, PHDE_RQ_MAX);
  const double f = 1.0 + ctx->pivot_check_tol;
  if (ctx->pivot_check_rule == PHDE_CHECK_EACH) {
    for (int j = 0; j < cc; j++)
      if (!(rl[j] <= f * rk[j])) return false;
    return true;
  }
  double sl = 0, sk = 0;
  for (int j = 0; j < cc; j++) {
    sl += rl[j];
    sk += rk[j];
  }
  return sl <= f * sk;  // false for NaN quotients
}

static int layout_learned(phde_ctx *ctx, const phde_layout_opts *o, double *coords_out, int64_t *sources_out,
                          phde_layout_extra *extra, phde_layout_stats *st) {
  const bool checked = o->strategy == PHDE_STRAT_LEARNED_CHECKED;
  phde_layout_opts ol = *o, ok = *o;
  ol.strategy = PHDE_STRAT_LEARNED;
  ok.strategy = PHDE_STRAT_KCENTERS;
  phde_layout_stats sl, sk;
  memset(&sl, 0, sizeof(sl));
  memset(&sk, 0, sizeof(sk));
  const int64_t n = ctx->n;
  std::vector<double> xk;
  std::vector<int64_t> srck;
  int rc;
  if (checked) {  // the Kcenters reference layout first, kept on the host
    xk.resize((size_t)n * o->c);
    srck.resize((size_t)3 * o->k);
    ctx->want_rq = true;
    rc = layout_impl(ctx, &ok, xk.data(), srck.data(), nullptr, &sk);
    ctx->want_rq = false;
    if (rc) return rc;
  }
  rc = layout_impl(ctx, &ol, coords_out, sources_out, extra, &sl);
  int outcome = PHDE_OUTCOME_LEARNED;
  if (rc == PHDE_ERR_TOO_LARGE || rc == PHDE_ERR_TOO_FEW_PIVOTS) {
    cudaStreamSynchronize(ctx->stream);
    outcome = PHDE_OUTCOME_FAILED;
  } else if (rc) {
    return rc;
  } else if (checked && !pivots_accepted(ctx, sl.rayleigh, sk.rayleigh, o->c)) {
    outcome = PHDE_OUTCOME_REJECTED;
  }
  if (outcome != PHDE_OUTCOME_LEARNED) {
    if (checked && !(extra && (extra->basis || extra->gram || extra->evecs || extra->evals))) {
      memcpy(coords_out, xk.data(), sizeof(double) * xk.size());
      if (sources_out) memcpy(sources_out, srck.data(), sizeof(int64_t) * sk.npasses);
    } else {
      const double check_ms = sk.ms_total;
      ctx->want_rq = true;
      rc = layout_impl(ctx, &ok, coords_out, sources_out, extra, &sk);
      ctx->want_rq = false;
      if (rc) return rc;
      sk.ms_total += check_ms;
    }
  }
  if (st) {
    const phde_layout_stats &ret = outcome == PHDE_OUTCOME_LEARNED ? sl : sk;
    *st = ret;
    st->pivot_outcome = outcome;
    memcpy(st->rayleigh, sl.rayleigh, sizeof(st->rayleigh));
    memcpy(st->rayleigh_kcenters, sk.rayleigh, sizeof(st->rayleigh_kcenters));
    st->ms_check = checked ? sk.ms_total : 0.0;
    st->ms_total = sl.ms_total + sk.ms_total;  // every layout this call computed
  }
  return PHDE_OK;
}

int phde_layout(phde_ctx *ctx, const phde_layout_opts *o, double *coords_out, int64_t *sources_out,
                phde_layout_extra *extra, phde_layout_stats *st) {
  if (st) memset(st, 0, sizeof(*st));
  if (!ctx || !o || !coords_out) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_layout: null argument");
  if (ctx->n <= 0) return phde_fail(ctx, PHDE_ERR_NO_GRAPH, "phde_layout: no graph uploaded");
  if (o->algo < 0 || o->algo > 3) return phde_fail(ctx, PHDE_ERR_INVALID, "Unrecognized algorithm");
  if (o->strategy < 0 || o->strategy > 4) return phde_fail(ctx, PHDE_ERR_INVALID, "Unrecognized Strategy");
  if ((o->strategy == PHDE_STRAT_LEARNED || o->strategy == PHDE_STRAT_LEARNED_CHECKED) && o->algo != PHDE_ALGO_PARHDE)
    return phde_fail(ctx, PHDE_ERR_INVALID, "learned pivots are implemented for ParHDE");
  if (o->eig != PHDE_EIG_POWER && o->eig != PHDE_EIG_EXACT) return phde_fail(ctx, PHDE_ERR_INVALID, "unknown eigensolver");
  if (o->precision != PHDE_PREC_FP64 && o->precision != PHDE_PREC_MIXED && o->precision != PHDE_PREC_EXACT)
    return phde_fail(ctx, PHDE_ERR_INVALID, "unknown precision");
  if (o->k < 1 || o->k > PHDE_MAX_K || o->k >= ctx->n || o->c < 1 || o->c > o->k)
    return phde_fail(ctx, PHDE_ERR_K_RANGE, "need 1 <= k <= 256, k < n and 1 <= c <= k");
  if (o->algo == PHDE_ALGO_WPARHDE && !ctx->weighted)
    return phde_fail(ctx, PHDE_ERR_WEIGHTS, "Weighted ParHDE code requires the weighted edges");
  if (o->algo != PHDE_ALGO_WPARHDE && ctx->weighted)
    return phde_fail(ctx, PHDE_ERR_WEIGHTS, "ParHDE code doesn't requires the weighted edges");
  if (o->precision == PHDE_PREC_MIXED && o->algo != PHDE_ALGO_PARHDE)
    return phde_fail(ctx, PHDE_ERR_INVALID, "mixed precision is implemented for ParHDE; use PHDE_PREC_FP64");
  if (o->precision == PHDE_PREC_EXACT && o->algo != PHDE_ALGO_PARHDE)
    return phde_fail(ctx, PHDE_ERR_INVALID, "the exact-Gram path is implemented for ParHDE; use PHDE_PREC_FP64");
  cudaSetDevice(ctx->device);
  const bool learned = o->strategy == PHDE_STRAT_LEARNED || o->strategy == PHDE_STRAT_LEARNED_CHECKED;
  int rc = learned ? layout_learned(ctx, o, coords_out, sources_out, extra, st)
                   : layout_impl(ctx, o, coords_out, sources_out, extra, st);
  if (st) st->status = rc;
  if (rc != PHDE_OK) cudaStreamSynchronize(ctx->stream);
  return rc;
}

int phde_distances(phde_ctx *ctx, const int64_t *sources, int nsrc, int32_t *out) {
  if (!ctx || !sources || !out || nsrc < 1) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_distances: bad arguments");
  if (ctx->n <= 0) return phde_fail(ctx, PHDE_ERR_NO_GRAPH, "phde_distances: no graph uploaded");
  for (int i = 0; i < nsrc; i++)
    if (sources[i] < 0 || sources[i] >= ctx->n) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_distances: source out of range");
  cudaSetDevice(ctx->device);
  const int64_t n = ctx->n;
  int64_t *d_src = (int64_t *)phde_buf(ctx, "dist.src", sizeof(int64_t) * nsrc);
  int64_t *d_src2 = (int64_t *)phde_buf(ctx, "dist.src2", sizeof(int64_t) * nsrc);
  ull *sumsq = (ull *)phde_buf(ctx, "dist.sumsq", sizeof(ull) * nsrc);
  if (!d_src || !d_src2 || !sumsq) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemcpyAsync(d_src, sources, sizeof(int64_t) * nsrc, cudaMemcpyHostToDevice, ctx->stream));
  int rc;
  if (!ctx->weighted) {
    // sources in groups of 256: one bitset sweep per level for each group (single BFS passes below 4)
    const int G = std::min(nsrc, 256);
    int32_t *D = (int32_t *)phde_buf(ctx, "dist.D", sizeof(int32_t) * n * G);
    if (!D) return PHDE_ERR_OOM;
    for (int s0 = 0; s0 < nsrc; s0 += G) {
      const int ns = std::min(G, nsrc - s0);
      if (ns >= 4)
        rc = phde_msbfs(ctx, d_src + s0, ns, D, nullptr, nullptr);
      else
        rc = phde_run_bfs_passes(ctx, ns, 1, d_src + s0, D, d_src2, sumsq, nullptr, 0);
      if (rc) return rc;
      PHDE_CK(ctx, cudaMemcpyAsync(out + (int64_t)s0 * n, D, sizeof(int32_t) * n * ns, cudaMemcpyDeviceToHost,
                                   ctx->stream));
      if ((rc = phde_check_device_err(ctx, "BFS"))) return rc;
    }
    return PHDE_OK;
  }
  int32_t *col = (int32_t *)phde_buf(ctx, "dist.col", sizeof(int32_t) * n);
  if (!col) return PHDE_ERR_OOM;
  for (int i = 0; i < nsrc; i++) {
    if ((rc = phde_run_sssp(ctx, d_src + i, col, 10000, nullptr))) return rc;
    PHDE_CK(ctx, cudaMemcpyAsync(out + (int64_t)i * n, col, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if ((rc = phde_check_device_err(ctx, "SSSP"))) return rc;
  }
  return PHDE_OK;
}

int phde_kcenters(phde_ctx *ctx, int passes, int variant, int32_t *dist_out, int64_t *sources_out) {
  if (!ctx || passes < 1 || !sources_out || (variant != 0 && variant != 2))
    return phde_fail(ctx, PHDE_ERR_INVALID, "phde_kcenters: bad arguments");
  if (ctx->n <= 0) return phde_fail(ctx, PHDE_ERR_NO_GRAPH, "phde_kcenters: no graph uploaded");
  cudaSetDevice(ctx->device);
  const int64_t n = ctx->n;
  int64_t *d_src = (int64_t *)phde_buf(ctx, "kcx.src", sizeof(int64_t) * (passes + 2));
  ull *sumsq = (ull *)phde_buf(ctx, "kcx.sumsq", sizeof(ull) * passes);
  if (!d_src || !sumsq) return PHDE_ERR_OOM;
  int rc;
  if (!ctx->weighted) {
    int32_t *D = (int32_t *)phde_buf(ctx, "kcx.D", sizeof(int32_t) * n * passes);
    if (!D) return PHDE_ERR_OOM;
    if ((rc = phde_run_bfs_passes(ctx, passes, variant, nullptr, D, d_src, sumsq, nullptr, 1))) return rc;
    if (dist_out) PHDE_CK(ctx, cudaMemcpyAsync(dist_out, D, sizeof(int32_t) * n * passes, cudaMemcpyDeviceToHost, ctx->stream));
  } else {
    int32_t *col = (int32_t *)phde_buf(ctx, "kcx.col", sizeof(int32_t) * n);
    int32_t *min_d = (int32_t *)phde_buf(ctx, "kcx.min_d", sizeof(int32_t) * n);
    int64_t *hist = (int64_t *)phde_buf(ctx, "kcx.hist", sizeof(int64_t) * passes);
    int64_t *cur = (int64_t *)phde_buf(ctx, "kcx.cur", sizeof(int64_t) * 2);
    if (!col || !min_d || !hist || !cur) return PHDE_ERR_OOM;
    if ((rc = phde_fill_i32(ctx, min_d, n, 0x7fffffff))) return rc;
    PHDE_CK(ctx, cudaMemsetAsync(cur, 0, sizeof(int64_t) * 2, ctx->stream));
    PHDE_CK(ctx, cudaMemsetAsync(sumsq, 0, sizeof(ull) * passes, ctx->stream));
    for (int r = 0; r < passes; r++) {
      PHDE_CK(ctx, cudaMemcpyAsync(d_src + r, cur, sizeof(int64_t), cudaMemcpyDeviceToDevice, ctx->stream));
      if ((rc = phde_run_sssp(ctx, cur, col, 10000, nullptr))) return rc;
      if ((rc = phde_run_select(ctx, col, min_d, r, r != 0, hist, cur + 1, sumsq + r))) return rc;
      PHDE_CK(ctx, cudaMemcpyAsync(cur, cur + 1, sizeof(int64_t), cudaMemcpyDeviceToDevice, ctx->stream));
      if (dist_out)
        PHDE_CK(ctx, cudaMemcpyAsync(dist_out + (int64_t)r * n, col, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    }
  }
  PHDE_CK(ctx, cudaMemcpyAsync(sources_out, d_src, sizeof(int64_t) * passes, cudaMemcpyDeviceToHost, ctx->stream));
  return phde_check_device_err(ctx, "Kcenters");
}

// ---- reference-shaped distance drop-ins ----
static thread_local phde_ctx *g_default_ctx = nullptr;

static phde_ctx *default_ctx() {
  if (!g_default_ctx) {
    int dev = 0;
    if (const char *d = getenv("PHDE_DEVICE")) dev = atoi(d);
    if (phde_create(&g_default_ctx, dev) != PHDE_OK) g_default_ctx = nullptr;
  }
  return g_default_ctx;
}

int phde_DOBFS(const uint32_t *row, const uint32_t *col, long source, long numNodes, long numEdges, double *dists,
               int alpha, int beta) {
  (void)alpha;
  (void)beta;
  phde_ctx *ctx = default_ctx();
  if (!ctx) return PHDE_ERR_CUDA;
  if (!dists || source < 0 || source >= numNodes) return PHDE_ERR_INVALID;
  int rc = phde_graph_upload(ctx, row, 4, col, nullptr, numNodes, numEdges);
  if (rc) return rc;
  std::vector<int32_t> d((size_t)numNodes);
  int64_t s = source;
  if ((rc = phde_distances(ctx, &s, 1, d.data()))) return rc;
  for (long v = 0; v < numNodes; v++)
    if (d[v] >= 0) dists[v] = (double)d[v];  // unreached entries are left as they were (bfs.cc:144-185)
  return PHDE_OK;
}

int phde_DeltaStep(const uint32_t *row, const uint32_t *col, const int32_t *weights, long source, long numNodes,
                   long numEdges, double *dist, int32_t delta) {
  (void)delta;
  phde_ctx *ctx = default_ctx();
  if (!ctx) return PHDE_ERR_CUDA;
  if (!dist || !weights || source < 0 || source >= numNodes) return PHDE_ERR_INVALID;
  int rc = phde_graph_upload(ctx, row, 4, col, weights, numNodes, numEdges);
  if (rc) return rc;
  std::vector<int32_t> d((size_t)numNodes);
  int64_t s = source;
  if ((rc = phde_distances(ctx, &s, 1, d.data()))) return rc;
  for (long v = 0; v < numNodes; v++) dist[v] = (double)d[v];  // every entry, kDistInf when unreached (sssp.cc:137-139)
  return PHDE_OK;
}

int phde_pivot_scores(phde_ctx *ctx, float *scores, int32_t *warm_dist, int64_t *candidates, int ncand) {
  if (!ctx || ncand < 0 || ncand > PHDE_LEARNED_CANDIDATES) return phde_fail(ctx, PHDE_ERR_INVALID, "pivot scores: bad arguments");
  if (ctx->n <= 0) return phde_fail(ctx, PHDE_ERR_NO_GRAPH, "pivot scores: no graph uploaded");
  if (ctx->weighted) return phde_fail(ctx, PHDE_ERR_WEIGHTS, "learned pivots are implemented for unweighted graphs");
  cudaSetDevice(ctx->device);
  const int64_t n = ctx->n;
  const int P0 = (int)std::min<int64_t>(PHDE_LEARNED_WARM, n);
  int32_t *D = (int32_t *)phde_buf(ctx, "ps.D", sizeof(int32_t) * n * P0);
  int64_t *d_src = (int64_t *)phde_buf(ctx, "ps.src", sizeof(int64_t) * (P0 + 2));
  ull *sumsq = (ull *)phde_buf(ctx, "ps.sumsq", sizeof(ull) * P0);
  if (!D || !d_src || !sumsq) return PHDE_ERR_OOM;
  if (ctx->pivot_model.empty()) {
    const float *w0;
    int cnt;
    if (phde_default_pivot_model(&w0, &cnt)) return phde_fail(ctx, PHDE_ERR_INVALID, "built-in pivot model has the wrong size");
    ctx->pivot_model.assign(w0, w0 + cnt);
  }
  int rc = phde_run_bfs_passes(ctx, P0, 0, nullptr, D, d_src, sumsq, nullptr, 1);
  if (rc || (rc = phde_check_device_err(ctx, "pivot scores: warm start"))) return rc;
  const int32_t *mind0 = (const int32_t *)phde_buf(ctx, "kc.min_d", sizeof(int32_t) * n);
  if (!mind0) return PHDE_ERR_OOM;
  std::vector<int64_t> cand;
  std::vector<float> cscore;
  if ((rc = phde_pivot_candidates(ctx, ctx->pivot_model.data(), std::max(ncand, 1), mind0, cand, cscore))) return rc;
  const float *score = (const float *)phde_buf(ctx, "lp.score", sizeof(float) * n);
  if (!score) return PHDE_ERR_OOM;
  if (scores) PHDE_CK(ctx, cudaMemcpyAsync(scores, score, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
  if (warm_dist) PHDE_CK(ctx, cudaMemcpyAsync(warm_dist, mind0, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (candidates)
    for (int i = 0; i < ncand; i++) candidates[i] = i < (int)cand.size() ? cand[i] : -1;
  return PHDE_OK;
}

int phde_set_pivot_check(phde_ctx *ctx, int rule, double tolerance) {
  if (!ctx || (rule != PHDE_CHECK_SUM && rule != PHDE_CHECK_EACH) || !(tolerance >= 0.0 && tolerance < 10.0))
    return phde_fail(ctx, PHDE_ERR_INVALID, "pivot check: rule PHDE_CHECK_SUM or PHDE_CHECK_EACH, tolerance in [0, 10)");
  ctx->pivot_check_rule = rule;
  ctx->pivot_check_tol = tolerance;
  return PHDE_OK;
}

int phde_set_pivot_model(phde_ctx *ctx, const float *weights, int count) {
  const float *w0;
  int cnt = 0;
  phde_default_pivot_model(&w0, &cnt);
  if (!ctx || !weights || count != cnt) return phde_fail(ctx, PHDE_ERR_INVALID, "pivot model: wrong weight count");
  ctx->pivot_model.assign(weights, weights + count);
  return PHDE_OK;
}

int phde_selftest_barrier_timeout(phde_ctx *ctx, int timeout_ms) {
  if (!ctx || timeout_ms < 1 || timeout_ms > 10000) return PHDE_ERR_INVALID;
  cudaSetDevice(ctx->device);
  int rc = phde_reset_sync(ctx);
  if (rc) return rc;
  barrier_timeout_kernel<<<1, 32, 0, ctx->stream>>>(ctx->d_sync, ctx->d_err, (uint64_t)timeout_ms * 1000000ull);
  PHDE_LAUNCHED(ctx);
  int e = 0;
  PHDE_CK(ctx, cudaMemcpyAsync(&e, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  if ((rc = phde_reset_sync(ctx))) return rc;
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return e;
}

}  // extern "C"
