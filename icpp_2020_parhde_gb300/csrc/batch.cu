// batch.cu -- many independent graphs laid out by one call (phde_batch_upload, phde_layout_batched).
//
// The reference lays out one graph per DrawingBase::run(); a caller with many graphs loops.  Here the
// batch is uploaded as the disjoint union of its graphs (vertex ranges vbase[b]..vbase[b+1], graph id
// per vertex), and every stage runs for all graphs at once:
//   Kcenters      one persistent launch (kcenters.cu, batched variant): each pass is one BFS per graph,
//                 all graphs' sources in the same level-0 frontier (the components never meet, so every
//                 distance is the single-graph one), per-graph farthest-vertex keys and exact sums;
//   CGS2          the blocked CGS2 of bcgs.cu per graph, on "segments" -- row ranges of one graph, one
//                 CTA each -- so a CTA stages its graph's coefficients in shared memory, and per-segment
//                 partial Gram matrices are summed per graph in segment order (deterministic);
//   SpMM          the FP32 Laplacian SpMM of mixed.cu on the union (the union's Laplacian is
//                 block-diagonal);
//   Gram          S_b^T L S_b per graph from segment partials;
//   eigensolve    one shared-memory Jacobi CTA per graph (eigen.cu);
//   coordinates   X_b = S_b Y_b per segment, FP64 column norms per graph.
// Nothing between the Kcenters launch and the coordinate copy waits on the host, so after the first call
// the whole sequence is captured once into a CUDA graph and replayed.  The segment length (rows per CTA) is
// picked by a small autotuner: each candidate length is timed on the caller's own batch at the first call.
// Options outside that pipeline (FP64 or exact arithmetic, k above 32, the power iteration, the other
// algorithms) lay the graphs out one after another with the single-graph pipeline (layout_per_graph): each
// graph's CSR is cut out of the union on the device and laid out as if uploaded alone.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "bcgs_gs.cuh"
#include "ctx.h"

int phde_degrees(phde_ctx *ctx, double *deg);
int phde_lap_spmm_mixed(phde_ctx *ctx, const double *deg, const float *S, float *LS, int k);
int phde_eigensolve_batched(phde_ctx *ctx, const double *d_M, int N, int c, int count, double *d_K,
                            double *d_evals, double *d_Y, int *d_st);
int phde_run_bfs_batched_blocks(phde_ctx *ctx, int P, const int32_t *d_order, int32_t *d_D, int64_t *d_sources,
                                unsigned long long *d_sumsq, unsigned long long *d_edges);
int phde_batch_learned_pivots(phde_ctx *ctx, int P, const float *d_weights, int32_t *D, int64_t *sources,
                              unsigned long long *sumsq, unsigned long long *edges);
int phde_default_pivot_model(const float **w, int *count);

namespace {

constexpr int BB = 32;   // candidates per CGS2 block
constexpr int GT = 256;  // threads per segment CTA
constexpr int QCH = 64;  // Gram rows per segment partial
constexpr int RT = 32;   // rows per staged tile
constexpr int MAXC = 4;  // coordinates

// ---- upload: union CSR from the graphs' own arrays ----

__device__ __forceinline__ int upper_index(const int64_t *base, int B, int64_t x) {  // largest b with base[b] <= x
  int lo = 0, hi = B;  // base[0] = 0 <= x; answer in [lo, hi)
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (base[mid] <= x)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Offsets: graph b's n_b + 1 local offsets are staged at vbase[b] + b (uint32 or int64 per `wide`).
// Adjacency: staged in place; ids are shifted by the graph's vertex base.  Checks per graph: offsets
// start at 0, end at nnz_b, neighbours < n_b.  Graphs with no edges are skipped by the edge search
// (equal ebase entries).
__global__ void batch_union_kernel(const void *staged_off, int wide, const int64_t *vbase, const int64_t *ebase,
                                   int B, int64_t N, int64_t E, int64_t *off, uint32_t *adj, int32_t *gid, int *bad) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int fail = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < N; v += stride) {
    const int b = upper_index(vbase, B, v);
    const int64_t li = v - vbase[b], si = vbase[b] + b + li;
    const int64_t lo = wide ? ((const int64_t *)staged_off)[si] : (int64_t)((const uint32_t *)staged_off)[si];
    const int64_t hi = wide ? ((const int64_t *)staged_off)[si + 1] : (int64_t)((const uint32_t *)staged_off)[si + 1];
    off[v] = ebase[b] + lo;
    gid[v] = b;
    if (li == 0 && lo != 0) fail = 1;
    if (v + 1 == vbase[b + 1] && hi != ebase[b + 1] - ebase[b]) fail = 1;
    if (hi < lo) fail = 1;
  }
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride) {
    const int b = upper_index(ebase, B, e);
    const uint32_t u = adj[e];
    if ((int64_t)u >= vbase[b + 1] - vbase[b]) fail = 1;
    adj[e] = (uint32_t)(u + vbase[b]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) off[N] = E;
  if (fail) atomicExch(bad, 1);
}

// ---- CGS2 on segments ----

struct Seg {
  const int32_t *graph;  // [nseg]
  const int64_t *r0, *r1;
  const int *first;      // [B + 1]: segments of graph b are first[b] .. first[b+1]-1
  int nseg;
};

// 1 / ||D[:, p]|| per graph and pass (sumsq is [p * B + b]).
__global__ void batch_inv_norms_kernel(const ull *sumsq, int PB, float *inv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < PB; i += gridDim.x * blockDim.x)
    inv[i] = (float)(1.0 / sqrt((double)sumsq[i]));
}

// X[v][c] = D[(rc0 + c) * N + v] * inv[(rc0 + c) * B + g(v)]; columns >= bc are zero.
__global__ void batch_load_kernel(const int32_t *D, int64_t N, int B, int rc0, int bc, const float *inv,
                                  const int32_t *gid, float *X) {
  __shared__ float tile[BB][RT + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t r0 = (int64_t)blockIdx.x * RT; r0 < N; r0 += (int64_t)gridDim.x * RT) {
    __syncthreads();
    for (int c = warp; c < BB; c += nw) {
      const int64_t r = r0 + lane;
      float x = 0.f;
      if (c < bc && r < N) x = (float)D[(int64_t)(rc0 + c) * N + r] * inv[(int64_t)(rc0 + c) * B + gid[r]];
      tile[c][lane] = x;
    }
    __syncthreads();
    for (int rr = warp; rr < RT; rr += nw)
      if (r0 + rr < N) X[(r0 + rr) * BB + lane] = tile[lane][rr];
  }
}

// Per-segment partial Gram: part[s][qq][i] = sum_{v in segment} A[v][q] * w[v] * Bm[v][i], q < nq (+ a ones
// row at q == nq when `ones`), i < nb.  nq is the graph's accepted count (jcount[b], proj mode) or fixed.
__global__ void __launch_bounds__(GT) batch_gram_kernel(Seg sg, const float *A, int lda, const int *jcount, int nq_fixed,
                                                        int ones, const float *Bm, int ldb, int nb, const double *w,
                                                        float *part) {
  __shared__ __align__(16) float At[RT][QCH];
  __shared__ float Xt[RT][BB];
  const int s = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int b = sg.graph[s];
  const int nq = jcount ? jcount[4 * b] : nq_fixed;
  const int64_t rb = sg.r0[s], re = sg.r1[s];
  float acc[8];
#pragma unroll
  for (int m = 0; m < 8; m++) acc[m] = 0.f;
  // staging as in bcgs.cu: one column per thread, the next tile prefetched into registers
  const int q = threadIdx.x % QCH, r1 = threadIdx.x / QCH;
  const float cst = (q == nq && ones) ? 1.f : 0.f;
  const int xi = threadIdx.x % BB, r2 = threadIdx.x / BB;
  constexpr int NA = RT / (GT / QCH), NX = RT / (GT / BB);
  float pa[NA], px[NX];
  auto fetch = [&](int64_t r0) {
#pragma unroll
    for (int t = 0; t < NA; t++) {
      const int64_t row = r0 + r1 + t * (GT / QCH);
      pa[t] = row < re ? (q < nq ? A[row * lda + q] : cst) : 0.f;
    }
#pragma unroll
    for (int t = 0; t < NX; t++) {
      const int64_t row = r0 + r2 + t * (GT / BB);
      px[t] = (row < re && xi < nb) ? Bm[row * ldb + xi] * (w ? (float)w[row] : 1.f) : 0.f;
    }
  };
  if (rb < re) fetch(rb);
  for (int64_t r0 = rb; r0 < re; r0 += RT) {
    __syncthreads();
#pragma unroll
    for (int t = 0; t < NA; t++) At[r1 + t * (GT / QCH)][q] = pa[t];
#pragma unroll
    for (int t = 0; t < NX; t++) Xt[r2 + t * (GT / BB)][xi] = px[t];
    __syncthreads();
    if (r0 + RT < re) fetch(r0 + RT);
#pragma unroll 4
    for (int rr = 0; rr < RT; rr++) {
      const float x = Xt[rr][lane];
      const float4 a0 = *(const float4 *)&At[rr][warp * 8];
      const float4 a1 = *(const float4 *)&At[rr][warp * 8 + 4];
      acc[0] = fmaf(a0.x, x, acc[0]);
      acc[1] = fmaf(a0.y, x, acc[1]);
      acc[2] = fmaf(a0.z, x, acc[2]);
      acc[3] = fmaf(a0.w, x, acc[3]);
      acc[4] = fmaf(a1.x, x, acc[4]);
      acc[5] = fmaf(a1.y, x, acc[5]);
      acc[6] = fmaf(a1.z, x, acc[6]);
      acc[7] = fmaf(a1.w, x, acc[7]);
    }
  }
  float *dst = part + ((int64_t)s * QCH + warp * 8) * BB + lane;
#pragma unroll
  for (int m = 0; m < 8; m++) dst[m * BB] = acc[m];
}

// Sum a graph's segment partials (segment order) for Gram row q = blockIdx.y of graph b = blockIdx.x.
//   mode 0: projection coefficients C[b][q][i] (FP32): sum / <q, D q> for q < j_b, sum / nnz_b for q == j_b;
//   mode 1: block Gram G[b][member][q][i] (FP64, 32 x 32; G points at the member);
//   mode 2: the k x k matrix M[b][q + i*k] (FP64, column-major), q, i < k.
__global__ void batch_reduce_kernel(Seg sg, const float *part, int mode, const int *jcount, const double *dden, int k,
                                    const int64_t *ebase, float *C, double *G) {
  const int b = blockIdx.x, q = blockIdx.y, i = threadIdx.x;
  const int nq = mode == 0 ? jcount[4 * b] : (mode == 1 ? BB : k);
  if (q > nq || (mode != 0 && q == nq)) return;
  double t = 0;
  for (int s = sg.first[b]; s < sg.first[b + 1]; s++) t += (double)part[((int64_t)s * QCH + q) * BB + i];
  if (mode == 0)
    C[((int64_t)b * QCH + q) * BB + i] = (float)(q < nq ? t / dden[(int64_t)b * (k + 1) + q]
                                                         : t / (double)(ebase[b + 1] - ebase[b]));
  else if (mode == 1)  // graph b's pair [Gd, G2] at b * 2 * 32 * 32; the caller offsets G by the pair member
    G[((int64_t)b * 2 * BB + q) * BB + i] = t;
  else if (i < k)
    G[(int64_t)b * k * k + q + (int64_t)i * k] = t;
}

// X[v][i] -= sum_{q < j_b} S[v][q] C_b[q][i] + C_b[j_b][i] over the segment's rows (warp per row).
__global__ void __launch_bounds__(GT) batch_update_kernel(Seg sg, const float *S, int lda, const int *jcount,
                                                          const float *C, float *X) {
  __shared__ float Cs[QCH][BB];
  const int s = blockIdx.x, b = sg.graph[s];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int nq = jcount[4 * b];
  for (int idx = threadIdx.x; idx < (nq + 1) * BB; idx += GT) Cs[idx / BB][idx % BB] = C[(int64_t)b * QCH * BB + idx];
  __syncthreads();
  for (int64_t v = sg.r0[s] + warp; v < sg.r1[s]; v += nw) {
    float p = Cs[nq][lane];
    for (int q = 0; q < nq; q++) p = fmaf(S[v * lda + q], Cs[q][lane], p);
    X[v * BB + lane] -= p;
  }
}

// Per graph (one CTA of four warps each): the accept/discard loop of bcgs_gs.cuh.
// st[4b..]: [0] accepted so far, [1] discarded, [2] candidates consumed, [3] accepted in this block.
__global__ void __launch_bounds__(bcgs_gs::NW * 32) batch_block_gs_kernel(const double *Gall, int bc, int k, int rc0,
                                                                          int P, int *stall, double *dlog,
                                                                          float *Rall) {
  __shared__ bcgs_gs::Smem S;
  __shared__ int res[3];
  const int b = blockIdx.x;
  const double *Gd = Gall + (int64_t)b * 2 * BB * BB, *G2 = Gd + BB * BB;
  int *st = stall + 4 * b;
  const int j0 = st[0];
  bcgs_gs::run(S, Gd, G2, bc, k, j0, dlog + (int64_t)b * P + rc0, Rall + (int64_t)b * BB * BB, res, res + 1, res + 2);
  __syncthreads();
  if (threadIdx.x == 0) {
    st[0] = j0 + res[0];
    st[1] += res[1];
    st[2] += res[2];
    st[3] = res[0];
  }
}

// S[v][j0_b + a] = sum_i X[v][i] R_b[i][a], a < nacc_b, with per-segment sums of deg * S^2 per column.
__global__ void __launch_bounds__(GT) batch_form_kernel(Seg sg, const float *X, const float *Rall, const int *stall,
                                                        float *S, int lda, const double *deg, double *fpart) {
  __shared__ float Rs[BB][BB + 1];
  __shared__ double red[GT / 32][BB];
  const int s = blockIdx.x, b = sg.graph[s];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int nacc = stall[4 * b + 3], j0 = stall[4 * b] - nacc;
  for (int idx = threadIdx.x; idx < BB * BB; idx += GT) Rs[idx / BB][idx % BB] = Rall[(int64_t)b * BB * BB + idx];
  __syncthreads();
  double dsum = 0;
  if (nacc > 0)
    for (int64_t v = sg.r0[s] + warp; v < sg.r1[s]; v += nw) {
      const float x = X[v * BB + lane];
      float val = 0.f;
#pragma unroll 8
      for (int i = 0; i < BB; i++) val = fmaf(__shfl_sync(PHDE_FULL_MASK, x, i), Rs[i][lane], val);
      if (lane < nacc) {
        S[v * lda + j0 + lane] = val;
        dsum += (double)val * (double)val * deg[v];
      }
    }
  red[warp][lane] = dsum;
  __syncthreads();
  if (warp == 0) {
    double t = 0;
    for (int w = 0; w < nw; w++) t += red[w][lane];
    fpart[(int64_t)s * BB + lane] = t;
  }
}

// <q, D q> of graph b's new columns, from its segments' partials in order.
__global__ void batch_dd_kernel(Seg sg, const double *fpart, const int *stall, int k, double *dden) {
  const int b = blockIdx.x, a = threadIdx.x;
  const int nacc = stall[4 * b + 3], j0 = stall[4 * b] - nacc;
  if (a >= nacc) return;
  double t = 0;
  for (int s = sg.first[b]; s < sg.first[b + 1]; s++) t += fpart[(int64_t)s * BB + a];
  dden[(int64_t)b * (k + 1) + j0 + a] = t;
}

// Coordinates of a segment's rows: X_b = S_b Y_b (FP32 products and row sums), written column-major per
// graph at out + c * vbase[b]; per-segment sums of squares per coordinate.
__global__ void __launch_bounds__(GT) batch_coords_kernel(Seg sg, const float *S, int k, const double *Yall, int c,
                                                          const int64_t *vbase, double *out, double *cpart) {
  __shared__ float Ys[BB * MAXC];
  __shared__ double red[GT / 32][MAXC];
  const int s = blockIdx.x, b = sg.graph[s];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const double *Y = Yall + (int64_t)b * k * c;  // column-major k x c
  for (int idx = threadIdx.x; idx < k * c; idx += GT) Ys[(idx % k) * c + idx / k] = (float)Y[idx];
  __syncthreads();
  const int64_t vb = vbase[b], nb = vbase[b + 1] - vb;
  double ss[MAXC] = {0, 0, 0, 0};
  for (int64_t v = sg.r0[s] + warp; v < sg.r1[s]; v += nw) {
    float acc[MAXC] = {0.f, 0.f, 0.f, 0.f};
    if (lane < k) {
      const float sv = S[v * k + lane];
#pragma unroll
      for (int t = 0; t < MAXC; t++)
        if (t < c) acc[t] = sv * Ys[lane * c + t];
    }
#pragma unroll
    for (int t = 0; t < MAXC; t++) {
      if (t >= c) break;
      const float x = warp_sum(acc[t]);
      if (lane == 0) {
        out[c * vb + (int64_t)t * nb + (v - vb)] = (double)x;
        ss[t] = fma((double)x, (double)x, ss[t]);
      }
    }
  }
  if (lane == 0)
    for (int t = 0; t < MAXC; t++) red[warp][t] = ss[t];
  __syncthreads();
  if (threadIdx.x < MAXC) {
    double t = 0;
    for (int w = 0; w < nw; w++) t += red[w][threadIdx.x];
    cpart[(int64_t)s * MAXC + threadIdx.x] = t;
  }
}

// Unit-norm columns per graph: inv[b][t] from the graph's segment sums, then every row scaled.
__global__ void batch_norms_kernel(Seg sg, const double *cpart, int c, int B, double *inv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B * c; i += gridDim.x * blockDim.x) {
    const int b = i / c, t = i % c;
    double tot = 0;
    for (int s = sg.first[b]; s < sg.first[b + 1]; s++) tot += cpart[(int64_t)s * MAXC + t];
    inv[i] = 1.0 / sqrt(tot);
  }
}
// Rayleigh quotient of every graph's coordinates: y^T M_b y over ||X_b y||^2 = 1 / inv^2 (one warp per graph).
__global__ void batch_rq_kernel(const double *M, const double *Y, const double *inv, int k, int c, double *rq) {
  const int b = blockIdx.x, lane = threadIdx.x;
  const double *Mb = M + (int64_t)b * k * k, *Yb = Y + (int64_t)b * k * c;
  for (int t = 0; t < c; t++) {
    double s = 0;
    for (int p = lane; p < k; p += 32) {
      double u = 0;
      for (int q = 0; q < k; q++) u = fma(Mb[p + q * k], Yb[q + t * k], u);
      s = fma(Yb[p + t * k], u, s);
    }
    s = warp_sum(s);
    const double iv = inv[(int64_t)b * c + t];
    if (lane == 0) rq[(int64_t)b * c + t] = s * iv * iv;
  }
}

__global__ void batch_scale_kernel(const int32_t *gid, const int64_t *vbase, int64_t N, int c, const double *inv,
                                   double *out) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < N; v += (int64_t)gridDim.x * blockDim.x) {
    const int b = gid[v];
    const int64_t vb = vbase[b], nb = vbase[b + 1] - vb;
    for (int t = 0; t < c; t++) out[c * vb + (int64_t)t * nb + (v - vb)] *= inv[(int64_t)b * c + t];
  }
}

int grid_rows(phde_ctx *ctx, int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->nsm * 8));
}

}  // namespace

// ------------------------------------------------------------------------------------------------
extern "C" int phde_batch_upload(phde_ctx *ctx, const phde_graph_desc *graphs, int count) {
  if (!ctx) return PHDE_ERR_INVALID;
  if (!graphs || count < 1) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_batch_upload: bad arguments");
  const int wide = graphs[0].offset_bytes == 8;
  std::vector<int64_t> vb(count + 1, 0), eb(count + 1, 0);
  for (int b = 0; b < count; b++) {
    const phde_graph_desc &g = graphs[b];
    if (!g.offsets || g.n <= 0 || g.nnz < 0 || (!g.adj && g.nnz > 0) || (g.offset_bytes != 4 && g.offset_bytes != 8) ||
        (g.offset_bytes == 8) != (wide != 0))
      return phde_fail(ctx, PHDE_ERR_INVALID,
                       "phde_batch_upload: graph " + std::to_string(b) + ": bad arguments (offset widths must agree)");
    vb[b + 1] = vb[b] + g.n;
    eb[b + 1] = eb[b] + g.nnz;
  }
  const int64_t N = vb[count], E = eb[count];
  if (N >= 0xffffffffll || E >= 0xffffffffll)
    return phde_fail(ctx, PHDE_ERR_INVALID, "phde_batch_upload: the batch must hold fewer than 2^32 vertices and entries");
  PHDE_CK(ctx, cudaSetDevice(ctx->device));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  // device CSR of the union (grow-only, as phde_graph_upload)
  if (N + 1 > ctx->off_cap || !ctx->d_off) {
    cudaFree(ctx->d_off);
    ctx->d_off = nullptr;
    ctx->off_cap = 0;
    PHDE_CK(ctx, cudaMalloc(&ctx->d_off, sizeof(int64_t) * (N + 1)));
    ctx->off_cap = N + 1;
  }
  if (E > ctx->adj_cap || !ctx->d_adj) {
    cudaFree(ctx->d_adj);
    ctx->d_adj = nullptr;
    ctx->adj_cap = 0;
    PHDE_CK(ctx, cudaMalloc(&ctx->d_adj, sizeof(uint32_t) * std::max<int64_t>(E, 1)));
    ctx->adj_cap = std::max<int64_t>(E, 1);
    cudaFree(ctx->d_w);
    ctx->d_w = nullptr;
  }
  if (N > ctx->gid_cap || !ctx->d_gid) {
    cudaFree(ctx->d_gid);
    ctx->d_gid = nullptr;
    ctx->gid_cap = 0;
    PHDE_CK(ctx, cudaMalloc(&ctx->d_gid, sizeof(int32_t) * N));
    ctx->gid_cap = N;
  }
  cudaFree(ctx->d_vbase);
  ctx->d_vbase = nullptr;
  PHDE_CK(ctx, cudaMalloc(&ctx->d_vbase, sizeof(int64_t) * 2 * (count + 1)));
  const size_t ow = wide ? 8 : 4;
  unsigned char *staged = (unsigned char *)phde_buf(ctx, "batch.staged_off", ow * (size_t)(N + count));
  int *bad = (int *)phde_buf(ctx, "upload.bad", sizeof(int));
  if (!staged || !bad) return PHDE_ERR_OOM;
  for (int b = 0; b < count; b++) {
    PHDE_CK(ctx, cudaMemcpyAsync(staged + ow * (size_t)(vb[b] + b), graphs[b].offsets, ow * (size_t)(graphs[b].n + 1),
                                 cudaMemcpyHostToDevice, ctx->stream));
    if (graphs[b].nnz > 0)
      PHDE_CK(ctx, cudaMemcpyAsync(ctx->d_adj + eb[b], graphs[b].adj, sizeof(uint32_t) * graphs[b].nnz,
                                   cudaMemcpyHostToDevice, ctx->stream));
  }
  int64_t *d_eb = ctx->d_vbase + (count + 1);
  PHDE_CK(ctx, cudaMemcpyAsync(ctx->d_vbase, vb.data(), sizeof(int64_t) * (count + 1), cudaMemcpyHostToDevice, ctx->stream));
  PHDE_CK(ctx, cudaMemcpyAsync(d_eb, eb.data(), sizeof(int64_t) * (count + 1), cudaMemcpyHostToDevice, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
  batch_union_kernel<<<grid_rows(ctx, std::max(N, E)), 256, 0, ctx->stream>>>(staged, wide, ctx->d_vbase, d_eb, count, N,
                                                                               E, ctx->d_off, ctx->d_adj, ctx->d_gid, bad);
  PHDE_LAUNCHED(ctx);
  int h = 0;
  PHDE_CK(ctx, cudaMemcpyAsync(&h, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->n = N;
  ctx->nnz = E;
  ctx->weighted = false;
  ctx->graph_epoch++;
  if (h) {
    ctx->n = ctx->nnz = 0;
    ctx->batch_B = 0;
    return phde_fail(ctx, PHDE_ERR_CSR, "phde_batch_upload: a graph's offsets must start at 0, never decrease and end "
                                        "at its nnz; its neighbours must be below its n");
  }
  ctx->batch_B = count;
  ctx->batch_warm_key = -1;  // a new batch: its buffers are sized anew before any capture
  ctx->batch_last_c = 0;
  ctx->batch_vbase = vb;
  ctx->batch_ebase = eb;
  // graphs largest first (the one-CTA-per-graph Kcenters takes them in this order)
  std::vector<int32_t> order(count);
  for (int b = 0; b < count; b++) order[b] = b;
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t x, int32_t y) { return vb[x + 1] - vb[x] > vb[y + 1] - vb[y]; });
  cudaFree(ctx->d_order);
  ctx->d_order = nullptr;
  PHDE_CK(ctx, cudaMalloc(&ctx->d_order, sizeof(int32_t) * count));
  PHDE_CK(ctx, cudaMemcpy(ctx->d_order, order.data(), sizeof(int32_t) * count, cudaMemcpyHostToDevice));
  const char *mode = getenv("PHDE_BATCH_BFS");
  ctx->batch_blocks = mode ? std::string(mode) == "blocks" : count >= ctx->nsm / 2;
  return PHDE_OK;
}

namespace {

// Everything from the Kcenters launch to the coordinate copy, with no host synchronisation (so that it
// can be captured into a CUDA graph).  Buffers are allocated by the caller beforehand.
struct BatchBufs {
  double *deg;
  int32_t *D;
  int64_t *src;
  ull *sumsq;
  ull *edges;
  float *inv, *X, *part, *C, *R, *S, *LS;
  double *G, *dden, *fpart, *M, *K, *ev, *Y, *cpart, *cinv, *out;
  int *st, *est;
  double *dlog;
  double *rq;              // [B][c] Rayleigh quotients
  bool learned = false;    // learned pivots (batch_learned.cu) instead of Kcenters
  const float *weights = nullptr;  // the pivot model on the device
  Seg sg;
};

int batch_pipeline(phde_ctx *ctx, const BatchBufs &q, int k, int c) {
  const int B = ctx->batch_B, P = 3 * k;
  const int64_t N = ctx->n;
  int rc;
  const int64_t *d_eb = ctx->d_vbase + (B + 1);
  if ((rc = phde_degrees(ctx, q.deg))) return rc;
  // Kcenters: one CTA per graph when the batch has enough graphs to fill the GPU (block barriers only),
  // else the whole-grid batched variant (every pass one BFS of the union)
  if (q.learned)
    rc = phde_batch_learned_pivots(ctx, P, q.weights, q.D, q.src, q.sumsq, q.edges);
  else if (ctx->batch_blocks)
    rc = phde_run_bfs_batched_blocks(ctx, P, ctx->d_order, q.D, q.src, q.sumsq, q.edges);
  else
    rc = phde_run_bfs_passes(ctx, P, 3, nullptr, q.D, q.src, q.sumsq, q.edges, 1);
  if (rc) return rc;
  batch_inv_norms_kernel<<<(P * B + 255) / 256, 256, 0, ctx->stream>>>(q.sumsq, P * B, q.inv);
  PHDE_LAUNCHED(ctx);
  PHDE_CK(ctx, cudaMemsetAsync(q.st, 0, sizeof(int) * 4 * B, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(q.dlog, 0xff, sizeof(double) * (size_t)P * B, ctx->stream));
  const int ns = q.sg.nseg;
  for (int rc0 = 0; rc0 < P; rc0 += BB) {
    const int bc = std::min(BB, P - rc0);
    batch_load_kernel<<<grid_rows(ctx, N), GT, 0, ctx->stream>>>(q.D, N, B, rc0, bc, q.inv, ctx->d_gid, q.X);
    PHDE_LAUNCHED(ctx);
    for (int pass = 0; pass < 2; pass++) {
      batch_gram_kernel<<<ns, GT, 0, ctx->stream>>>(q.sg, q.S, k, q.st, 0, 1, q.X, BB, BB, q.deg, q.part);
      PHDE_LAUNCHED(ctx);
      batch_reduce_kernel<<<dim3(B, k + 1), BB, 0, ctx->stream>>>(q.sg, q.part, 0, q.st, q.dden, k, d_eb, q.C, nullptr);
      PHDE_LAUNCHED(ctx);
      batch_update_kernel<<<ns, GT, 0, ctx->stream>>>(q.sg, q.S, k, q.st, q.C, q.X);
      PHDE_LAUNCHED(ctx);
    }
    for (int wsel = 0; wsel < 2; wsel++) {
      batch_gram_kernel<<<ns, GT, 0, ctx->stream>>>(q.sg, q.X, BB, nullptr, BB, 0, q.X, BB, BB,
                                                    wsel == 0 ? q.deg : nullptr, q.part);
      PHDE_LAUNCHED(ctx);
      // block Gram of graph b goes to G[b][wsel] (2 x 32 x 32 per graph)
      batch_reduce_kernel<<<dim3(B, BB), BB, 0, ctx->stream>>>(q.sg, q.part, 1, q.st, nullptr, k, d_eb, nullptr,
                                                               q.G + wsel * BB * BB);
      PHDE_LAUNCHED(ctx);
    }
    batch_block_gs_kernel<<<B, bcgs_gs::NW * 32, 0, ctx->stream>>>(q.G, bc, k, rc0, P, q.st, q.dlog, q.R);
    PHDE_LAUNCHED(ctx);
    batch_form_kernel<<<ns, GT, 0, ctx->stream>>>(q.sg, q.X, q.R, q.st, q.S, k, q.deg, q.fpart);
    PHDE_LAUNCHED(ctx);
    batch_dd_kernel<<<B, BB, 0, ctx->stream>>>(q.sg, q.fpart, q.st, k, q.dden);
    PHDE_LAUNCHED(ctx);
  }
  if ((rc = phde_lap_spmm_mixed(ctx, q.deg, q.S, q.LS, k))) return rc;
  batch_gram_kernel<<<ns, GT, 0, ctx->stream>>>(q.sg, q.S, k, nullptr, k, 0, q.LS, k, k, nullptr, q.part);
  PHDE_LAUNCHED(ctx);
  batch_reduce_kernel<<<dim3(B, k), BB, 0, ctx->stream>>>(q.sg, q.part, 2, q.st, nullptr, k, d_eb, nullptr, q.M);
  PHDE_LAUNCHED(ctx);
  if ((rc = phde_eigensolve_batched(ctx, q.M, k, c, B, q.K, q.ev, q.Y, q.est))) return rc;
  batch_coords_kernel<<<ns, GT, 0, ctx->stream>>>(q.sg, q.S, k, q.Y, c, ctx->d_vbase, q.out, q.cpart);
  PHDE_LAUNCHED(ctx);
  batch_norms_kernel<<<(B * c + 255) / 256, 256, 0, ctx->stream>>>(q.sg, q.cpart, c, B, q.cinv);
  PHDE_LAUNCHED(ctx);
  batch_rq_kernel<<<B, 32, 0, ctx->stream>>>(q.M, q.Y, q.cinv, k, c, q.rq);
  PHDE_LAUNCHED(ctx);
  batch_scale_kernel<<<grid_rows(ctx, N), 256, 0, ctx->stream>>>(ctx->d_gid, ctx->d_vbase, N, c, q.cinv, q.out);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

// Segments of at most `seg_rows` rows, none crossing a graph boundary.
void build_segments(const std::vector<int64_t> &vb, int64_t seg_rows, std::vector<int32_t> &g, std::vector<int64_t> &r0,
                    std::vector<int64_t> &r1, std::vector<int> &first) {
  const int B = (int)vb.size() - 1;
  g.clear();
  r0.clear();
  r1.clear();
  first.assign(B + 1, 0);
  for (int b = 0; b < B; b++) {
    first[b] = (int)g.size();
    for (int64_t v = vb[b]; v < vb[b + 1]; v += seg_rows) {
      g.push_back(b);
      r0.push_back(v);
      r1.push_back(std::min(vb[b + 1], v + seg_rows));
    }
  }
  first[B] = (int)g.size();
}

}  // namespace

namespace {

// Graph b's CSR cut out of the union with local vertex ids: off_b[i] = off[v0 + i] - off[v0], adj_b[e] =
// adj[e0 + e] - v0.
__global__ void batch_extract_kernel(const int64_t *off, const uint32_t *adj, int64_t v0, int64_t nb, int64_t e0,
                                     int64_t mb, int64_t *off_b, uint32_t *adj_b) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= nb; i += stride) off_b[i] = off[v0 + i] - e0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < mb; e += stride)
    adj_b[e] = adj[e0 + e] - (uint32_t)v0;
}

// The context's view of the uploaded union, put back when a per-graph layout returns (also on errors).
struct UnionView {
  phde_ctx *ctx;
  int64_t *off;
  uint32_t *adj;
  int32_t *w;
  int64_t n, nnz;
  int B;
  bool weighted, want_rq;
  explicit UnionView(phde_ctx *c)
      : ctx(c), off(c->d_off), adj(c->d_adj), w(c->d_w), n(c->n), nnz(c->nnz), B(c->batch_B),
        weighted(c->weighted), want_rq(c->want_rq) {}
  ~UnionView() {
    ctx->d_off = off;
    ctx->d_adj = adj;
    ctx->d_w = w;
    ctx->n = n;
    ctx->nnz = nnz;
    ctx->batch_B = B;
    ctx->weighted = weighted;
    ctx->want_rq = want_rq;
    ctx->graph_epoch++;  // a value no cache holds: every per-graph plan is rebuilt for the union
  }
};

// Every graph of the batch through phde_layout in turn (options the fused pipeline does not cover).  The
// coordinates land where phde_layout_batched puts them; the Rayleigh quotients of each graph's coordinates
// (phde_batch_rayleigh) come from its layout; the stats add up the graphs' times, passes and launches.
int layout_per_graph(phde_ctx *ctx, const phde_layout_opts *o, double *coords_out, phde_layout_stats *stats) {
  const int B = ctx->batch_B, c = o->c;
  int64_t nmax = 0, mmax = 0;
  for (int b = 0; b < B; b++) {
    nmax = std::max(nmax, ctx->batch_vbase[b + 1] - ctx->batch_vbase[b]);
    mmax = std::max(mmax, ctx->batch_ebase[b + 1] - ctx->batch_ebase[b]);
  }
  int64_t *off_b = (int64_t *)phde_buf(ctx, "pg.off", sizeof(int64_t) * (nmax + 1));
  uint32_t *adj_b = (uint32_t *)phde_buf(ctx, "pg.adj", sizeof(uint32_t) * std::max<int64_t>(mmax, 1));
  double *rq = (double *)phde_buf(ctx, "batch.rq", sizeof(double) * (size_t)B * c);
  if (!off_b || !adj_b || !rq) return PHDE_ERR_OOM;
  std::vector<double> h_rq((size_t)B * c, 0.0);
  phde_layout_stats sum;
  memset(&sum, 0, sizeof(sum));
  const int64_t launches0 = ctx->launches;
  {
    UnionView keep(ctx);
    for (int b = 0; b < B; b++) {
      const int64_t v0 = ctx->batch_vbase[b], nb = ctx->batch_vbase[b + 1] - v0;
      const int64_t e0 = ctx->batch_ebase[b], mb = ctx->batch_ebase[b + 1] - e0;
      const int g = (int)std::max<int64_t>(1, std::min<int64_t>((std::max(nb + 1, mb) + 255) / 256, (int64_t)ctx->nsm * 8));
      batch_extract_kernel<<<g, 256, 0, ctx->stream>>>(keep.off, keep.adj, v0, nb, e0, mb, off_b, adj_b);
      PHDE_LAUNCHED(ctx);
      ctx->d_off = off_b;
      ctx->d_adj = adj_b;
      ctx->d_w = nullptr;
      ctx->weighted = false;
      ctx->n = nb;
      ctx->nnz = mb;
      ctx->batch_B = 0;
      ctx->want_rq = true;
      ctx->graph_epoch++;  // the graph's own plans
      phde_layout_stats sb;
      const int rc = phde_layout(ctx, o, coords_out + (int64_t)c * v0, nullptr, nullptr, &sb);
      if (rc) return phde_fail(ctx, rc, "phde_layout_batched: graph " + std::to_string(b) + ": " + ctx->err);
      for (int j = 0; j < c && j < PHDE_RQ_MAX; j++) h_rq[(size_t)b * c + j] = sb.rayleigh[j];
      sum.npasses = std::max(sum.npasses, sb.npasses);
      sum.naccepted = b == 0 ? sb.naccepted : std::min(sum.naccepted, sb.naccepted);
      sum.ndiscarded += sb.ndiscarded;
      sum.eig_iters = std::max(sum.eig_iters, sb.eig_iters);
      sum.ms_dist += sb.ms_dist;
      sum.ms_orth += sb.ms_orth;
      sum.ms_mmult += sb.ms_mmult;
      sum.ms_eig += sb.ms_eig;
      sum.ms_coords += sb.ms_coords;
      sum.ms_total += sb.ms_total;
      sum.edges_examined += sb.edges_examined;
    }
  }
  PHDE_CK(ctx, cudaMemcpyAsync(rq, h_rq.data(), sizeof(double) * h_rq.size(), cudaMemcpyHostToDevice, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->batch_last_c = c;
  if (stats) {
    *stats = sum;
    stats->status = PHDE_OK;
    stats->gpu_launches = (int)(ctx->launches - launches0);
  }
  return PHDE_OK;
}

}  // namespace

extern "C" int phde_layout_batched(phde_ctx *ctx, const phde_layout_opts *o, double *coords_out,
                                   phde_layout_stats *stats) {
  if (!ctx) return PHDE_ERR_INVALID;
  if (!o || !coords_out) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_layout_batched: bad arguments");
  if (ctx->batch_B < 1) return phde_fail(ctx, PHDE_ERR_NO_GRAPH, "phde_layout_batched: no batch uploaded");
  const bool learned = o->strategy == PHDE_STRAT_LEARNED;
  const int k = o->k, c = o->c, B = ctx->batch_B, P = 3 * k;
  // the fused pipeline: ParHDE, Kcenters or learned pivots, mixed precision, Jacobi, k <= 32, c <= 4
  const bool fused = o->algo == PHDE_ALGO_PARHDE && (o->strategy == PHDE_STRAT_KCENTERS || learned) &&
                     o->precision == PHDE_PREC_MIXED && o->eig == PHDE_EIG_EXACT && k <= BB && c <= MAXC;
  if (k < 2 || c < 1 || c > k) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_layout_batched: need 2 <= k and 1 <= c <= k");
  for (int b = 0; b < B; b++)
    if (ctx->batch_vbase[b + 1] - ctx->batch_vbase[b] <= P)
      return phde_fail(ctx, PHDE_ERR_K_RANGE,
                       "phde_layout_batched: graph " + std::to_string(b) + " has no more vertices than 3k pivots");
  if (!fused) {
    PHDE_CK(ctx, cudaSetDevice(ctx->device));
    return layout_per_graph(ctx, o, coords_out, stats);
  }
  for (int b = 0; b < B; b++) {
    if (learned && ctx->batch_vbase[b + 1] - ctx->batch_vbase[b] <= PHDE_LEARNED_CANDIDATES)
      return phde_fail(ctx, PHDE_ERR_K_RANGE,
                       "phde_layout_batched: learned pivots need more than 256 vertices per graph (graph " +
                           std::to_string(b) + ")");
  }
  PHDE_CK(ctx, cudaSetDevice(ctx->device));
  const int64_t N = ctx->n;
  ctx->kernel_ms = 0;
  ctx->kernel_launches = 0;
  ctx->kev_pending = false;
  BatchBufs q;
  q.deg = (double *)phde_buf(ctx, "layout.deg", sizeof(double) * N);
  q.D = (int32_t *)phde_buf(ctx, "layout.D", sizeof(int32_t) * N * P);
  q.src = (int64_t *)phde_buf(ctx, "batch.src", sizeof(int64_t) * P * B);
  q.sumsq = (ull *)phde_buf(ctx, "batch.sumsq", sizeof(ull) * P * B);
  q.edges = (ull *)phde_buf(ctx, "layout.edges", sizeof(ull));
  q.inv = (float *)phde_buf(ctx, "batch.inv", sizeof(float) * P * B);
  q.X = (float *)phde_buf(ctx, "bcgs.X", sizeof(float) * N * BB);
  q.S = (float *)phde_buf(ctx, "layout.S32", sizeof(float) * N * k);
  q.LS = (float *)phde_buf(ctx, "layout.LS32", sizeof(float) * N * k);
  q.C = (float *)phde_buf(ctx, "batch.C", sizeof(float) * B * QCH * BB);
  q.R = (float *)phde_buf(ctx, "batch.R", sizeof(float) * B * BB * BB);
  q.G = (double *)phde_buf(ctx, "batch.G", sizeof(double) * B * 2 * BB * BB);
  q.dden = (double *)phde_buf(ctx, "batch.dden", sizeof(double) * B * (k + 1));
  q.M = (double *)phde_buf(ctx, "batch.M", sizeof(double) * B * k * k);
  q.K = (double *)phde_buf(ctx, "batch.K", sizeof(double) * B * k * k);
  q.ev = (double *)phde_buf(ctx, "batch.ev", sizeof(double) * B * k);
  q.Y = (double *)phde_buf(ctx, "batch.Y", sizeof(double) * B * k * c);
  q.cinv = (double *)phde_buf(ctx, "batch.cinv", sizeof(double) * B * c);
  q.out = (double *)phde_buf(ctx, "batch.out", sizeof(double) * N * c);
  q.st = (int *)phde_buf(ctx, "batch.st", sizeof(int) * 4 * B);
  q.est = (int *)phde_buf(ctx, "batch.est", sizeof(int) * 2 * B);
  q.dlog = (double *)phde_buf(ctx, "batch.dlog", sizeof(double) * P * B);
  q.rq = (double *)phde_buf(ctx, "batch.rq", sizeof(double) * B * c);
  q.learned = learned;
  if (learned) {  // the model goes to the device before the (captured) sequence, on every call
    if (ctx->pivot_model.empty()) {
      const float *w0;
      int cnt;
      if (phde_default_pivot_model(&w0, &cnt)) return phde_fail(ctx, PHDE_ERR_INVALID, "built-in pivot model has the wrong size");
      ctx->pivot_model.assign(w0, w0 + cnt);
    }
    float *dw = (float *)phde_buf(ctx, "lpb.w", sizeof(float) * ctx->pivot_model.size());
    if (!dw) return PHDE_ERR_OOM;
    PHDE_CK(ctx, cudaMemcpyAsync(dw, ctx->pivot_model.data(), sizeof(float) * ctx->pivot_model.size(),
                                 cudaMemcpyHostToDevice, ctx->stream));
    q.weights = dw;
  }
  if (!q.deg || !q.D || !q.src || !q.sumsq || !q.edges || !q.inv || !q.X || !q.S || !q.LS || !q.C || !q.R || !q.G ||
      !q.dden || !q.M || !q.K || !q.ev || !q.Y || !q.cinv || !q.out || !q.st || !q.est || !q.dlog || !q.rq)
    return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(q.edges, 0, sizeof(ull), ctx->stream));

  // ---- segment length: autotuned once per uploaded batch (each candidate timed on this batch) ----
  auto set_segments = [&](int64_t seg_rows) -> int {
    std::vector<int32_t> g;
    std::vector<int64_t> r0, r1;
    std::vector<int> first;
    build_segments(ctx->batch_vbase, seg_rows, g, r0, r1, first);
    const int ns = (int)g.size();
    int32_t *dg = (int32_t *)phde_buf(ctx, "batch.seg_g", sizeof(int32_t) * ns);
    int64_t *d0 = (int64_t *)phde_buf(ctx, "batch.seg_r0", sizeof(int64_t) * ns);
    int64_t *d1 = (int64_t *)phde_buf(ctx, "batch.seg_r1", sizeof(int64_t) * ns);
    int *df = (int *)phde_buf(ctx, "batch.seg_first", sizeof(int) * (B + 1));
    float *part = (float *)phde_buf(ctx, "batch.part", sizeof(float) * (size_t)ns * QCH * BB);
    double *fpart = (double *)phde_buf(ctx, "batch.fpart", sizeof(double) * (size_t)ns * BB);
    double *cpart = (double *)phde_buf(ctx, "batch.cpart", sizeof(double) * (size_t)ns * MAXC);
    if (!dg || !d0 || !d1 || !df || !part || !fpart || !cpart) return PHDE_ERR_OOM;
    PHDE_CK(ctx, cudaMemcpyAsync(dg, g.data(), sizeof(int32_t) * ns, cudaMemcpyHostToDevice, ctx->stream));
    PHDE_CK(ctx, cudaMemcpyAsync(d0, r0.data(), sizeof(int64_t) * ns, cudaMemcpyHostToDevice, ctx->stream));
    PHDE_CK(ctx, cudaMemcpyAsync(d1, r1.data(), sizeof(int64_t) * ns, cudaMemcpyHostToDevice, ctx->stream));
    PHDE_CK(ctx, cudaMemcpyAsync(df, first.data(), sizeof(int) * (B + 1), cudaMemcpyHostToDevice, ctx->stream));
    PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));  // the host vectors go out of scope
    q.sg = Seg{dg, d0, d1, df, ns};
    q.part = part;
    q.fpart = fpart;
    q.cpart = cpart;
    return PHDE_OK;
  };
  int rc;
  // the tuned length is kept for batches of the same shape (count, vertices, entries, k); the captured
  // graph is rebuilt after every upload (the device CSR may have moved)
  const int64_t shape = ((int64_t)B * 1000003 + N) * 1000003 + ctx->nnz;
  const bool tune = ctx->batch_tuned_shape != shape || ctx->batch_tuned_k != k;
  if (ctx->batch_graph && ctx->batch_graph_epoch != ctx->graph_epoch) {
    cudaGraphExecDestroy(ctx->batch_graph);
    ctx->batch_graph = nullptr;
  }
  if (tune) {
    static const int64_t kCandidates[] = {2048, 4096, 8192, 16384, 32768};
    float best = 1e30f;
    int64_t best_rows = 8192;
    for (int64_t rows : kCandidates) {
      if ((rc = set_segments(rows))) return rc;
      cudaEventRecord(ctx->ev[0], ctx->stream);
      if ((rc = batch_pipeline(ctx, q, k, c))) return rc;
      cudaEventRecord(ctx->ev[1], ctx->stream);
      if ((rc = phde_check_device_err(ctx, "batched layout (tuning)"))) return rc;
      float ms = 0;
      cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
      if (ms < best) {
        best = ms;
        best_rows = rows;
      }
    }
    ctx->batch_seg_rows = best_rows;
    ctx->batch_tuned_shape = shape;
    ctx->batch_tuned_k = k;
    ctx->batch_tune_ms = best;
    if (ctx->batch_graph) {
      cudaGraphExecDestroy(ctx->batch_graph);
      ctx->batch_graph = nullptr;
    }
  }
  if ((rc = set_segments(ctx->batch_seg_rows))) return rc;
  const int64_t launches0 = ctx->launches;
  // ---- run: replay the captured graph, or capture it (first call after tuning), or launch directly ----
  const int key_c = c * 8 + o->strategy;  // the captured sequence depends on c and the pivot strategy
  if (ctx->batch_graph && (ctx->batch_graph_c != key_c || ctx->batch_graph_ws != ctx->ws_epoch)) {
    cudaGraphExecDestroy(ctx->batch_graph);
    ctx->batch_graph = nullptr;
  }
  cudaEventRecord(ctx->ev[0], ctx->stream);
  bool replayed = false, ran = false;
  if (ctx->batch_warm_key != key_c) {
    // the first call with this sequence runs it directly (it allocates its buffers); the next one captures it
    if ((rc = batch_pipeline(ctx, q, k, c))) return rc;
    ran = true;
    ctx->batch_warm_key = key_c;
    ctx->batch_no_graph = false;
  } else if (ctx->batch_graph) {
    PHDE_CK(ctx, cudaGraphLaunch(ctx->batch_graph, ctx->stream));
    ctx->launches += ctx->batch_graph_launches;
    replayed = true;
  } else if (!ctx->batch_no_graph) {
    const int64_t ws0 = ctx->ws_epoch;
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const int64_t l0 = ctx->launches;
      const int prc = batch_pipeline(ctx, q, k, c);
      const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
      cudaGraphExec_t exec = nullptr;
      if (prc == PHDE_OK && ce == cudaSuccess && graph && ctx->ws_epoch == ws0 &&
          cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
        ctx->batch_graph = exec;
        ctx->batch_graph_epoch = ctx->graph_epoch;
        ctx->batch_graph_c = key_c;
        ctx->batch_graph_ws = ctx->ws_epoch;
        ctx->batch_graph_launches = ctx->launches - l0;
        PHDE_CK(ctx, cudaGraphLaunch(exec, ctx->stream));
        replayed = true;
      } else {
        ctx->batch_no_graph = true;  // capture unsupported here: launch directly from now on
      }
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      ctx->err.clear();
    } else {
      cudaGetLastError();
      ctx->batch_no_graph = true;
    }
  }
  if (!replayed && !ran && (rc = batch_pipeline(ctx, q, k, c))) return rc;
  // the caller's buffer is not part of the captured graph: copy after it
  PHDE_CK(ctx, cudaMemcpyAsync(coords_out, q.out, sizeof(double) * N * c, cudaMemcpyDeviceToHost, ctx->stream));
  cudaEventRecord(ctx->ev[1], ctx->stream);
  ctx->kev_pending = false;  // the Kcenters events belong to the capture
  if ((rc = phde_check_device_err(ctx, "batched layout"))) return rc;
  std::vector<int> st(4 * B), est(2 * B);
  PHDE_CK(ctx, cudaMemcpyAsync(st.data(), q.st, sizeof(int) * 4 * B, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaMemcpyAsync(est.data(), q.est, sizeof(int) * 2 * B, cudaMemcpyDeviceToHost, ctx->stream));
  ull h_edges = 0;
  PHDE_CK(ctx, cudaMemcpyAsync(&h_edges, q.edges, sizeof(ull), cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
  int naccepted_min = k, ndisc = 0, sweeps = 0;
  for (int b = 0; b < B; b++) {
    naccepted_min = std::min(naccepted_min, st[4 * b]);
    ndisc += st[4 * b + 1];
    sweeps = std::max(sweeps, est[b]);
    if (est[B + b] != PHDE_OK)
      return phde_fail(ctx, est[B + b], "batched layout: Jacobi eigensolver did not converge for graph " + std::to_string(b));
  }
  if (naccepted_min < k)
    return phde_fail(ctx, PHDE_ERR_TOO_FEW_PIVOTS, "batched layout: a graph has fewer than k independent pivot columns");
  ctx->batch_last_c = c;
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    stats->status = PHDE_OK;
    stats->npasses = P;
    stats->naccepted = k;
    stats->ndiscarded = ndisc;
    stats->eig_iters = sweeps;
    stats->gpu_launches = (int)(ctx->launches - launches0);
    stats->ms_total = ms;
    stats->edges_examined = (int64_t)h_edges;
    stats->batch_graph_replay = replayed ? 1 : 0;
    stats->batch_seg_rows = (int)ctx->batch_seg_rows;
    stats->ms_batch_tune = tune ? ctx->batch_tune_ms : 0.0;
  }
  return PHDE_OK;
}

// The last phde_layout_batched call's Rayleigh quotients, graph b's coordinate t at rq_out[b * c + t].
extern "C" int phde_batch_rayleigh(phde_ctx *ctx, double *rq_out) {
  if (!ctx || !rq_out) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_batch_rayleigh: bad arguments");
  if (ctx->batch_B < 1 || ctx->batch_last_c < 1)
    return phde_fail(ctx, PHDE_ERR_NO_GRAPH, "phde_batch_rayleigh: no batched layout computed");
  const size_t cnt = (size_t)ctx->batch_B * ctx->batch_last_c;
  const double *rq = (const double *)phde_buf(ctx, "batch.rq", sizeof(double) * cnt);
  if (!rq) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemcpyAsync(rq_out, rq, sizeof(double) * cnt, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return PHDE_OK;
}
