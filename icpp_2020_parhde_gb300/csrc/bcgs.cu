// bcgs.cu -- blocked CGS2 D-orthogonalisation for the mixed-precision path (PHDE_PREC_MIXED).
//
// The reference orthogonalises the distance columns one at a time (ParHDE.cpp:190-285): every candidate x
// (L2-normalised) gets c_q = <x, D q> / <q, D q> against the accepted columns q and the constant column,
// x -= sum c_q q, and is discarded when ||x|| < 1e-3, else appended as x / ||x||, until k are accepted.
// Column at a time, that is a chain of grid-wide reductions per candidate.  Here candidates go in blocks
// of 32:
//   1. X (n x 32, FP32 row-major) = the block's normalised distance columns;
//   2. two projection passes against the accepted basis S and the constant column u0 (CGS2): the
//      tall-skinny Gram G = [S u0]^T D X (FP32 products over row slabs, FP64 across slabs), the
//      coefficients G / <q, D q>, and X -= [S u0] C;
//   3. the block's own Gram matrices Gd = X^T D X and G2 = X^T X (32 x 32);
//   4. one warp runs the reference's accept/discard loop over the block's candidates in the 32-dim
//      coefficient space, in FP64: candidate i is t = e_i, projected twice against the block's accepted
//      vectors r_a (c_a = t^T Gd r_a / r_a^T Gd r_a), its norm is sqrt(t^T G2 t), and it is discarded
//      below 1e-3 or accepted as t / norm -- so the acceptance order and rule are the reference's;
//   5. the accepted columns S[:, j + a] = X r_a, with their exact <q, D q> for later denominators.
// In exact arithmetic this equals column-at-a-time classical Gram-Schmidt (X after step 2 is D-orthogonal
// to S, so <x_i, D q_a> is the same whether x_i was projected on S first or not); step 2's second pass
// and step 4's second pass are the re-orthogonalisation that FP32 needs on these nearly collinear
// columns.  Seven launches per 32 candidates replace seven grid barriers per candidate.
#include <cmath>
#include <vector>

#include "bcgs_gs.cuh"
#include "ctx.h"

namespace {

constexpr int BB = 32;       // candidates per block
constexpr int GT = 256;      // threads of the Gram / update kernels
constexpr int QCH = 64;      // Gram rows (basis columns) per CTA along grid.y
constexpr int RT = 32;       // rows per staged tile
constexpr int ST_LD = 36;
constexpr int RED_THREADS = 1024;  // cross-CTA reductions    // row stride of the transposed S tile: 16-byte aligned, 4-way staging conflicts

// D[:, rc0 + c] / ||D[:, rc0 + c]|| into X[:, c] (row-major n x 32; columns >= bc are zero).
__global__ void bcgs_load_kernel(const int32_t *D, int64_t n, int rc0, int bc, const ull *sumsq, float *X) {
  __shared__ float tile[BB][RT + 1];
  __shared__ float inv[BB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (threadIdx.x < BB)
    inv[threadIdx.x] = threadIdx.x < bc ? (float)(1.0 / sqrt((double)sumsq[rc0 + threadIdx.x])) : 0.f;
  for (int64_t r0 = (int64_t)blockIdx.x * RT; r0 < n; r0 += (int64_t)gridDim.x * RT) {
    __syncthreads();
    for (int c = warp; c < BB; c += nw) {
      const int64_t r = r0 + lane;
      tile[c][lane] = (c < bc && r < n) ? (float)D[(int64_t)(rc0 + c) * n + r] * inv[c] : 0.f;
    }
    __syncthreads();
    for (int rr = warp; rr < RT; rr += nw)
      if (r0 + rr < n) X[(r0 + rr) * BB + lane] = tile[lane][rr];
  }
}

// Partial Gram products over each CTA's row slab (QC Gram rows per CTA along grid.y):
//   part[((y * gridDim.x + x) * R + qq) * 32 + i] = sum_r A[r][q] * w[r] * X[r][i],   q = y * QC + qq,
// where A[r][q] is the basis (row-major, leading dimension lda) for q < nq, 1 for q == nq when `ones` (the
// constant column), 0 beyond; R = QC.  SELF (A = X, QC = 32): both X^T D X (rows 0..31) and X^T X (rows
// 32..63) from one read of X, R = 64.  FP32 products, FP32 slab sums; staging of the next 32-row tile is
// prefetched into registers while the current one is multiplied.
template <int QC, bool SELF>
__global__ void __launch_bounds__(GT) bcgs_gram_kernel(const float *A, int lda, int nq, int ones, const float *X,
                                                       const double *w, int64_t n, float *part) {
  constexpr int QPW = QC / 8;  // Gram rows per warp (eight warps)
  constexpr int NR = SELF ? 2 * QC : QC;
  __shared__ __align__(16) float At[RT][QC];
  __shared__ float Xt[RT][BB];
  __shared__ float Xw[SELF ? RT : 1][BB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int qbase = blockIdx.y * QC;
  const int64_t per = ((n + gridDim.x - 1) / gridDim.x + RT - 1) / RT * RT;
  const int64_t rb = (int64_t)blockIdx.x * per, re = min(n, rb + per);
  float acc[QPW], acc2[SELF ? QPW : 1];
#pragma unroll
  for (int m = 0; m < QPW; m++) acc[m] = 0.f;
#pragma unroll
  for (int m = 0; m < (SELF ? QPW : 1); m++) acc2[m] = 0.f;
  const int q = threadIdx.x % QC, r1 = threadIdx.x / QC, qq = qbase + q;
  const float cst = (qq == nq && ones) ? 1.f : 0.f;
  const int xi = threadIdx.x % BB, r2 = threadIdx.x / BB;
  constexpr int NA = RT / (GT / QC), NX = RT / (GT / BB);
  float pa[NA], px[NX], pw[NX];
  auto fetch = [&](int64_t r0) {
#pragma unroll
    for (int t = 0; t < NA; t++) {
      const int64_t row = r0 + r1 + t * (GT / QC);
      pa[t] = row < re ? (qq < nq ? A[row * lda + qq] : cst) : 0.f;
    }
#pragma unroll
    for (int t = 0; t < NX; t++) {
      const int64_t row = r0 + r2 + t * (GT / BB);
      const float x = row < re ? X[row * BB + xi] : 0.f;
      const float wf = (w && row < re) ? (float)w[row] : 1.f;
      px[t] = SELF ? x : x * wf;
      pw[t] = x * wf;
    }
  };
  if (rb < re) fetch(rb);
  for (int64_t r0 = rb; r0 < re; r0 += RT) {
    __syncthreads();
#pragma unroll
    for (int t = 0; t < NA; t++) At[r1 + t * (GT / QC)][q] = pa[t];
#pragma unroll
    for (int t = 0; t < NX; t++) {
      Xt[r2 + t * (GT / BB)][xi] = px[t];
      if (SELF) Xw[r2 + t * (GT / BB)][xi] = pw[t];
    }
    __syncthreads();
    if (r0 + RT < re) fetch(r0 + RT);
#pragma unroll 4
    for (int rr = 0; rr < RT; rr++) {
      const float x = Xt[rr][lane];
      float av[QPW];
      if constexpr (QPW % 4 == 0) {
#pragma unroll
        for (int m = 0; m < QPW; m += 4) {
          const float4 a4 = *(const float4 *)&At[rr][warp * QPW + m];
          av[m] = a4.x;
          av[m + 1] = a4.y;
          av[m + 2] = a4.z;
          av[m + 3] = a4.w;
        }
      } else {
#pragma unroll
        for (int m = 0; m < QPW; m++) av[m] = At[rr][warp * QPW + m];
      }
#pragma unroll
      for (int m = 0; m < QPW; m++) acc[m] = fmaf(av[m], x, acc[m]);
      if constexpr (SELF) {
        const float xw = Xw[rr][lane];
#pragma unroll
        for (int m = 0; m < QPW; m++) acc2[m] = fmaf(av[m], xw, acc2[m]);
      }
    }
  }
  float *dst = part + ((int64_t)(blockIdx.y * gridDim.x + blockIdx.x) * NR + warp * QPW) * BB + lane;
  if constexpr (SELF) {
    // rows 0..QC-1: X^T D X (weighted), rows QC..2QC-1: X^T X
#pragma unroll
    for (int m = 0; m < QPW; m++) {
      dst[m * BB] = acc2[m];
      dst[(QC + m) * BB] = acc[m];
    }
  } else {
#pragma unroll
    for (int m = 0; m < QPW; m++) dst[m * BB] = acc[m];
  }
}

// The projection Gram of the first block, when only the constant column is accepted: per-CTA sums of
// w_r X[r][i] (the constant column's Gram row), in the layout bcgs_reduce_kernel reads with one row per CTA.
__global__ void __launch_bounds__(GT) bcgs_u0_kernel(const float *X, const double *w, int64_t n, float *part) {
  __shared__ float red[GT / 32][BB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  float acc = 0.f;
  for (int64_t r = (int64_t)blockIdx.x * nw + warp; r < n; r += (int64_t)gridDim.x * nw)
    acc = fmaf(X[r * BB + lane], (float)w[r], acc);
  red[warp][lane] = acc;
  __syncthreads();
  if (warp == 0) {
    float t = 0.f;
    for (int i = 0; i < nw; i++) t += red[i][lane];
    part[(int64_t)blockIdx.x * BB + lane] = t;
  }
}

// Sum the partials of Gram row q (one CTA per row, fixed order: deterministic) in FP64.
//   mode 0 (projection): C[q][i] = sum / <q, D q> for q < nq, sum / (n * den0) for q == nq (the constant
//                        column's coefficient times its entry 1/sqrt(n)); FP32 out.
//   mode 1 (block Gram): G[q][i] = sum, FP64 out.
__global__ void __launch_bounds__(RED_THREADS) bcgs_reduce_kernel(const float *part, int ncta, int nq, int mode,
                                                                  const double *dden, double n_den0, float *C,
                                                                  double *G, int rows) {
  __shared__ double red[RED_THREADS / 32][BB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // Gram row q; `rows` partial rows per CTA (the kernel's QC, 2 QC for the block Grams)
  const int q = blockIdx.x, y = mode == 0 ? q / rows : 0, qq = mode == 0 ? q % rows : q;
  // four independent sums per thread (the partials come from L2: hide its latency), combined in order
  const float *base = part + ((int64_t)y * ncta * rows + qq) * BB + lane;
  const int64_t cs = (int64_t)rows * BB;
  double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  int c = warp;
  for (; c + 3 * nw < ncta; c += 4 * nw) {
    s0 += (double)__ldcg(base + c * cs);
    s1 += (double)__ldcg(base + (c + nw) * cs);
    s2 += (double)__ldcg(base + (c + 2 * nw) * cs);
    s3 += (double)__ldcg(base + (c + 3 * nw) * cs);
  }
  for (; c < ncta; c += nw) s0 += (double)__ldcg(base + c * cs);
  const double s = (s0 + s1) + (s2 + s3);
  red[warp][lane] = s;
  __syncthreads();
  if (warp == 0) {
    double t = 0;
    for (int w = 0; w < nw; w++) t += red[w][lane];
    if (mode == 0)
      C[q * BB + lane] = (float)(q < nq ? t / dden[q] : t / n_den0);
    else
      G[q * BB + lane] = t;
  }
}

// X[r][i] -= sum_{q < nq} S[r][q] C[q][i] + C[nq][i]   (C[nq] = the constant column's term).
// A warp per 4 rows of a 32-row tile; the tile of S is staged transposed so 4 rows come in one load.
__global__ void __launch_bounds__(GT) bcgs_update_kernel(const float *S, int lda, int nq, const float *C, float *X,
                                                         int64_t n) {
  extern __shared__ __align__(16) float smu[];
  float *Cs = smu;                          // [(nq + 1) * 32]
  float *St = smu + (nq + 1) * BB;          // [nq][ST_LD]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int idx = threadIdx.x; idx < (nq + 1) * BB; idx += GT) Cs[idx] = C[idx];
  for (int64_t r0 = (int64_t)blockIdx.x * RT; r0 < n; r0 += (int64_t)gridDim.x * RT) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < RT * nq; idx += GT) {
      const int r = idx / nq, q = idx % nq;
      St[q * ST_LD + r] = r0 + r < n ? S[(r0 + r) * lda + q] : 0.f;
    }
    __syncthreads();
    const float c0 = Cs[nq * BB + lane];
    float p0 = c0, p1 = c0, p2 = c0, p3 = c0;
    for (int q = 0; q < nq; q++) {
      const float cq = Cs[q * BB + lane];
      const float4 s4 = *(const float4 *)&St[q * ST_LD + warp * 4];
      p0 = fmaf(s4.x, cq, p0);
      p1 = fmaf(s4.y, cq, p1);
      p2 = fmaf(s4.z, cq, p2);
      p3 = fmaf(s4.w, cq, p3);
    }
    const int64_t r = r0 + warp * 4;
    if (r < n) X[r * BB + lane] -= p0;
    if (r + 1 < n) X[(r + 1) * BB + lane] -= p1;
    if (r + 2 < n) X[(r + 2) * BB + lane] -= p2;
    if (r + 3 < n) X[(r + 3) * BB + lane] -= p3;
  }
}

// The block's accept/discard loop (bcgs_gs.cuh), one CTA of four warps.
// st: [0] accepted so far (j), [1] discarded, [2] candidates consumed, [3] accepted in this block.
__global__ void __launch_bounds__(bcgs_gs::NW * 32) bcgs_block_gs_kernel(const double *Gd, const double *G2, int bc,
                                                                         int k, int rc0, int *st, double *dlog,
                                                                         float *R) {
  __shared__ bcgs_gs::Smem S;
  __shared__ int res[3];
  const int j0 = st[0];
  bcgs_gs::run(S, Gd, G2, bc, k, j0, dlog + rc0, R, res, res + 1, res + 2);
  __syncthreads();
  if (threadIdx.x == 0) {
    st[0] = j0 + res[0];
    st[1] += res[1];
    st[2] += res[2];
    st[3] = res[0];
  }
}

// S[r][j0 + a] = sum_i X[r][i] R[i][a] for a < nacc, with per-CTA partial sums of deg * S^2 per column.
__global__ void __launch_bounds__(GT) bcgs_form_kernel(const float *X, const float *R, int nacc, float *S, int lda,
                                                       int j0, const double *deg, int64_t n, double *part) {
  __shared__ float Rs[BB][BB + 1];
  __shared__ double red[GT / 32][BB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int idx = threadIdx.x; idx < BB * BB; idx += GT) Rs[idx / BB][idx % BB] = R[idx];
  __syncthreads();
  // deg * v^2 in FP32, summed in FP32 over 16 rows and in FP64 beyond (GB300's FP64 rate is 1/64 of FP32,
  // and three FP64 operations per element would bound the kernel)
  double dsum = 0;
  float fsum = 0.f;
  int cnt = 0;
  for (int64_t r = (int64_t)blockIdx.x * nw + warp; r < n; r += (int64_t)gridDim.x * nw) {
    const float x = X[r * BB + lane];
    float v = 0.f;
#pragma unroll 8
    for (int i = 0; i < BB; i++) v = fmaf(__shfl_sync(PHDE_FULL_MASK, x, i), Rs[i][lane], v);
    if (lane < nacc) {
      S[r * lda + j0 + lane] = v;
      fsum = fmaf(v * v, (float)deg[r], fsum);
    }
    if (++cnt == 16) {
      dsum += (double)fsum;
      fsum = 0.f;
      cnt = 0;
    }
  }
  dsum += (double)fsum;
  red[warp][lane] = dsum;
  __syncthreads();
  if (warp == 0) {
    double t = 0;
    for (int w = 0; w < nw; w++) t += red[w][lane];
    part[(int64_t)blockIdx.x * BB + lane] = t;
  }
}

// <q, D q> of the block's new columns from the form kernel's partials (fixed order: warp w sums CTAs
// w, w + 32, ..., then the warps' sums are added in warp order).
__global__ void __launch_bounds__(RED_THREADS) bcgs_dd_kernel(const double *part, int ncta, int nacc, int j0,
                                                              double *dden) {
  __shared__ double red[RED_THREADS / 32][BB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double t = 0;
  for (int c = warp; c < ncta; c += nw) t += part[(int64_t)c * BB + lane];
  red[warp][lane] = t;
  __syncthreads();
  if (warp == 0) {
    double u = 0;
    for (int w = 0; w < nw; w++) u += red[w][lane];
    if (lane < nacc) dden[j0 + lane] = u;
  }
}

}  // namespace

int phde_bcgs2_mixed(phde_ctx *ctx, const int32_t *D, int P, const ull *sumsq, const double *deg, float *S, int k,
                     int *h_state, double *h_dlog) {
  const int64_t n = ctx->n;
  if (ctx->weighted) return phde_fail(ctx, PHDE_ERR_INVALID, "blocked CGS2 takes unweighted graphs");
  const int ncta = ctx->nsm * 6;  // Gram row slabs (several CTAs per SM hide the staging latency)
  const int ncta_tc = ctx->nsm * 2;  // tensor-core Gram: two CTAs per SM (88 KB of stages each)
  const int ncta_g = ctx->tc_gram_cgs2 ? ncta_tc : ncta;
  const int nqc_max = (k + 1 + QCH - 1) / QCH;
  float *X = (float *)phde_buf(ctx, "bcgs.X", sizeof(float) * n * BB);
  float *part = (float *)phde_buf(ctx, "bcgs.part", sizeof(float) * (size_t)nqc_max * ncta * QCH * BB);
  float *C = (float *)phde_buf(ctx, "bcgs.C", sizeof(float) * (size_t)(k + 1) * BB);
  double *G = (double *)phde_buf(ctx, "bcgs.G", sizeof(double) * 2 * BB * BB);
  float *R = (float *)phde_buf(ctx, "bcgs.R", sizeof(float) * BB * BB);
  double *dden = (double *)phde_buf(ctx, "bcgs.dden", sizeof(double) * (k + 1));
  double *fpart = (double *)phde_buf(ctx, "bcgs.fpart", sizeof(double) * ncta * BB);
  int *st = (int *)phde_buf(ctx, "bcgs.state", sizeof(int) * 4);
  double *dlog = (double *)phde_buf(ctx, "bcgs.dlog", sizeof(double) * P);
  if (!X || !part || !C || !G || !R || !dden || !fpart || !st || !dlog) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(dlog, 0xff, sizeof(double) * P, ctx->stream));  // NaN: accepted
  PHDE_CK(ctx, cudaMemsetAsync(st, 0, sizeof(int) * 4, ctx->stream));
  const double n_den0 = (double)ctx->nnz;  // n * <u0, D u0> = sum of degrees
  const int g_rows = (int)std::max<int64_t>(1, std::min<int64_t>((n + RT - 1) / RT, (int64_t)ctx->nsm * 8));
  const size_t upd_smem_max = sizeof(float) * ((size_t)(k + 1) * BB + (size_t)k * ST_LD);
  PHDE_CK(ctx, cudaFuncSetAttribute(bcgs_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)std::max<size_t>(upd_smem_max, 48 * 1024)));
  int j = 0;
  int hst[4] = {0, 0, 0, 0};
  for (int rc0 = 0; rc0 < P && j < k; rc0 += BB) {
    const int bc = std::min(BB, P - rc0);
    bcgs_load_kernel<<<g_rows, GT, 0, ctx->stream>>>(D, n, rc0, bc, sumsq, X);
    PHDE_LAUNCHED(ctx);
    const int nqt = j + 1;
    const int qc = ctx->tc_gram_cgs2 ? QCH : nqt <= 8 ? 8 : (nqt <= 32 ? 32 : 64), nqc = (nqt + qc - 1) / qc;
    for (int pass = 0; pass < 2; pass++) {
      if (j == 0) {
        bcgs_u0_kernel<<<ncta, GT, 0, ctx->stream>>>(X, deg, n, part);
      } else if (ctx->tc_gram_cgs2) {
        const int rc = phde_tc_gram32(ctx, S, k, j, 1, X, deg, n, ncta_tc, nqc, 0, part);
        if (rc) return rc;
      } else if (qc == 8)
        bcgs_gram_kernel<8, false><<<dim3(ncta, nqc), GT, 0, ctx->stream>>>(S, k, j, 1, X, deg, n, part);
      else if (qc == 32)
        bcgs_gram_kernel<32, false><<<dim3(ncta, nqc), GT, 0, ctx->stream>>>(S, k, j, 1, X, deg, n, part);
      else
        bcgs_gram_kernel<64, false><<<dim3(ncta, nqc), GT, 0, ctx->stream>>>(S, k, j, 1, X, deg, n, part);
      if (j == 0 || !ctx->tc_gram_cgs2) PHDE_LAUNCHED(ctx);
      if (j == 0)  // one Gram row (the constant column) per CTA
        bcgs_reduce_kernel<<<1, RED_THREADS, 0, ctx->stream>>>(part, ncta, 0, 0, dden, n_den0, C, nullptr, 1);
      else
        bcgs_reduce_kernel<<<nqt, RED_THREADS, 0, ctx->stream>>>(part, ncta_g, j, 0, dden, n_den0, C, nullptr, qc);
      PHDE_LAUNCHED(ctx);
      const size_t smem = sizeof(float) * ((size_t)nqt * BB + (size_t)j * ST_LD);
      bcgs_update_kernel<<<g_rows, GT, smem, ctx->stream>>>(S, k, j, C, X, n);
      PHDE_LAUNCHED(ctx);
    }
    // block Grams X^T D X and X^T X in one pass; G holds them one after the other (64 rows of 32)
    if (ctx->tc_gram_cgs2) {
      const int rc = phde_tc_gram32(ctx, nullptr, 0, 0, 0, X, deg, n, ncta_tc, 1, 1, part);
      if (rc) return rc;
    } else {
      bcgs_gram_kernel<32, true><<<dim3(ncta, 1), GT, 0, ctx->stream>>>(X, BB, BB, 0, X, deg, n, part);
      PHDE_LAUNCHED(ctx);
    }
    bcgs_reduce_kernel<<<2 * BB, RED_THREADS, 0, ctx->stream>>>(part, ncta_g, BB, 1, nullptr, 0.0, nullptr, G, 2 * BB);
    PHDE_LAUNCHED(ctx);
    bcgs_block_gs_kernel<<<1, bcgs_gs::NW * 32, 0, ctx->stream>>>(G, G + BB * BB, bc, k, rc0, st, dlog, R);
    PHDE_LAUNCHED(ctx);
    PHDE_CK(ctx, cudaMemcpyAsync(hst, st, sizeof(hst), cudaMemcpyDeviceToHost, ctx->stream));
    PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    const int nacc = hst[3];
    if (nacc > 0) {
      bcgs_form_kernel<<<ncta, GT, 0, ctx->stream>>>(X, R, nacc, S, k, j, deg, n, fpart);
      PHDE_LAUNCHED(ctx);
      bcgs_dd_kernel<<<1, RED_THREADS, 0, ctx->stream>>>(fpart, ncta, nacc, j, dden);
      PHDE_LAUNCHED(ctx);
    }
    j = hst[0];
  }
  h_state[0] = hst[0];
  h_state[1] = hst[1];
  h_state[2] = hst[2];
  h_state[3] = 0;
  PHDE_CK(ctx, cudaMemcpyAsync(h_dlog, dlog, sizeof(double) * P, cudaMemcpyDeviceToHost, ctx->stream));
  return PHDE_OK;
}
