// tcgram.cu -- tall-skinny Gram products G = A^T diag(w) B on the 5th-generation tensor cores (tcgen05), for
// the mixed-precision path: the CGS2 projections [S u0]^T D X and block Grams X^T D X, X^T X
// (ParHDE.cpp:190-285's inner products, blocked), and S^T (L S) (DrawingBase.cpp:221-244).
//
// The inputs are FP32 and GB300's tensor cores take 16-bit operands, so every value is split into three
// BF16 parts, v = hi + mid + lo (8 + 8 + 8 significand bits: the whole FP32 significand).  The A operand of
// one MMA (M = 128 rows) stacks the hi, mid and lo parts of 32 Gram rows (rows 96..127 are zero), and each
// K step runs three MMAs, against the hi, mid and lo parts of B, into one FP32 accumulator in TMEM: its
// rows r, 32 + r and 64 + r then hold hi(a) b, mid(a) b and lo(a) b for Gram row r -- all nine partial
// products, so the result is FP32-faithful (products of the full FP32 inputs, FP32 accumulation over the
// CTA's rows) and the three rows are added in FP64 at the end.
//
// Per CTA: eight producer warps stage 64-row chunks of A and B from global memory (any leading dimension,
// any alignment: plain coalesced loads), split them and store them in the canonical K-major layout without
// swizzle (8-row x 16-byte core matrices; core matrices adjacent in K 128 bytes apart, 8-row groups 1024
// bytes apart); a ninth warp issues the MMAs from one thread.  Two stages with a full and an empty mbarrier
// each: the producers arrive on `full` after their stores, the issuer waits for it, and its tcgen05.commit
// arrives on `empty` when the MMAs have read the stage -- no block-wide barrier in the main loop.  At the
// end the accumulators are read with tcgen05.ld (each warp reads its own 32-lane quarter) and combined.  Every mbarrier wait is bounded by %globaltimer; on expiry the kernel records
// PHDE_ERR_TIMEOUT, waits once more (bounded) for its MMAs, frees its TMEM and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>

#include "ctx.h"
#include "tc_common.cuh"

namespace {

constexpr int PRODUCERS = 256;             // staging threads (warps 0..7); warp 8 issues the MMAs
constexpr int TC_THREADS = PRODUCERS + 32;
constexpr int A_TILE_BYTES = 128 * KC * 2; // one stacked A operand: 128 rows x 64 K of BF16 (16 KB)

}  // namespace

// Arguments of one Gram launch (host-visible: the launchers in mixed.cu and bcgs.cu fill it).
struct TcGramArgs {
  const float *A;
  int lda, acols;     // A: n x acols used, row-major with leading dimension lda
  int ones_col;       // an A column (index >= acols) that reads as 1.0 (the constant column), -1 for none
  int self_weighted;  // A tile 0 = w * B's columns, tile 1 = B's columns (block Grams X^T D X and X^T X)
  const float *B;
  int ldb, bcols;     // B: n x bcols used
  int weight_b;       // multiply B rows by (float) w[row]
  const double *w;
  int64_t n;
  int64_t rows_per;   // rows per CTA along the row-split grid dimension
  int ldo;            // output: OUT 1 row stride (elements)
  float *out32;       // OUT 0: [(tile * ncta + cta) * (32 MT) + row] * N + col
  double *out64;      // OUT 1: [split][(a0 + row) * ldo + b0 + col]
  int64_t out64_split;
  int tiles_b;        // OUT 1: tiles along B (grid.x = tiles_a * tiles_b)
  int *err;
  uint64_t timeout_ns;
};

// MT: A tiles of 32 Gram rows per CTA (1 or 2); N: B columns per CTA (32 or 64); OUT: 0 -> FP32 partials
// for the CGS2 reductions (grid.x = row splits, grid.y = A tiles), 1 -> FP64 partials (grid.x = A x B tiles,
// grid.y = row splits).
template <int MT, int N, int OUT>
__global__ void __launch_bounds__(TC_THREADS) tc_gram_kernel(TcGramArgs g) {
  constexpr int B_PART_BYTES = N * KC * 2;
  constexpr int STAGE_BYTES = MT * A_TILE_BYTES + 3 * B_PART_BYTES;
  constexpr uint32_t NCOLS = MT * N;  // TMEM columns: a power of two >= 32 for the shapes used
  constexpr uint32_t IDESC = idesc_bf16(128, N);
  extern __shared__ __align__(1024) uint8_t sm[];
  __shared__ __align__(8) uint64_t s_full[2], s_empty[2];
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail, s_committed;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int cta_rows = OUT == 0 ? blockIdx.x : blockIdx.y;
  const int tile = OUT == 0 ? blockIdx.y : blockIdx.x;
  const int a0 = OUT == 0 ? tile * 32 * MT : (tile / g.tiles_b) * 32 * MT;
  const int b0 = OUT == 0 ? 0 : (tile % g.tiles_b) * N;
  const int64_t r0 = (int64_t)cta_rows * g.rows_per, r1 = min(g.n, r0 + g.rows_per);
  const int nchunks = r1 > r0 ? (int)((r1 - r0 + KC - 1) / KC) : 0;

  if (nchunks == 0) {  // no rows: zero partials
    for (int i = tid; i < 32 * MT * N; i += TC_THREADS) {
      const int row = i / N, col = i % N;
      if (OUT == 0) {
        g.out32[((int64_t)(tile * gridDim.x + cta_rows) * (32 * MT) + row) * N + col] = 0.f;
      } else if (a0 + row < g.acols && b0 + col < g.bcols) {
        g.out64[(int64_t)cta_rows * g.out64_split + (int64_t)(a0 + row) * g.ldo + b0 + col] = 0.0;
      }
    }
    return;
  }

  if (tid == 0) {
    for (int s = 0; s < 2; s++) {
      mbar_init(smem_u32(&s_full[s]), PRODUCERS);
      mbar_init(smem_u32(&s_empty[s]), 1);
    }
    fence_mbar_init();
    s_fail = 0;
    s_committed = 0;
  }
  if (warp == 0) tmem_alloc(smem_u32(&s_tmem), NCOLS);
  // the zero rows 96..127 of every stacked A operand, both stages
  for (int s = 0; s < 2; s++)
    for (int t = 0; t < MT; t++) {
      uint4 *z = (uint4 *)(sm + s * STAGE_BYTES + t * A_TILE_BYTES + 96 * KC * 2);
      for (int i = tid; i < 32 * KC * 2 / 16; i += TC_THREADS) z[i] = make_uint4(0, 0, 0, 0);
    }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  volatile int *fail = &s_fail;

  if (warp < PRODUCERS / 32) {
    // Producers.  Staging units: (column, 8-row group); A: MT * 32 columns, B: N columns.  Unit
    // tid + j * PRODUCERS of thread tid; the A units fill whole multiples of the producers, so j alone says A
    // or B.  All loads of a chunk are issued before any of its values is stored, and the next chunk's loads
    // right after this chunk's stores, so they are in flight while the tensor core runs.
    constexpr int A_UNITS = MT * 32 * (KC / 8), B_UNITS = N * (KC / 8);
    constexpr int UPT = (A_UNITS + B_UNITS) / PRODUCERS;
    static_assert(A_UNITS % PRODUCERS == 0 && B_UNITS % PRODUCERS == 0, "units must fill the producers");
    auto load_chunk = [&](int c, float (&v)[UPT][8]) {
      // branch-free: every load is unconditional, at a valid address (a row past the block reads the block's
      // last row, a column outside the operand reads column 0), and the value is masked afterwards -- a
      // conditional load per element splits the loads into separately waited groups
      const int64_t rb = r0 + (int64_t)c * KC;
#pragma unroll
      for (int j = 0; j < UPT; j++) {
        const int u = tid + j * PRODUCERS;
        const bool is_a = u < A_UNITS;
        const int ub = u - A_UNITS;
        const int col = is_a ? u % (MT * 32) : ub % N;  // A: Gram row of this CTA; B: column
        const int rg = is_a ? u / (MT * 32) : ub / N;
        const float *base;
        int64_t ld;
        bool valid, weighted;
        float constant = 0.f;
        if (is_a && g.self_weighted) {  // tile 0: w * B, tile 1: B (B's columns 0..31)
          const int bc = col & 31;
          base = g.B + (bc < g.bcols ? bc : 0);
          ld = g.ldb;
          valid = bc < g.bcols;
          weighted = col < 32;
        } else if (is_a) {
          const int acol = a0 + col;
          valid = acol < g.acols;
          base = valid ? g.A + acol : g.B;
          ld = valid ? g.lda : g.ldb;
          weighted = false;
          constant = acol == g.ones_col ? 1.f : 0.f;
        } else {
          const int bcol = b0 + col;
          valid = bcol < g.bcols;
          base = g.B + (valid ? bcol : 0);
          ld = g.ldb;
          weighted = g.weight_b != 0;
        }
#pragma unroll
        for (int i = 0; i < 8; i++) {
          const int64_t row = rb + rg * 8 + i;
          const bool in = row < r1;
          const int64_t rr = in ? row : r1 - 1;
          const float x = __ldg(base + rr * ld);
          const float wv = weighted ? (float)__ldg(g.w + rr) : 1.f;
          v[j][i] = in ? (valid ? x * wv : constant) : 0.f;
        }
      }
    };
    auto store_chunk = [&](uint8_t *st, const float (&v)[UPT][8]) {
#pragma unroll
      for (int j = 0; j < UPT; j++) {
        const int u = tid + j * PRODUCERS;
        if (u < A_UNITS) {
          const int col = u % (MT * 32), rg = u / (MT * 32);
          const int t = col >> 5, cr = col & 31;
          uint8_t *at = st + t * A_TILE_BYTES;
          store_split8(v[j], at + core_off(cr, rg), at + core_off(32 + cr, rg), at + core_off(64 + cr, rg));
        } else {
          const int ub = u - A_UNITS;
          const int col = ub % N, rg = ub / N;
          uint8_t *bt = st + MT * A_TILE_BYTES;
          store_split8(v[j], bt + core_off(col, rg), bt + B_PART_BYTES + core_off(col, rg),
                       bt + 2 * B_PART_BYTES + core_off(col, rg));
        }
      }
    };
    float v[UPT][8];
    load_chunk(0, v);
    for (int c = 0; c < nchunks; c++) {
      const int s = c & 1;
      if (c >= 2 && !mbar_wait(smem_u32(&s_empty[s]), (uint32_t)(((c >> 1) - 1) & 1), g.timeout_ns, fail)) {
        *fail = 1;
        break;
      }
      if (*fail) break;
      store_chunk(sm + s * STAGE_BYTES, v);
      fence_async_smem();  // this thread's stores, visible to the tensor core's reads
      mbar_arrive(smem_u32(&s_full[s]));
      if (c + 1 < nchunks) load_chunk(c + 1, v);
    }
  } else if (lane == 0) {
    // The MMA issuer: for each chunk, once every producer has stored it, three MMAs per K step and A tile;
    // the commit frees the stage when they have read it.
    int c = 0;
    for (; c < nchunks; c++) {
      const int s = c & 1;
      if (!mbar_wait(smem_u32(&s_full[s]), (uint32_t)((c >> 1) & 1), g.timeout_ns, fail)) {
        *fail = 1;
        break;
      }
      tc_fence_after();
      const uint32_t st_addr = smem_u32(sm + s * STAGE_BYTES);
#pragma unroll
      for (int ks = 0; ks < KC / 16; ks++)
#pragma unroll
        for (int t = 0; t < MT; t++) {
          const uint64_t ad = smem_desc(st_addr + t * A_TILE_BYTES + ks * 2 * CORE_LBO);
#pragma unroll
          for (int p = 0; p < 3; p++) {
            const uint64_t bd = smem_desc(st_addr + MT * A_TILE_BYTES + p * B_PART_BYTES + ks * 2 * CORE_LBO);
            mma_bf16(tmem + (uint32_t)(t * N), ad, bd, IDESC, (c > 0 || ks > 0 || p > 0) ? 1u : 0u);
          }
        }
      mma_commit(smem_u32(&s_empty[s]));
    }
    s_committed = c;
  }
  __syncthreads();
  // the last commit covers every MMA issued before it
  const int last = s_committed - 1;
  bool ok = *fail == 0;
  if (last >= 0 && !mbar_wait(smem_u32(&s_empty[last & 1]), (uint32_t)((last >> 1) & 1), g.timeout_ns, nullptr))
    *fail = 1;
  __syncthreads();
  if (*fail) {
    ok = false;
    if (tid == 0) atomicCAS(g.err, 0, PHDE_ERR_TIMEOUT);
  }
  tc_fence_after();

  // read the accumulators: warp w < 8 reads lane quarter q = w & 3 of tile w >> 2
  float *red = (float *)sm;  // [MT][2][32][N]: the mid and lo rows, handed to the hi rows' warps
  const int q = warp & 3, t = warp >> 2;
  float vals[N];
  if (t < MT && ok) {
#pragma unroll
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(t * N + c0), v);
#pragma unroll
      for (int i = 0; i < 16; i++) vals[c0 + i] = v[i];
    }
    if (q == 1 || q == 2) {
      float *dst = red + ((t * 2 + (q - 1)) * 32 + lane) * N;
#pragma unroll
      for (int i = 0; i < N; i++) dst[i] = vals[i];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (t < MT && q == 0) {
    const int row = t * 32 + lane;  // Gram row within the CTA
    const float *mid = red + ((t * 2 + 0) * 32 + lane) * N, *lo = red + ((t * 2 + 1) * 32 + lane) * N;
#pragma unroll
    for (int i = 0; i < N; i++) {
      const double v = ok ? ((double)vals[i] + (double)mid[i]) + (double)lo[i] : 0.0;
      if (OUT == 0) {
        g.out32[((int64_t)(tile * gridDim.x + cta_rows) * (32 * MT) + row) * N + i] = (float)v;
      } else if (a0 + row < g.acols && b0 + i < g.bcols) {
        g.out64[(int64_t)cta_rows * g.out64_split + (int64_t)(a0 + row) * g.ldo + b0 + i] = v;
      }
    }
  }
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, NCOLS);
  }
}

namespace {

// out[i] = sum over splits of part[s * split + i], FP64, fixed order.
__global__ void tc_sum_parts_kernel(const double *part, int nsplit, int64_t split, int64_t count, double *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0;
    for (int p = 0; p < nsplit; p++) s += part[(int64_t)p * split + i];
    out[i] = s;
  }
}

template <int MT, int N, int OUT>
int launch(phde_ctx *ctx, const TcGramArgs &a, dim3 grid) {
  constexpr int STAGE_BYTES = MT * A_TILE_BYTES + 3 * N * KC * 2;
  constexpr int SMEM = 2 * STAGE_BYTES;
  static bool attr_set[64] = {};
  if (!attr_set[ctx->device & 63]) {
    PHDE_CK(ctx, cudaFuncSetAttribute(tc_gram_kernel<MT, N, OUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
    attr_set[ctx->device & 63] = true;
  }
  tc_gram_kernel<MT, N, OUT><<<grid, TC_THREADS, SMEM, ctx->stream>>>(a);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

}  // namespace

// G (FP64 partials, [split][acols x bcols] row-major at out64) = A^T diag(w) B over row splits.
int phde_tc_gram64(phde_ctx *ctx, const float *A, int lda, int acols, const float *B, int ldb, int bcols,
                   const double *w, int64_t n, int nsplit, double *out64) {
  TcGramArgs a{};
  a.A = A;
  a.lda = lda;
  a.acols = acols;
  a.ones_col = -1;
  a.B = B;
  a.ldb = ldb;
  a.bcols = bcols;
  a.weight_b = w != nullptr;
  a.w = w;
  a.n = n;
  a.rows_per = ((n + nsplit - 1) / nsplit + KC - 1) / KC * KC;
  a.ldo = bcols;
  a.out64 = out64;
  a.out64_split = (int64_t)acols * bcols;
  a.tiles_b = (bcols + 63) / 64;
  a.err = ctx->d_err;
  a.timeout_ns = ctx->timeout_ns;
  const int tiles_a = (acols + 63) / 64;
  return launch<2, 64, 1>(ctx, a, dim3((unsigned)(tiles_a * a.tiles_b), (unsigned)nsplit));
}

// The CGS2 partial layout of bcgs.cu: projection (self == 0): rows 0..63 of A chunk y = [S u0] columns
// 64 y .. 64 y + 63 (u0 = column nq), B = w X; block Grams (self == 1): rows 0..31 X^T D X, 32..63 X^T X.
int phde_tc_gram32(phde_ctx *ctx, const float *A, int lda, int nq, int ones, const float *X, const double *w,
                   int64_t n, int ncta, int nqc, int self, float *part) {
  TcGramArgs a{};
  a.A = A;
  a.lda = lda;
  a.acols = self ? 0 : nq;
  a.ones_col = (!self && ones) ? nq : -1;
  a.self_weighted = self;
  a.B = X;
  a.ldb = 32;
  a.bcols = 32;
  a.weight_b = self ? 0 : 1;
  a.w = w;
  a.n = n;
  a.rows_per = ((n + ncta - 1) / ncta + KC - 1) / KC * KC;
  a.out32 = part;
  a.err = ctx->d_err;
  a.timeout_ns = ctx->timeout_ns;
  return launch<2, 32, 0>(ctx, a, dim3((unsigned)ncta, (unsigned)nqc));
}

// Diagnostics: G = A^T diag(w) B (acols x bcols, row-major FP64) for host arrays, through the tensor-core
// kernel; the rows are split over `nsplit` CTAs per tile (0: one per 4096 rows).
extern "C" int phde_gram_f32(phde_ctx *ctx, const float *A, int lda, int acols, const float *B, int ldb, int bcols,
                             const double *w, int64_t n, int nsplit, double *G) {
  if (!ctx) return PHDE_ERR_INVALID;
  if (!A || !B || !G || n < 0 || acols < 1 || bcols < 1 || lda < acols || ldb < bcols || acols > 1024 ||
      bcols > 1024)
    return phde_fail(ctx, PHDE_ERR_INVALID, "phde_gram_f32: bad arguments");
  PHDE_CK(ctx, cudaSetDevice(ctx->device));
  if (nsplit <= 0) nsplit = (int)std::max<int64_t>(1, std::min<int64_t>((n + 4095) / 4096, 4096));
  float *dA = (float *)phde_buf(ctx, "gram.A", sizeof(float) * std::max<int64_t>(1, n * lda));
  float *dB = (float *)phde_buf(ctx, "gram.B", sizeof(float) * std::max<int64_t>(1, n * ldb));
  double *dw = w ? (double *)phde_buf(ctx, "gram.w", sizeof(double) * std::max<int64_t>(1, n)) : nullptr;
  double *part = (double *)phde_buf(ctx, "gram.part", sizeof(double) * (size_t)nsplit * acols * bcols);
  double *dG = (double *)phde_buf(ctx, "gram.G", sizeof(double) * (size_t)acols * bcols);
  if (!dA || !dB || (w && !dw) || !part || !dG) return PHDE_ERR_OOM;
  if (n > 0) {
    PHDE_CK(ctx, cudaMemcpyAsync(dA, A, sizeof(float) * n * lda, cudaMemcpyHostToDevice, ctx->stream));
    PHDE_CK(ctx, cudaMemcpyAsync(dB, B, sizeof(float) * n * ldb, cudaMemcpyHostToDevice, ctx->stream));
    if (w) PHDE_CK(ctx, cudaMemcpyAsync(dw, w, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  }
  PHDE_CK(ctx, cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
  int rc = phde_tc_gram64(ctx, dA, lda, acols, dB, ldb, bcols, dw, n, nsplit, part);
  if (rc) return rc;
  const int64_t cnt = (int64_t)acols * bcols;
  tc_sum_parts_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((cnt + 255) / 256, 1024)), 256, 0,
                        ctx->stream>>>(part, nsplit, cnt, cnt, dG);
  PHDE_LAUNCHED(ctx);
  PHDE_CK(ctx, cudaMemcpyAsync(G, dG, sizeof(double) * cnt, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return phde_check_device_err(ctx, "phde_gram_f32");
}
