// msbfs.cu -- multi-source breadth-first search with per-vertex source bitsets (one persistent launch).
//
// Up to 64*W sources (W <= 4 words) are searched together.  Every vertex keeps a `seen` bitset (bit b:
// source b has reached it) and the frontier bitset of the current level.  One level is a pull sweep:
// an unsaturated vertex ORs the frontier words of its neighbours, keeps the bits it has not seen,
// records hop distance L+1 for each of them and publishes them as its next-level frontier.  The
// adjacency is read once per level for all sources, and a vertex every source has reached drops out.
// Rows above MS_HEAVY neighbours (R-MAT hubs) are cut into chunks whose partial ORs are combined with
// atomicOr before the same finalisation; OR is order-free, so the result is deterministic.
//
// Used where all sources are known up front -- random pivot strategies, learned pivots, and
// phde_distances -- so the reference's one-BFS-per-pivot loop (ParHDE.cpp:158-175,
// DrawingBase.cpp:173-190) becomes one sweep per level.  Hop distances are unique: every column equals
// the one-source BFS column bit for bit.
#include "ctx.h"

namespace {

constexpr int MS_THREADS = 512;
constexpr int MS_MAXW = 4;
constexpr int64_t MS_HEAVY = 1024;
constexpr int64_t MS_CHUNK = 1024;

struct MsArgs {
  const int64_t *off;
  const uint32_t *adj;
  int64_t n;
  int W;           // words per vertex
  int nsrc;        // sources this sweep
  const int64_t *src;
  int32_t *D;      // column b of this sweep at D + b*n (int32, pre-filled with -1)
  ull *seen;       // [n*W]
  ull *front[2];   // [n*W] each, double buffered
  ull *hacc;       // [n*W] partial ORs of heavy rows (zeroed)
  const int64_t *heavy_rows;  // rows with degree > MS_HEAVY
  int64_t nheavy;
  const int64_t *chunk_row;   // heavy-row chunks: row and first edge
  const int64_t *chunk_e0;
  int64_t nchunks;
  unsigned *active;           // [3] new-bit flags: level L sets slot L%3 and clears slot (L+1)%3
  int *levels_out;
  GridSync *gs;
  int *err;
  uint64_t timeout_ns;
};

__device__ __forceinline__ void ms_finalise(const MsArgs &a, int64_t v, const ull *acc, ull *fnext, int32_t L,
                                            bool &any) {
  for (int w = 0; w < a.W; w++) {
    const ull s = a.seen[v * a.W + w];
    const ull nw = acc[w] & ~s;
    fnext[v * a.W + w] = nw;
    if (nw) {
      any = true;
      a.seen[v * a.W + w] = s | nw;
      ull m = nw;
      while (m) {
        const int b = __ffsll((long long)m) - 1;
        m &= m - 1;
        a.D[(int64_t)(w * 64 + b) * a.n + v] = L + 1;
      }
    }
  }
}

__global__ void __launch_bounds__(MS_THREADS) msbfs_kernel(MsArgs a) {
  const int64_t n = a.n;
  const int W = a.W;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, gts = (int64_t)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  const int64_t gw = gt >> 5, gws = gts >> 5;
  // full mask of the valid source bits per word
  ull full[MS_MAXW];
  for (int w = 0; w < MS_MAXW; w++) {
    const int bits = a.nsrc - 64 * w;
    full[w] = bits >= 64 ? ~0ull : (bits <= 0 ? 0ull : ((1ull << bits) - 1ull));
  }
  // level 0: every source sees itself
  if (gt == 0)
    for (int b = 0; b < a.nsrc; b++) {
      const int64_t s = a.src[b];
      atomicOr(a.seen + s * W + (b >> 6), 1ull << (b & 63));
      atomicOr(a.front[0] + s * W + (b >> 6), 1ull << (b & 63));
      a.D[(int64_t)b * n + s] = 0;
    }
  if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
  int32_t L = 0;
  for (;; L++) {
    const ull *fcur = a.front[L & 1];
    ull *fnext = a.front[(L + 1) & 1];
    // slot (L+1)%3 was last read after level L-2's final barrier, which every block has passed
    if (gt == 0) a.active[(L + 1) % 3] = 0u;
    bool any = false;
    // light rows: one thread per vertex
    for (int64_t v = gt; v < n; v += gts) {
      const int64_t e0 = a.off[v], e1 = a.off[v + 1];
      if (e1 - e0 > MS_HEAVY) continue;
      bool sat = true;
      for (int w = 0; w < W; w++) sat &= (a.seen[v * W + w] == full[w]);
      if (sat) {
        for (int w = 0; w < W; w++) fnext[v * W + w] = 0ull;
        continue;
      }
      ull acc[MS_MAXW] = {0ull, 0ull, 0ull, 0ull};
      for (int64_t e = e0; e < e1; e++) {
        const int64_t u = __ldg(a.adj + e);
        for (int w = 0; w < W; w++) acc[w] |= __ldcg(fcur + u * W + w);
      }
      ms_finalise(a, v, acc, fnext, L, any);
    }
    // heavy-row chunks: one warp per chunk, OR-reduced, combined with atomicOr
    for (int64_t c = gw; c < a.nchunks; c += gws) {
      const int64_t v = a.chunk_row[c], e0 = a.chunk_e0[c], e1 = min(a.off[v + 1], e0 + MS_CHUNK);
      ull acc[MS_MAXW] = {0ull, 0ull, 0ull, 0ull};
      for (int64_t e = e0 + lane; e < e1; e += 32) {
        const int64_t u = __ldg(a.adj + e);
        for (int w = 0; w < W; w++) acc[w] |= __ldcg(fcur + u * W + w);
      }
      for (int w = 0; w < W; w++) {
        ull x = acc[w];
        for (int o = 16; o > 0; o >>= 1) x |= __shfl_xor_sync(PHDE_FULL_MASK, x, o);
        if (lane == 0 && x) atomicOr(a.hacc + v * W + w, x);
      }
    }
    if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
    for (int64_t h = gt; h < a.nheavy; h += gts) {
      const int64_t v = a.heavy_rows[h];
      ull acc[MS_MAXW] = {0ull, 0ull, 0ull, 0ull};
      for (int w = 0; w < W; w++) {
        acc[w] = __ldcg(a.hacc + v * W + w);
        a.hacc[v * W + w] = 0ull;
      }
      ms_finalise(a, v, acc, fnext, L, any);
    }
    if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(a.active + (L % 3), 1u);
    if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
    if (__ldcg(a.active + (L % 3)) == 0u) break;
  }
  if (gt == 0) *a.levels_out = L + 1;
}

__global__ void ms_heavy_plan_kernel(const int64_t *off, int64_t n, int64_t *heavy_rows, int64_t *chunk_row,
                                     int64_t *chunk_e0, ull *counts) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e0 = off[v], deg = off[v + 1] - e0;
    if (deg <= MS_HEAVY) continue;
    heavy_rows[atomicAdd(counts, 1ull)] = v;
    const int64_t nch = (deg + MS_CHUNK - 1) / MS_CHUNK;
    const int64_t base = (int64_t)atomicAdd(counts + 1, (ull)nch);
    for (int64_t c = 0; c < nch; c++) {
      chunk_row[base + c] = v;
      chunk_e0[base + c] = e0 + c * MS_CHUNK;
    }
  }
}

// sum of squares of every distance column (exact integers)
__global__ void col_sumsq_kernel(const int32_t *D, int64_t n, int ncols, ull *out, int *unreached) {
  __shared__ ull red[32];
  for (int c = blockIdx.y; c < ncols; c += gridDim.y) {
    ull s = 0;
    int bad = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      const int32_t d = D[(int64_t)c * n + i];
      if (d < 0) bad = 1;
      else s += (ull)d * (ull)d;
    }
    s = block_sum(s, red);
    if (threadIdx.x == 0) atomicAdd(out + c, s);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(unreached, 1);
  }
}

}  // namespace

// Distance columns for `nsrc` given sources (device array) into D (n * nsrc, column-major, int32,
// -1 when unreached); sweeps of up to 256 sources.  If sumsq != nullptr, also the exact sum of squares
// of every column, and *h_unreached = whether any entry stayed unreached (synchronises).
int phde_msbfs(phde_ctx *ctx, const int64_t *d_src, int nsrc, int32_t *D, unsigned long long *sumsq,
               int *h_unreached) {
  const int64_t n = ctx->n;
  if (nsrc < 1) return PHDE_OK;
  const int Wmax = MS_MAXW;
  ull *seen = (ull *)phde_buf(ctx, "ms.seen", sizeof(ull) * n * Wmax);
  ull *f0 = (ull *)phde_buf(ctx, "ms.f0", sizeof(ull) * n * Wmax);
  ull *f1 = (ull *)phde_buf(ctx, "ms.f1", sizeof(ull) * n * Wmax);
  ull *hacc = (ull *)phde_buf(ctx, "ms.hacc", sizeof(ull) * n * Wmax);
  const int64_t cap_h = ctx->nnz / MS_HEAVY + 1, cap_c = ctx->nnz / MS_CHUNK + cap_h + 1;
  int64_t *hrows = (int64_t *)phde_buf(ctx, "ms.hrows", sizeof(int64_t) * cap_h);
  int64_t *crow = (int64_t *)phde_buf(ctx, "ms.crow", sizeof(int64_t) * cap_c);
  int64_t *ce0 = (int64_t *)phde_buf(ctx, "ms.ce0", sizeof(int64_t) * cap_c);
  ull *counts = (ull *)phde_buf(ctx, "ms.counts", sizeof(ull) * 2);
  unsigned *active = (unsigned *)phde_buf(ctx, "ms.active", sizeof(unsigned) * 3);
  int *levels = (int *)phde_buf(ctx, "ms.levels", sizeof(int));
  int *unr = (int *)phde_buf(ctx, "ms.unreached", sizeof(int));
  if (!seen || !f0 || !f1 || !hacc || !hrows || !crow || !ce0 || !counts || !active || !levels || !unr)
    return PHDE_ERR_OOM;
  if (ctx->ms_plan_epoch != ctx->graph_epoch) {
    PHDE_CK(ctx, cudaMemsetAsync(counts, 0, sizeof(ull) * 2, ctx->stream));
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->nsm * 8));
    ms_heavy_plan_kernel<<<g, 256, 0, ctx->stream>>>(ctx->d_off, n, hrows, crow, ce0, counts);
    PHDE_LAUNCHED(ctx);
    ull h[2];
    PHDE_CK(ctx, cudaMemcpyAsync(h, counts, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->ms_nheavy = (int64_t)h[0];
    ctx->ms_nchunks = (int64_t)h[1];
    ctx->ms_plan_epoch = ctx->graph_epoch;
  }
  PHDE_CK(ctx, cudaMemsetAsync(D, 0xff, sizeof(int32_t) * (size_t)n * nsrc, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(hacc, 0, sizeof(ull) * n * Wmax, ctx->stream));
  int per_sm = 0;
  PHDE_CK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, msbfs_kernel, MS_THREADS, 0));
  if (per_sm < 1) return phde_fail(ctx, PHDE_ERR_CUDA, "msbfs kernel cannot be resident");
  per_sm = std::min(per_sm, 4);
  for (int s0 = 0; s0 < nsrc; s0 += 64 * Wmax) {
    const int ns = std::min(nsrc - s0, 64 * Wmax);
    const int W = (ns + 63) / 64;
    PHDE_CK(ctx, cudaMemsetAsync(seen, 0, sizeof(ull) * n * W, ctx->stream));
    PHDE_CK(ctx, cudaMemsetAsync(f0, 0, sizeof(ull) * n * W, ctx->stream));
    PHDE_CK(ctx, cudaMemsetAsync(active, 0, sizeof(unsigned) * 3, ctx->stream));
    int rc = phde_reset_sync(ctx);
    if (rc) return rc;
    MsArgs a;
    a.off = ctx->d_off;
    a.adj = ctx->d_adj;
    a.n = n;
    a.W = W;
    a.nsrc = ns;
    a.src = d_src + s0;
    a.D = D + (int64_t)s0 * n;
    a.seen = seen;
    a.front[0] = f0;
    a.front[1] = f1;
    a.hacc = hacc;
    a.heavy_rows = hrows;
    a.nheavy = ctx->ms_nheavy;
    a.chunk_row = crow;
    a.chunk_e0 = ce0;
    a.nchunks = ctx->ms_nchunks;
    a.active = active;
    a.levels_out = levels;
    a.gs = ctx->d_sync;
    a.err = ctx->d_err;
    a.timeout_ns = ctx->timeout_ns;
    void *args[] = {&a};
    cudaEventRecord(ctx->kev[0], ctx->stream);
    PHDE_CK(ctx, cudaLaunchCooperativeKernel((const void *)msbfs_kernel, dim3(ctx->nsm * per_sm), dim3(MS_THREADS),
                                             args, 0, ctx->stream));
    PHDE_LAUNCHED(ctx);
    cudaEventRecord(ctx->kev[1], ctx->stream);
    ctx->kev_pending = true;
    if ((rc = phde_check_device_err(ctx, "multi-source BFS"))) return rc;
  }
  if (sumsq) {
    PHDE_CK(ctx, cudaMemsetAsync(sumsq, 0, sizeof(ull) * nsrc, ctx->stream));
    PHDE_CK(ctx, cudaMemsetAsync(unr, 0, sizeof(int), ctx->stream));
    const int gx = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 64));
    col_sumsq_kernel<<<dim3(gx, std::min(nsrc, 1024)), 256, 0, ctx->stream>>>(D, n, nsrc, sumsq, unr);
    PHDE_LAUNCHED(ctx);
    int h = 0;
    PHDE_CK(ctx, cudaMemcpyAsync(&h, unr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (h_unreached) *h_unreached = h;
  }
  return PHDE_OK;
}
