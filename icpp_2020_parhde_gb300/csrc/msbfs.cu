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
#include <vector>

#include "ctx.h"

namespace {

constexpr int MS_THREADS = 512;
constexpr int MS_MAXW = 4;
constexpr int64_t MS_HEAVY = 256;  // rows above this are cut into chunks (one warp per chunk)
constexpr int64_t MS_CHUNK = 256;
constexpr int MS_GROUP = 8;        // lanes per light row

struct MsArgs {
  const int64_t *off;
  const uint32_t *adj;
  int64_t n;
  int W;           // words per vertex
  int nsrc;        // sources this sweep
  const int64_t *src;
  uint16_t *R;     // row-major n x RW distance record: R[v*RW + b] = level + 1 (0 = unreached)
  int RW;          // row width (all sources of all sweeps, a multiple of 64)
  int col0;        // first source of this sweep within the row
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

// 4-bit group -> 4 x 16-bit lanes of ones (the lanes whose source bit is set)
__constant__ ull kNibbleLanes[16] = {
    0x0000000000000000ull, 0x000000000000ffffull, 0x00000000ffff0000ull, 0x00000000ffffffffull,
    0x0000ffff00000000ull, 0x0000ffff0000ffffull, 0x0000ffffffff0000ull, 0x0000ffffffffffffull,
    0xffff000000000000ull, 0xffff00000000ffffull, 0xffff0000ffff0000ull, 0xffff0000ffffffffull,
    0xffffffff00000000ull, 0xffffffff0000ffffull, 0xffffffffffff0000ull, 0xffffffffffffffffull};

__device__ __forceinline__ void ms_finalise(const MsArgs &a, int64_t v, const ull *acc, ull *fnext, int32_t L,
                                            bool &any) {
  const ull lvl = 0x0001000100010001ull * (ull)(uint16_t)(L + 2);  // level L+1, stored +1
  for (int w = 0; w < a.W; w++) {
    const ull s = a.seen[v * a.W + w];
    const ull nw = acc[w] & ~s;
    fnext[v * a.W + w] = nw;
    if (nw) {
      any = true;
      a.seen[v * a.W + w] = s | nw;
      ull *row = (ull *)(a.R + v * a.RW + a.col0 + 64 * w);  // 16 groups of 4 sources, 8 bytes each
      for (int gi = 0; gi < 16; gi++) {
        const unsigned nib = (unsigned)(nw >> (4 * gi)) & 15u;
        if (nib) row[gi] |= kNibbleLanes[nib] & lvl;
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
      a.R[s * a.RW + a.col0 + b] = 1;  // level 0
    }
  if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
  int32_t L = 0;
  for (;; L++) {
    const ull *fcur = a.front[L & 1];
    ull *fnext = a.front[(L + 1) & 1];
    // slot (L+1)%3 was last read after level L-2's final barrier, which every block has passed
    if (gt == 0) a.active[(L + 1) % 3] = 0u;
    bool any = false;
    // light rows: a group of MS_GROUP lanes per vertex, neighbours strided across the group.  A warp holds
    // 32/MS_GROUP groups with consecutive ids; the loop runs over the warp's first group id so its trip
    // count is warp-uniform and every lane reaches the group shuffles.
    {
      const int gl = lane & (MS_GROUP - 1);
      const int64_t gstr = gts / MS_GROUP;                         // groups in the grid
      const int64_t wfirst = (gt >> 5) * (32 / MS_GROUP);          // this warp's first group id
      for (int64_t i0 = wfirst; i0 < n; i0 += gstr) {
        const int64_t v = i0 + (lane / MS_GROUP);
        bool act = v < n;
        int64_t e0 = 0, e1 = 0;
        if (act) {
          e0 = a.off[v];
          e1 = a.off[v + 1];
          if (e1 - e0 > MS_HEAVY) act = false;
        }
        bool sat = true;
        if (act)
          for (int w = 0; w < W; w++) sat &= (a.seen[v * W + w] == full[w]);
        ull acc[MS_MAXW] = {0ull, 0ull, 0ull, 0ull};
        if (act && !sat)
          for (int64_t e = e0 + gl; e < e1; e += MS_GROUP) {
            const int64_t u = __ldg(a.adj + e);
            for (int w = 0; w < W; w++) acc[w] |= __ldcg(fcur + u * W + w);
          }
        for (int w = 0; w < MS_MAXW; w++)
          for (int o = MS_GROUP / 2; o > 0; o >>= 1) acc[w] |= __shfl_xor_sync(PHDE_FULL_MASK, acc[w], o, MS_GROUP);
        if (act && gl == 0) {
          if (sat) {
            for (int w = 0; w < W; w++) fnext[v * W + w] = 0ull;
          } else {
            ms_finalise(a, v, acc, fnext, L, any);
          }
        }
      }
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

// D[p*n + v] = R[v*RW + cols[p]] - 1 for the requested columns, through 32-row shared-memory tiles;
// per-column exact sums of squares and an unreached flag on the way.
__global__ void gather_columns_kernel(const uint16_t *R, int64_t n, int RW, const int *cols, int ncols, int32_t *D,
                                      ull *sumsq, int *unreached) {
  extern __shared__ uint16_t tile[];  // [32][RW]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int bad = 0;
  for (int64_t v0 = (int64_t)blockIdx.x * 32; v0 < n; v0 += (int64_t)gridDim.x * 32) {
    const int rows = n - v0 < 32 ? (int)(n - v0) : 32;
    __syncthreads();
    const ull *src = (const ull *)(R + v0 * RW);
    ull *dst = (ull *)tile;
    for (int i = threadIdx.x; i < rows * RW / 4; i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    for (int p = warp; p < ncols; p += nw) {
      int d = -1;
      if (lane < rows) {
        d = (int)tile[lane * RW + cols[p]] - 1;
        D[(int64_t)p * n + v0 + lane] = d;
        bad |= d < 0;
      }
      const ull sq = d > 0 ? (ull)d * (ull)d : 0ull;
      const ull tot = warp_sum(sq);
      if (lane == 0 && tot) atomicAdd(sumsq + p, tot);
    }
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(unreached, 1);
}

}  // namespace

// Heavy-row chunk plan of the multi-source BFS (rows above MS_HEAVY, chunks of MS_CHUNK edges), built once
// per uploaded graph; also used by the learned-pivot feature kernel.
int phde_heavy_chunks(phde_ctx *ctx, const int64_t **chunk_row, const int64_t **chunk_e0, int64_t *nchunks,
                      int64_t *chunk) {
  const int64_t n = ctx->n;
  const int64_t cap_h = ctx->nnz / MS_HEAVY + 1, cap_c = ctx->nnz / MS_CHUNK + cap_h + 1;
  int64_t *hrows = (int64_t *)phde_buf(ctx, "ms.hrows", sizeof(int64_t) * cap_h);
  int64_t *crow = (int64_t *)phde_buf(ctx, "ms.crow", sizeof(int64_t) * cap_c);
  int64_t *ce0 = (int64_t *)phde_buf(ctx, "ms.ce0", sizeof(int64_t) * cap_c);
  ull *counts = (ull *)phde_buf(ctx, "ms.counts", sizeof(ull) * 2);
  if (!hrows || !crow || !ce0 || !counts) return PHDE_ERR_OOM;
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
  *chunk_row = crow;
  *chunk_e0 = ce0;
  *nchunks = ctx->ms_nchunks;
  *chunk = MS_CHUNK;
  return PHDE_OK;
}

// Multi-source BFS from `nsrc` sources (device array; sweeps of up to 256).  The result is the row-major
// record R (n x RW uint16, RW = nsrc rounded up to 64; level + 1, 0 = unreached), returned through *R_out.
int phde_msbfs_record(phde_ctx *ctx, const int64_t *d_src, int nsrc, uint16_t **R_out, int *RW_out) {
  const int64_t n = ctx->n;
  if (nsrc < 1) return PHDE_ERR_INVALID;
  const int RW = (nsrc + 63) / 64 * 64;
  const int Wmax = MS_MAXW;
  uint16_t *R = (uint16_t *)phde_buf(ctx, "ms.R", sizeof(uint16_t) * n * RW);
  ull *seen = (ull *)phde_buf(ctx, "ms.seen", sizeof(ull) * n * Wmax);
  ull *f0 = (ull *)phde_buf(ctx, "ms.f0", sizeof(ull) * n * Wmax);
  ull *f1 = (ull *)phde_buf(ctx, "ms.f1", sizeof(ull) * n * Wmax);
  ull *hacc = (ull *)phde_buf(ctx, "ms.hacc", sizeof(ull) * n * Wmax);
  unsigned *active = (unsigned *)phde_buf(ctx, "ms.active", sizeof(unsigned) * 3);
  int *levels = (int *)phde_buf(ctx, "ms.levels", sizeof(int));
  if (!R || !seen || !f0 || !f1 || !hacc || !active || !levels) return PHDE_ERR_OOM;
  const int64_t *crow, *ce0;
  int64_t nch, chunk;
  int rc0 = phde_heavy_chunks(ctx, &crow, &ce0, &nch, &chunk);
  if (rc0) return rc0;
  const int64_t *hrows = (const int64_t *)phde_buf(ctx, "ms.hrows", 0);
  PHDE_CK(ctx, cudaMemsetAsync(R, 0, sizeof(uint16_t) * (size_t)n * RW, ctx->stream));
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
    a.R = R;
    a.RW = RW;
    a.col0 = s0;
    a.seen = seen;
    a.front[0] = f0;
    a.front[1] = f1;
    a.hacc = hacc;
    a.heavy_rows = hrows;
    a.nheavy = ctx->ms_nheavy;
    a.chunk_row = crow;
    a.chunk_e0 = ce0;
    a.nchunks = nch;
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
  *R_out = R;
  *RW_out = RW;
  return PHDE_OK;
}

// Columns `h_cols` of the record into D (n x ncols int32 column-major, -1 unreached); optional exact sums
// of squares per column and the unreached flag (synchronises when either is requested).
int phde_record_columns(phde_ctx *ctx, const uint16_t *R, int RW, const int *h_cols, int ncols, int32_t *D,
                        unsigned long long *sumsq, int *h_unreached) {
  const int64_t n = ctx->n;
  int *dcols = (int *)phde_buf(ctx, "ms.cols", sizeof(int) * ncols);
  ull *ssq = sumsq ? sumsq : (ull *)phde_buf(ctx, "ms.ssq_tmp", sizeof(ull) * ncols);
  int *unr = (int *)phde_buf(ctx, "ms.unreached", sizeof(int));
  if (!dcols || !ssq || !unr) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemcpyAsync(dcols, h_cols, sizeof(int) * ncols, cudaMemcpyHostToDevice, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(ssq, 0, sizeof(ull) * ncols, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(unr, 0, sizeof(int), ctx->stream));
  const size_t smem = sizeof(uint16_t) * 32 * (size_t)RW;
  PHDE_CK(ctx, cudaFuncSetAttribute(gather_columns_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 31) / 32, (int64_t)ctx->nsm * 4));
  gather_columns_kernel<<<g, 512, smem, ctx->stream>>>(R, n, RW, dcols, ncols, D, ssq, unr);
  PHDE_LAUNCHED(ctx);
  if (sumsq || h_unreached) {
    int h = 0;
    PHDE_CK(ctx, cudaMemcpyAsync(&h, unr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (h_unreached) *h_unreached = h;
  }
  return PHDE_OK;
}

// All columns, in source order (what phde_distances and the random strategies need).
int phde_msbfs(phde_ctx *ctx, const int64_t *d_src, int nsrc, int32_t *D, unsigned long long *sumsq,
               int *h_unreached) {
  uint16_t *R;
  int RW;
  int rc = phde_msbfs_record(ctx, d_src, nsrc, &R, &RW);
  if (rc) return rc;
  std::vector<int> cols(nsrc);
  for (int i = 0; i < nsrc; i++) cols[i] = i;
  return phde_record_columns(ctx, R, RW, cols.data(), nsrc, D, sumsq, h_unreached);
}
