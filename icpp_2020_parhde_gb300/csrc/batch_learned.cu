// batch_learned.cu -- learned pivots for batched layouts (phde_layout_batched with PHDE_STRAT_LEARNED).
//
// The single-graph learned strategy (api.cu, learned.cu, msbfs.cu) per graph of a batch, every step over the
// disjoint union at once and without a host round trip, so that the whole batched layout stays one captured
// sequence:
//   warm start    PHDE_LEARNED_WARM exact Kcenters passes of every graph (the batched Kcenters of kcenters.cu);
//   scores        the per-vertex features and the MLP (learned.cu), each graph's features normalised by its
//                 own maxima -- the scores a single-graph call gives that graph;
//   candidates    each graph's 256 best-scored vertices (score descending, index ascending on ties), one CTA per
//                 graph: a radix select on the scores' bits and a bitonic sort;
//   one sweep     the multi-source BFS from all graphs' candidates together, graph b's candidate i searching
//                 with bit i (the components never meet, so the bits do not mix);
//   order         farthest-point selection per graph on the exact candidate distances, seeded with the warm
//                 pivots (one CTA per graph; the host loop of the single-graph strategy, lowest index on ties);
//   columns       the chosen candidates' distance columns into D with their exact sums of squares per graph.
// The rest is the batched pipeline of batch.cu.
#include <algorithm>
#include <vector>

#include "ctx.h"

int phde_run_bfs_batched_blocks(phde_ctx *ctx, int P, const int32_t *d_order, int32_t *d_D, int64_t *d_sources,
                                unsigned long long *d_sumsq, unsigned long long *d_edges);
int phde_batch_scores(phde_ctx *ctx, const float *d_weights, const int32_t *d_d0, const float **score_out);
int phde_msbfs_record_batched(phde_ctx *ctx, const int64_t *d_src, int nlist, int period, uint16_t **R_out,
                              int *RW_out);

namespace {

constexpr int BL_M = PHDE_LEARNED_CANDIDATES;  // candidates per graph
constexpr int TM_THREADS = 512;

__device__ __forceinline__ uint32_t score_key(float s) { return __float_as_uint(s); }  // scores are >= 0

// Graph b's BL_M best-scored vertices, best first (score descending, then index ascending): cand[b * BL_M + i].
// Every graph has more than BL_M vertices.
__global__ void __launch_bounds__(TM_THREADS) batch_topm_kernel(const float *score, const int64_t *vbase,
                                                                int64_t *cand) {
  __shared__ unsigned hist[2048];
  __shared__ unsigned s_bin, s_need, s_cnt, s_eq;
  __shared__ unsigned s_wtot[TM_THREADS / 32];
  __shared__ unsigned long long keys[BL_M];
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t v0 = vbase[b], v1 = vbase[b + 1];
  // radix select of the BL_M-th largest key: 11, 11 and 10 bits from the top
  unsigned prefix = 0, mask = 0, need = BL_M;
  const int shifts[3] = {21, 10, 0}, widths[3] = {11, 11, 10};
  for (int pass = 0; pass < 3; pass++) {
    const int sh = shifts[pass], nb = 1 << widths[pass];
    for (int i = tid; i < nb; i += TM_THREADS) hist[i] = 0;
    __syncthreads();
    for (int64_t v = v0 + tid; v < v1; v += TM_THREADS) {
      const uint32_t key = score_key(score[v]);
      if ((key & mask) == prefix) atomicAdd(&hist[(key >> sh) & (nb - 1)], 1u);
    }
    __syncthreads();
    if (tid == 0) {
      unsigned acc = 0;
      int bin = nb - 1;
      for (; bin > 0; bin--) {
        if (acc + hist[bin] >= need) break;
        acc += hist[bin];
      }
      s_bin = (unsigned)bin;
      s_need = need - acc;  // keys of this bin still to take
    }
    __syncthreads();
    prefix |= s_bin << sh;
    mask |= (unsigned)(nb - 1) << sh;
    need = s_need;
    __syncthreads();
  }
  // prefix is now the threshold key T: every key above it, and the `need` lowest-index keys equal to it
  if (tid == 0) {
    s_cnt = 0;
    s_eq = 0;
  }
  __syncthreads();
  for (int64_t base = v0; base < v1; base += TM_THREADS) {
    const int64_t v = base + tid;
    uint32_t key = 0;
    bool gt = false, eq = false;
    if (v < v1) {
      key = score_key(score[v]);
      gt = key > prefix;
      eq = key == prefix;
    }
    if (gt) keys[atomicAdd(&s_cnt, 1u)] = ((ull)(~key) << 32) | (ull)(v - v0);
    // equal keys in index order: block-wide rank through the warps' ballots
    const unsigned bal = __ballot_sync(PHDE_FULL_MASK, eq);
    if (lane == 0) s_wtot[warp] = __popc(bal);
    __syncthreads();
    unsigned before = s_eq;
    for (int w = 0; w < warp; w++) before += s_wtot[w];
    const unsigned rank = before + __popc(bal & ((1u << lane) - 1u));
    unsigned tot = 0;
    for (int w = 0; w < TM_THREADS / 32; w++) tot += s_wtot[w];
    if (eq && rank < need) keys[BL_M - need + rank] = ((ull)(~key) << 32) | (ull)(v - v0);
    __syncthreads();
    if (tid == 0) s_eq += tot;
    __syncthreads();
  }
  // bitonic sort of the BL_M keys, ascending: score descending, local index ascending
  for (int size = 2; size <= BL_M; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      __syncthreads();
      if (tid < BL_M) {
        const int j = tid ^ stride;
        if (j > tid) {
          const bool up = (tid & size) == 0;
          const ull x = keys[tid], y = keys[j];
          if ((x > y) == up) {
            keys[tid] = y;
            keys[j] = x;
          }
        }
      }
    }
  __syncthreads();
  if (tid < BL_M) cand[(int64_t)b * BL_M + tid] = v0 + (int64_t)(keys[tid] & 0xffffffffull);
}

// Farthest-point order of graph b's candidates (one CTA of BL_M threads, thread i = candidate i): the minimum
// distance to the warm pivots, then P - P0 times the unused candidate farthest from every pivot taken (lowest
// index on ties), its record column folded into the minima.  ord[b][p] = candidate index, sources[(P0 + p) B + b].
__global__ void __launch_bounds__(BL_M) batch_fps_kernel(const int32_t *D, int64_t N, int P0, int P, const uint16_t *R,
                                                         int RW, const int64_t *cand, int B, int *ord,
                                                         int64_t *sources) {
  __shared__ ull red[32];
  const int b = blockIdx.x, i = threadIdx.x;
  const int64_t c = cand[(int64_t)b * BL_M + i];
  int32_t mind = INT32_MAX;
  for (int p = 0; p < P0; p++) mind = min(mind, D[(int64_t)p * N + c]);
  bool used = false;
  const int Pn = P - P0;
  for (int step = 0; step < Pn; step++) {
    const ull key = used ? 0ull : (((ull)(uint32_t)mind + 1ull) << 32) | (ull)(0xffffffffu - (uint32_t)i);
    const ull best = block_max_u64(key, red);
    const int ib = (int)(0xffffffffu - (uint32_t)(best & 0xffffffffull));
    if (i == ib) used = true;
    if (i == 0) {
      ord[(int64_t)b * Pn + step] = ib;
      sources[(int64_t)(P0 + step) * B + b] = cand[(int64_t)b * BL_M + ib];
    }
    mind = min(mind, (int32_t)R[c * RW + ib] - 1);
  }
}

// D[(P0 + p) N + v] = R[v][ord[g(v)][p]] - 1 through 32-row shared-memory tiles; exact sums of squares per
// (column, graph) into sumsq[(P0 + p) B + g], one atomic per warp when its 32 rows share a graph.
__global__ void batch_record_cols_kernel(const uint16_t *R, int RW, int64_t N, const int32_t *gid, const int *ord,
                                         int P0, int P, int B, int32_t *D, ull *sumsq) {
  extern __shared__ uint16_t tile[];  // [32][RW + 2]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int TLD = RW + 2, hw = RW / 2, Pn = P - P0;
  for (int64_t v0 = (int64_t)blockIdx.x * 32; v0 < N; v0 += (int64_t)gridDim.x * 32) {
    const int rows = N - v0 < 32 ? (int)(N - v0) : 32;
    __syncthreads();
    const uint32_t *src = (const uint32_t *)(R + v0 * RW);
    uint32_t *dst = (uint32_t *)tile;
    for (int i = threadIdx.x; i < rows * hw; i += blockDim.x) {
      const int r = i / hw, cc = i - r * hw;
      dst[r * (TLD / 2) + cc] = src[i];
    }
    __syncthreads();
    const int g = lane < rows ? gid[v0 + lane] : -1;
    const int g0 = __shfl_sync(PHDE_FULL_MASK, g, 0);
    const bool one = __all_sync(PHDE_FULL_MASK, g == g0 || g < 0);
    for (int p = warp; p < Pn; p += nw) {
      uint32_t sq = 0;
      if (lane < rows) {
        const int d = (int)tile[lane * TLD + ord[(int64_t)g * Pn + p]] - 1;
        D[(int64_t)(P0 + p) * N + v0 + lane] = d;
        sq = (uint32_t)(d * d);
      }
      if (one) {
        // d < 2^16: the halves of d^2 sum without overflow over a warp
        const ull tot = ((ull)__reduce_add_sync(PHDE_FULL_MASK, sq >> 16) << 16) +
                        (ull)__reduce_add_sync(PHDE_FULL_MASK, sq & 0xffffu);
        if (lane == 0 && tot) atomicAdd(sumsq + (int64_t)(P0 + p) * B + g0, tot);
      } else if (sq) {
        atomicAdd(sumsq + (int64_t)(P0 + p) * B + g, (ull)sq);
      }
    }
  }
}

}  // namespace

// Learned pivots of every graph of the uploaded batch: D (N x P int32, column-major), sources[p * B + b] and the
// exact column sums of squares sumsq[p * B + b] for all P = 3k passes, as the batched Kcenters gives them.
// d_weights: the pivot model on the device.  No host synchronisation.
int phde_batch_learned_pivots(phde_ctx *ctx, int P, const float *d_weights, int32_t *D, int64_t *sources, ull *sumsq,
                              ull *edges) {
  const int64_t N = ctx->n;
  const int B = ctx->batch_B;
  const int P0 = std::min(P, PHDE_LEARNED_WARM);
  int rc;
  if (ctx->batch_blocks)
    rc = phde_run_bfs_batched_blocks(ctx, P0, ctx->d_order, D, sources, sumsq, edges);
  else
    rc = phde_run_bfs_passes(ctx, P0, 3, nullptr, D, sources, sumsq, edges, 1);
  if (rc) return rc;
  if (P0 == P) return PHDE_OK;
  const int32_t *mind0 = (const int32_t *)phde_buf(ctx, "kc.min_d", sizeof(int32_t) * N);
  int64_t *cand = (int64_t *)phde_buf(ctx, "lpb.cand", sizeof(int64_t) * (size_t)B * BL_M);
  int *ord = (int *)phde_buf(ctx, "lpb.ord", sizeof(int) * (size_t)B * (P - P0));
  if (!mind0 || !cand || !ord) return PHDE_ERR_OOM;
  const float *score;
  if ((rc = phde_batch_scores(ctx, d_weights, mind0, &score))) return rc;
  batch_topm_kernel<<<B, TM_THREADS, 0, ctx->stream>>>(score, ctx->d_vbase, cand);
  PHDE_LAUNCHED(ctx);
  uint16_t *R;
  int RW;
  if ((rc = phde_msbfs_record_batched(ctx, cand, B * BL_M, BL_M, &R, &RW))) return rc;
  batch_fps_kernel<<<B, BL_M, 0, ctx->stream>>>(D, N, P0, P, R, RW, cand, B, ord, sources);
  PHDE_LAUNCHED(ctx);
  PHDE_CK(ctx, cudaMemsetAsync(sumsq + (int64_t)P0 * B, 0, sizeof(ull) * (size_t)(P - P0) * B, ctx->stream));
  const size_t smem = sizeof(uint16_t) * 32 * (size_t)(RW + 2);
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((N + 31) / 32, (int64_t)ctx->nsm * 8));
  batch_record_cols_kernel<<<grid, 256, smem, ctx->stream>>>(R, RW, N, ctx->d_gid, ord, P0, P, B, D, sumsq);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}
