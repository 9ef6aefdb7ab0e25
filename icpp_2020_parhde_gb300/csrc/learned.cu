// learned.cu -- learned pivot proposal: per-vertex features and the pivot-scoring MLP.
//
// Kcenters picks pivots one at a time (ParHDE.cpp:118-157): every pivot needs the BFS of the previous
// one, so 3k dependent passes run back to back.  The learned strategy runs the first PHDE_LEARNED_WARM
// pivots as exact Kcenters passes (the farthest-first rule of ParHDE.cpp:118-157), then proposes the
// rest at once.  With d0(v) = the warm start's minimum distance from v to its pivots (Kcenters' own
// selection key):
//     f0 = log(1+deg v) / log(1+max deg)
//     f1 = log(1+sum of neighbour degrees) / log(1+max of that sum)
//     f2 = d0(v) / max d0
//     f3 = |{u in N(v): d0(u) > d0(v)}| / deg v   (share of neighbours farther from the pivots)
//   score = MLP(f): 4 -> 64 -> 64 -> 1, ReLU, FP32 (weights trained on the pivots Kcenters picks after
//           the warm start, train/train_pivot_mlp.py, compiled in from pivot_mlp_weights.h)
// The host takes the M best-scored vertices as candidates, runs ONE multi-source BFS from all of them,
// and picks the remaining pivots among them by farthest-point selection on exact distances, seeded with
// the warm-start pivots.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ctx.h"
#include "pivot_mlp_weights.h"
#include "tc_common.cuh"

namespace {

constexpr int MLP_IN = 4, MLP_H = 64;
constexpr int MLP_WEIGHTS = MLP_H * MLP_IN + MLP_H + MLP_H * MLP_H + MLP_H + MLP_H + 1;

// neighbour-degree sum and outward-neighbour count.  Rows up to FEAT_HEAVY neighbours: a group of 8 lanes
// per vertex; heavier rows (R-MAT hubs): one warp per chunk of the multi-source BFS plan, integer
// atomicAdd (exact, order-free).  hop2/outw are zeroed before the launch.
constexpr int64_t FEAT_HEAVY = 256;
// pk[v] = degree(v) << 32 | (uint32) d0[v]: what the feature pass gathers per neighbour, in one 8-byte load
__global__ void feature_pack_kernel(const int64_t *off, const int32_t *d0, int64_t n, ull *pk) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
    pk[v] = ((ull)(off[v + 1] - off[v]) << 32) | (ull)(uint32_t)d0[v];
}

__device__ __forceinline__ void feature_edge(ull pku, int32_t dv, ull &h, unsigned &o) {
  h += pku >> 32;
  o += (int32_t)(uint32_t)pku > dv ? 1u : 0u;
}

__global__ void feature_raw_kernel(const int64_t *off, const uint32_t *adj, const int32_t *d0, const ull *pk, int64_t n,
                                   const int64_t *chunk_row, const int64_t *chunk_e0, int64_t nchunks, int64_t chunk,
                                   ull *hop2, uint32_t *outw) {
  const int lane = threadIdx.x & 31, gl = lane & 7;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, gts = (int64_t)gridDim.x * blockDim.x;
  const int64_t gstr = gts / 8, wfirst = (gt >> 5) * 4;
  for (int64_t i0 = wfirst; i0 < n; i0 += gstr) {
    const int64_t v = i0 + (lane >> 3);
    ull h = 0;
    unsigned o = 0;
    bool act = v < n;
    if (act) {
      const int64_t e0 = off[v], e1 = off[v + 1];
      if (e1 - e0 > FEAT_HEAVY) {
        act = false;
      } else {
        const int32_t dv = d0[v];
        int64_t e = e0 + gl;
        for (; e + 24 < e1; e += 32) {  // four gathers in flight per lane: the loop is latency bound
          const uint32_t u0 = __ldg(adj + e), u1 = __ldg(adj + e + 8), u2 = __ldg(adj + e + 16), u3 = __ldg(adj + e + 24);
          const ull p0 = __ldg(pk + u0), p1 = __ldg(pk + u1), p2 = __ldg(pk + u2), p3 = __ldg(pk + u3);
          feature_edge(p0, dv, h, o);
          feature_edge(p1, dv, h, o);
          feature_edge(p2, dv, h, o);
          feature_edge(p3, dv, h, o);
        }
        for (; e < e1; e += 8) feature_edge(__ldg(pk + __ldg(adj + e)), dv, h, o);
      }
    }
    for (int s = 4; s > 0; s >>= 1) {
      h += __shfl_xor_sync(PHDE_FULL_MASK, h, s, 8);
      o += __shfl_xor_sync(PHDE_FULL_MASK, o, s, 8);
    }
    if (act && gl == 0) {
      hop2[v] = h;
      outw[v] = o;
    }
  }
  const int64_t gw = gt >> 5, gws = gts >> 5;
  for (int64_t c = gw; c < nchunks; c += gws) {
    const int64_t v = chunk_row[c], e0 = chunk_e0[c], e1 = min(off[v + 1], e0 + chunk);
    const int32_t dv = d0[v];
    ull h = 0;
    unsigned o = 0;
    for (int64_t e = e0 + lane; e < e1; e += 32) feature_edge(__ldg(pk + __ldg(adj + e)), dv, h, o);
    h = warp_sum(h);
    o = warp_sum(o);
    if (lane == 0) {
      atomicAdd(hop2 + v, h);
      atomicAdd(outw + v, o);
    }
  }
}

// Per-graph maxima of a batch (the disjoint union, graph of each vertex in gid): maxes[3 b .. 3 b + 2].  A warp
// whose 32 vertices lie in one graph reduces first and adds one atomic per value.
__global__ void feature_max_batched_kernel(const int64_t *off, const int32_t *d0, const ull *hop2, const int32_t *gid,
                                           int64_t n, ull *maxes) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~31ll; base < n; base += stride) {
    const int64_t v = base + lane;
    ull mdeg = 0, mhop = 0, md0 = 0;
    int g = -1;
    if (v < n) {
      mdeg = (ull)(off[v + 1] - off[v]);
      mhop = hop2[v];
      md0 = (ull)(d0[v] < 0 ? 0 : d0[v]);
      g = gid[v];
    }
    const int g0 = __shfl_sync(PHDE_FULL_MASK, g, 0);
    if (__all_sync(PHDE_FULL_MASK, g == g0)) {
      mdeg = warp_max_u64(mdeg);
      mhop = warp_max_u64(mhop);
      md0 = warp_max_u64(md0);
      if (lane == 0) {
        atomicMax(maxes + 3 * g0, mdeg);
        atomicMax(maxes + 3 * g0 + 1, mhop);
        atomicMax(maxes + 3 * g0 + 2, md0);
      }
    } else if (g >= 0) {
      atomicMax(maxes + 3 * g, mdeg);
      atomicMax(maxes + 3 * g + 1, mhop);
      atomicMax(maxes + 3 * g + 2, md0);
    }
  }
}

__global__ void feature_max_kernel(const int64_t *off, const int32_t *d0, const ull *hop2, int64_t n, ull *maxes) {
  __shared__ ull red[32];
  ull mdeg = 0, mhop = 0, md0 = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    mdeg = max(mdeg, (ull)(off[v + 1] - off[v]));
    mhop = max(mhop, hop2[v]);
    md0 = max(md0, (ull)(d0[v] < 0 ? 0 : d0[v]));
  }
  mdeg = block_max_u64(mdeg, red);
  mhop = block_max_u64(mhop, red);
  md0 = block_max_u64(md0, red);
  if (threadIdx.x == 0) {
    atomicMax(maxes, mdeg);
    atomicMax(maxes + 1, mhop);
    atomicMax(maxes + 2, md0);
  }
}

// Scores of 128 vertices per tile and 256 threads: features -> F[128][4]; layer 1 (4 -> 64, ReLU) -> H[64][128]
// (hidden unit major); layer 2 (64 -> 64, ReLU) as a register-tiled product, thread (vg, og) computing
// vertices 8 vg .. 8 vg + 7 times hidden units 4 og .. 4 og + 3 (32 FMAs per 12 shared-memory words); the
// output unit's dot product over the 64 hidden units summed across the 16 threads of a vertex group with
// shuffles; then the sigmoid and the score histogram.
constexpr int MLP_TILE = 128;
// gid (batches): the features of vertex v are normalised by its own graph's maxima, maxes[3 gid[v] ..]; no
// histogram when nbins is 0.
__global__ void __launch_bounds__(256) mlp_score_kernel(const int64_t *off, const int32_t *d0, const ull *hop2,
                                                        const uint32_t *outw, const ull *maxes, int64_t n,
                                                        const float *weights, float *score, unsigned *hist,
                                                        int nbins, const int32_t *gid) {
  __shared__ float W1[MLP_H][MLP_IN], b1[MLP_H], b2[MLP_H], w3[MLP_H];
  __shared__ __align__(16) float W2t[MLP_H][MLP_H];  // W2t[i][o] = W2[o][i]
  __shared__ float F[MLP_TILE][MLP_IN + 1];
  __shared__ float s_b3;
  // dynamic: H[i][v] (layer-1 output i of tile vertex v), then the per-block score histogram [nbins]
  extern __shared__ __align__(16) float s_dyn[];
  float(*H)[MLP_TILE] = (float(*)[MLP_TILE])s_dyn;
  unsigned *s_hist = (unsigned *)(s_dyn + MLP_H * MLP_TILE);
  const int tid = threadIdx.x;
  for (int i = tid; i < MLP_H * MLP_IN; i += blockDim.x) W1[i / MLP_IN][i % MLP_IN] = weights[i];
  const float *gb1 = weights + MLP_H * MLP_IN, *gW2 = gb1 + MLP_H, *gb2 = gW2 + MLP_H * MLP_H, *gw3 = gb2 + MLP_H;
  for (int i = tid; i < MLP_H; i += blockDim.x) {
    b1[i] = gb1[i];
    b2[i] = gb2[i];
    w3[i] = gw3[i];
  }
  for (int i = tid; i < MLP_H * MLP_H; i += blockDim.x) W2t[i % MLP_H][i / MLP_H] = gW2[i];
  if (tid == 0) s_b3 = gw3[MLP_H];
  for (int i = tid; i < nbins; i += blockDim.x) s_hist[i] = 0u;
  const float ldeg = logf(1.f + (float)maxes[0]), lhop = logf(1.f + (float)maxes[1]);
  const float md0 = maxes[2] ? (float)maxes[2] : 1.f;
  const int og = tid & 15, vg = tid >> 4;  // hidden units 4 og .. 4 og + 3, tile vertices 8 vg .. 8 vg + 7
  for (int64_t t0 = (int64_t)blockIdx.x * MLP_TILE; t0 < n; t0 += (int64_t)gridDim.x * MLP_TILE) {
    __syncthreads();  // the weights (first tile) or the previous tile's H and F are no longer read
    if (tid < MLP_TILE) {
      const int64_t v = t0 + tid;
      float f0 = 0.f, f1 = 0.f, f2 = 0.f, f3 = 0.f;
      if (v < n) {
        float ld = ldeg, lh = lhop, m0 = md0;
        if (gid) {  // this vertex's graph's maxima
          const ull *mx = maxes + 3 * (int64_t)gid[v];
          ld = logf(1.f + (float)mx[0]);
          lh = logf(1.f + (float)mx[1]);
          m0 = mx[2] ? (float)mx[2] : 1.f;
        }
        const float deg = (float)(off[v + 1] - off[v]);
        f0 = ld > 0.f ? logf(1.f + deg) / ld : 0.f;
        f1 = lh > 0.f ? logf(1.f + (float)hop2[v]) / lh : 0.f;
        f2 = (float)(d0[v] < 0 ? 0 : d0[v]) / m0;
        f3 = deg > 0.f ? (float)outw[v] / deg : 0.f;
      }
      F[tid][0] = f0;
      F[tid][1] = f1;
      F[tid][2] = f2;
      F[tid][3] = f3;
    }
    __syncthreads();
    // layer 1: thread (vg, og) fills H[4 og .. 4 og + 3][8 vg .. 8 vg + 7]
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const int v = vg * 8 + j;
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int o = og * 4 + u;
        float a = b1[o];
#pragma unroll
        for (int i = 0; i < MLP_IN; i++) a = fmaf(W1[o][i], F[v][i], a);
        H[o][v] = a > 0.f ? a : 0.f;
      }
    }
    __syncthreads();
    // layer 2 tile: acc[j][u] for vertex 8 vg + j and hidden unit 4 og + u
    float acc[8][4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const float b = b2[og * 4 + u];
#pragma unroll
      for (int j = 0; j < 8; j++) acc[j][u] = b;
    }
#pragma unroll 4
    for (int i = 0; i < MLP_H; i++) {
      const float4 ha = *(const float4 *)&H[i][vg * 8], hb = *(const float4 *)&H[i][vg * 8 + 4];
      const float4 w = *(const float4 *)&W2t[i][og * 4];
      const float hv[8] = {ha.x, ha.y, ha.z, ha.w, hb.x, hb.y, hb.z, hb.w};
      const float wv[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
      for (int j = 0; j < 8; j++)
#pragma unroll
        for (int u = 0; u < 4; u++) acc[j][u] = fmaf(wv[u], hv[j], acc[j][u]);
    }
    // output unit: sum over hidden units of w3 * ReLU(layer 2), the 16 threads of a vertex group combined
    float part[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      float p = 0.f;
#pragma unroll
      for (int u = 0; u < 4; u++) p = fmaf(w3[og * 4 + u], acc[j][u] > 0.f ? acc[j][u] : 0.f, p);
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) p += __shfl_xor_sync(PHDE_FULL_MASK, p, o);
      part[j] = p;
    }
    // lane og < 8 of the group finishes vertex 8 vg + og; the histogram count is aggregated over the warp's
    // lanes with the same bin (scores crowd into few bins, so per-vertex atomics would serialise)
    int bin = -1;
    if (og < 8) {
      float outv = part[0];
#pragma unroll
      for (int j = 1; j < 8; j++)
        if (og == j) outv = part[j];
      const int64_t v = t0 + vg * 8 + og;
      if (v < n) {
        const float pr = 1.f / (1.f + expf(-(s_b3 + outv)));
        score[v] = pr;
        if (nbins > 0) {
          bin = (int)(pr * nbins);
          bin = bin < 0 ? 0 : (bin >= nbins ? nbins - 1 : bin);
        }
      }
    }
    const unsigned same = __match_any_sync(PHDE_FULL_MASK, bin);
    if (bin >= 0 && (tid & 31) == __ffs(same) - 1) atomicAdd(s_hist + bin, (unsigned)__popc(same));
  }
  __syncthreads();
  for (int i = tid; i < nbins; i += blockDim.x)
    if (s_hist[i]) atomicAdd(hist + i, s_hist[i]);
}

// vertices whose score bin is >= bmin, compacted (order fixed afterwards on the host)
__global__ void collect_kernel(const float *score, int64_t n, int bmin, int nbins, int64_t *cand, float *cscore,
                               unsigned *count, unsigned cap) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    const float p = score[v];
    int bin = (int)(p * nbins);
    bin = bin < 0 ? 0 : (bin >= nbins ? nbins - 1 : bin);
    if (bin >= bmin) {
      const unsigned at = atomicAdd(count, 1u);
      if (at < cap) {
        cand[at] = v;
        cscore[at] = p;
      }
    }
  }
}

// Distances of every candidate to the warm-start pivots: sub[i*P0 + j] = D[j*n + cand_i]; and to the other
// candidates from the row-major record: csub[i*M + j] = R[cand_i*RW + j] - 1.
__global__ void cand_distances_kernel(const int32_t *D, int P0, const uint16_t *R, int RW, int64_t n,
                                      const int64_t *cand, int M, int32_t *sub, int32_t *csub) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < M * (M + P0); idx += gridDim.x * blockDim.x) {
    const int i = idx / (M + P0), j = idx % (M + P0);
    if (j < P0)
      sub[i * P0 + j] = D[(int64_t)j * n + cand[i]];
    else if (R)
      csub[i * M + (j - P0)] = (int32_t)R[cand[i] * RW + (j - P0)] - 1;
  }
}

// Level mode: csub[i][j] = the level whose frontier array has source j's bit at vertex cand[i] (-1: none);
// thread per (candidate, source word).
__global__ void cand_distances_lvl_kernel(const ull *lvl, int nlev, int W, int64_t n, const int64_t *cand, int M,
                                          int32_t *csub) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < M * W; idx += gridDim.x * blockDim.x) {
    const int i = idx / W, w = idx - i * W;
    const int64_t v = cand[i];
    const int nb = min(64, M - 64 * w);
    const ull valid = nb >= 64 ? ~0ull : ((1ull << nb) - 1ull);
    ull seen = 0;
    for (int L = 0; L < nlev; L++) {
      const ull x = lvl[((int64_t)L * n + v) * W + w] & valid;
      seen |= x;
      for (ull y = x; y; y &= y - 1) csub[i * M + 64 * w + __ffsll((long long)y) - 1] = L;
    }
    for (ull y = valid & ~seen; y; y &= y - 1) csub[i * M + 64 * w + __ffsll((long long)y) - 1] = -1;
  }
}

// The same scores with layer 2 on the tensor cores (tcgen05): per tile of 128 vertices the layer-1 outputs H
// (128 x 64, FP32) and, once per CTA, W2 (64 x 64) are split into three BF16 parts each and stored K-major in
// shared memory; one thread issues the MMAs of six part products (hi.hi, hi.mid, mid.hi, hi.lo, lo.hi, mid.mid
// -- the three dropped ones are below 2^-24 of the product) into an FP32 accumulator of 128 TMEM lanes x 64
// columns; warps 0..3 read their lane quarter (one vertex per lane) and finish: bias, ReLU, the output unit,
// the sigmoid and the histogram, while warps 4..7 compute the next tile's features.  FP32-faithful: the scores
// agree with the CUDA-core kernel to FP32 rounding.
// Every mbarrier wait is bounded; on expiry the kernel records PHDE_ERR_TIMEOUT and returns after its MMAs.
constexpr int TM_THREADS = 256;
constexpr int TM_B_PART = MLP_H * MLP_H * 2;     // one BF16 part of W2: 64 x 64 (8 KB)
constexpr int TM_A_PART = MLP_TILE * MLP_H * 2;  // one BF16 part of H: 128 x 64 (16 KB)
constexpr int TM_SMEM = 3 * TM_B_PART + 3 * TM_A_PART;
constexpr uint32_t TM_IDESC = idesc_bf16(128, MLP_H);

__global__ void __launch_bounds__(TM_THREADS) mlp_score_tc_kernel(const int64_t *off, const int32_t *d0,
                                                                  const ull *hop2, const uint32_t *outw,
                                                                  const ull *maxes, int64_t n, const float *weights,
                                                                  float *score, unsigned *hist, int nbins,
                                                                  const int32_t *gid, int *err,
                                                                  uint64_t timeout_ns) {
  extern __shared__ __align__(1024) uint8_t tsm[];  // B parts [3][64 x 64], A parts [3][128 x 64], histogram
  uint8_t *Bp = tsm, *Ap = tsm + 3 * TM_B_PART;
  unsigned *s_hist = (unsigned *)(tsm + TM_SMEM);
  __shared__ float W1[MLP_H][MLP_IN], b1[MLP_H], b2[MLP_H], w3[MLP_H];
  __shared__ float F[MLP_TILE][MLP_IN + 1];
  __shared__ float s_b3;
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < MLP_H * MLP_IN; i += blockDim.x) W1[i / MLP_IN][i % MLP_IN] = weights[i];
  const float *gb1 = weights + MLP_H * MLP_IN, *gW2 = gb1 + MLP_H, *gb2 = gW2 + MLP_H * MLP_H, *gw3 = gb2 + MLP_H;
  for (int i = tid; i < MLP_H; i += blockDim.x) {
    b1[i] = gb1[i];
    b2[i] = gb2[i];
    w3[i] = gw3[i];
  }
  if (tid == 0) s_b3 = gw3[MLP_H];
  for (int i = tid; i < nbins; i += blockDim.x) s_hist[i] = 0u;
  // B = W2 (row o = output unit, K = input unit), K-major: unit (o, 8-group g)
  for (int u = tid; u < MLP_H * (MLP_H / 8); u += blockDim.x) {
    const int o = u / (MLP_H / 8), g = u % (MLP_H / 8);
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = gW2[o * MLP_H + 8 * g + i];
    store_split8(v, Bp + core_off(o, g), Bp + TM_B_PART + core_off(o, g), Bp + 2 * TM_B_PART + core_off(o, g));
  }
  if (tid == 0) {
    mbar_init(smem_u32(&s_bar), 1);
    fence_mbar_init();
    s_fail = 0;
  }
  if (warp == 0) tmem_alloc(smem_u32(&s_tmem), MLP_H);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  const float ldeg = logf(1.f + (float)maxes[0]), lhop = logf(1.f + (float)maxes[1]);
  const float md0 = maxes[2] ? (float)maxes[2] : 1.f;
  // warps 4..7 compute the features of tile vertex tid - 128, one tile ahead: their loads for the next tile
  // are in flight while the tensor core and warps 0..3 finish the current one
  float f0 = 0.f, f1 = 0.f, f2 = 0.f, f3 = 0.f;
  auto features = [&](int64_t t0) {
    const int64_t v = t0 + (tid - MLP_TILE);
    f0 = f1 = f2 = f3 = 0.f;
    if (v < n) {
      float ld = ldeg, lh = lhop, m0 = md0;
      if (gid) {  // this vertex's graph's maxima
        const ull *mx = maxes + 3 * (int64_t)gid[v];
        ld = logf(1.f + (float)mx[0]);
        lh = logf(1.f + (float)mx[1]);
        m0 = mx[2] ? (float)mx[2] : 1.f;
      }
      const float deg = (float)(off[v + 1] - off[v]);
      f0 = ld > 0.f ? logf(1.f + deg) / ld : 0.f;
      f1 = lh > 0.f ? logf(1.f + (float)hop2[v]) / lh : 0.f;
      f2 = (float)(d0[v] < 0 ? 0 : d0[v]) / m0;
      f3 = deg > 0.f ? (float)outw[v] / deg : 0.f;
    }
  };
  const int64_t tstride = (int64_t)gridDim.x * MLP_TILE;
  if (tid >= MLP_TILE) features((int64_t)blockIdx.x * MLP_TILE);
  uint32_t parity = 0;
  bool issued = false;  // an MMA group not yet waited for (thread 0's view; all threads wait below)
  for (int64_t t0 = (int64_t)blockIdx.x * MLP_TILE; t0 < n; t0 += tstride) {
    if (tid >= MLP_TILE) {
      F[tid - MLP_TILE][0] = f0;
      F[tid - MLP_TILE][1] = f1;
      F[tid - MLP_TILE][2] = f2;
      F[tid - MLP_TILE][3] = f3;
    }
    __syncthreads();  // F ready; the previous tile's accumulator read (the barrier at the loop's end)
    // layer 1 (4 -> 64, ReLU) into the A parts: thread (v = tid % 128, half = tid / 128) takes hidden units
    // 32 half .. 32 half + 31, four 8-unit K groups
    {
      const int v = tid & (MLP_TILE - 1), half = tid >> 7;
#pragma unroll
      for (int gq = 0; gq < 4; gq++) {
        const int g = 4 * half + gq;
        float h[8];
#pragma unroll
        for (int i = 0; i < 8; i++) {
          const int o = 8 * g + i;
          float acc = b1[o];
#pragma unroll
          for (int f = 0; f < MLP_IN; f++) acc = fmaf(W1[o][f], F[v][f], acc);
          h[i] = acc > 0.f ? acc : 0.f;
        }
        store_split8(h, Ap + core_off(v, g), Ap + TM_A_PART + core_off(v, g), Ap + 2 * TM_A_PART + core_off(v, g));
      }
    }
    fence_async_smem();  // the A stores, visible to the tensor core
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
      const uint32_t a0 = smem_u32(Ap), b0 = smem_u32(Bp);
      const int pa[6] = {0, 0, 1, 0, 2, 1}, pb[6] = {0, 1, 0, 2, 0, 1};
#pragma unroll
      for (int ks = 0; ks < MLP_H / 16; ks++)
#pragma unroll
        for (int q = 0; q < 6; q++)
          mma_bf16(tmem, smem_desc(a0 + pa[q] * TM_A_PART + ks * 2 * CORE_LBO),
                   smem_desc(b0 + pb[q] * TM_B_PART + ks * 2 * CORE_LBO), TM_IDESC, (ks > 0 || q > 0) ? 1u : 0u);
      mma_commit(smem_u32(&s_bar));
    }
    issued = true;
    if (tid >= MLP_TILE && t0 + tstride < n) features(t0 + tstride);
    const bool ok = mbar_wait(smem_u32(&s_bar), parity, timeout_ns, nullptr);
    parity ^= 1u;
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicCAS(err, 0, PHDE_ERR_TIMEOUT);
      s_fail = 1;
      break;
    }
    issued = false;
    tc_fence_after();
    // output unit: lane l of warp w < 4 holds vertex 32 w + l's 64 layer-2 sums
    int bin = -1;
    if (warp < 4) {
      float sum = 0.f;
#pragma unroll
      for (int c0 = 0; c0 < MLP_H; c0 += 16) {
        float vv[16];
        tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, vv);
#pragma unroll
        for (int i = 0; i < 16; i++) {
          const float a = vv[i] + b2[c0 + i];
          sum = fmaf(w3[c0 + i], a > 0.f ? a : 0.f, sum);
        }
      }
      const int64_t v = t0 + 32 * warp + lane;
      if (v < n) {
        const float pr = 1.f / (1.f + expf(-(s_b3 + sum)));
        score[v] = pr;
        if (nbins > 0) {
          bin = (int)(pr * nbins);
          bin = bin < 0 ? 0 : (bin >= nbins ? nbins - 1 : bin);
        }
      }
      const unsigned same = __match_any_sync(PHDE_FULL_MASK, bin);
      if (bin >= 0 && lane == __ffs(same) - 1) atomicAdd(s_hist + bin, (unsigned)__popc(same));
    }
    tc_fence_before();
    __syncthreads();  // the accumulator and the A parts are free for the next tile
  }
  if (s_fail && issued) {  // a timed-out MMA group: wait once more (bounded) before the TMEM goes
    mbar_wait(smem_u32(&s_bar), parity ^ 1u, timeout_ns, nullptr);
  }
  __syncthreads();
  for (int i = tid; i < nbins; i += blockDim.x)
    if (s_hist[i]) atomicAdd(hist + i, s_hist[i]);
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, MLP_H);
  }
}

// The scoring grid: every CTA resident at once (a grid-stride loop over 128-vertex tiles gives each the same
// share, and a second, partial wave of CTAs would double the time of the first).
int mlp_grid(phde_ctx *ctx, int64_t n, size_t smem, int *grid) {
  int per_sm = 0;
  PHDE_CK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mlp_score_kernel, 256, smem));
  per_sm = std::max(per_sm, 1);
  *grid = (int)std::max<int64_t>(1, std::min<int64_t>((n + MLP_TILE - 1) / MLP_TILE, (int64_t)ctx->nsm * per_sm));
  return PHDE_OK;
}

// The scores of every vertex: the tensor-core kernel (PHDE_MLP_CUDA_CORES=1: the CUDA-core one).  Every CTA
// resident at once (grid-stride over 128-vertex tiles).
int launch_scores(phde_ctx *ctx, const int32_t *d_d0, const ull *hop2, const uint32_t *outw, const ull *maxes,
                  int64_t n, const float *wts, float *score, unsigned *hist, int nbins, const int32_t *gid) {
  if (getenv("PHDE_MLP_CUDA_CORES")) {
    const size_t mlp_smem = sizeof(float) * MLP_H * MLP_TILE + sizeof(unsigned) * nbins;
    PHDE_CK(ctx, cudaFuncSetAttribute(mlp_score_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_smem));
    int gm = 0;
    if (int rc = mlp_grid(ctx, n, mlp_smem, &gm)) return rc;
    mlp_score_kernel<<<gm, 256, mlp_smem, ctx->stream>>>(ctx->d_off, d_d0, hop2, outw, maxes, n, wts, score, hist,
                                                         nbins, gid);
    PHDE_LAUNCHED(ctx);
    return PHDE_OK;
  }
  const size_t smem = TM_SMEM + sizeof(unsigned) * nbins;
  PHDE_CK(ctx, cudaFuncSetAttribute(mlp_score_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // all of the unified L1/shared storage as shared memory: two CTAs of ~96 KB per SM
  PHDE_CK(ctx, cudaFuncSetAttribute(mlp_score_tc_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                    (int)cudaSharedmemCarveoutMaxShared));
  int per_sm = 0;
  PHDE_CK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mlp_score_tc_kernel, TM_THREADS, smem));
  // the occupancy query can assume the default carveout: count the CTAs the shared memory holds as well (no
  // CTA waits on another, so any grid is safe; the TMEM of four CTAs is half of an SM's)
  cudaFuncAttributes fa;
  int smem_sm = 0, resv = 0;
  PHDE_CK(ctx, cudaFuncGetAttributes(&fa, mlp_score_tc_kernel));
  PHDE_CK(ctx, cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device));
  PHDE_CK(ctx, cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, ctx->device));
  per_sm = std::max(per_sm, smem_sm / (int)(smem + fa.sharedSizeBytes + resv));
  per_sm = std::max(1, std::min(per_sm, 4));  // 64 TMEM columns each
  const int grid =
      (int)std::max<int64_t>(1, std::min<int64_t>((n + MLP_TILE - 1) / MLP_TILE, (int64_t)ctx->nsm * per_sm));
  mlp_score_tc_kernel<<<grid, TM_THREADS, smem, ctx->stream>>>(ctx->d_off, d_d0, hop2, outw, maxes, n, wts, score,
                                                               hist, nbins, gid, ctx->d_err, ctx->timeout_ns);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

}  // namespace

int phde_default_pivot_model(const float **w, int *count) {
  *w = kPivotMlpWeights;
  *count = (int)(sizeof(kPivotMlpWeights) / sizeof(float));
  return *count == MLP_WEIGHTS ? PHDE_OK : PHDE_ERR_INVALID;
}

// Score every vertex and return the M best candidates (score descending, index ascending on ties) in
// h_cand; d_d0 holds the warm start's minimum distance to its pivots.  Synchronises.
int phde_pivot_candidates(phde_ctx *ctx, const float *h_weights, int M, const int32_t *d_d0,
                          std::vector<int64_t> &h_cand, std::vector<float> &h_score) {
  const int64_t n = ctx->n;
  const int nbins = 4096;
  ull *hop2 = (ull *)phde_buf(ctx, "lp.hop2", sizeof(ull) * n);
  uint32_t *outw = (uint32_t *)phde_buf(ctx, "lp.outw", sizeof(uint32_t) * n);
  ull *maxes = (ull *)phde_buf(ctx, "lp.max", sizeof(ull) * 3);
  ull *pk = (ull *)phde_buf(ctx, "lp.pack", sizeof(ull) * n);
  float *score = (float *)phde_buf(ctx, "lp.score", sizeof(float) * n);
  unsigned *hist = (unsigned *)phde_buf(ctx, "lp.hist", sizeof(unsigned) * nbins);
  float *wts = (float *)phde_buf(ctx, "lp.w", sizeof(float) * MLP_WEIGHTS);
  const unsigned cap = (unsigned)std::max<int64_t>(4 * M, 65536);
  int64_t *cand = (int64_t *)phde_buf(ctx, "lp.cand", sizeof(int64_t) * cap);
  float *cscore = (float *)phde_buf(ctx, "lp.cscore", sizeof(float) * cap);
  unsigned *count = (unsigned *)phde_buf(ctx, "lp.count", sizeof(unsigned));
  if (!hop2 || !outw || !maxes || !pk || !score || !hist || !wts || !cand || !cscore || !count) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(maxes, 0, sizeof(ull) * 3, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(hist, 0, sizeof(unsigned) * nbins, ctx->stream));
  PHDE_CK(ctx, cudaMemcpyAsync(wts, h_weights, sizeof(float) * MLP_WEIGHTS, cudaMemcpyHostToDevice, ctx->stream));
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->nsm * 8));
  const int64_t *crow, *ce0;
  int64_t nch, chunk;
  int rc = phde_heavy_chunks(ctx, &crow, &ce0, &nch, &chunk);
  if (rc) return rc;
  PHDE_CK(ctx, cudaMemsetAsync(hop2, 0, sizeof(ull) * n, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(outw, 0, sizeof(uint32_t) * n, ctx->stream));
  feature_pack_kernel<<<g, 256, 0, ctx->stream>>>(ctx->d_off, d_d0, n, pk);
  PHDE_LAUNCHED(ctx);
  feature_raw_kernel<<<g, 256, 0, ctx->stream>>>(ctx->d_off, ctx->d_adj, d_d0, pk, n, crow, ce0, nch, chunk, hop2,
                                                 outw);
  PHDE_LAUNCHED(ctx);
  feature_max_kernel<<<g, 256, 0, ctx->stream>>>(ctx->d_off, d_d0, hop2, n, maxes);
  PHDE_LAUNCHED(ctx);
  PHDE_CK(ctx, cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
  if ((rc = launch_scores(ctx, d_d0, hop2, outw, maxes, n, wts, score, hist, nbins, nullptr))) return rc;
  std::vector<unsigned> hh(nbins);
  PHDE_CK(ctx, cudaMemcpyAsync(hh.data(), hist, sizeof(unsigned) * nbins, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  // lowest bin such that the bins at or above it hold at least M vertices
  int bmin = nbins - 1;
  int64_t acc = 0;
  for (; bmin > 0; bmin--) {
    acc += hh[bmin];
    if (acc >= M) break;
  }
  PHDE_CK(ctx, cudaMemsetAsync(count, 0, sizeof(unsigned), ctx->stream));
  collect_kernel<<<g, 256, 0, ctx->stream>>>(score, n, bmin, nbins, cand, cscore, count, cap);
  PHDE_LAUNCHED(ctx);
  unsigned hc = 0;
  PHDE_CK(ctx, cudaMemcpyAsync(&hc, count, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  hc = std::min(hc, cap);
  std::vector<int64_t> c(hc);
  std::vector<float> cs(hc);
  PHDE_CK(ctx, cudaMemcpyAsync(c.data(), cand, sizeof(int64_t) * hc, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaMemcpyAsync(cs.data(), cscore, sizeof(float) * hc, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<int> ord(hc);
  for (unsigned i = 0; i < hc; i++) ord[i] = (int)i;
  std::sort(ord.begin(), ord.end(), [&](int x, int y) { return cs[x] != cs[y] ? cs[x] > cs[y] : c[x] < c[y]; });
  const int take = (int)std::min<int64_t>(M, hc);
  h_cand.resize(take);
  h_score.resize(take);
  for (int i = 0; i < take; i++) {
    h_cand[i] = c[ord[i]];
    h_score[i] = cs[ord[i]];
  }
  return PHDE_OK;
}

int phde_cand_distances(phde_ctx *ctx, const int32_t *D, int P0, const uint16_t *R, int RW, const int64_t *d_cand,
                        int M, std::vector<int32_t> &h_sub, std::vector<int32_t> &h_csub, const MsLevels *lv) {
  int32_t *sub = (int32_t *)phde_buf(ctx, "lp.sub", sizeof(int32_t) * (size_t)M * std::max(P0, 1));
  int32_t *csub = (int32_t *)phde_buf(ctx, "lp.csub", sizeof(int32_t) * (size_t)M * M);
  if (!sub || !csub) return PHDE_ERR_OOM;
  const int total = M * (M + P0);
  cand_distances_kernel<<<(total + 255) / 256, 256, 0, ctx->stream>>>(D, P0, lv ? nullptr : R, RW, ctx->n, d_cand, M,
                                                                      sub, csub);
  PHDE_LAUNCHED(ctx);
  if (lv) {
    cand_distances_lvl_kernel<<<(M * lv->W + 127) / 128, 128, 0, ctx->stream>>>(lv->lvl, lv->nlev, lv->W, ctx->n,
                                                                                d_cand, M, csub);
    PHDE_LAUNCHED(ctx);
  }
  h_sub.resize((size_t)M * P0);
  h_csub.resize((size_t)M * M);
  if (P0 > 0)
    PHDE_CK(ctx, cudaMemcpyAsync(h_sub.data(), sub, sizeof(int32_t) * M * P0, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaMemcpyAsync(h_csub.data(), csub, sizeof(int32_t) * M * M, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return PHDE_OK;
}

// Scores of every vertex of an uploaded batch (features normalised per graph) into the context's "lp.score"
// buffer; d_d0 is the warm start's minimum distance.  No synchronisation (part of the captured batched layout).
// d_weights: the model on the device (the caller copies it before the captured sequence).
int phde_batch_scores(phde_ctx *ctx, const float *d_weights, const int32_t *d_d0, const float **score_out) {
  const int64_t n = ctx->n;
  const int B = ctx->batch_B;
  ull *hop2 = (ull *)phde_buf(ctx, "lp.hop2", sizeof(ull) * n);
  uint32_t *outw = (uint32_t *)phde_buf(ctx, "lp.outw", sizeof(uint32_t) * n);
  ull *maxes = (ull *)phde_buf(ctx, "lpb.max", sizeof(ull) * 3 * B);
  ull *pk = (ull *)phde_buf(ctx, "lp.pack", sizeof(ull) * n);
  float *score = (float *)phde_buf(ctx, "lp.score", sizeof(float) * n);
  if (!hop2 || !outw || !maxes || !pk || !score) return PHDE_ERR_OOM;
  const int64_t *crow, *ce0;
  int64_t nch, chunk;
  int rc = phde_heavy_chunks(ctx, &crow, &ce0, &nch, &chunk);
  if (rc) return rc;
  PHDE_CK(ctx, cudaMemsetAsync(maxes, 0, sizeof(ull) * 3 * B, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(hop2, 0, sizeof(ull) * n, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(outw, 0, sizeof(uint32_t) * n, ctx->stream));
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->nsm * 8));
  feature_pack_kernel<<<g, 256, 0, ctx->stream>>>(ctx->d_off, d_d0, n, pk);
  PHDE_LAUNCHED(ctx);
  feature_raw_kernel<<<g, 256, 0, ctx->stream>>>(ctx->d_off, ctx->d_adj, d_d0, pk, n, crow, ce0, nch, chunk, hop2,
                                                 outw);
  PHDE_LAUNCHED(ctx);
  feature_max_batched_kernel<<<g, 256, 0, ctx->stream>>>(ctx->d_off, d_d0, hop2, ctx->d_gid, n, maxes);
  PHDE_LAUNCHED(ctx);
  if (int rc2 = launch_scores(ctx, d_d0, hop2, outw, maxes, n, d_weights, score, nullptr, 0, ctx->d_gid)) return rc2;
  *score_out = score;
  return PHDE_OK;
}
