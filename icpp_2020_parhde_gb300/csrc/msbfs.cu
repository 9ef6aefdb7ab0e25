// msbfs.cu -- multi-source breadth-first search with per-vertex source bitsets (one persistent launch).
//
// Up to 64*W sources (W <= 4 words) are searched together.  Every vertex keeps a `seen` bitset (bit b:
// source b has reached it) and the frontier bitset of the current level.  A level computes, for each
// vertex that can gain bits, the OR of its neighbours' frontier words, keeps the bits it has not seen,
// records hop distance L+1 for each of them (16-bit record, row per vertex) and publishes them as its
// next-level frontier word.  Two ways to pick the vertices of a level:
//   dense  -- every vertex not yet finished, in 32-vertex tiles: a `done` bitmap (saturated, both frontier
//             words zero) lets a warp skip 32 finished vertices with one load;
//   sparse -- when the frontier's out-edges are few (below nnz / 16): only the frontier's neighbours can
//             gain bits, so they are claimed once (a per-vertex level stamp), listed, and pulled; the
//             stale output words of two levels back are cleared from their list.  The frontier of a
//             sparse level is a (vertex, edge prefix) list that the previous level built (or that is
//             rebuilt by one scan of the frontier words after a dense level), walked edge-balanced.
// In dense levels rows of at most MS_SMALL neighbours are pulled by one lane each (a tile's 32 rows by one warp),
// the other light rows by groups of 8 lanes; rows above MS_HEAVY neighbours (R-MAT hubs) are cut into
// chunks whose partial ORs are combined with atomicOr before the same finalisation.  OR is order-free, so
// the result is deterministic.
//
// Used where all sources are known up front -- random pivot strategies, learned pivots, and
// phde_distances -- so the reference's one-BFS-per-pivot loop (ParHDE.cpp:158-175,
// DrawingBase.cpp:173-190) becomes one sweep per level.  Hop distances are unique: every column equals
// the one-source BFS column bit for bit.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ctx.h"

namespace {

constexpr int MS_THREADS = 512;
constexpr int MS_MAXW = 4;
constexpr int64_t MS_HEAVY = 256;  // rows above this are cut into chunks (one warp per chunk)
constexpr int64_t MS_CHUNK = 256;
constexpr int MS_GROUP = 8;        // lanes per light row
constexpr int MS_TILE_CHUNK = 4;   // dense levels: 32-vertex tiles a warp takes from the level counter at once
constexpr int64_t MS_SMALL = 40;  // dense levels: rows up to this many neighbours are pulled by one lane each
// dense levels on index-local graphs (mesh-like numberings): a CTA takes MS_WIN consecutive vertices and
// stages the frontier words of those and of MS_WIN on each side in shared memory, where most of their
// neighbours' words are then found
constexpr int MS_WIN = 1024;
constexpr int MS_WIN_SAMPLE = 16;  // the locality estimate reads the rows of every 16th vertex
constexpr int GATHER_SMEM_COLS = 1024;  // columns whose sums of squares are kept per CTA

struct MsArgs {
  const int64_t *off;
  const uint32_t *adj;
  int64_t n;
  int nsrc;        // sources this sweep (the word count W is the kernel's template argument)
  const int64_t *src;
  // batches (period > 0): src holds nlist sources and entry i searches with bit i % period -- each graph's
  // candidates share the bit positions, the components never meet; the level-0 frontier list is left for
  // the first level to build (built_f false)
  int nlist, period;
  uint16_t *R;     // row-major n x RW distance record: R[v*RW + b] = level + 1 (0 = unreached); null in level mode
  // level mode (lvl non-null): no record; the frontier words of every level stay, level L's in
  // lvl[L * n * W ..] (array 0: the sources; arrays 0 and 1 zeroed by the host, array L + 2 cleared during
  // level L), so bit b of vertex v is set in exactly the array of its distance from source b.  lcap: the
  // last array allocated.
  ull *lvl;
  int lcap;
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
  // vertices given new bits at level L, with edge prefixes (count << 32 | edges in lctr): slot L % 4; the
  // sources are slot 3 (level -1).  Level L reads its frontier from slot (L-1) % 4, clears the stale
  // output words of slot (L-2) % 4 when it runs sparse, and resets slot (L+1) % 4.
  uint32_t *qv[4], *qe[4];
  ull *lctr;                  // [4] list positions (count << 32 | edges) of the lists built by sparse levels
  ull *lstat;                 // [4] the same totals for every level (dense levels count without a list)
  int32_t *stamp;             // [n] claim stamps of sparse levels (L + 1), zeroed
  uint32_t *cand;             // [n] candidates of a sparse level
  unsigned *ccount;           // [2] candidate counters, by level parity
  ull *cedge;                 // [2] the candidates' total degree, by level parity
  unsigned *tctr;             // [4] dense levels: next 32-vertex tile to hand out, slot L % 4 (reset one level ahead)
  int64_t sparse_edges;       // a level runs sparse when its frontier has fewer out-edges
  int *levels_out;
  ull *trace;                 // optional [2*trace_cap]: per level end time (ns) and vertices given new bits
  int trace_cap;
  uint32_t *done;             // [n/32] bitmap: saturated with both frontier words zero (or a hub row): skipped
  // [3][n/32] frontier bitmaps: bit v of fbm[L % 3] <=> vertex v's frontier word of level L is nonzero.  A pull
  // tests a neighbour's bit (one L1/L2-resident word) before gathering its 32-byte word, so levels with a
  // small frontier skip most gathers.  Level L reads fbm[L % 3], sets fbm[(L+1) % 3] and clears fbm[(L+2) % 3]
  // (read during level L-1, written again during level L+1).
  uint32_t *fbm[3];
  int win;                    // dense levels stage frontier windows in shared memory (MS_WIN)
  GridSync *gs;
  int *err;
  uint64_t timeout_ns;
};

// Frontier words of one vertex through the L2 (other blocks wrote them during the previous level).
// Frontier words of one vertex, kept in L2 (evict-last): every level gathers them from many neighbours.
template <int W>
__device__ __forceinline__ void ld_front(const ull *p, ull (&x)[W], uint64_t keep) {
  if constexpr (W == 4) {
    ld_cg_hint32(p, keep, x);  // one L2 request for the vertex's 32 bytes
  } else if constexpr (W == 2) {
#pragma unroll
    for (int h = 0; h < W / 2; h++) {
      const uint4 a = ld_cg_hint(p + 2 * h, keep);
      x[2 * h] = ((ull)a.y << 32) | a.x;
      x[2 * h + 1] = ((ull)a.w << 32) | a.z;
    }
  } else {
#pragma unroll
    for (int w = 0; w < W; w++) x[w] = __ldcg(p + w);
  }
}

template <int W>
__device__ __forceinline__ void ld_words(const ull *p, ull (&x)[W]) {
  if constexpr (W == 4) {
    asm volatile("ld.global.cg.v4.u64 {%0, %1, %2, %3}, [%4];" : "=l"(x[0]), "=l"(x[1]), "=l"(x[2]), "=l"(x[3]) : "l"(p));
  } else if constexpr (W == 2) {
    const uint4 a = __ldcg((const uint4 *)p);
    x[0] = ((ull)a.y << 32) | a.x;
    x[1] = ((ull)a.w << 32) | a.z;
  } else {
#pragma unroll
    for (int w = 0; w < W; w++) x[w] = __ldcg(p + w);
  }
}

// A neighbour's frontier words: from the shared-memory window when u lies in it (WIN), else through L2 --
// after the frontier-bitmap test when use_bm (the window holds zero words for vertices outside the frontier).
// Returns false when the words are known to be zero (not read).
template <int W, bool WIN>
__device__ __forceinline__ bool gather_front(const ull *fcur, const ull *swin, int64_t wlo, const uint32_t *fbm_cur,
                                             bool use_bm, uint32_t u, ull (&x)[W], uint64_t keep) {
  if constexpr (WIN) {
    const uint64_t d = (uint64_t)((int64_t)u - wlo);
    if (d < (uint64_t)(3 * MS_WIN)) {
#pragma unroll
      for (int w = 0; w < W; w++) x[w] = swin[d * W + w];
      return true;
    }
  }
  if (use_bm && !((__ldcg(fbm_cur + (u >> 5)) >> (u & 31)) & 1u)) return false;
  ld_front<W>(fcur + (int64_t)u * W, x, keep);
  return true;
}

// Record word for 4 sources: the 4 bits of `nib` select which of the four 16-bit lanes get value `val`.
__device__ __forceinline__ ull nibble_lanes(unsigned nib, unsigned val) {
  const ull e = (ull)(nib & 1u) | ((ull)(nib & 2u) << 15) | ((ull)(nib & 4u) << 30) | ((ull)(nib & 8u) << 45);
  return e * (ull)val;  // the lanes do not overlap: no carries
}

// New bits of vertex v at level L (OR of its neighbours' frontier words `acc`, seen words `s`), finalised
// by the MS_GROUP lanes of its group: lane gl writes record words gl, gl+8, ... (4 sources per word) and
// seen/frontier word gl.  Returns whether any bit is new.
template <int W>
__device__ __forceinline__ bool ms_group_finalise(const MsArgs &a, int64_t v, const ull (&acc)[W], const ull (&s)[W],
                                                  ull *fnext, int32_t L, int gl) {
  const unsigned val = (unsigned)(L + 2);  // level L+1, stored +1
  ull nw[W];
  bool any = false;
#pragma unroll
  for (int w = 0; w < W; w++) {
    nw[w] = acc[w] & ~s[w];
    any |= nw[w] != 0ull;
  }
  if (a.R) {
    ull *row = (ull *)(a.R + v * a.RW + a.col0);
#pragma unroll
    for (int i = 0; i < 2 * W; i++) {
      const int gi = gl + 8 * (i & 1);
      const unsigned nib = (unsigned)(nw[i >> 1] >> (4 * gi)) & 15u;
      if (nib) red_or_hint(row + gl + 8 * i, nibble_lanes(nib, val), l2_policy_evict_first());  // a reduction in L2
    }
  }
#pragma unroll
  for (int w = 0; w < W; w++)
    if (w == gl) {
      fnext[v * W + w] = nw[w];
      if (nw[w]) a.seen[v * W + w] = s[w] | nw[w];
    }
  return any;
}

// Same, one thread for the whole row (heavy rows: few).
template <int W>
__device__ __forceinline__ bool ms_thread_finalise(const MsArgs &a, int64_t v, const ull (&acc)[W], ull *fnext,
                                                   int32_t L) {
  const unsigned val = (unsigned)(L + 2);
  bool any = false;
  ull *row = a.R ? (ull *)(a.R + v * a.RW + a.col0) : nullptr;
#pragma unroll
  for (int w = 0; w < W; w++) {
    const ull s = a.seen[v * W + w];
    const ull nw = acc[w] & ~s;
    fnext[v * W + w] = nw;
    if (nw) {
      any = true;
      a.seen[v * W + w] = s | nw;
      if (row)
        for (int gi = 0; gi < 16; gi++) {
          const unsigned nib = (unsigned)(nw >> (4 * gi)) & 15u;
          if (nib) atomicOr(row + 16 * w + gi, nibble_lanes(nib, val));
        }
    }
  }
  return any;
}

// One vertex v pulled by its MS_GROUP-lane group (gl = lane in group): OR of the neighbours' frontier words,
// new bits finalised.  Every lane of the warp must call it (the group shuffles are warp-wide); lanes whose
// group has no vertex pass act = false.  Returns through `newbits` whether v got new bits (group leader).
__device__ __forceinline__ bool fbit(const uint32_t *bm, uint32_t u) { return (__ldcg(bm + (u >> 5)) >> (u & 31)) & 1u; }

template <int W, bool WIN = false>
__device__ __forceinline__ void ms_pull_vertex(const MsArgs &a, const ull (&full)[W], const ull *fcur, ull *fnext,
                                               const uint32_t *fbm_cur, uint32_t *fbm_next, bool use_bm, int32_t L,
                                               int64_t v, bool act, int gl, bool mark_done, bool &newbits,
                                               uint32_t &deg, const ull *swin = nullptr, int64_t wlo = 0) {
  newbits = false;
  int64_t e0 = 0, e1 = 0;
  deg = 0;
  if (act) {
    e0 = a.off[v];
    e1 = a.off[v + 1];
    deg = (uint32_t)(e1 - e0);
    if (e1 - e0 > MS_HEAVY) act = false;  // hub rows go by chunks
  }
  ull s[W];
  bool sat = true;
#pragma unroll
  for (int w = 0; w < W; w++) s[w] = 0ull;
  if (act) {
    ld_words<W>(a.seen + v * W, s);
#pragma unroll
    for (int w = 0; w < W; w++) sat &= (s[w] == full[w]);
  }
  ull acc[W];
#pragma unroll
  for (int w = 0; w < W; w++) acc[w] = 0ull;
  const uint64_t stream = l2_policy_evict_first(), keep = l2_policy_evict_last();
  if (act && !sat)
    for (int64_t e = e0 + gl; e < e1; e += 2 * MS_GROUP) {
      const int64_t e2 = e + MS_GROUP;
      const uint32_t u0 = ld_nc_hint(a.adj + e, stream);
      const uint32_t u1 = e2 < e1 ? ld_nc_hint(a.adj + e2, stream) : u0;
      // gather only the neighbours in this level's frontier (their bitmap bit): an empty word adds nothing
      ull x0[W];
      if (gather_front<W, WIN>(fcur, swin, wlo, fbm_cur, use_bm, u0, x0, keep)) {
#pragma unroll
        for (int w = 0; w < W; w++) acc[w] |= x0[w];
      }
      ull x1[W];
      if (e2 < e1 && gather_front<W, WIN>(fcur, swin, wlo, fbm_cur, use_bm, u1, x1, keep)) {
#pragma unroll
        for (int w = 0; w < W; w++) acc[w] |= x1[w];
      }
    }
#pragma unroll
  for (int w = 0; w < W; w++)
#pragma unroll
    for (int o = MS_GROUP / 2; o > 0; o >>= 1) acc[w] |= __shfl_xor_sync(PHDE_FULL_MASK, acc[w], o, MS_GROUP);
  // every lane of the group read `seen` above, before the shuffles; the writes come after them
  if (act) {
    if (sat) {
      // saturated: clear this level's output word; once the current word is empty too, the vertex is
      // finished for the rest of the sweep
#pragma unroll
      for (int w = 0; w < W; w++)
        if (w == gl) fnext[v * W + w] = 0ull;
      if (mark_done && gl == 0 && !fbit(fbm_cur, (uint32_t)v)) atomicOr(a.done + (v >> 5), 1u << (v & 31));
    } else if (ms_group_finalise<W>(a, v, acc, s, fnext, L, gl) && gl == 0) {
      newbits = true;
      atomicOr(fbm_next + (v >> 5), 1u << (v & 31));
    }
  }
}

// One light row v (neighbours e0 .. e1, at most MS_SMALL) pulled by one lane: the gathers four at a time, then
// the finalisation (record nibbles by L2 reductions).  newbits: v got new bits; finished: v is saturated and
// not in this level's frontier (its `done` bit may be set).
template <int W, bool WIN>
__device__ __forceinline__ void ms_pull_light(const MsArgs &a, const ull (&full)[W], const ull *fcur, ull *fnext,
                                              const uint32_t *fbm_cur, bool use_bm, int32_t L, int64_t v, int64_t e0,
                                              int64_t e1, bool &newbits, bool &finished, const ull *swin,
                                              int64_t wlo) {
  newbits = finished = false;
  ull s[W];
  ld_words<W>(a.seen + v * W, s);
  bool sat = true;
#pragma unroll
  for (int w = 0; w < W; w++) sat &= (s[w] == full[w]);
  if (sat) {
#pragma unroll
    for (int w = 0; w < W; w++) fnext[v * W + w] = 0ull;
    finished = !fbit(fbm_cur, (uint32_t)v);
    return;
  }
  const uint64_t stream = l2_policy_evict_first(), keep = l2_policy_evict_last();
  ull acc[W];
#pragma unroll
  for (int w = 0; w < W; w++) acc[w] = 0ull;
  for (int64_t e = e0; e < e1; e += 4) {
    uint32_t u[4];
#pragma unroll
    for (int j = 0; j < 4; j++) u[j] = e + j < e1 ? ld_nc_hint(a.adj + e + j, stream) : 0u;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      ull x[W];
      if (e + j < e1 && gather_front<W, WIN>(fcur, swin, wlo, fbm_cur, use_bm, u[j], x, keep)) {
#pragma unroll
        for (int w = 0; w < W; w++) acc[w] |= x[w];
      }
    }
  }
  const unsigned val = (unsigned)(L + 2);  // level L+1, stored +1
  ull *row = a.R ? (ull *)(a.R + v * a.RW + a.col0) : nullptr;
  const uint64_t rec = l2_policy_evict_first();
#pragma unroll
  for (int w = 0; w < W; w++) {
    const ull nw = acc[w] & ~s[w];
    fnext[v * W + w] = nw;
    if (nw) {
      newbits = true;
      a.seen[v * W + w] = s[w] | nw;
      if (row)
        for (ull m = nw; m;) {
          const int gi = (__ffsll((long long)m) - 1) >> 2;
          red_or_hint(row + 16 * w + gi, nibble_lanes((unsigned)(nw >> (4 * gi)) & 15u, val), rec);
          m &= ~(15ull << (4 * gi));
        }
    }
  }
}

// One 32-vertex tile t of a dense level, by one warp: the unfinished vertices (the tile's `done` word); rows of
// at most MS_SMALL neighbours by their own lane (the tile's frontier-bitmap and `done` bits out as one atomic
// each), the other light rows by the warp's four 8-lane groups in turn.  WIN: neighbours' words from the
// shared-memory window starting at vertex wlo where they lie in it.
template <int W, bool WIN>
__device__ __forceinline__ void ms_dense_tile(const MsArgs &a, const ull (&full)[W], const ull *fcur, ull *fnext,
                                              const uint32_t *fbm_cur, uint32_t *fbm_next, bool use_bm, int32_t L,
                                              int64_t t, const ull *swin, int64_t wlo, ull &my_stat) {
  const int64_t n = a.n;
  const int lane = threadIdx.x & 31, gl = lane & (MS_GROUP - 1), grp = lane / MS_GROUP;
  const int64_t v0 = t * 32;
  const unsigned valid = n - v0 >= 32 ? 0xffffffffu : ((1u << (n - v0)) - 1u);
  // one read of the tile's word, broadcast: the warp sets bits of it below
  unsigned todo = __shfl_sync(PHDE_FULL_MASK, lane == 0 ? __ldcg(a.done + t) : 0u, 0);
  todo = ~todo & valid;
  if (todo) {
    const int64_t v = v0 + lane;
    const bool mine = (todo >> lane) & 1u;
    int64_t e0 = 0, e1 = 0;
    if (mine) {
      e0 = a.off[v];
      e1 = a.off[v + 1];
    }
    const bool light = mine && e1 - e0 <= MS_SMALL;
    const unsigned lmask = __ballot_sync(PHDE_FULL_MASK, light);
    todo &= ~lmask;
    bool nb = false, fin = false;
    if (light) ms_pull_light<W, WIN>(a, full, fcur, fnext, fbm_cur, use_bm, L, v, e0, e1, nb, fin, swin, wlo);
    const unsigned nbm = __ballot_sync(PHDE_FULL_MASK, nb), finm = __ballot_sync(PHDE_FULL_MASK, fin);
    if (lane == 0 && nbm) atomicOr(fbm_next + t, nbm);
    if (lane == 0 && finm) atomicOr(a.done + t, finm);
    if (nb) my_stat += (1ull << 32) | (ull)(e1 - e0);
  }
  while (todo) {
    // the grp-th set bit of todo (none: act = false)
    unsigned rest = todo;
    for (int j = 0; j < grp && rest; j++) rest &= rest - 1u;
    const bool act = rest != 0u;
    const int64_t v = v0 + (act ? __ffs(rest) - 1 : 0);
    bool nb;
    uint32_t dv;
    ms_pull_vertex<W, WIN>(a, full, fcur, fnext, fbm_cur, fbm_next, use_bm, L, v, act, gl, true, nb, dv, swin, wlo);
    if (nb) my_stat += (1ull << 32) | (ull)dv;
    for (int j = 0; j < 32 / MS_GROUP && todo; j++) todo &= todo - 1u;
  }
}

template <int W>
__global__ void __launch_bounds__(MS_THREADS, 2) msbfs_kernel(MsArgs a) {
  extern __shared__ __align__(16) ull ms_dyn[];  // the frontier window of index-local dense levels (a.win)
  const int64_t n = a.n;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, gts = (int64_t)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31, gl = lane & (MS_GROUP - 1), grp = lane / MS_GROUP;
  const int64_t gw = gt >> 5, gws = gts >> 5;
  // full mask of the valid source bits per word
  ull full[W];
#pragma unroll
  for (int w = 0; w < W; w++) {
    const int bits = a.nsrc - 64 * w;
    full[w] = bits >= 64 ? ~0ull : (bits <= 0 ? 0ull : ((1ull << bits) - 1ull));
  }
  // level 0: every source sees itself; hub rows never enter the light pull (their bit in `done`)
  if (a.period > 0) {
    ull my = 0;  // (sources << 32 | their edges) of this thread, for the level-0 frontier totals
    for (int64_t i = gt; i < a.nlist; i += gts) {
      const int b = (int)(i % a.period);
      const int64_t s = a.src[i];
      atomicOr(a.seen + s * W + (b >> 6), 1ull << (b & 63));
      atomicOr(a.front[0] + s * W + (b >> 6), 1ull << (b & 63));
      atomicOr(a.fbm[0] + (s >> 5), 1u << (s & 31));
      if (a.R) a.R[s * a.RW + a.col0 + b] = 1;
      my += (1ull << 32) | (ull)(a.off[s + 1] - a.off[s]);
    }
    my = warp_sum(my);
    if ((threadIdx.x & 31) == 0 && my) atomicAdd(a.lstat + 3, my);
  } else if (gt == 0)
    for (int b = 0; b < a.nsrc; b++) {
      const int64_t s = a.src[b];
      atomicOr(a.seen + s * W + (b >> 6), 1ull << (b & 63));
      atomicOr(a.front[0] + s * W + (b >> 6), 1ull << (b & 63));
      atomicOr(a.fbm[0] + (s >> 5), 1u << (s & 31));
      if (a.R) a.R[s * a.RW + a.col0 + b] = 1;  // level 0
    }
  for (int64_t h = gt; h < a.nheavy; h += gts) {
    const int64_t v = a.heavy_rows[h];
    atomicOr(a.done + (v >> 5), 1u << (v & 31));
  }
  // the sources are the frontier of level 0 (list slot 3)
  if (gt == 0 && a.period == 0) {
    ull run = 0;
    for (int b = 0; b < a.nsrc; b++) {
      const int64_t s = a.src[b];
      a.qv[3][b] = (uint32_t)s;
      a.qe[3][b] = (uint32_t)run;
      run += (ull)(a.off[s + 1] - a.off[s]);
    }
    a.lctr[3] = a.lstat[3] = ((ull)a.nsrc << 32) | run;
  }
  __shared__ PushScratch psc;
  __shared__ ull s_stat;
  __shared__ unsigned s_tile;
  bool built_f = a.period == 0, built_z = true;  // lists of levels L-1 and L-2 exist (sparse levels build them)
  if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
  int32_t L = 0;
  for (;; L++) {
    if (L > 65533) {  // the 16-bit record holds levels up to 65534; every block sees the same L
      if (gt == 0) atomicCAS(a.err, 0, PHDE_ERR_TOO_LARGE);
      return;
    }
    if (a.lvl && L + 1 > a.lcap) {  // more levels than the arrays allow (uniform): the caller uses the record
      if (gt == 0) atomicCAS(a.err, 0, PHDE_ERR_TOO_LARGE);
      return;
    }
    const int64_t nW = n * W;
    const ull *fcur = a.lvl ? a.lvl + (int64_t)L * nW : a.front[L & 1];
    ull *fnext = a.lvl ? a.lvl + (int64_t)(L + 1) * nW : a.front[(L + 1) & 1];
    if (a.lvl && L + 2 <= a.lcap) {  // the array level L + 1 writes, cleared one level ahead
      ull *ahead = a.lvl + (int64_t)(L + 2) * nW;
      for (int64_t i = gt; i < nW; i += gts) ahead[i] = 0ull;
    }
    const uint32_t *fbm_cur = a.fbm[L % 3];
    uint32_t *fbm_next = a.fbm[(L + 1) % 3];
    {
      uint32_t *fbm_old = a.fbm[(L + 2) % 3];
      for (int64_t i = gt; i < (n + 31) / 32; i += gts) fbm_old[i] = 0u;
    }
    const int so = L & 3, sf = (L + 3) & 3, sz = (L + 2) & 3;
    // slot (L+1)%4 and the other candidate counter were last used by level L-1, finished at its barrier
    if (gt == 0) {
      a.lctr[(L + 1) & 3] = 0ull;
      a.lstat[(L + 1) & 3] = 0ull;
      a.ccount[(L + 1) & 1] = 0u;
      a.cedge[(L + 1) & 1] = 0ull;
      a.tctr[(L + 1) & 3] = 0u;
    }
    if (threadIdx.x == 0) s_stat = 0ull;
    ull my_stat = 0;  // dense: this thread's (count << 32 | edges) of vertices given new bits
    // the frontier's totals: its list counter if the previous level built one, else its count
    const ull fstat = built_f ? __ldcg(a.lctr + sf) : __ldcg(a.lstat + sf);
    const uint32_t fedges = (uint32_t)(fstat & 0xffffffffull);
    // test the frontier bitmap before each gather while the frontier holds at most a quarter of the vertices
    // (above that, most neighbours are in it and the test only lengthens the dependent chain)
    const bool use_bm = (int64_t)(fstat >> 32) <= n / 4;
    const bool sparse = (int64_t)fedges < a.sparse_edges;
    bool push = false;  // a sparse level that pushes (set below, uniform)
    if (sparse) {
      if (!built_f) {
        // the previous level ran dense: list its frontier (the vertices with a nonzero current word)
        for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += gts) {
          const int64_t v = base + threadIdx.x;
          bool nz = false;
          uint32_t dv = 0;
          if (v < n) {
            ull x[W];
            ld_words<W>(fcur + v * W, x);
#pragma unroll
            for (int w = 0; w < W; w++) nz |= x[w] != 0ull;
            if (nz) dv = (uint32_t)(a.off[v + 1] - a.off[v]);
          }
          block_push(nz, (uint32_t)v, dv, a.qv[sf], a.qe[sf], a.lctr + sf, &psc);
        }
      }
      // stale output words (the vertices given bits at level L-2) go to zero: from its list, or all (level
      // mode: the array is fresh)
      if (a.lvl) {
      } else if (built_z) {
        const uint32_t zcnt = (uint32_t)(__ldcg(a.lctr + sz) >> 32);
        for (int64_t i = gt; i < zcnt; i += gts) {
          const int64_t v = a.qv[sz][i];
#pragma unroll
          for (int w = 0; w < W; w++) fnext[v * W + w] = 0ull;
        }
      } else {
        for (int64_t i = gt; i < n * W; i += gts) fnext[i] = 0ull;
      }
      if (!built_f && !grid_sync(a.gs, a.err, a.timeout_ns)) return;
      // new bits can only appear next to the frontier: claim those neighbours once (stamp L+1), edge-balanced
      // over the frontier's edges, skipping finished vertices, and add up the candidates' degrees.  Then either
      // pull every candidate's neighbours (work in proportion to the candidates' edges) or, when those are
      // more than twice the frontier's -- hubs next to a small frontier, as in R-MAT's first levels -- push:
      // every frontier edge (u, v) ORs u's frontier word into v's accumulator (hacc, zero outside a level),
      // work in proportion to the frontier's edges but an L2 reduction per word.
      const ull fctr = __ldcg(a.lctr + sf);
      const uint32_t fcnt = (uint32_t)(fctr >> 32), fe = (uint32_t)(fctr & 0xffffffffull);
      const uint32_t *fqv = a.qv[sf], *fqe = a.qe[sf];
      unsigned *cc = a.ccount + (L & 1);
      ull *ce = a.cedge + (L & 1);
      const uint64_t keep = l2_policy_evict_last();
      // `done` also marks the hub rows (dense levels pull them by chunks): those stay candidates
      auto target = [&](int64_t e, uint32_t &u) -> int64_t {  // v of frontier edge e, or -1 when finished
        const uint32_t slot = owner_slot(fqe, fcnt, (uint32_t)e);
        u = fqv[slot];
        const uint32_t v = __ldg(a.adj + a.off[u] + (e - (int64_t)fqe[slot]));
        bool skip = (__ldcg(a.done + (v >> 5)) >> (v & 31)) & 1u;
        if (skip) skip = a.off[v + 1] - a.off[v] <= MS_HEAVY;
        return skip ? -1 : (int64_t)v;
      };
      for (int64_t base = gw * 32; base < fe; base += gws * 32) {
        const int64_t e = base + lane;
        bool mine = false;
        uint32_t v = 0;
        ull dsum = 0;
        if (e < fe) {
          uint32_t u;
          const int64_t t = target(e, u);
          if (t >= 0) {
            v = (uint32_t)t;
            mine = atomicMax(a.stamp + v, L + 1) < L + 1;
            if (mine) dsum = (ull)(a.off[v + 1] - a.off[v]);
          }
        }
        const unsigned bal = __ballot_sync(PHDE_FULL_MASK, mine);
        unsigned slot0 = 0;
        dsum = warp_sum(dsum);
        if (lane == 0 && bal) {
          slot0 = atomicAdd(cc, (unsigned)__popc(bal));
          atomicAdd(ce, dsum);
        }
        slot0 = __shfl_sync(PHDE_FULL_MASK, slot0, 0);
        if (mine) a.cand[slot0 + __popc(bal & ((1u << lane) - 1u))] = v;
      }
      if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
      const unsigned nc = __ldcg(cc);
      push = __ldcg(ce) > 2ull * fe;  // uniform
      if (push) {
        for (int64_t base = gw * 32; base < fe; base += gws * 32) {
          const int64_t e = base + lane;
          if (e < fe) {
            uint32_t u;
            const int64_t v = target(e, u);
            if (v >= 0) {
              ull x[W];
              ld_front<W>(fcur + (int64_t)u * W, x, keep);
#pragma unroll
              for (int w = 0; w < W; w++)
                if (x[w]) red_or_hint(a.hacc + v * W + w, x[w], keep);
            }
          }
        }
        if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
        // finalise the candidates (thread per candidate, the accumulator cleared for the next level); the
        // block-uniform loop lets block_push list the vertices given new bits
        for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x; i0 < nc; i0 += (int64_t)gridDim.x * blockDim.x) {
          const int64_t i = i0 + threadIdx.x;
          bool nb = false;
          uint32_t v = 0, dv = 0;
          if (i < nc) {
            v = a.cand[i];
            ull acc[W];
#pragma unroll
            for (int w = 0; w < W; w++) {
              acc[w] = __ldcg(a.hacc + (int64_t)v * W + w);
              a.hacc[(int64_t)v * W + w] = 0ull;
            }
            nb = ms_thread_finalise<W>(a, v, acc, fnext, L);
            if (nb) {
              atomicOr(fbm_next + (v >> 5), 1u << (v & 31));
              dv = (uint32_t)(a.off[v + 1] - a.off[v]);
            } else {
              // saturated (or nothing new): finished for the rest of the sweep once its current word is empty
              bool sat = true;
#pragma unroll
              for (int w = 0; w < W; w++) sat &= __ldcg(a.seen + (int64_t)v * W + w) == full[w];
              if (sat && !fbit(fbm_cur, v)) atomicOr(a.done + (v >> 5), 1u << (v & 31));
            }
          }
          block_push(nb, v, dv, a.qv[so], a.qe[so], a.lctr + so, &psc);
        }
      } else {
        // pull the candidates (hub rows by chunks below); the block-uniform loop lets block_push list the
        // vertices given new bits
        const int gpb = blockDim.x / MS_GROUP;  // groups per block
        for (int64_t i0 = (int64_t)blockIdx.x * gpb; i0 < nc; i0 += (int64_t)gridDim.x * gpb) {
          const int64_t i = i0 + threadIdx.x / MS_GROUP;
          const bool act = i < nc;
          const int64_t v = act ? (int64_t)a.cand[i] : 0;
          bool nb;
          uint32_t dv;
          ms_pull_vertex<W>(a, full, fcur, fnext, fbm_cur, fbm_next, use_bm, L, v, act, gl, true, nb, dv);
          block_push(nb, (uint32_t)v, dv, a.qv[so], a.qe[so], a.lctr + so, &psc);
        }
      }
    } else {
      // light rows, 32-vertex tiles per warp: one load of the done bitmap skips finished vertices (ms_dense_tile)
      const int64_t ntiles = (n + 31) / 32;
      unsigned *tc = a.tctr + (L & 3);
      if (a.win) {
        // index-local graph: the CTA takes MS_WIN vertices at a time from the level counter, stages the frontier
        // words of [vs - MS_WIN, vs + 2 MS_WIN) and its warps work through the tiles with that window
        const int64_t nst = (n + MS_WIN - 1) / MS_WIN;
        const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
        for (;;) {
          __syncthreads();  // the previous window is consumed and s_tile read
          if (threadIdx.x == 0) s_tile = atomicAdd(tc, 1u);
          __syncthreads();
          const int64_t st = s_tile;
          if (st >= nst) break;  // uniform
          const int64_t vs = st * MS_WIN, wlo = vs - MS_WIN;
          const int64_t t0 = vs / 32, t1 = min(t0 + MS_WIN / 32, ntiles);
          bool any = false;  // an unfinished vertex in the super-tile (else no staging)
          for (int64_t tt = t0 + threadIdx.x; tt < t1; tt += blockDim.x) {
            const int64_t b0 = tt * 32;
            const unsigned valid = n - b0 >= 32 ? 0xffffffffu : ((1u << (n - b0)) - 1u);
            any |= (~__ldcg(a.done + tt) & valid) != 0u;
          }
          if (!__syncthreads_or(any)) continue;
          for (int64_t j = threadIdx.x; j < 3 * MS_WIN; j += blockDim.x) {
            const int64_t gv = wlo + j;
            ull x[W];
#pragma unroll
            for (int w = 0; w < W; w++) x[w] = 0ull;
            if (gv >= 0 && gv < n) ld_words<W>(fcur + gv * W, x);
#pragma unroll
            for (int w = 0; w < W; w++) ms_dyn[j * W + w] = x[w];
          }
          __syncthreads();
          for (int64_t tt = t0 + warp; tt < t1; tt += nwarps)
            ms_dense_tile<W, true>(a, full, fcur, fnext, fbm_cur, fbm_next, use_bm, L, tt, ms_dyn, wlo, my_stat);
        }
      } else {
        // warps take MS_TILE_CHUNK tiles at a time from a level counter, so warps that meet heavy
        // neighbourhoods do not hold the level's end back
        int64_t t = 0, tend = 0;
        for (;; t++) {
          if (t >= tend) {
            unsigned tb = 0;
            if (lane == 0) tb = atomicAdd(tc, (unsigned)MS_TILE_CHUNK);
            t = (int64_t)__shfl_sync(PHDE_FULL_MASK, tb, 0);
            if (t >= ntiles) break;
            tend = min(t + MS_TILE_CHUNK, ntiles);
          }
          ms_dense_tile<W, false>(a, full, fcur, fnext, fbm_cur, fbm_next, use_bm, L, t, nullptr, 0, my_stat);
        }
      }
    }
    // heavy-row chunks (a push level finalised every candidate, hubs included): one warp per chunk,
    // OR-reduced, combined with atomicOr; a pull level takes its candidates only
    for (int64_t c = push ? a.nchunks : gw; c < a.nchunks; c += gws) {
      const int64_t v = a.chunk_row[c], e0 = a.chunk_e0[c], e1 = min(a.off[v + 1], e0 + MS_CHUNK);
      if (sparse && __ldcg(a.stamp + v) != L + 1) continue;
      ull acc[W];
      ld_words<W>(a.seen + v * W, acc);  // seen changes only in the finalisation after the barrier
      bool sat = true;
#pragma unroll
      for (int w = 0; w < W; w++) {
        sat &= acc[w] == full[w];
        acc[w] = 0ull;
      }
      if (sat) continue;  // the row's finalisation writes zero new bits either way
      const uint64_t stream = l2_policy_evict_first(), keep = l2_policy_evict_last();
      for (int64_t e = e0 + lane; e < e1; e += 32) {
        const uint32_t u = ld_nc_hint(a.adj + e, stream);
        if (use_bm && !fbit(fbm_cur, u)) continue;
        ull x[W];
        ld_front<W>(fcur + (int64_t)u * W, x, keep);
#pragma unroll
        for (int w = 0; w < W; w++) acc[w] |= x[w];
      }
#pragma unroll
      for (int w = 0; w < W; w++) {
        ull x = acc[w];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x |= __shfl_xor_sync(PHDE_FULL_MASK, x, o);
        if (lane == 0 && x) atomicOr(a.hacc + v * W + w, x);
      }
    }
    if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
    for (int64_t h = push ? a.nheavy : gt; h < a.nheavy; h += gts) {
      const int64_t v = a.heavy_rows[h];
      ull acc[W];
#pragma unroll
      for (int w = 0; w < W; w++) {
        acc[w] = __ldcg(a.hacc + v * W + w);
        a.hacc[v * W + w] = 0ull;
      }
      if (ms_thread_finalise<W>(a, v, acc, fnext, L)) {
        atomicOr(fbm_next + (v >> 5), 1u << (v & 31));
        const uint32_t dv = (uint32_t)(a.off[v + 1] - a.off[v]);
        if (sparse) {
          const ull pos = atomicAdd(a.lctr + so, (1ull << 32) | (ull)dv);
          a.qv[so][(uint32_t)(pos >> 32)] = (uint32_t)v;
          a.qe[so][(uint32_t)(pos >> 32)] = (uint32_t)(pos & 0xffffffffull);
        } else {
          my_stat += (1ull << 32) | (ull)dv;
        }
      }
    }
    // this level's totals: the list counter (sparse) or one atomic per block (dense)
    if (!sparse) {
      my_stat = warp_sum(my_stat);
      if (lane == 0 && my_stat) atomicAdd(&s_stat, my_stat);
      __syncthreads();
      if (threadIdx.x == 0 && s_stat) atomicAdd(a.lstat + so, s_stat);
    }
    if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
    built_z = built_f;
    built_f = sparse;
    const ull ostat = sparse ? __ldcg(a.lctr + so) : __ldcg(a.lstat + so);
    const unsigned tot = (unsigned)(ostat >> 32);
    if (a.trace && gt == 0 && L < a.trace_cap) {
      a.trace[2 * L] = global_timer_ns();
      a.trace[2 * L + 1] = tot;
    }
    if (tot == 0u) break;
  }
  if (gt == 0) *a.levels_out = L + 1;
}

// The heavy-row plan, and the graph's index locality: over the rows of every MS_WIN_SAMPLE-th vertex (their
// first 64 neighbours), the neighbours within MS_WIN of the row's index (counts[2]) against all (counts[3]).
__global__ void ms_heavy_plan_kernel(const int64_t *off, const uint32_t *adj, int64_t n, int64_t *heavy_rows,
                                     int64_t *chunk_row, int64_t *chunk_e0, ull *counts) {
  ull near = 0, seen = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e0 = off[v], deg = off[v + 1] - e0;
    if (v % MS_WIN_SAMPLE == 0)
      for (int64_t e = e0; e < e0 + min(deg, (int64_t)64); e++) {
        const int64_t d = (int64_t)adj[e] - v;
        near += (d >= -MS_WIN && d <= MS_WIN) ? 1ull : 0ull;
        seen++;
      }
    if (deg <= MS_HEAVY) continue;
    heavy_rows[atomicAdd(counts, 1ull)] = v;
    const int64_t nch = (deg + MS_CHUNK - 1) / MS_CHUNK;
    const int64_t base = (int64_t)atomicAdd(counts + 1, (ull)nch);
    for (int64_t c = 0; c < nch; c++) {
      chunk_row[base + c] = v;
      chunk_e0[base + c] = e0 + c * MS_CHUNK;
    }
  }
  near = warp_sum(near);
  seen = warp_sum(seen);
  if ((threadIdx.x & 31) == 0 && seen) {
    atomicAdd(counts + 2, near);
    atomicAdd(counts + 3, seen);
  }
}

// D[p*n + v] = R[v*RW + cols[p]] - 1 for the requested columns, through 32-row shared-memory tiles;
// per-column exact sums of squares and an unreached flag on the way.
__global__ void gather_columns_kernel(const uint16_t *R, int64_t n, int RW, const int *cols, int ncols, int32_t *D,
                                      ull *sumsq, int *unreached) {
  extern __shared__ uint16_t tile[];  // [32][RW + 2]: the padded row stride puts consecutive rows in
                                      // consecutive banks (a plain 512-byte stride maps every lane to one bank)
  __shared__ ull s_ssq[GATHER_SMEM_COLS];  // per-CTA column sums; column p is always summed by warp p % nw
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int TLD = RW + 2, hw = RW / 2;  // row stride in 16-bit entries; 32-bit words per row
  for (int p = threadIdx.x; p < GATHER_SMEM_COLS; p += blockDim.x) s_ssq[p] = 0ull;
  int bad = 0;
  for (int64_t v0 = (int64_t)blockIdx.x * 32; v0 < n; v0 += (int64_t)gridDim.x * 32) {
    const int rows = n - v0 < 32 ? (int)(n - v0) : 32;
    __syncthreads();
    const uint32_t *src = (const uint32_t *)(R + v0 * RW);
    uint32_t *dst = (uint32_t *)tile;
    for (int i = threadIdx.x; i < rows * hw; i += blockDim.x) {
      const int r = i / hw, c = i - r * hw;
      dst[r * (TLD / 2) + c] = src[i];
    }
    __syncthreads();
    for (int p = warp; p < ncols; p += nw) {
      int d = -1;
      if (lane < rows) {
        d = (int)tile[lane * TLD + cols[p]] - 1;
        D[(int64_t)p * n + v0 + lane] = d;
        bad |= d < 0;
      }
      // d < 2^16, so d * d < 2^32: the warp sums its high and low 16-bit halves with one 32-bit reduction
      // each (no overflow: 32 * 2^16 fits), instead of a 64-bit shuffle tree
      const uint32_t sq = d > 0 ? (uint32_t)d * (uint32_t)d : 0u;
      const ull tot = ((ull)__reduce_add_sync(PHDE_FULL_MASK, sq >> 16) << 16) +
                      (ull)__reduce_add_sync(PHDE_FULL_MASK, sq & 0xffffu);
      if (lane == 0 && tot) {
        if (p < GATHER_SMEM_COLS)
          s_ssq[p] += tot;
        else
          atomicAdd(sumsq + p, tot);
      }
    }
  }
  __syncthreads();
  for (int p = threadIdx.x; p < ncols && p < GATHER_SMEM_COLS; p += blockDim.x)
    if (s_ssq[p]) atomicAdd(sumsq + p, s_ssq[p]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(unreached, 1);
}

// The same columns from a level-mode sweep: per 32-vertex tile, thread (row, source word) walks the levels and
// writes every source's distance into the tile (-1: never reached), then the columns are taken as above.
__global__ void level_columns_kernel(const ull *lvl, int nlev, int W, int64_t n, const int *cols, int ncols, int32_t *D,
                                     ull *sumsq, int *unreached) {
  __shared__ int16_t tile[32][64 * MS_MAXW + 2];
  __shared__ ull s_ssq[GATHER_SMEM_COLS];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int p = threadIdx.x; p < GATHER_SMEM_COLS; p += blockDim.x) s_ssq[p] = 0ull;
  int bad = 0;
  for (int64_t v0 = (int64_t)blockIdx.x * 32; v0 < n; v0 += (int64_t)gridDim.x * 32) {
    const int rows = n - v0 < 32 ? (int)(n - v0) : 32;
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * W; e += blockDim.x) {
      const int r = e / W, w = e - r * W;
      if (r >= rows) continue;
      ull seen = 0;
      for (int L = 0; L < nlev; L++) {
        const ull x = __ldg(lvl + ((int64_t)L * n + v0 + r) * W + w);
        seen |= x;
        for (ull y = x; y; y &= y - 1) tile[r][64 * w + __ffsll((long long)y) - 1] = (int16_t)L;
      }
      for (ull y = ~seen; y; y &= y - 1) tile[r][64 * w + __ffsll((long long)y) - 1] = (int16_t)-1;
    }
    __syncthreads();
    for (int p = warp; p < ncols; p += nw) {
      int d = -1;
      if (lane < rows) {
        d = (int)tile[lane][cols[p]];
        D[(int64_t)p * n + v0 + lane] = d;
        bad |= d < 0;
      }
      const uint32_t sq = d > 0 ? (uint32_t)d * (uint32_t)d : 0u;
      const ull tot = ((ull)__reduce_add_sync(PHDE_FULL_MASK, sq >> 16) << 16) +
                      (ull)__reduce_add_sync(PHDE_FULL_MASK, sq & 0xffffu);
      if (lane == 0 && tot) {
        if (p < GATHER_SMEM_COLS)
          s_ssq[p] += tot;
        else
          atomicAdd(sumsq + p, tot);
      }
    }
  }
  __syncthreads();
  for (int p = threadIdx.x; p < ncols && p < GATHER_SMEM_COLS; p += blockDim.x)
    if (s_ssq[p]) atomicAdd(sumsq + p, s_ssq[p]);
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
  ull *counts = (ull *)phde_buf(ctx, "ms.counts", sizeof(ull) * 4);
  if (!hrows || !crow || !ce0 || !counts) return PHDE_ERR_OOM;
  if (ctx->ms_plan_epoch != ctx->graph_epoch) {
    PHDE_CK(ctx, cudaMemsetAsync(counts, 0, sizeof(ull) * 4, ctx->stream));
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->nsm * 8));
    ms_heavy_plan_kernel<<<g, 256, 0, ctx->stream>>>(ctx->d_off, ctx->d_adj, n, hrows, crow, ce0, counts);
    PHDE_LAUNCHED(ctx);
    ull h[4];
    PHDE_CK(ctx, cudaMemcpyAsync(h, counts, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->ms_nheavy = (int64_t)h[0];
    ctx->ms_nchunks = (int64_t)h[1];
    // index-local when at least 90 % of the sampled neighbours lie within MS_WIN: 2-D RGGs and meshes numbered
    // by cell (100 %; the window pays there), not 3-D RGGs (63 %: the staging costs more than the gathers it
    // saves) nor R-MAT (a few per cent)
    ctx->ms_local = h[3] > 0 && 10 * h[2] >= 9 * h[3];
    ctx->ms_plan_epoch = ctx->graph_epoch;
  }
  *chunk_row = crow;
  *chunk_e0 = ce0;
  *nchunks = ctx->ms_nchunks;
  *chunk = MS_CHUNK;
  return PHDE_OK;
}

// The sweep: sources d_src (nlist entries; bit = entry, or entry % period for batches), optionally without
// host synchronisation (sync false: no error read-back and no level count -- for captured sequences).
// Level mode (lvl_cap > 0, one sweep of at most 256 sources, no batch): no record, the per-level frontier arrays
// 0 .. lvl_cap are kept and returned through *lv; more levels than lvl_cap give PHDE_ERR_TOO_LARGE.
static int msbfs_run(phde_ctx *ctx, const int64_t *d_src, int nsrc, int nlist, int period, bool sync, uint16_t **R_out,
                     int *RW_out, int lvl_cap = 0, MsLevels *lv = nullptr) {
  const int64_t n = ctx->n;
  if (nsrc < 1 || (period > 0 && (nsrc != period || period > 64 * MS_MAXW))) return PHDE_ERR_INVALID;
  if (lvl_cap > 0 && (nsrc > 64 * MS_MAXW || period > 0 || !lv || !sync)) return PHDE_ERR_INVALID;
  int last_nlev = 0;
  const int RW = (nsrc + 63) / 64 * 64;
  const int Wmax = MS_MAXW;
  uint16_t *R = nullptr;
  ull *seen = (ull *)phde_buf(ctx, "ms.seen", sizeof(ull) * n * Wmax);
  ull *f0, *f1, *lvl = nullptr;
  if (lvl_cap > 0) {
    const int W1 = (nsrc + 63) / 64;
    lvl = (ull *)phde_buf(ctx, "ms.lvl", sizeof(ull) * (size_t)(lvl_cap + 1) * n * W1);
    if (!lvl) return PHDE_ERR_OOM;
    f0 = lvl;
    f1 = lvl + n * W1;
  } else {
    R = (uint16_t *)phde_buf(ctx, "ms.R", sizeof(uint16_t) * n * RW);
    f0 = (ull *)phde_buf(ctx, "ms.f0", sizeof(ull) * n * Wmax);
    f1 = (ull *)phde_buf(ctx, "ms.f1", sizeof(ull) * n * Wmax);
  }
  ull *hacc = (ull *)phde_buf(ctx, "ms.hacc", sizeof(ull) * n * Wmax);
  int *levels = (int *)phde_buf(ctx, "ms.levels", sizeof(int));
  const int64_t nw32 = (n + 31) / 32, lcap = n + 256;  // a level list holds each vertex once; the sources' may repeat
  uint32_t *bms = (uint32_t *)phde_buf(ctx, "ms.done", sizeof(uint32_t) * nw32);
  uint32_t *fbm = (uint32_t *)phde_buf(ctx, "ms.fbm", sizeof(uint32_t) * 3 * nw32);
  uint32_t *lists = (uint32_t *)phde_buf(ctx, "ms.lists", sizeof(uint32_t) * 8 * lcap);  // qv[4], qe[4]
  uint32_t *cand = (uint32_t *)phde_buf(ctx, "ms.cand", sizeof(uint32_t) * n);
  int32_t *stamp = (int32_t *)phde_buf(ctx, "ms.stamp", sizeof(int32_t) * n);
  const size_t ctr_bytes = sizeof(ull) * 10 + sizeof(unsigned) * 6;  // lctr[4], lstat[4], cedge[2], ccount[2], tctr[4]
  ull *lctr = (ull *)phde_buf(ctx, "ms.lctr", ctr_bytes);
  if ((!R && !lvl) || !seen || !f0 || !f1 || !hacc || !levels || !bms || !fbm || !lists || !cand || !stamp || !lctr)
    return PHDE_ERR_OOM;
  const int64_t *crow, *ce0;
  int64_t nch, chunk;
  int rc0 = phde_heavy_chunks(ctx, &crow, &ce0, &nch, &chunk);
  if (rc0) return rc0;
  const int64_t *hrows = (const int64_t *)phde_buf(ctx, "ms.hrows", 0);
  if (R) PHDE_CK(ctx, cudaMemsetAsync(R, 0, sizeof(uint16_t) * (size_t)n * RW, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(hacc, 0, sizeof(ull) * n * Wmax, ctx->stream));
  // optional per-level trace (PHDE_MSBFS_TRACE=<file>): end time and vertices given new bits per level
  const char *trace_path = getenv("PHDE_MSBFS_TRACE");
  const int trace_cap = 4096;
  ull *trace = trace_path ? (ull *)phde_buf(ctx, "ms.trace", sizeof(ull) * 2 * trace_cap) : nullptr;
  for (int s0 = 0; s0 < nsrc; s0 += 64 * Wmax) {
    const int ns = std::min(nsrc - s0, 64 * Wmax);
    const int W = (ns + 63) / 64;
    const void *fn = W == 1 ? (const void *)msbfs_kernel<1>
                   : W == 2 ? (const void *)msbfs_kernel<2>
                   : W == 3 ? (const void *)msbfs_kernel<3>
                            : (const void *)msbfs_kernel<4>;
    // dense levels of index-local graphs stage frontier windows (PHDE_MSBFS_WINDOW=0 or 1 picks outright)
    const char *we = getenv("PHDE_MSBFS_WINDOW");
    const bool win = we ? atoi(we) != 0 : ctx->ms_local;
    const size_t dyn = win ? sizeof(ull) * 3 * MS_WIN * W : 0;
    PHDE_CK(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    // with a window, all of the unified L1/shared storage as shared memory (two CTAs per SM); without, the
    // default split
    PHDE_CK(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                      win ? (int)cudaSharedmemCarveoutMaxShared : (int)cudaSharedmemCarveoutDefault));
    int per_sm = 0;
    PHDE_CK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, MS_THREADS, dyn));
    if (per_sm < 1) return phde_fail(ctx, PHDE_ERR_CUDA, "msbfs kernel cannot be resident");
    per_sm = std::min(per_sm, 4);
    PHDE_CK(ctx, cudaMemsetAsync(seen, 0, sizeof(ull) * n * W, ctx->stream));
    PHDE_CK(ctx, cudaMemsetAsync(f0, 0, sizeof(ull) * n * W, ctx->stream));
    PHDE_CK(ctx, cudaMemsetAsync(f1, 0, sizeof(ull) * n * W, ctx->stream));  // level 1 writes candidates only
    PHDE_CK(ctx, cudaMemsetAsync(lctr, 0, ctr_bytes, ctx->stream));
    PHDE_CK(ctx, cudaMemsetAsync(bms, 0, sizeof(uint32_t) * nw32, ctx->stream));
    PHDE_CK(ctx, cudaMemsetAsync(fbm, 0, sizeof(uint32_t) * 3 * nw32, ctx->stream));
    PHDE_CK(ctx, cudaMemsetAsync(stamp, 0, sizeof(int32_t) * n, ctx->stream));
    int rc = phde_reset_sync(ctx);
    if (rc) return rc;
    MsArgs a;
    a.off = ctx->d_off;
    a.adj = ctx->d_adj;
    a.n = n;
    a.nsrc = ns;
    a.src = d_src + s0;
    a.nlist = period > 0 ? nlist : ns;
    a.period = period;
    a.R = R;
    a.RW = RW;
    a.col0 = s0;
    a.lvl = lvl;
    a.lcap = lvl_cap;
    a.seen = seen;
    a.front[0] = f0;
    a.front[1] = f1;
    a.hacc = hacc;
    a.heavy_rows = hrows;
    a.nheavy = ctx->ms_nheavy;
    a.chunk_row = crow;
    a.chunk_e0 = ce0;
    a.nchunks = nch;
    for (int i = 0; i < 4; i++) {
      a.qv[i] = lists + (int64_t)i * lcap;
      a.qe[i] = lists + (int64_t)(4 + i) * lcap;
    }
    a.lctr = lctr;
    a.lstat = lctr + 4;
    a.cedge = lctr + 8;
    a.ccount = (unsigned *)(lctr + 10);
    a.tctr = a.ccount + 2;
    a.stamp = stamp;
    a.cand = cand;
    a.sparse_edges = std::max<int64_t>(ctx->nnz / 16, 1);
    a.levels_out = levels;
    a.trace = trace;
    a.trace_cap = trace_cap;
    a.done = bms;
    for (int i = 0; i < 3; i++) a.fbm[i] = fbm + (int64_t)i * nw32;
    a.win = win ? 1 : 0;
    a.gs = ctx->d_sync;
    a.err = ctx->d_err;
    a.timeout_ns = ctx->timeout_ns;
    void *args[] = {&a};
    const double before = ctx->kernel_ms;
    cudaEventRecord(ctx->kev[0], ctx->stream);
    PHDE_CK(ctx, cudaLaunchCooperativeKernel(fn, dim3(ctx->nsm * per_sm), dim3(MS_THREADS), args, dyn, ctx->stream));
    PHDE_LAUNCHED(ctx);
    cudaEventRecord(ctx->kev[1], ctx->stream);
    ctx->kev_pending = true;
    if (!sync) {  // captured batched layouts: no host wait; the error word is read after the whole sequence
      ctx->kev_pending = false;
      continue;
    }
    if ((rc = phde_check_device_err(ctx, "multi-source BFS"))) return rc;  // synchronises, collects the time
    ctx->msbfs_ms += ctx->kernel_ms - before;
    int nlev = 0;
    PHDE_CK(ctx, cudaMemcpyAsync(&nlev, levels, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->msbfs_levels += nlev;
    last_nlev = nlev;
    if (trace) {
      int nl = 0;
      std::vector<ull> h(2 * trace_cap);
      PHDE_CK(ctx, cudaMemcpyAsync(&nl, levels, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      PHDE_CK(ctx, cudaMemcpyAsync(h.data(), trace, sizeof(ull) * h.size(), cudaMemcpyDeviceToHost, ctx->stream));
      PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
      if (FILE *f = fopen(trace_path, "a")) {
        fprintf(f, "# sweep col0=%d W=%d levels=%d grid=%d\n", s0, W, nl, ctx->nsm * per_sm);
        for (int l = 0; l < std::min(nl, trace_cap); l++)
          fprintf(f, "%d,%llu,%llu\n", l, (unsigned long long)(l ? h[2 * l] - h[2 * l - 2] : 0ull),
                  (unsigned long long)h[2 * l + 1]);
        fclose(f);
      }
    }
  }
  *R_out = R;
  *RW_out = RW;
  if (lv) {
    lv->lvl = lvl;
    lv->W = (nsrc + 63) / 64;
    lv->nlev = last_nlev;  // one sweep
  }
  return PHDE_OK;
}

// Multi-source BFS from `nsrc` sources (device array; sweeps of up to 256).  The result is the row-major
// record R (n x RW uint16, RW = nsrc rounded up to 64; level + 1, 0 = unreached), returned through *R_out.
int phde_msbfs_record(phde_ctx *ctx, const int64_t *d_src, int nsrc, uint16_t **R_out, int *RW_out) {
  return msbfs_run(ctx, d_src, nsrc, nsrc, 0, true, R_out, RW_out);
}

// The same search in level mode (no record; see msbfs_run): the frontier arrays of levels 0 .. lv->nlev - 1.
int phde_msbfs_levels(phde_ctx *ctx, const int64_t *d_src, int nsrc, int lvl_cap, MsLevels *lv) {
  uint16_t *R;
  int RW;
  return msbfs_run(ctx, d_src, nsrc, nsrc, 0, true, &R, &RW, lvl_cap, lv);
}

// A batch's candidates in one sweep: d_src holds nlist vertices, entry i searching with bit i % period
// (period <= 256: every graph's candidates take bits 0 .. period-1).  No host synchronisation.
int phde_msbfs_record_batched(phde_ctx *ctx, const int64_t *d_src, int nlist, int period, uint16_t **R_out,
                              int *RW_out) {
  return msbfs_run(ctx, d_src, period, nlist, period, false, R_out, RW_out);
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
  const size_t smem = sizeof(uint16_t) * 32 * (size_t)(RW + 2);
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

// Columns `h_cols` (source indices) of a level-mode sweep into D, as phde_record_columns.
int phde_level_columns(phde_ctx *ctx, const MsLevels *lv, const int *h_cols, int ncols, int32_t *D,
                       unsigned long long *sumsq, int *h_unreached) {
  const int64_t n = ctx->n;
  int *dcols = (int *)phde_buf(ctx, "ms.cols", sizeof(int) * ncols);
  ull *ssq = sumsq ? sumsq : (ull *)phde_buf(ctx, "ms.ssq_tmp", sizeof(ull) * ncols);
  int *unr = (int *)phde_buf(ctx, "ms.unreached", sizeof(int));
  if (!dcols || !ssq || !unr) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemcpyAsync(dcols, h_cols, sizeof(int) * ncols, cudaMemcpyHostToDevice, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(ssq, 0, sizeof(ull) * ncols, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(unr, 0, sizeof(int), ctx->stream));
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 31) / 32, (int64_t)ctx->nsm * 4));
  level_columns_kernel<<<g, 256, 0, ctx->stream>>>(lv->lvl, lv->nlev, lv->W, n, dcols, ncols, D, ssq, unr);
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
