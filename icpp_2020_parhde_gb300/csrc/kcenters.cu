// kcenters.cu -- Kcenters pivot distances: P breadth-first searches in ONE persistent cooperative launch.
//
// Replaces the serial Kcenters loop of variants/ParHDE.cpp:118-157 (and DrawingBase.cpp:119-172), whose
// every pass calls gapbs DOBFS (gapbs/bfs.cc:144-185) and then an OpenMP min/argmax reduction.  Each pass
// here is a level-synchronous direction-optimising BFS over the device CSR, followed by the Kcenters
// selection folded into one sweep; grid barriers (bounded waits) separate the levels, so the 3k
// dependent passes cost no host round trip.
//
// Per level, with frontier F_L (vertices at hop distance L):
//   top-down  : edge-balanced -- thread e takes the e-th out-edge of F_L, finds its owner vertex by
//               binary search over the frontier's start-edge prefix array, and claims the neighbour
//               with a CAS on its distance entry (-1 -> L+1);
//   bottom-up : every unvisited vertex scans its neighbours for one in the frontier and stops at the
//               first; the frontier is a bitmap (one bit per vertex) that every block copies into
//               shared memory at the start of the level when it fits (80 KB for 646k vertices), so the
//               membership test is a shared-memory hit;
//   both append the new frontier with block-aggregated 64-bit atomics that keep (slot, edge prefix)
//   together, so the next top-down step is load balanced even around hub vertices.
// The top-down / bottom-up switch has the reference's form (bfs.cc:159-183): go bottom-up when the
// frontier's out-edges exceed edges_to_check / alpha, stay there while the frontier grows or exceeds
// n / beta, beta = 18 as there, alpha = 6 instead of 15: on the GPU a bottom-up level scans every
// unvisited vertex, and at the frontier sizes between the two rules (R-MAT 22: 8.7 M out-edges) the
// top-down level is the faster one (130-235 us against 300-320 us).  Hop distances are unique, so the
// result is bit-exact whatever the direction schedule.
//
// Selection (ParHDE.cpp:127-155): min_d[v] = min(min_d[v], d_p[v]); the next source is the vertex of
// largest min_d, lowest index first (a 64-bit atomicMax on (min_d << 32) | ~v); if that vertex is in
// the history, the duplicate fix-up takes the highest-index vertex with the same min_d that is not.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ctx.h"

namespace {

constexpr int KC_THREADS = 1024;

struct KcArgs {
  const int64_t *off;
  const uint32_t *adj;
  int64_t n, nnz;
  int32_t *D;  // n * P, column-major, pre-filled with -1
  int P;
  int variant;  // 0: ParHDE history (raw argmax), 1: fixed sources, 2: DrawingBase history (used source)
  int require_all;  // an unreached vertex is an error (always for the Kcenters variants)
  const int64_t *fixed_src;
  int64_t *sources;
  int32_t *min_d;   // [n], INT32_MAX initially
  ull *sumsq;       // [P]
  ull *keys;        // [P]
  ull *fixkey;      // [P]
  uint32_t *qv0, *qv1, *qe0, *qe1;
  uint32_t *bm[3];  // frontier bitmaps, W words each, rotating with the global step (zero initially)
  int64_t W;        // words per bitmap
  int smem_bm;      // copy the frontier bitmap into shared memory for bottom-up levels
  ull *ctr;         // [4] ring of (count << 32 | edges)
  ull *edges;       // [1] adjacency entries read
  ull *trace;       // optional timeline: per level {globaltimer, pass<<40 | level<<32 | in_bu, frontier count, edges}
  int trace_cap;    // entries of 4 words
  GridSync *gs;
  int *err;
  uint64_t timeout_ns;
  int alpha, beta;
  // batched layouts: the graph is the disjoint union of B graphs (vertex ranges vbase[b]..vbase[b+1]);
  // every pass runs one BFS per graph, all from the same launch, and the selection is per graph.  Then
  // sources, keys and sumsq are indexed [p * B + b], and gid[v] is v's graph.
  int B;
  const int64_t *vbase;
  const int32_t *gid;
  ull *qinit;       // [1] level-0 queue counter of the pass (count << 32 | edges)
};

// Per-graph fold of a batched pass: the max of `key` and the sum of `ssq` over the lanes of one graph
// (a warp covers consecutive vertices, so almost always one graph), one atomic per graph per warp.
__device__ __forceinline__ void batch_fold(ull *keys, ull *sumsq, int g, ull key, ull ssq, bool valid) {
  const int lane = threadIdx.x & 31;
  const int g0 = __shfl_sync(PHDE_FULL_MASK, g, 0);
  if (__all_sync(PHDE_FULL_MASK, valid && g == g0)) {
    const ull km = warp_max_u64(key);
    const ull ss = warp_sum(ssq);
    if (lane == 0) {
      atomicMax(keys + g0, km);
      if (ss) atomicAdd(sumsq + g0, ss);
    }
  } else if (valid) {
    atomicMax(keys + g, key);
    if (ssq) atomicAdd(sumsq + g, ssq);
  }
}

__global__ void __launch_bounds__(KC_THREADS) kcenters_bfs_kernel(KcArgs a) {
  __shared__ PushScratch psc;
  __shared__ ull red[32];
  extern __shared__ uint32_t s_hist[];  // [P]: every block keeps the same selection history, then the bitmap
  uint32_t *s_bm = s_hist + ((a.P + 3) & ~3);
  const int64_t n = a.n;
  const int tid = threadIdx.x;
  const int64_t gstride = (int64_t)gridDim.x * blockDim.x;
  const int64_t gbase = (int64_t)blockIdx.x * blockDim.x;
  int64_t src = a.variant == 1 ? a.fixed_src[0] : 0;
  uint32_t step = 0;
  ull edges_local = 0;

  for (int p = 0; p < a.P; p++) {
    int32_t *Dp = a.D + (int64_t)p * n;
    int64_t s_off = 0;
    uint32_t sdeg = 0;
    uint32_t f_cnt = 1, f_edges = 0;
    if (a.B == 0) {
      if (tid == 0) {
        Dp[src] = 0;
        // the level-0 frontier bitmap holds only the source (the previous pass left it empty)
        atomicOr(a.bm[step % 3] + (src >> 5), 1u << (src & 31));
        if (blockIdx.x == 0) a.sources[p] = src;
      }
      __syncthreads();
      s_off = a.off[src];
      sdeg = (uint32_t)(a.off[src + 1] - s_off);
      f_edges = sdeg;
    } else {
      // batched: block 0 queues every graph's source (vertex 0 of the graph, then the previous pass's
      // farthest vertex) as the level-0 frontier, in graph order
      if (blockIdx.x == 0) {
        if (tid == 0) *a.qinit = 0ull;
        __syncthreads();
        uint32_t *q0v = (step & 1) ? a.qv1 : a.qv0;
        uint32_t *q0e = (step & 1) ? a.qe1 : a.qe0;
        for (int b0 = 0; b0 < a.B; b0 += blockDim.x) {
          const int b = b0 + tid;
          uint32_t v = 0, dv = 0;
          if (b < a.B) {
            v = p == 0 ? (uint32_t)a.vbase[b]
                       : 0xffffffffu - (uint32_t)(__ldcg(a.keys + (int64_t)(p - 1) * a.B + b) & 0xffffffffull);
            dv = (uint32_t)(a.off[v + 1] - a.off[v]);
            Dp[v] = 0;
            atomicOr(a.bm[step % 3] + (v >> 5), 1u << (v & 31));
            a.sources[(int64_t)p * a.B + b] = v;
          }
          block_push(b < a.B, v, dv, q0v, q0e, a.qinit, &psc);
        }
      }
      if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
      const ull q = __ldcg(a.qinit);
      f_cnt = (uint32_t)(q >> 32);
      f_edges = (uint32_t)(q & 0xffffffffull);
    }
    int64_t edges_to_check = a.nnz, scout = f_edges;
    bool in_bu = false;
    int64_t awake = 0, old_awake = 0;
    int32_t L = 0;

    while (f_cnt > 0) {
      if (!in_bu) {
        if (scout > edges_to_check / a.alpha) {
          in_bu = true;
          awake = f_cnt;
        } else {
          edges_to_check -= scout;
        }
      }
      if (in_bu) old_awake = awake;
      const uint32_t *qin_v = (step & 1) ? a.qv1 : a.qv0;
      const uint32_t *qin_e = (step & 1) ? a.qe1 : a.qe0;
      uint32_t *qout_v = (step & 1) ? a.qv0 : a.qv1;
      uint32_t *qout_e = (step & 1) ? a.qe0 : a.qe1;
      ull *octr = a.ctr + (step & 3);
      if (blockIdx.x == 0 && tid == 0) a.ctr[(step + 2) & 3] = 0ull;
      const uint32_t *bm_cur = a.bm[step % 3];
      uint32_t *bm_next = a.bm[(step + 1) % 3];
      {  // the bitmap of the previous level becomes the next level's (empty) output
        uint32_t *bm_clr = a.bm[(step + 2) % 3];
        for (int64_t w = gbase + tid; w < a.W; w += gstride) bm_clr[w] = 0u;
      }

      if (!in_bu) {
        const int64_t E = f_edges;
        for (int64_t base = gbase; base < E; base += gstride) {
          const int64_t e = base + tid;
          bool claimed = false;
          uint32_t v = 0, dv = 0;
          if (e < E) {
            int64_t j;
            if (L == 0 && a.B == 0) {
              j = s_off + e;
            } else {
              const uint32_t s = owner_slot(qin_e, f_cnt, (uint32_t)e);
              j = a.off[qin_v[s]] + (e - (int64_t)qin_e[s]);
            }
            v = __ldg(a.adj + j);
            edges_local++;
            if (Dp[v] == -1 && atomicCAS(Dp + v, -1, L + 1) == -1) {
              claimed = true;
              dv = (uint32_t)(a.off[v + 1] - a.off[v]);
              atomicOr(bm_next + (v >> 5), 1u << (v & 31));
            }
          }
          block_push(claimed, v, dv, qout_v, qout_e, octr, &psc);
        }
      } else {
        if (a.smem_bm) {
          for (int64_t w = tid; w < a.W; w += blockDim.x) s_bm[w] = __ldcg(bm_cur + w);
          __syncthreads();
        }
        const uint32_t *front = a.smem_bm ? s_bm : bm_cur;
        for (int64_t base = gbase; base < n; base += gstride) {
          const int64_t v = base + tid;
          bool found = false;
          uint32_t dv = 0;
          if (v < n && Dp[v] == -1) {
            const int64_t j0 = a.off[v], j1 = a.off[v + 1];
            // four neighbours per round (their adjacency entries, then their bitmap words, all in flight): a
            // vertex far from the frontier tests every neighbour, one dependent L2 round trip each otherwise
            for (int64_t j = j0; j < j1 && !found; j += 4) {
              uint32_t u[4], word[4];
#pragma unroll
              for (int q = 0; q < 4; q++) u[q] = j + q < j1 ? __ldg(a.adj + j + q) : 0u;
#pragma unroll
              for (int q = 0; q < 4; q++)
                word[q] = j + q < j1 ? (a.smem_bm ? front[u[q] >> 5] : __ldcg(front + (u[q] >> 5))) : 0u;
#pragma unroll
              for (int q = 0; q < 4; q++) {
                if (found || j + q >= j1) continue;
                edges_local++;  // counted up to the first frontier neighbour, as a one-at-a-time scan would
                found = (word[q] >> (u[q] & 31)) & 1u;
              }
            }
            if (found) {
              Dp[v] = L + 1;
              dv = (uint32_t)(j1 - j0);
            }
          }
          // one bitmap word per warp: the warp covers 32 consecutive, 32-aligned vertices
          const uint32_t bal = __ballot_sync(PHDE_FULL_MASK, found);
          const int64_t v0 = v - (tid & 31);
          if ((tid & 31) == 0 && v0 < n) bm_next[v0 >> 5] = bal;
          block_push(found, (uint32_t)v, dv, qout_v, qout_e, octr, &psc);
        }
      }
      if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
      const ull out = __ldcg(octr);
      f_cnt = (uint32_t)(out >> 32);
      f_edges = (uint32_t)(out & 0xffffffffull);
      if (a.trace && blockIdx.x == 0 && tid == 0 && step < (uint32_t)a.trace_cap) {
        ull *tr = a.trace + 4 * (size_t)step;
        tr[0] = global_timer_ns();
        tr[1] = ((ull)p << 40) | ((ull)(uint32_t)L << 32) | (in_bu ? 1ull : 0ull);
        tr[2] = f_cnt;
        tr[3] = f_edges;
      }
      if (in_bu) {
        awake = f_cnt;
        if (!(awake >= old_awake || awake > n / a.beta)) {
          in_bu = false;
          scout = 1;
        }
      } else {
        scout = f_edges;
      }
      L++;
      step++;
    }

    // ---- fold the finished column: min distance, farthest vertex, sum of squares ----
    ull kbest = 0, ssq = 0;
    int bad = 0;
    if (a.B > 0) {  // batched: per-graph keys and sums; the grid-stride loop keeps warps together
      for (int64_t base = gbase; base < n; base += gstride) {
        const int64_t v = base + tid;
        ull key = 0, sq = 0;
        int g = -1;
        const bool valid = v < n;
        if (valid) {
          const int32_t d = Dp[v];
          g = a.gid[v];
          if (d < 0) {
            bad = 1;
          } else {
            sq = (ull)d * (ull)d;
            int32_t m = a.min_d[v];
            if (d < m) {
              m = d;
              a.min_d[v] = m;
            }
            key = ((ull)(uint32_t)m << 32) | (ull)(0xffffffffu - (uint32_t)v);
          }
        }
        batch_fold(a.keys + (int64_t)p * a.B, a.sumsq + (int64_t)p * a.B, g, key, sq, valid);
      }
      if (__syncthreads_or(bad)) {
        if (tid == 0) atomicCAS(a.err, 0, PHDE_ERR_DISCONNECTED);
        return;
      }
      if (p + 1 == a.P) break;
      if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
      continue;
    }
    for (int64_t v = gbase + tid; v < n; v += gstride) {
      const int32_t d = Dp[v];
      if (d < 0) {
        bad = 1;
        continue;
      }
      ssq += (ull)d * (ull)d;
      if (a.variant != 1) {
        int32_t m = a.min_d[v];
        if (d < m) {
          m = d;
          a.min_d[v] = m;
        }
        const ull key = ((ull)(uint32_t)m << 32) | (ull)(0xffffffffu - (uint32_t)v);
        kbest = key > kbest ? key : kbest;
      }
    }
    if ((a.variant != 1 || a.require_all) && __syncthreads_or(bad)) {
      if (tid == 0) atomicCAS(a.err, 0, PHDE_ERR_DISCONNECTED);
      return;
    }
    ssq = block_sum(ssq, red);
    if (tid == 0) atomicAdd(a.sumsq + p, ssq);
    if (a.variant != 1) {
      kbest = block_max_u64(kbest, red);
      if (tid == 0) atomicMax(a.keys + p, kbest);
    }
    if (p + 1 == a.P) break;
    if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;

    if (a.variant == 1) {
      src = a.fixed_src[p + 1];
      continue;
    }
    const ull key = __ldcg(a.keys + p);
    const uint32_t raw = 0xffffffffu - (uint32_t)(key & 0xffffffffull);
    const int32_t maxval = (int32_t)(key >> 32);
    int hit = 0;
    for (int i = tid; i < p; i += blockDim.x) hit |= (s_hist[i] == raw);
    hit = __syncthreads_or(hit);
    int64_t next = raw;
    if (p >= 1 && hit) {
      // duplicate fix-up (ParHDE.cpp:144-154 at one thread): highest-index vertex with the same
      // minimum distance that is not in the history
      for (int64_t v = gbase + tid; v < n; v += gstride) {
        if (a.min_d[v] != maxval) continue;
        bool inh = false;
        for (int i = 0; i < p && !inh; i++) inh = (s_hist[i] == (uint32_t)v);
        if (!inh) atomicMax(a.fixkey + p, (ull)v + 1ull);
      }
      if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
      const ull fk = __ldcg(a.fixkey + p);
      if (fk) next = (int64_t)(fk - 1ull);
    }
    __syncthreads();
    if (tid == 0) s_hist[p] = a.variant == 2 ? (uint32_t)src : raw;
    __syncthreads();
    src = next;
  }
  ull etot = block_sum(edges_local, red);
  if (tid == 0 && a.edges) atomicAdd(a.edges, etot);
}

// ---------------------------------------------------------------------------------------------
// Batched Kcenters with one CTA per graph (batches of small graphs).  A grid-wide level barrier costs
// more than a small graph's whole level, and every grid-wide level waits for the deepest graph of the
// batch; here each CTA takes whole graphs from a work list (largest first) and runs their 3k passes with
// block barriers only.  Per pass: a level-synchronous top-down BFS from the pass's source over queues in
// the graph's own slice of the union's queue arrays -- a thread per frontier vertex, its neighbours' loads
// issued in batches of eight before the claims (atomicCAS on the distance entry; appends through a
// shared-memory counter) --, then the Kcenters fold over the graph's vertices (min distance,
// farthest vertex with the lowest index on ties -- the key (min_d << 32) | ~v --, exact sum of squares).
// Same outputs as the batched variant of kcenters_bfs_kernel: D columns over the union, sources, keys and
// sums indexed [p * B + b].
struct KbArgs {
  const int64_t *off;
  const uint32_t *adj;
  int64_t N;
  int32_t *D;
  int P, B;
  const int64_t *vbase;
  const int32_t *order;  // graphs, largest first
  unsigned *next;        // work-list counter (zeroed)
  int64_t *sources;
  int32_t *min_d;
  ull *sumsq;
  uint32_t *q0, *q1;     // [N] each: frontier vertices
  ull *edges;
  int *err;
};

constexpr int KB_THREADS = 1024;

__global__ void __launch_bounds__(KB_THREADS) kcenters_block_kernel(KbArgs a) {
  __shared__ int s_graph;
  // level L appends through s_c[L % 3]; after the level every thread reads it, and
  // thread 0 clears s_c[(L + 2) % 3] -- last read before this level's final barrier, next used two levels on
  __shared__ ull s_c[3];
  __shared__ ull red[32];
  __shared__ int64_t s_src;
  const int tid = threadIdx.x;
  ull edges_local = 0;
  for (;;) {
    if (tid == 0) s_graph = (int)atomicAdd(a.next, 1u);
    __syncthreads();
    const int gi = s_graph;
    __syncthreads();
    if (gi >= a.B) break;
    const int b = a.order[gi];
    const int64_t vb = a.vbase[b], nb = a.vbase[b + 1] - vb;
    int64_t src = vb;  // Kcenters starts at the graph's vertex 0
    for (int p = 0; p < a.P; p++) {
      int32_t *Dp = a.D + (int64_t)p * a.N;
      if (tid == 0) {
        Dp[src] = 0;
        a.q0[vb] = (uint32_t)src;
        s_c[0] = 0ull;
        s_c[1] = 0ull;
      }
      uint32_t cnt = 1;
      const uint32_t *qin = a.q0 + vb;
      uint32_t *qout = a.q1 + vb;
      int32_t L = 0;
      __syncthreads();
      while (cnt > 0) {
        unsigned *c = (unsigned *)(s_c + (L % 3));
        // a thread per frontier vertex; its neighbours in batches of 8 with every load of a batch in flight
        // before the claims (a level's critical path is its chain of memory round trips)
        for (uint32_t i = tid; i < cnt; i += blockDim.x) {
          const uint32_t u = qin[i];
          const int64_t e1 = a.off[u + 1];
          for (int64_t e0 = a.off[u]; e0 < e1; e0 += 8) {
            uint32_t vv[8];
#pragma unroll
            for (int t = 0; t < 8; t++) vv[t] = e0 + t < e1 ? __ldg(a.adj + e0 + t) : 0xffffffffu;
            int old[8];  // all eight claims issued before any result is used
#pragma unroll
            for (int t = 0; t < 8; t++) old[t] = vv[t] != 0xffffffffu ? atomicCAS(Dp + vv[t], -1, L + 1) : 0;
#pragma unroll
            for (int t = 0; t < 8; t++) {
              if (vv[t] == 0xffffffffu) continue;
              edges_local++;
              if (old[t] == -1) qout[atomicAdd(c, 1u)] = vv[t];
            }
          }
        }
        __syncthreads();
        cnt = *c;
        if (tid == 0) s_c[(L + 2) % 3] = 0ull;
        const uint32_t *tq = qin;
        qin = qout;
        qout = (uint32_t *)tq;
        L++;
      }
      // fold: min distance, farthest vertex (lowest index on ties), exact sum of squares
      ull kbest = 0, ssq = 0;
      int bad = 0;
      for (int64_t v = vb + tid; v < vb + nb; v += blockDim.x) {
        const int32_t d = __ldcg(Dp + v);
        if (d < 0) {
          bad = 1;
          continue;
        }
        ssq += (ull)d * (ull)d;
        int32_t m = a.min_d[v];
        if (d < m) {
          m = d;
          a.min_d[v] = m;
        }
        const ull key = ((ull)(uint32_t)m << 32) | (ull)(0xffffffffu - (uint32_t)v);
        kbest = key > kbest ? key : kbest;
      }
      bad = __syncthreads_or(bad);
      ssq = block_sum(ssq, red);
      kbest = block_max_u64(kbest, red);
      if (tid == 0) {
        a.sumsq[(int64_t)p * a.B + b] = ssq;
        a.sources[(int64_t)p * a.B + b] = src;
        if (bad) atomicCAS(a.err, 0, PHDE_ERR_DISCONNECTED);
        s_src = (int64_t)(0xffffffffu - (uint32_t)(kbest & 0xffffffffull));
      }
      __syncthreads();
      src = s_src;
      if (bad) break;
    }
  }
  const ull etot = block_sum(edges_local, red);
  if (tid == 0 && a.edges) atomicAdd(a.edges, etot);
}

__global__ void fill_i32_kernel(int32_t *p, int64_t n, int32_t v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

}  // namespace

int phde_fill_i32(phde_ctx *ctx, int32_t *p, int64_t n, int32_t v) {
  int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->nsm * 8);
  if (blocks < 1) blocks = 1;
  fill_i32_kernel<<<blocks, 256, 0, ctx->stream>>>(p, n, v);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

int phde_run_bfs_passes(phde_ctx *ctx, int P, int variant, const int64_t *d_fixed_src, int32_t *d_D,
                        int64_t *d_sources, unsigned long long *d_sumsq, unsigned long long *d_edges, int require_all) {
  const int64_t n = ctx->n;
  if (ctx->nnz >= (int64_t)0xffffffffll || n >= (int64_t)0xffffffffll)
    return phde_fail(ctx, PHDE_ERR_INVALID, "graphs with 2^32 or more vertices or adjacency entries are not supported");
  // variant 3: batched ParHDE Kcenters over the uploaded batch (per-graph sources, keys and sums)
  const int B = variant == 3 ? ctx->batch_B : 0;
  if (variant == 3 && B < 1) return phde_fail(ctx, PHDE_ERR_INVALID, "no batch uploaded");
  const int64_t PB = (int64_t)P * (B ? B : 1);
  int32_t *min_d = (int32_t *)phde_buf(ctx, "kc.min_d", sizeof(int32_t) * n);
  ull *keys = (ull *)phde_buf(ctx, "kc.keys", sizeof(ull) * PB);
  ull *fixkey = (ull *)phde_buf(ctx, "kc.fixkey", sizeof(ull) * P);
  ull *qinit = (ull *)phde_buf(ctx, "kc.qinit", sizeof(ull));
  uint32_t *qv0 = (uint32_t *)phde_buf(ctx, "q.v0", sizeof(uint32_t) * n);
  uint32_t *qv1 = (uint32_t *)phde_buf(ctx, "q.v1", sizeof(uint32_t) * n);
  uint32_t *qe0 = (uint32_t *)phde_buf(ctx, "q.e0", sizeof(uint32_t) * n);
  uint32_t *qe1 = (uint32_t *)phde_buf(ctx, "q.e1", sizeof(uint32_t) * n);
  ull *ctr = (ull *)phde_buf(ctx, "q.ctr", sizeof(ull) * 4);
  const int64_t W = (n + 31) / 32;
  uint32_t *bms = (uint32_t *)phde_buf(ctx, "kc.bitmaps", sizeof(uint32_t) * 3 * W);
  if (!bms) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(bms, 0, sizeof(uint32_t) * 3 * W, ctx->stream));
  if (!min_d || !keys || !fixkey || !qinit || !qv0 || !qv1 || !qe0 || !qe1 || !ctr) return PHDE_ERR_OOM;

  PHDE_CK(ctx, cudaMemsetAsync(d_D, 0xff, sizeof(int32_t) * (size_t)n * (size_t)P, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(keys, 0, sizeof(ull) * PB, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(fixkey, 0, sizeof(ull) * P, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(ctr, 0, sizeof(ull) * 4, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(d_sumsq, 0, sizeof(ull) * PB, ctx->stream));
  int rc = phde_fill_i32(ctx, min_d, n, 0x7fffffff);
  if (rc) return rc;
  if ((rc = phde_reset_sync(ctx))) return rc;

  int per_sm = 0;
  // shared memory: the selection history, then (when it fits two blocks per SM) the frontier bitmap
  const size_t hist_bytes = sizeof(uint32_t) * (size_t)((P + 3) & ~3);
  const size_t bm_bytes = sizeof(uint32_t) * (size_t)W;
  const int smem_bm = hist_bytes + bm_bytes <= 100 * 1024;
  const size_t smem = hist_bytes + (smem_bm ? bm_bytes : 0);
  PHDE_CK(ctx, cudaFuncSetAttribute(kcenters_bfs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  PHDE_CK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kcenters_bfs_kernel, KC_THREADS, smem));
  if (per_sm < 1) return phde_fail(ctx, PHDE_ERR_CUDA, "kcenters kernel cannot be resident");
  per_sm = std::min(per_sm, 2);
  KcArgs a;
  a.off = ctx->d_off;
  a.adj = ctx->d_adj;
  a.n = n;
  a.nnz = ctx->nnz;
  a.D = d_D;
  a.P = P;
  a.variant = variant == 3 ? 0 : variant;
  a.B = B;
  a.vbase = ctx->d_vbase;
  a.gid = ctx->d_gid;
  a.qinit = qinit;
  a.require_all = require_all || variant != 1;
  a.fixed_src = d_fixed_src;
  a.sources = d_sources;
  a.min_d = min_d;
  a.sumsq = d_sumsq;
  a.keys = keys;
  a.fixkey = fixkey;
  a.qv0 = qv0;
  a.qv1 = qv1;
  a.qe0 = qe0;
  a.qe1 = qe1;
  a.ctr = ctr;
  a.bm[0] = bms;
  a.bm[1] = bms + W;
  a.bm[2] = bms + 2 * W;
  a.W = W;
  a.smem_bm = smem_bm;
  a.edges = d_edges;
  // PHDE_BFS_TRACE=<file>: write the per-level timeline of this launch as CSV after it completes
  const char *trace_file = getenv("PHDE_BFS_TRACE");
  const int trace_cap = 1 << 16;
  a.trace = nullptr;
  a.trace_cap = 0;
  if (trace_file) {
    a.trace = (ull *)phde_buf(ctx, "kc.trace", sizeof(ull) * 4 * trace_cap);
    if (a.trace) {
      PHDE_CK(ctx, cudaMemsetAsync(a.trace, 0, sizeof(ull) * 4 * trace_cap, ctx->stream));
      a.trace_cap = trace_cap;
    }
  }
  a.gs = ctx->d_sync;
  a.err = ctx->d_err;
  a.timeout_ns = ctx->timeout_ns;
  a.alpha = 6;
  a.beta = 18;
  void *args[] = {&a};
  cudaEventRecord(ctx->kev[0], ctx->stream);
  PHDE_CK(ctx, cudaLaunchCooperativeKernel((const void *)kcenters_bfs_kernel, dim3(ctx->nsm * per_sm),
                                           dim3(KC_THREADS), args, smem, ctx->stream));
  PHDE_LAUNCHED(ctx);
  cudaEventRecord(ctx->kev[1], ctx->stream);
  ctx->kev_pending = true;
  if (a.trace) {
    std::vector<ull> h((size_t)4 * trace_cap);
    PHDE_CK(ctx, cudaMemcpyAsync(h.data(), a.trace, sizeof(ull) * 4 * trace_cap, cudaMemcpyDeviceToHost, ctx->stream));
    PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (FILE *f = fopen(trace_file, "w")) {
      fprintf(f, "step,t_ns,pass,level,bottom_up,frontier,frontier_edges\n");
      for (int i = 0; i < trace_cap && h[4 * i]; i++)
        fprintf(f, "%d,%llu,%llu,%llu,%llu,%llu,%llu\n", i, h[4 * i], h[4 * i + 1] >> 40, (h[4 * i + 1] >> 32) & 0xff,
                h[4 * i + 1] & 1, h[4 * i + 2], h[4 * i + 3]);
      fclose(f);
    }
  }
  return PHDE_OK;
}

// Batched Kcenters, one CTA per graph (see kcenters_block_kernel).  d_order lists the graphs largest first.
int phde_run_bfs_batched_blocks(phde_ctx *ctx, int P, const int32_t *d_order, int32_t *d_D, int64_t *d_sources,
                                unsigned long long *d_sumsq, unsigned long long *d_edges) {
  const int64_t N = ctx->n;
  const int B = ctx->batch_B;
  int32_t *min_d = (int32_t *)phde_buf(ctx, "kc.min_d", sizeof(int32_t) * N);
  uint32_t *q0 = (uint32_t *)phde_buf(ctx, "q.v0", sizeof(uint32_t) * N);
  uint32_t *q1 = (uint32_t *)phde_buf(ctx, "q.v1", sizeof(uint32_t) * N);
  unsigned *next = (unsigned *)phde_buf(ctx, "kb.next", sizeof(unsigned));
  if (!min_d || !q0 || !q1 || !next) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(d_D, 0xff, sizeof(int32_t) * (size_t)N * (size_t)P, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(next, 0, sizeof(unsigned), ctx->stream));
  int rc = phde_fill_i32(ctx, min_d, N, 0x7fffffff);
  if (rc) return rc;
  KbArgs a;
  a.off = ctx->d_off;
  a.adj = ctx->d_adj;
  a.N = N;
  a.D = d_D;
  a.P = P;
  a.B = B;
  a.vbase = ctx->d_vbase;
  a.order = d_order;
  a.next = next;
  a.sources = d_sources;
  a.min_d = min_d;
  a.sumsq = d_sumsq;
  a.q0 = q0;
  a.q1 = q1;
  a.edges = d_edges;
  a.err = ctx->d_err;
  int per_sm = 0;
  PHDE_CK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kcenters_block_kernel, KB_THREADS, 0));
  const int grid = std::max(1, std::min(B, ctx->nsm * std::max(per_sm, 1)));
  kcenters_block_kernel<<<grid, KB_THREADS, 0, ctx->stream>>>(a);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}
