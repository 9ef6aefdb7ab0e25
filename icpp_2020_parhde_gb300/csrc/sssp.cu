// sssp.cu -- exact weighted shortest paths for WParHDE, one persistent cooperative launch per source.
//
// Replaces gapbs DeltaStep (gapbs/sssp.cc:53-140) as called from WParHDE (WParHDE.cpp:116 through
// DrawingBase.cpp:116).  The reference runs delta-stepping with thread-local bins of width delta and
// CAS-min relaxations; this kernel keeps the same bucketing idea in a GPU shape (near-far):
//   near set  : vertices whose tentative distance is below the current band limit T, processed in
//               rounds; every round relaxes all out-edges of the near frontier, edge-balanced exactly
//               like the top-down BFS step (owner found by binary search over the frontier's
//               start-edge prefix array), with atomicMin on the distance;
//   far pile  : improved vertices at or beyond T; when the near frontier empties, T jumps to the band
//               holding the smallest far distance and the pile is split into the new near frontier and
//               what stays far.
// Both lists are de-duplicated with per-vertex stamps.  Shortest-path distances are unique, so the
// result is bit-exact against the reference whatever the band width or relaxation order.
#include <algorithm>
#include <cstdlib>

#include "ctx.h"

namespace {

constexpr int SS_THREADS = 1024;
constexpr int32_t SSSP_INF = 0x7fffffff / 2;  // kDistInf, gapbs/sssp.cc:50

struct SsArgs {
  const int64_t *off;
  const uint32_t *adj;
  const int32_t *w;
  int64_t n;
  const int64_t *src;
  int32_t *dist;  // [n], SSSP_INF initially
  int32_t delta;
  int lmax;                         // block-local relaxation rounds per grid round
  uint32_t *qv0, *qv1, *qe0, *qe1;  // near frontier (vertex, start-edge prefix)
  uint32_t *qo0, *qo1;              // near frontier: the vertex's first adjacency index
  uint32_t *far0, *far1;            // far pile
  int32_t *stamp_near, *stamp_far;  // [n], -1 initially
  ull *ctr;                         // [4] near ring
  unsigned *farctr;                 // [2]
  ull *minfar;                      // [2], alternating by phase
  ull *edges;  // [0] += adjacency entries read, [1] += rounds; may be null
  GridSync *gs;
  int *err;
  uint64_t timeout_ns;
};

constexpr int SS_LQ = SS_THREADS;  // block-local queue capacity (one entry per thread for its prefix scan)

// The block-local queue: vertices a block improved below the band limit, relaxed again by the same block
// before the grid barrier.
struct LocalQ {
  uint32_t v[2][SS_LQ], deg[2][SS_LQ], first[2][SS_LQ], off[2][SS_LQ];  // first: exclusive prefix of deg
  uint32_t cnt[2];  // entries claimed (may exceed SS_LQ: the excess went to the grid queue)
  uint32_t total;   // edges of the buffer being relaxed
  uint32_t warp_sum[32];
};

// One edge u -> v (index j).  Returns the flags of what the improvement asks for: near (below the band
// limit T) or far; atomicMin has already lowered dist[v].  ov/dv: v's adjacency start and out-degree.
__device__ __forceinline__ void relax_edge(const SsArgs &a, uint32_t u, int64_t j, int64_t T, uint32_t &v, bool &near,
                                           bool &far, uint32_t &ov, uint32_t &dv) {
  v = __ldg(a.adj + j);
  const int32_t du = __ldcg(a.dist + u);
  const int32_t nd = du + __ldg(a.w + j);
  if (nd < __ldcg(a.dist + v)) {
    const int64_t ov0 = __ldg(a.off + v), ov1 = __ldg(a.off + v + 1);  // in flight with the atomic
    const int32_t old = atomicMin(a.dist + v, nd);
    if (nd < old) {
      near = nd < T;
      far = !near;
      ov = (uint32_t)ov0;
      dv = (uint32_t)(ov1 - ov0);
    }
  }
}

// Offers near improvements to local buffer b (warp-aggregated slot claims in shared memory); those that do
// not fit fall back to the grid queue, de-duplicated by the round's stamp.  Far improvements are
// de-duplicated by the phase's stamp.  On return to_near / to_far are the grid-queue and far-pile flags.
__device__ __forceinline__ void place(const SsArgs &a, LocalQ &lq, int b, bool local_ok, uint32_t v, uint32_t dv,
                                      uint32_t ov, int32_t it, int32_t phase, bool &to_near, bool &to_far) {
  const int lane = threadIdx.x & 31;
  bool want = local_ok && to_near;
  const unsigned m = __ballot_sync(PHDE_FULL_MASK, want);
  if (m) {
    const int leader = __ffs(m) - 1;
    uint32_t wb = 0;
    if (lane == leader) wb = atomicAdd(&lq.cnt[b], (uint32_t)__popc(m));
    wb = __shfl_sync(PHDE_FULL_MASK, wb, leader);
    if (want) {
      const uint32_t slot = wb + __popc(m & ((1u << lane) - 1u));
      if (slot < SS_LQ) {
        lq.v[b][slot] = v;
        lq.deg[b][slot] = dv;
        lq.off[b][slot] = ov;
        to_near = false;  // handled locally
      }
    }
  }
  if (to_near) to_near = atomicExch(a.stamp_near + v, it + 1) != it + 1;
  if (to_far) to_far = atomicExch(a.stamp_far + v, phase) != phase;
}

template <int MINB>
__global__ void __launch_bounds__(SS_THREADS, MINB) sssp_nearfar_kernel(SsArgs a) {
  __shared__ Push2Scratch psc;
  __shared__ uint32_t s_win[SS_THREADS / 32][32];
  __shared__ ull red[32];
  extern __shared__ __align__(16) unsigned char ss_dyn[];  // the LocalQ, present only when a.lmax > 0
  LocalQ &lq = *reinterpret_cast<LocalQ *>(ss_dyn);
  const int tid = threadIdx.x;
  const int64_t gstride = (int64_t)gridDim.x * blockDim.x;
  const int64_t gbase = (int64_t)blockIdx.x * blockDim.x;
  const int64_t src = *a.src;
  if (blockIdx.x == 0 && tid == 0) {
    a.dist[src] = 0;
    a.qv0[0] = (uint32_t)src;
    a.qe0[0] = 0;
    a.qo0[0] = (uint32_t)a.off[src];
    a.stamp_near[src] = 0;
  }
  ull edges_local = 0;
  uint32_t f_cnt = 1, f_edges = (uint32_t)(a.off[src + 1] - a.off[src]);
  unsigned far_cnt = 0;
  int64_t T = a.delta;
  int32_t it = 0, phase = 0;
  uint32_t step = 0;
  if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;

  while (true) {
    // ---- relaxation rounds over the near frontier ----
    while (f_cnt > 0) {
      const uint32_t *qin_v = (step & 1) ? a.qv1 : a.qv0;
      const uint32_t *qin_e = (step & 1) ? a.qe1 : a.qe0;
      const uint32_t *qin_o = (step & 1) ? a.qo1 : a.qo0;
      uint32_t *qout_v = (step & 1) ? a.qv0 : a.qv1;
      uint32_t *qout_e = (step & 1) ? a.qe0 : a.qe1;
      uint32_t *qout_o = (step & 1) ? a.qo0 : a.qo1;
      ull *octr = a.ctr + (step & 3);
      uint32_t *far_in = (phase & 1) ? a.far1 : a.far0;
      unsigned *fctr = a.farctr + (phase & 1);
      if (blockIdx.x == 0 && tid == 0) a.ctr[(step + 1) & 3] = 0ull;
      const int64_t E = f_edges;
      const bool local_on = a.lmax > 0;
      if (local_on) {
        if (tid == 0) lq.cnt[0] = lq.cnt[1] = 0;
        __syncthreads();
      }
      for (int64_t base = gbase; base < E; base += gstride) {
        const int64_t e = base + tid, e0w = base + (tid & ~31);
        bool to_near = false, to_far = false;
        uint32_t v = 0, dv = 0, ov = 0;
        if (e0w < E) {  // warp-uniform
          uint32_t es;
          const uint32_t s = warp_owner_slots(qin_e, f_cnt, (uint32_t)e0w, s_win[tid >> 5], es);
          if (e < E) {
            const uint32_t u = qin_v[s];
            const int64_t j = (int64_t)qin_o[s] + (e - (int64_t)es);  // qin_o[s] = off[u], loaded with u
            edges_local++;
            relax_edge(a, u, j, T, v, to_near, to_far, ov, dv);
          }
        }
        place(a, lq, 0, local_on, v, dv, ov, it, phase, to_near, to_far);
        block_push2(to_near, v, dv, qout_v, qout_e, octr, to_far, far_in, fctr, &psc, qout_o, ov);
      }
      // ---- block-local rounds: relax what this block improved, without a grid barrier; the last local
      // round (and any overflow of the local queue) sends its improvements to the grid queue ----
      int cur = 0;
      for (int li = 0; li < a.lmax; li++) {
        __syncthreads();  // the buffer's entries are written
        const uint32_t cnt = min(lq.cnt[cur], (uint32_t)SS_LQ);
        if (cnt == 0) break;
        {  // exclusive prefix of the out-degrees, one entry per thread
          const int lane = tid & 31, w = tid >> 5;
          const uint32_t d = (uint32_t)tid < cnt ? lq.deg[cur][tid] : 0u;
          uint32_t x = d;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(PHDE_FULL_MASK, x, o);
            if (lane >= o) x += y;
          }
          if (lane == 31) lq.warp_sum[w] = x;
          __syncthreads();
          if (w == 0) {
            const uint32_t ws_ = lane < (int)(blockDim.x >> 5) ? lq.warp_sum[lane] : 0u;
            uint32_t y = ws_;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
              const uint32_t z = __shfl_up_sync(PHDE_FULL_MASK, y, o);
              if (lane >= o) y += z;
            }
            lq.warp_sum[lane] = y - ws_;
            if (lane == 31) lq.total = y;
          }
          __syncthreads();
          if ((uint32_t)tid < cnt) lq.first[cur][tid] = lq.warp_sum[w] + x - d;
          if (tid == 0) lq.cnt[cur ^ 1] = 0;
          __syncthreads();
        }
        const uint32_t total = lq.total;
        for (uint32_t eb = 0; eb < total; eb += blockDim.x) {
          const uint32_t e = eb + tid;
          bool to_near = false, to_far = false;
          uint32_t v = 0, dv = 0, ov = 0;
          if (e < total) {
            uint32_t lo = 0, hi = cnt;  // the entry owning local edge e
            while (hi - lo > 1) {
              const uint32_t mid = (lo + hi) >> 1;
              if (lq.first[cur][mid] <= e)
                lo = mid;
              else
                hi = mid;
            }
            const uint32_t u = lq.v[cur][lo];
            const int64_t j = (int64_t)lq.off[cur][lo] + (e - lq.first[cur][lo]);
            edges_local++;
            relax_edge(a, u, j, T, v, to_near, to_far, ov, dv);
          }
          place(a, lq, cur ^ 1, li + 1 < a.lmax, v, dv, ov, it, phase, to_near, to_far);
          block_push2(to_near, v, dv, qout_v, qout_e, octr, to_far, far_in, fctr, &psc, qout_o, ov);
        }
        cur ^= 1;
      }
      if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
      const ull out = __ldcg(octr);
      f_cnt = (uint32_t)(out >> 32);
      f_edges = (uint32_t)(out & 0xffffffffull);
      it++;
      step++;
    }
    // ---- near frontier empty: move to the band of the closest far vertex ----
    far_cnt = __ldcg(a.farctr + (phase & 1));
    if (far_cnt == 0) break;
    const uint32_t *far_in = (phase & 1) ? a.far1 : a.far0;
    uint32_t *far_out = (phase & 1) ? a.far0 : a.far1;
    unsigned *fout_ctr = a.farctr + ((phase + 1) & 1);
    ull *mslot = a.minfar + (phase & 1);
    ull mloc = ~0ull;
    for (int64_t i = gbase + tid; i < far_cnt; i += gstride) {
      const int32_t d = __ldcg(a.dist + far_in[i]);
      if (d >= T) mloc = (ull)d < mloc ? (ull)d : mloc;
    }
    const ull bm = block_max_u64(~mloc, red);  // block minimum through the complement
    if (tid == 0 && bm != 0ull) atomicMin(mslot, ~bm);
    if (blockIdx.x == 0 && tid == 0) {
      *fout_ctr = 0u;
      a.minfar[(phase + 1) & 1] = ~0ull;
    }
    if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
    const ull mf = __ldcg(mslot);
    const int64_t T_old = T;
    if (mf != ~0ull) T = ((int64_t)mf / a.delta + 1) * (int64_t)a.delta;
    // split the pile: this is a step of its own, writing the next round's input queue
    uint32_t *qout_v = (step & 1) ? a.qv0 : a.qv1;
    uint32_t *qout_e = (step & 1) ? a.qe0 : a.qe1;
    uint32_t *qout_o = (step & 1) ? a.qo0 : a.qo1;
    ull *octr = a.ctr + (step & 3);
    if (blockIdx.x == 0 && tid == 0) a.ctr[(step + 1) & 3] = 0ull;
    for (int64_t base = gbase; base < (int64_t)far_cnt; base += gstride) {
      const int64_t i = base + tid;
      bool to_near = false, keep = false;
      uint32_t v = 0, dv = 0, ov = 0;
      if (i < far_cnt) {
        v = far_in[i];
        const int32_t d = __ldcg(a.dist + v);
        if (d >= T_old && d < T) {
          if (atomicExch(a.stamp_near + v, it + 1) != it + 1) {
            to_near = true;
            ov = (uint32_t)a.off[v];
            dv = (uint32_t)(a.off[v + 1] - ov);
          }
        } else if (d >= T) {
          keep = atomicExch(a.stamp_far + v, phase + 1) != phase + 1;
        }
      }
      block_push2(to_near, v, dv, qout_v, qout_e, octr, keep, far_out, fout_ctr, &psc, qout_o, ov);
    }
    if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
    const ull out = __ldcg(octr);
    f_cnt = (uint32_t)(out >> 32);
    f_edges = (uint32_t)(out & 0xffffffffull);
    it++;
    step++;
    phase++;
    if (f_cnt == 0 && __ldcg(a.farctr + (phase & 1)) == 0) break;
  }
  ull etot = block_sum(edges_local, red);
  if (tid == 0 && a.edges) atomicAdd(a.edges, etot);
  if (blockIdx.x == 0 && tid == 0 && a.edges) atomicAdd(a.edges + 1, (ull)it);  // rounds (relaxation + split)
}

// Fold one finished distance column into the Kcenters state (WParHDE.cpp:117-136).
__global__ void fold_kernel(const int32_t *col, int64_t n, int32_t *min_d, ull *key_out, ull *ssq_out, int *err) {
  __shared__ ull red[32];
  ull kbest = 0, ssq = 0;
  int bad = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    const int32_t d = col[v];
    if (d >= SSSP_INF || d < 0) {
      bad = 1;
      continue;
    }
    ssq += (ull)d * (ull)d;
    int32_t m = min_d[v];
    if (d < m) {
      m = d;
      min_d[v] = m;
    }
    const ull key = ((ull)(uint32_t)m << 32) | (ull)(0xffffffffu - (uint32_t)v);
    kbest = key > kbest ? key : kbest;
  }
  if (__syncthreads_or(bad)) {
    if (threadIdx.x == 0) atomicCAS(err, 0, PHDE_ERR_DISCONNECTED);
    return;
  }
  ssq = block_sum(ssq, red);
  kbest = block_max_u64(kbest, red);
  if (threadIdx.x == 0) {
    atomicAdd(ssq_out, ssq);
    atomicMax(key_out, kbest);
  }
}

// Choose the next source (one block): raw argmax, duplicate fix-up against the history of raw argmaxes
// (WParHDE.cpp:137-153), append the raw argmax to the history.
__global__ void select_kernel(const ull *key_in, const int32_t *min_d, int64_t n, int pass, int check_fix,
                              int64_t *hist, int64_t *next_src) {
  __shared__ ull red[32];
  const ull key = *key_in;
  const int64_t raw = (int64_t)(0xffffffffu - (uint32_t)(key & 0xffffffffull));
  const int32_t maxval = (int32_t)(key >> 32);
  int hit = 0;
  for (int i = threadIdx.x; i < pass; i += blockDim.x) hit |= (hist[i] == raw);
  hit = __syncthreads_or(hit);
  int64_t next = raw;
  if (check_fix && hit) {
    ull best = 0;
    for (int64_t v = threadIdx.x; v < n; v += blockDim.x) {
      if (min_d[v] != maxval) continue;
      bool inh = false;
      for (int i = 0; i < pass && !inh; i++) inh = hist[i] == v;
      if (!inh) best = (ull)v + 1 > best ? (ull)v + 1 : best;
    }
    best = block_max_u64(best, red);
    if (best) next = (int64_t)best - 1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    hist[pass] = raw;
    *next_src = next;
  }
}

}  // namespace

int phde_fill_i32(phde_ctx *ctx, int32_t *p, int64_t n, int32_t v);

namespace {
// sum of the (non-negative) edge weights, for the band width
__global__ void weight_sum_kernel(const int32_t *w, int64_t nnz, ull *sum) {
  ull s = 0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x)
    s += (ull)(w[e] > 0 ? w[e] : 0);
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(sum, s);
}
}  // namespace

int phde_run_sssp(phde_ctx *ctx, const int64_t *d_src, int32_t *d_col, int32_t delta, unsigned long long *d_edges) {
  const int64_t n = ctx->n;
  if (ctx->nnz >= (int64_t)0xffffffffll || n >= (int64_t)0xffffffffll)
    return phde_fail(ctx, PHDE_ERR_INVALID, "graphs with 2^32 or more vertices or adjacency entries are not supported");
  if (!ctx->d_w) return phde_fail(ctx, PHDE_ERR_WEIGHTS, "SSSP needs edge weights");
  // The band width changes the work, never the distances (they are unique).  The reference's width
  // (10000, WParHDE.cpp:104) is far above typical weights, which makes the search nearly Bellman-Ford: on
  // a 256^3 grid with weights in [1, 255] a band of 8 mean weights is three times faster (on a 64^3 grid,
  // where every round is short, the wide band is as fast or faster).  So graphs of 2^20 vertices or more
  // use min(delta, max(64, 8 * mean weight)); PHDE_SSSP_DELTA sets the band outright.
  if (const char *e = getenv("PHDE_SSSP_DELTA")) {
    delta = atoi(e);
  } else if (n >= (int64_t)1 << 20) {
    if (ctx->w_mean_epoch != ctx->graph_epoch) {
      ull *wsum = (ull *)phde_buf(ctx, "ss.wsum", sizeof(ull));
      if (!wsum) return PHDE_ERR_OOM;
      PHDE_CK(ctx, cudaMemsetAsync(wsum, 0, sizeof(ull), ctx->stream));
      const int g = (int)std::max<int64_t>(1, std::min<int64_t>((ctx->nnz + 255) / 256, (int64_t)ctx->nsm * 8));
      weight_sum_kernel<<<g, 256, 0, ctx->stream>>>(ctx->d_w, ctx->nnz, wsum);
      PHDE_LAUNCHED(ctx);
      ull h = 0;
      PHDE_CK(ctx, cudaMemcpyAsync(&h, wsum, sizeof(ull), cudaMemcpyDeviceToHost, ctx->stream));
      PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
      ctx->w_mean = ctx->nnz > 0 ? (double)h / (double)ctx->nnz : 1.0;
      ctx->w_mean_epoch = ctx->graph_epoch;
    }
    const double band = std::max(64.0, 8.0 * ctx->w_mean);
    if (band < (double)delta) delta = (int32_t)band;
  }
  if (delta < 1) delta = 1;
  uint32_t *qv0 = (uint32_t *)phde_buf(ctx, "q.v0", sizeof(uint32_t) * n);
  uint32_t *qv1 = (uint32_t *)phde_buf(ctx, "q.v1", sizeof(uint32_t) * n);
  uint32_t *qe0 = (uint32_t *)phde_buf(ctx, "q.e0", sizeof(uint32_t) * n);
  uint32_t *qe1 = (uint32_t *)phde_buf(ctx, "q.e1", sizeof(uint32_t) * n);
  uint32_t *qo0 = (uint32_t *)phde_buf(ctx, "ss.qo0", sizeof(uint32_t) * n);
  uint32_t *qo1 = (uint32_t *)phde_buf(ctx, "ss.qo1", sizeof(uint32_t) * n);
  uint32_t *far0 = (uint32_t *)phde_buf(ctx, "ss.far0", sizeof(uint32_t) * n);
  uint32_t *far1 = (uint32_t *)phde_buf(ctx, "ss.far1", sizeof(uint32_t) * n);
  int32_t *stn = (int32_t *)phde_buf(ctx, "ss.stamp_near", sizeof(int32_t) * n);
  int32_t *stf = (int32_t *)phde_buf(ctx, "ss.stamp_far", sizeof(int32_t) * n);
  ull *ctr = (ull *)phde_buf(ctx, "q.ctr", sizeof(ull) * 4);
  unsigned *farctr = (unsigned *)phde_buf(ctx, "ss.farctr", sizeof(unsigned) * 2);
  ull *minfar = (ull *)phde_buf(ctx, "ss.minfar", sizeof(ull) * 2);
  if (!qv0 || !qv1 || !qe0 || !qe1 || !qo0 || !qo1 || !far0 || !far1 || !stn || !stf || !ctr || !farctr || !minfar) return PHDE_ERR_OOM;
  int rc;
  if ((rc = phde_fill_i32(ctx, d_col, n, SSSP_INF))) return rc;
  PHDE_CK(ctx, cudaMemsetAsync(stn, 0xff, sizeof(int32_t) * n, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(stf, 0xff, sizeof(int32_t) * n, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(ctr, 0, sizeof(ull) * 4, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(farctr, 0, sizeof(unsigned) * 2, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(minfar, 0xff, sizeof(ull) * 2, ctx->stream));
  if ((rc = phde_reset_sync(ctx))) return rc;
  // Resident CTAs per SM: one (with the registers it wants) below 2^20 vertices, where rounds are short and
  // latency-bound (a 64^3 grid: 1.5 ms per pass against 2.1 ms with two), two (registers capped at 32) on
  // larger graphs (a 256^3 grid: 14.3 ms against 16.1 ms with one); PHDE_SSSP_CTAS=1 or 2 picks outright.
  const char *ce = getenv("PHDE_SSSP_CTAS");
  const int want = ce ? (atoi(ce) == 1 ? 1 : 2) : (n < ((int64_t)1 << 20) ? 1 : 2);
  const void *kfn = want == 1 ? (const void *)sssp_nearfar_kernel<1> : (const void *)sssp_nearfar_kernel<2>;
  // block-local rounds per grid round (PHDE_SSSP_LOCAL, none by default): each block keeps relaxing the
  // vertices it improved below the band limit (up to SS_LQ of them) this many times before the grid
  // barrier.  On a 256^3 grid four local rounds took 10-12.5 ms per pass on some runs and 43-50 ms on
  // others (same inputs, band 1024; band 512 stayed near 13 ms), against 14.6 ms without: the blocks that
  // run ahead inside the band relax with distances other blocks later lower, and how much of that is
  // wasted depends on timing.  Off until that is bounded.
  const char *le = getenv("PHDE_SSSP_LOCAL");
  const int lmax = le ? std::max(0, atoi(le)) : 0;
  const size_t dyn = lmax > 0 ? sizeof(LocalQ) : 0;  // the queue's shared memory, below the 48 KB default
  int per_sm = 0;
  PHDE_CK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, SS_THREADS, dyn));
  if (per_sm < 1) return phde_fail(ctx, PHDE_ERR_CUDA, "sssp kernel cannot be resident");
  per_sm = std::min(per_sm, want);
  SsArgs a;
  a.off = ctx->d_off;
  a.adj = ctx->d_adj;
  a.w = ctx->d_w;
  a.n = n;
  a.src = d_src;
  a.dist = d_col;
  a.delta = delta;
  a.lmax = lmax;
  a.qv0 = qv0;
  a.qv1 = qv1;
  a.qe0 = qe0;
  a.qe1 = qe1;
  a.qo0 = qo0;
  a.qo1 = qo1;
  a.far0 = far0;
  a.far1 = far1;
  a.stamp_near = stn;
  a.stamp_far = stf;
  a.ctr = ctr;
  a.farctr = farctr;
  a.minfar = minfar;
  a.edges = d_edges;
  a.gs = ctx->d_sync;
  a.err = ctx->d_err;
  a.timeout_ns = ctx->timeout_ns;
  void *args[] = {&a};
  cudaEventRecord(ctx->kev[0], ctx->stream);
  PHDE_CK(ctx, cudaLaunchCooperativeKernel(kfn, dim3(ctx->nsm * per_sm),
                                           dim3(SS_THREADS), args, dyn, ctx->stream));
  PHDE_LAUNCHED(ctx);
  cudaEventRecord(ctx->kev[1], ctx->stream);
  ctx->kev_pending = true;
  return PHDE_OK;
}

int phde_run_select(phde_ctx *ctx, const int32_t *d_col, int32_t *d_min, int pass, int check_fix, int64_t *d_hist,
                    int64_t *d_next_src, unsigned long long *d_sumsq) {
  ull *key = (ull *)phde_buf(ctx, "sel.key", sizeof(ull));
  if (!key) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(key, 0, sizeof(ull), ctx->stream));
  int blocks = (int)std::min<int64_t>((ctx->n + 511) / 512, (int64_t)ctx->nsm * 4);
  fold_kernel<<<std::max(blocks, 1), 512, 0, ctx->stream>>>(d_col, ctx->n, d_min, key, d_sumsq, ctx->d_err);
  PHDE_LAUNCHED(ctx);
  select_kernel<<<1, 1024, 0, ctx->stream>>>(key, d_min, ctx->n, pass, check_fix, d_hist, d_next_src);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}
