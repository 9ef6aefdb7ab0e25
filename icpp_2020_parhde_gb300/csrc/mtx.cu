// mtx.cu -- Matrix Market coordinate entries to the layout's CSR on the GPU (the work of the reference's
// mtx2csr tool, mtx2csr.cpp:117-296), and the copy of an uploaded graph back to the host.
//
// The reference builds per-vertex adjacency vectors on one thread, sorts them, drops parallel edges,
// labels components by BFS in vertex order, keeps the largest and relabels it in increasing order.  Here:
//   1. entries -> directed (src, dst, w) pairs, both directions; self loops dropped (symmetric input) or rows
//      shifted past the columns (a non-square general matrix is read as a bipartite graph);
//   2. radix sort by w, then stably by (src << 32 | dst): each (src, dst) run starts with its smallest weight,
//      which is the entry the reference keeps after sorting pairs;
//   3. first-of-run flags, exclusive scan, compaction: the deduplicated, row-sorted edge list;
//   4. connected components by lock-free union-find that hooks the larger root under the smaller, so every
//      component's root is its smallest vertex -- and the reference's "first component found in vertex
//      order" among equally large ones is the one with the smallest root;
//   5. the largest component's vertices renumbered by an exclusive scan (increasing, as the reference), new
//      offsets from its rows' degrees, every kept edge written at its row position.
// The result is the context's uploaded graph (int64 offsets, uint32 adjacency, int32 weights if given).
#include <algorithm>
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "ctx.h"

namespace {

constexpr ull KEY_NONE = ~0ull;

// Directed pairs of entry i at 2i and 2i+1 (1-indexed input).  bad: an index outside the matrix.
__global__ void mtx_directed_kernel(const uint32_t *u, const uint32_t *v, const int32_t *w, int64_t count, int64_t n1,
                                    int64_t n2, int symmetric, ull *key, uint32_t *wk, int *bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t a = u[i], b = v[i];
    const int32_t wt = w ? w[i] : 1;
    // weights sort as unsigned keys: flipping the sign bit orders int32 values
    const uint32_t wkey = (uint32_t)wt ^ 0x80000000u;
    ull k0 = KEY_NONE, k1 = KEY_NONE;
    if (a < 1 || b < 1 || (int64_t)a > n1 || (int64_t)b > (symmetric ? n1 : n2)) {
      atomicExch(bad, 1);
    } else if (symmetric) {
      if (a != b) {
        k0 = ((ull)(a - 1) << 32) | (ull)(b - 1);
        k1 = ((ull)(b - 1) << 32) | (ull)(a - 1);
      }
    } else {
      const ull row = (ull)(a - 1) + (ull)n2;  // rows after the columns
      k0 = (row << 32) | (ull)(b - 1);
      k1 = ((ull)(b - 1) << 32) | row;
    }
    key[2 * i] = k0;
    key[2 * i + 1] = k1;
    wk[2 * i] = wkey;
    wk[2 * i + 1] = wkey;
  }
}

__global__ void mtx_flags_kernel(const ull *key, int64_t m, uint32_t *flag) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    flag[i] = key[i] != KEY_NONE && (i == 0 || key[i] != key[i - 1]) ? 1u : 0u;
}

__global__ void mtx_compact_kernel(const ull *key, const uint32_t *wk, const uint32_t *flag, const uint32_t *pos,
                                   int64_t m, ull *ukey, int32_t *uw, int64_t *deg) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
    if (!flag[i]) continue;
    const ull k = key[i];
    ukey[pos[i]] = k;
    uw[pos[i]] = (int32_t)(wk[i] ^ 0x80000000u);
    atomicAdd((ull *)deg + (k >> 32), 1ull);
  }
}

__device__ __forceinline__ uint32_t uf_find(uint32_t *parent, uint32_t x) {
  // path halving; parents only ever decrease, so the walk ends at the root
  uint32_t p = parent[x];
  while (p != x) {
    const uint32_t gp = parent[p];
    if (gp != p) atomicMin(parent + x, gp);
    x = p;
    p = parent[x];
  }
  return x;
}

// Union of every edge's endpoints: the larger root goes under the smaller.  A CAS that loses to another
// thread's link retries from the new roots; each retry follows a completed link, and the retries are capped
// (an error rather than an unbounded loop).
__global__ void mtx_union_kernel(const ull *ukey, int64_t E, uint32_t *parent, int *err) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    const ull k = ukey[e];
    uint32_t a = (uint32_t)(k >> 32), b = (uint32_t)(k & 0xffffffffull);
    if (a > b) continue;  // each undirected edge once
    for (int tries = 0;; tries++) {
      if (tries > (1 << 20)) {
        atomicCAS(err, 0, PHDE_ERR_TIMEOUT);
        break;
      }
      const uint32_t ra = uf_find(parent, a), rb = uf_find(parent, b);
      if (ra == rb) break;
      const uint32_t hi = ra > rb ? ra : rb, lo = ra > rb ? rb : ra;
      if (atomicCAS(parent + hi, hi, lo) == hi) break;
      a = hi;
      b = lo;
    }
  }
}

// Roots, component sizes, and the largest component (ties: the smallest root).
__global__ void mtx_roots_kernel(uint32_t *parent, int64_t n, uint32_t *size, unsigned *ncomp) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t r = uf_find(parent, (uint32_t)v);
    parent[v] = r;
    atomicAdd(size + r, 1u);
    if (r == (uint32_t)v) atomicAdd(ncomp, 1u);
  }
}
__global__ void mtx_largest_kernel(const uint32_t *size, int64_t n, ull *best) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
    if (size[v]) atomicMax(best, ((ull)size[v] << 32) | (ull)(0xffffffffu - (uint32_t)v));
}
__global__ void mtx_keep_kernel(const uint32_t *parent, int64_t n, const ull *best, uint32_t *keep) {
  const uint32_t root = 0xffffffffu - (uint32_t)(*best & 0xffffffffull);
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
    keep[v] = parent[v] == root ? 1u : 0u;
}
__global__ void mtx_newdeg_kernel(const uint32_t *keep, const uint32_t *newid, const int64_t *deg, int64_t n,
                                  int64_t *ndeg) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x)
    if (keep[v]) ndeg[newid[v]] = deg[v];
}
__global__ void mtx_place_kernel(const ull *ukey, const int32_t *uw, int64_t E, const int64_t *rowstart,
                                 const uint32_t *keep, const uint32_t *newid, const int64_t *noff, uint32_t *adj,
                                 int32_t *w) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    const ull k = ukey[e];
    const uint32_t s = (uint32_t)(k >> 32), d = (uint32_t)(k & 0xffffffffull);
    if (!keep[s]) continue;
    const int64_t p = noff[newid[s]] + (e - rowstart[s]);
    adj[p] = newid[d];
    if (w) w[p] = uw[e];
  }
}
__global__ void narrow_offsets_kernel(const int64_t *in, int64_t count, uint32_t *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (uint32_t)in[i];
}

__global__ void mtx_iota_kernel(uint32_t *p, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = (uint32_t)i;
}

int grid_for(phde_ctx *ctx, int64_t work) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((work + 255) / 256, (int64_t)ctx->nsm * 8));
}

}  // namespace

extern "C" int phde_graph_from_entries(phde_ctx *ctx, const uint32_t *u, const uint32_t *v, const int32_t *w,
                                       int64_t count, int64_t n1, int64_t n2, int symmetric, phde_csr_info *info) {
  if (!ctx) return PHDE_ERR_INVALID;
  if (count < 0 || (count > 0 && (!u || !v)) || n1 < 1 || n2 < 1 || (symmetric && n1 != n2))
    return phde_fail(ctx, PHDE_ERR_INVALID, "phde_graph_from_entries: bad arguments");
  const int64_t N = symmetric ? n1 : n1 + n2, M2 = 2 * count;
  if (N >= 0xffffffffll || M2 >= 0xffffffffll)
    return phde_fail(ctx, PHDE_ERR_INVALID, "phde_graph_from_entries: n and 2 * entries must be below 2^32");
  PHDE_CK(ctx, cudaSetDevice(ctx->device));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  const int64_t M2a = std::max<int64_t>(M2, 1);
  uint32_t *du = (uint32_t *)phde_buf(ctx, "mtx.u", sizeof(uint32_t) * std::max<int64_t>(count, 1));
  uint32_t *dv = (uint32_t *)phde_buf(ctx, "mtx.v", sizeof(uint32_t) * std::max<int64_t>(count, 1));
  int32_t *dw = w ? (int32_t *)phde_buf(ctx, "mtx.w", sizeof(int32_t) * std::max<int64_t>(count, 1)) : nullptr;
  ull *key0 = (ull *)phde_buf(ctx, "mtx.key0", sizeof(ull) * M2a);
  ull *key1 = (ull *)phde_buf(ctx, "mtx.key1", sizeof(ull) * M2a);
  uint32_t *wk0 = (uint32_t *)phde_buf(ctx, "mtx.wk0", sizeof(uint32_t) * M2a);
  uint32_t *wk1 = (uint32_t *)phde_buf(ctx, "mtx.wk1", sizeof(uint32_t) * M2a);
  uint32_t *flag = (uint32_t *)phde_buf(ctx, "mtx.flag", sizeof(uint32_t) * M2a);
  uint32_t *pos = (uint32_t *)phde_buf(ctx, "mtx.pos", sizeof(uint32_t) * M2a);
  int *bad = (int *)phde_buf(ctx, "mtx.bad", sizeof(int) * 4);
  if (!du || !dv || (w && !dw) || !key0 || !key1 || !wk0 || !wk1 || !flag || !pos || !bad) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(bad, 0, sizeof(int) * 4, ctx->stream));
  if (count > 0) {
    PHDE_CK(ctx, cudaMemcpyAsync(du, u, sizeof(uint32_t) * count, cudaMemcpyHostToDevice, ctx->stream));
    PHDE_CK(ctx, cudaMemcpyAsync(dv, v, sizeof(uint32_t) * count, cudaMemcpyHostToDevice, ctx->stream));
    if (w) PHDE_CK(ctx, cudaMemcpyAsync(dw, w, sizeof(int32_t) * count, cudaMemcpyHostToDevice, ctx->stream));
    mtx_directed_kernel<<<grid_for(ctx, count), 256, 0, ctx->stream>>>(du, dv, dw, count, n1, n2, symmetric, key0, wk0,
                                                                        bad);
    PHDE_LAUNCHED(ctx);
  }
  // ---- sort by weight, then stably by (src, dst) ----
  cub::DoubleBuffer<ull> kb(key0, key1);
  cub::DoubleBuffer<uint32_t> wb(wk0, wk1);
  size_t t1 = 0, t2 = 0, t3 = 0;
  if (M2 > 0) {
    PHDE_CK(ctx, cub::DeviceRadixSort::SortPairs(nullptr, t1, wb, kb, (int64_t)M2, 0, 32, ctx->stream));
    PHDE_CK(ctx, cub::DeviceRadixSort::SortPairs(nullptr, t2, kb, wb, (int64_t)M2, 0, 64, ctx->stream));
  }
  PHDE_CK(ctx, cub::DeviceScan::ExclusiveSum(nullptr, t3, flag, pos, (int64_t)M2a, ctx->stream));
  const size_t tmp_bytes = std::max(std::max(t1, t2), std::max<size_t>(t3, 256));
  void *tmp = phde_buf(ctx, "mtx.cubtmp", tmp_bytes);
  if (!tmp) return PHDE_ERR_OOM;
  if (M2 > 0) {
    size_t tb = tmp_bytes;
    if (w) PHDE_CK(ctx, cub::DeviceRadixSort::SortPairs(tmp, tb, wb, kb, (int64_t)M2, 0, 32, ctx->stream));
    tb = tmp_bytes;
    PHDE_CK(ctx, cub::DeviceRadixSort::SortPairs(tmp, tb, kb, wb, (int64_t)M2, 0, 64, ctx->stream));
  }
  const ull *key = kb.Current();
  const uint32_t *wk = wb.Current();
  // ---- deduplicate (first of each (src, dst) run) ----
  if (M2 > 0) {
    mtx_flags_kernel<<<grid_for(ctx, M2), 256, 0, ctx->stream>>>(key, M2, flag);
    PHDE_LAUNCHED(ctx);
  } else {
    PHDE_CK(ctx, cudaMemsetAsync(flag, 0, sizeof(uint32_t), ctx->stream));
  }
  {
    size_t tb = tmp_bytes;
    PHDE_CK(ctx, cub::DeviceScan::ExclusiveSum(tmp, tb, flag, pos, (int64_t)M2a, ctx->stream));
  }
  uint32_t h2[2] = {0, 0};
  PHDE_CK(ctx, cudaMemcpyAsync(h2, pos + (M2a - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaMemcpyAsync(h2 + 1, flag + (M2a - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  int hbad = 0;
  PHDE_CK(ctx, cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (hbad) return phde_fail(ctx, PHDE_ERR_CSR, "phde_graph_from_entries: an entry's index is outside the matrix");
  const int64_t E = (int64_t)h2[0] + (int64_t)h2[1];
  ull *ukey = (ull *)phde_buf(ctx, "mtx.ukey", sizeof(ull) * std::max<int64_t>(E, 1));
  int32_t *uw = (int32_t *)phde_buf(ctx, "mtx.uw", sizeof(int32_t) * std::max<int64_t>(E, 1));
  int64_t *deg = (int64_t *)phde_buf(ctx, "mtx.deg", sizeof(int64_t) * (N + 1));
  int64_t *rowstart = (int64_t *)phde_buf(ctx, "mtx.rowstart", sizeof(int64_t) * (N + 1));
  uint32_t *parent = (uint32_t *)phde_buf(ctx, "mtx.parent", sizeof(uint32_t) * N);
  uint32_t *size = (uint32_t *)phde_buf(ctx, "mtx.size", sizeof(uint32_t) * N);
  uint32_t *keep = (uint32_t *)phde_buf(ctx, "mtx.keep", sizeof(uint32_t) * (N + 1));
  uint32_t *newid = (uint32_t *)phde_buf(ctx, "mtx.newid", sizeof(uint32_t) * (N + 1));
  int64_t *ndeg = (int64_t *)phde_buf(ctx, "mtx.ndeg", sizeof(int64_t) * (N + 1));
  ull *best = (ull *)phde_buf(ctx, "mtx.best", sizeof(ull) * 2);
  if (!ukey || !uw || !deg || !rowstart || !parent || !size || !keep || !newid || !ndeg || !best) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(deg, 0, sizeof(int64_t) * (N + 1), ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(size, 0, sizeof(uint32_t) * N, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(best, 0, sizeof(ull) * 2, ctx->stream));
  if (M2 > 0) {
    mtx_compact_kernel<<<grid_for(ctx, M2), 256, 0, ctx->stream>>>(key, wk, flag, pos, M2, ukey, uw, deg);
    PHDE_LAUNCHED(ctx);
  }
  // row starts of the deduplicated list (exclusive scan of the degrees; deg[N] = 0 closes it)
  size_t t4 = 0;
  PHDE_CK(ctx, cub::DeviceScan::ExclusiveSum(nullptr, t4, deg, rowstart, N + 1, ctx->stream));
  void *tmp2 = phde_buf(ctx, "mtx.cubtmp2", std::max<size_t>(t4, 256));
  if (!tmp2) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cub::DeviceScan::ExclusiveSum(tmp2, t4, deg, rowstart, N + 1, ctx->stream));
  // ---- components: union-find, roots = smallest vertex; the largest component (smallest root on ties) ----
  mtx_iota_kernel<<<grid_for(ctx, N), 256, 0, ctx->stream>>>(parent, N);
  PHDE_LAUNCHED(ctx);
  unsigned *ncomp = (unsigned *)(best + 1);
  if (E > 0) {
    mtx_union_kernel<<<grid_for(ctx, E), 256, 0, ctx->stream>>>(ukey, E, parent, bad + 1);
    PHDE_LAUNCHED(ctx);
  }
  mtx_roots_kernel<<<grid_for(ctx, N), 256, 0, ctx->stream>>>(parent, N, size, ncomp);
  PHDE_LAUNCHED(ctx);
  mtx_largest_kernel<<<grid_for(ctx, N), 256, 0, ctx->stream>>>(size, N, best);
  PHDE_LAUNCHED(ctx);
  mtx_keep_kernel<<<grid_for(ctx, N), 256, 0, ctx->stream>>>(parent, N, best, keep);
  PHDE_LAUNCHED(ctx);
  PHDE_CK(ctx, cudaMemsetAsync(keep + N, 0, sizeof(uint32_t), ctx->stream));
  size_t t5 = 0;
  PHDE_CK(ctx, cub::DeviceScan::ExclusiveSum(nullptr, t5, keep, newid, N + 1, ctx->stream));
  void *tmp3 = phde_buf(ctx, "mtx.cubtmp3", std::max<size_t>(t5, 256));
  if (!tmp3) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cub::DeviceScan::ExclusiveSum(tmp3, t5, keep, newid, N + 1, ctx->stream));
  ull hb[2] = {0, 0};
  uint32_t hn = 0;
  int herr = 0;
  PHDE_CK(ctx, cudaMemcpyAsync(hb, best, sizeof(hb), cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaMemcpyAsync(&hn, newid + N, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaMemcpyAsync(&herr, bad + 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (herr) return phde_fail(ctx, herr, "phde_graph_from_entries: component labelling did not settle");
  const int64_t Nn = hn;
  // ---- the kept component: new offsets, edges at their row positions ----
  PHDE_CK(ctx, cudaMemsetAsync(ndeg, 0, sizeof(int64_t) * (N + 1), ctx->stream));
  mtx_newdeg_kernel<<<grid_for(ctx, N), 256, 0, ctx->stream>>>(keep, newid, deg, N, ndeg);
  PHDE_LAUNCHED(ctx);
  if (Nn + 1 > ctx->off_cap || !ctx->d_off) {
    cudaFree(ctx->d_off);
    ctx->d_off = nullptr;
    ctx->off_cap = 0;
    PHDE_CK(ctx, cudaMalloc(&ctx->d_off, sizeof(int64_t) * (Nn + 1)));
    ctx->off_cap = Nn + 1;
  }
  size_t t6 = 0;
  PHDE_CK(ctx, cub::DeviceScan::ExclusiveSum(nullptr, t6, ndeg, ctx->d_off, Nn + 1, ctx->stream));
  void *tmp4 = phde_buf(ctx, "mtx.cubtmp4", std::max<size_t>(t6, 256));
  if (!tmp4) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cub::DeviceScan::ExclusiveSum(tmp4, t6, ndeg, ctx->d_off, Nn + 1, ctx->stream));
  int64_t nnz = 0;
  PHDE_CK(ctx, cudaMemcpyAsync(&nnz, ctx->d_off + Nn, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (nnz > ctx->adj_cap || !ctx->d_adj) {
    cudaFree(ctx->d_adj);
    ctx->d_adj = nullptr;
    ctx->adj_cap = 0;
    PHDE_CK(ctx, cudaMalloc(&ctx->d_adj, sizeof(uint32_t) * std::max<int64_t>(nnz, 1)));
    ctx->adj_cap = std::max<int64_t>(nnz, 1);
    cudaFree(ctx->d_w);
    ctx->d_w = nullptr;
  }
  if (w && !ctx->d_w) PHDE_CK(ctx, cudaMalloc(&ctx->d_w, sizeof(int32_t) * ctx->adj_cap));
  if (E > 0) {
    mtx_place_kernel<<<grid_for(ctx, E), 256, 0, ctx->stream>>>(ukey, uw, E, rowstart, keep, newid, ctx->d_off,
                                                                 ctx->d_adj, w ? ctx->d_w : nullptr);
    PHDE_LAUNCHED(ctx);
  }
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->n = Nn;
  ctx->nnz = nnz;
  ctx->weighted = w != nullptr;
  ctx->batch_B = 0;
  ctx->graph_epoch++;
  if (info) {
    info->n_in = N;
    info->nnz_dedup = E;
    info->ncomponents = (int64_t)(uint32_t)hb[1];
    info->n = Nn;
    info->nnz = nnz;
  }
  return PHDE_OK;
}

extern "C" int phde_graph_download(phde_ctx *ctx, uint32_t *offsets, uint32_t *adj, int32_t *weights) {
  if (!ctx) return PHDE_ERR_INVALID;
  if (ctx->n <= 0) return phde_fail(ctx, PHDE_ERR_NO_GRAPH, "phde_graph_download: no graph uploaded");
  if (!offsets || (!adj && ctx->nnz > 0)) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_graph_download: bad arguments");
  if (weights && !ctx->weighted) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_graph_download: the graph has no weights");
  PHDE_CK(ctx, cudaSetDevice(ctx->device));
  uint32_t *o32 = (uint32_t *)phde_buf(ctx, "download.off32", sizeof(uint32_t) * (ctx->n + 1));
  if (!o32) return PHDE_ERR_OOM;
  narrow_offsets_kernel<<<grid_for(ctx, ctx->n + 1), 256, 0, ctx->stream>>>(ctx->d_off, ctx->n + 1, o32);
  PHDE_LAUNCHED(ctx);
  PHDE_CK(ctx, cudaMemcpyAsync(offsets, o32, sizeof(uint32_t) * (ctx->n + 1), cudaMemcpyDeviceToHost, ctx->stream));
  if (ctx->nnz > 0) {
    PHDE_CK(ctx, cudaMemcpyAsync(adj, ctx->d_adj, sizeof(uint32_t) * ctx->nnz, cudaMemcpyDeviceToHost, ctx->stream));
    if (weights)
      PHDE_CK(ctx, cudaMemcpyAsync(weights, ctx->d_w, sizeof(int32_t) * ctx->nnz, cudaMemcpyDeviceToHost, ctx->stream));
  }
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return PHDE_OK;
}
