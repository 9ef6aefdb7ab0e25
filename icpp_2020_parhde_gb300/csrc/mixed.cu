// mixed.cu -- the mixed-precision dense stages of ParHDE (PHDE_PREC_MIXED).
//
// GB300 runs FP64 at 1/64 of its FP32 rate, so the FP64 path is bound by the FP64 pipe.  Here the
// n-sized work is FP32 and only what is k-sized or a cross-block sum is FP64:
//   cgs2_kernel      D-orthogonalisation of ParHDE.cpp:190-285 as CGS2: every candidate is projected
//                    twice against the accepted columns and the constant column (single-pass classical
//                    Gram-Schmidt in FP32 would lose orthogonality on these nearly collinear distance
//                    columns); FP32 products, FP64 sums across warps and blocks; same norm test
//                    (||x|| < 1e-3 discards, ParHDE.cpp:267) and the same acceptance order.
//   spmm32 kernels   LS = D*S - A*S with an FP32 basis (half the bytes of every neighbour gather; the
//                    R-MAT-20 basis is 129 MB and stays largely in the 129 MB L2), same heavy-row plan.
//   gram32_kernel    S^T LS with FP32 products accumulated in FP32 over 128-row spans and in FP64 across
//                    spans and blocks.
//   coords32_kernel  X = S*Y: FP32 products and row sums (S is FP32), FP64 column norms.
// The k x k eigensolve stays FP64 (eigen.cu).
#include <algorithm>

#include "ctx.h"
#include "spmm_plan.cuh"

namespace {

constexpr int C2_THREADS = 256;
constexpr int MAXQ = 8;  // columns per lane: k <= 256
constexpr int COORD_MAXC = 4;  // coordinates per FP32 coords pass

__device__ __forceinline__ double partials_sum(const double *part, double *red) {
  double s = 0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s += __ldcg(part + b);
  return block_sum(s, red);
}

struct Cgs2Args {
  const int32_t *D;
  int64_t n;
  int P;
  const ull *sumsq;
  const double *deg;
  float *S;  // row-major n x k
  int k;
  float *X;        // [n] candidate after the current pass
  double *part;    // [gridDim][k+2]
  double *part2;   // [gridDim]
  double *coef;    // [k+1]
  double *inv_den; // [k+1]
  int *state;
  double *dlog;
  GridSync *gs;
  int *err;
  uint64_t timeout_ns;
};

constexpr int TILE_LD = 33;
__device__ __forceinline__ void stage_tile32(const float *S, int64_t i0, int rows, int k, int c0, int nc, float *tile,
                                             int lane) {
  __syncwarp();
  if (lane < nc) {
    const float *src = S + i0 * k + c0 + lane;
#pragma unroll 8
    for (int r = 0; r < rows; r++) tile[r * TILE_LD + lane] = src[(int64_t)r * k];
  }
  __syncwarp();
}

__global__ void __launch_bounds__(C2_THREADS) cgs2_kernel(Cgs2Args a) {
  extern __shared__ double sm[];  // [nwarps][k+2] (coefficients as float in phase E), then float tiles
  __shared__ double red[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int64_t n = a.n;
  const int k = a.k, ld = k + 2;
  float *tile = (float *)(sm + nw * ld) + warp * 32 * TILE_LD;
  const int64_t gw = (int64_t)blockIdx.x * nw + warp, gws = (int64_t)gridDim.x * nw;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, gts = (int64_t)gridDim.x * blockDim.x;
  const double inv0 = 1.0 / sqrt((double)n);

  double acc0 = 0;
  for (int64_t i = gt; i < n; i += gts) acc0 += a.deg[i];
  acc0 = block_sum(acc0, red);
  if (threadIdx.x == 0) a.part2[blockIdx.x] = acc0 * inv0 * inv0;
  if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
  const double inv_den0 = 1.0 / partials_sum(a.part2, red);
  if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;

  int j = 1, ndisc = 0, ncand = 0;
  bool newcol = false;
  for (int rc = 0; rc < a.P; rc++) {
    if (j > k) break;
    ncand++;
    const int32_t *Dc = a.D + (int64_t)rc * n;
    const float inv_rc = (float)(1.0 / sqrt((double)__ldcg(a.sumsq + rc)));
    const int jm1 = j - 1;
    double ssq = 0;
    for (int pass = 0; pass < 2; pass++) {
      // ---- A: dots <v, D S_q> (q < j-1) and <v, D u0>; v = the candidate (pass 0) or X (pass 1) ----
      float accq[MAXQ];
#pragma unroll
      for (int t = 0; t < MAXQ; t++) accq[t] = 0.f;
      double vsum = 0;
      for (int64_t i0 = gw * 32; i0 < n; i0 += gws * 32) {
        const int64_t il = i0 + lane;
        float vdl = 0.f;
        if (il < n) {
          const float v = pass == 0 ? (float)Dc[il] * inv_rc : __ldcg(a.X + il);
          vdl = v * (float)a.deg[il];
        }
        vsum += (double)vdl;
        const int rows = n - i0 < 32 ? (int)(n - i0) : 32;
#pragma unroll
        for (int t = 0; t < MAXQ; t++) {
          const int c0 = 32 * t;
          if (c0 >= jm1) break;
          const int nc = jm1 - c0 < 32 ? jm1 - c0 : 32;
          stage_tile32(a.S, i0, rows, k, c0, nc, tile, lane);
          float acc = accq[t];
          for (int rr = 0; rr < rows; rr++) {
            const float vd = __shfl_sync(PHDE_FULL_MASK, vdl, rr);
            if (lane < nc) acc = fmaf(vd, tile[rr * TILE_LD + lane], acc);
          }
          accq[t] = acc;
          __syncwarp();
        }
      }
      vsum = warp_sum(vsum);
#pragma unroll
      for (int t = 0; t < MAXQ; t++) {
        const int q = lane + 32 * t;
        if (q < jm1) sm[warp * ld + q] = (double)accq[t];
      }
      if (lane == 0) sm[warp * ld + k] = vsum * inv0;
      __syncthreads();
      for (int q = threadIdx.x; q < k + 1; q += blockDim.x) {
        if (q < jm1 || q == k) {
          double s = 0;
          for (int w = 0; w < nw; w++) s += sm[w * ld + q];
          a.part[(int64_t)blockIdx.x * ld + q] = s;
        }
      }
      if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
      // ---- C: coefficients ----
      for (int q = blockIdx.x; q < j; q += gridDim.x) {
        const int slot = q == jm1 ? k : q;
        const bool fresh = pass == 0 && newcol && q == j - 2;
        double s = 0, sd = 0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
          s += __ldcg(a.part + (int64_t)b * ld + slot);
          if (fresh) sd += __ldcg(a.part + (int64_t)b * ld + k + 1);
        }
        s = block_sum(s, red);
        if (fresh) sd = block_sum(sd, red);
        if (threadIdx.x == 0) {
          double id;
          if (slot == k) {
            id = inv_den0;
          } else if (fresh) {
            id = 1.0 / sd;
            a.inv_den[q] = id;
          } else {
            id = __ldcg(a.inv_den + q);
          }
          a.coef[slot] = s * id;
        }
        __syncthreads();
      }
      if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
      // ---- E: v' = v - (sum_q coef_q S_q + coef_0 u0), thread per row ----
      float *cf = (float *)sm;
      __syncthreads();
      for (int q = threadIdx.x; q < jm1; q += blockDim.x) cf[q] = (float)__ldcg(a.coef + q);
      __syncthreads();
      const float c0u0 = (float)(__ldcg(a.coef + k) * inv0);
      ssq = 0;
      for (int64_t i0 = gw * 32; i0 < n; i0 += gws * 32) {
        const int rows = n - i0 < 32 ? (int)(n - i0) : 32;
        float p = 0.f;
        for (int c0 = 0; c0 < jm1; c0 += 32) {
          const int nc = jm1 - c0 < 32 ? jm1 - c0 : 32;
          stage_tile32(a.S, i0, rows, k, c0, nc, tile, lane);
          if (lane < rows)
            for (int q = 0; q < nc; q++) p = fmaf(cf[c0 + q], tile[lane * TILE_LD + q], p);
          __syncwarp();
        }
        if (lane < rows) {
          const int64_t i = i0 + lane;
          const float v = pass == 0 ? (float)Dc[i] * inv_rc : __ldcg(a.X + i);
          const float vp = v - (p + c0u0);
          a.X[i] = vp;
          ssq += (double)vp * (double)vp;
        }
      }
      if (pass == 1) {
        ssq = block_sum(ssq, red);
        if (threadIdx.x == 0) a.part2[blockIdx.x] = ssq;
      }
      if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
    }
    // ---- G: norm test and acceptance ----
    const double nrm = sqrt(partials_sum(a.part2, red));
    if (nrm < 0.001) {
      ndisc++;
      if (blockIdx.x == 0 && threadIdx.x == 0) a.dlog[rc] = nrm;
      newcol = false;
    } else {
      const float scale = (float)(1.0 / nrm);
      double dd = 0;
      for (int64_t i = gt; i < n; i += gts) {
        const float v = __ldcg(a.X + i) * scale;
        a.S[i * k + (j - 1)] = v;
        dd += (double)v * (double)v * a.deg[i];
      }
      dd = block_sum(dd, red);
      if (threadIdx.x == 0) a.part[(int64_t)blockIdx.x * ld + k + 1] = dd;
      j++;
      newcol = true;
      if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.state[0] = j - 1;
    a.state[1] = ndisc;
    a.state[2] = ncand;
  }
}

// ---- FP32 Laplacian SpMM ----
// A warp per row (light rows) or per chunk of a heavy row.  Lane l owns columns 2l, 2l+1 of every 64-column
// tile (float2 gathers: one 8-byte load per lane and neighbour row; k even), KT tiles (k <= 64 KT); the
// neighbour loop keeps four rows in flight.  Odd k uses the scalar variant (lane l: columns l + 32t).
template <int KT>
__device__ __forceinline__ void spmm32_acc2(const uint32_t *adj, const float *S, int k, int lane, int64_t e0,
                                            int64_t e1, float2 (&acc)[KT]) {
  int64_t e = e0;
  for (; e + 4 <= e1; e += 4) {
    const int64_t v0 = __ldg(adj + e), v1 = __ldg(adj + e + 1), v2 = __ldg(adj + e + 2), v3 = __ldg(adj + e + 3);
#pragma unroll
    for (int t = 0; t < KT; t++) {
      const int q = 2 * lane + 64 * t;
      if (q < k) {
        const float2 a0 = *(const float2 *)(S + v0 * k + q), a1 = *(const float2 *)(S + v1 * k + q);
        const float2 a2 = *(const float2 *)(S + v2 * k + q), a3 = *(const float2 *)(S + v3 * k + q);
        acc[t].x -= (a0.x + a1.x) + (a2.x + a3.x);
        acc[t].y -= (a0.y + a1.y) + (a2.y + a3.y);
      }
    }
  }
  for (; e < e1; e++) {
    const int64_t v = __ldg(adj + e);
#pragma unroll
    for (int t = 0; t < KT; t++) {
      const int q = 2 * lane + 64 * t;
      if (q < k) {
        const float2 a = *(const float2 *)(S + v * k + q);
        acc[t].x -= a.x;
        acc[t].y -= a.y;
      }
    }
  }
}

template <int KT>
__global__ void spmm32_light2_kernel(const int64_t *off, const uint32_t *adj, const double *deg, const float *S,
                                     float *LS, int64_t n, int k) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t gws = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = gw; i < n; i += gws) {
    const int64_t e0 = off[i], e1 = off[i + 1];
    if (e1 - e0 > SPMM_HEAVY) continue;
    const float di = (float)(e1 - e0);  // unweighted: the degree is the row length
    float2 acc[KT];
#pragma unroll
    for (int t = 0; t < KT; t++) {
      const int q = 2 * lane + 64 * t;
      acc[t] = make_float2(0.f, 0.f);
      if (q < k) {
        const float2 si = *(const float2 *)(S + i * k + q);
        acc[t] = make_float2(di * si.x, di * si.y);
      }
    }
    spmm32_acc2<KT>(adj, S, k, lane, e0, e1, acc);
#pragma unroll
    for (int t = 0; t < KT; t++) {
      const int q = 2 * lane + 64 * t;
      if (q < k) *(float2 *)(LS + i * k + q) = acc[t];
    }
  }
}

template <int KT>
__global__ void spmm32_chunk2_kernel(const uint32_t *adj, const float *S, const Chunk *chunks, int64_t nchunks,
                                     float *part, int k) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t gws = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = gw; c < nchunks; c += gws) {
    float2 acc[KT];
#pragma unroll
    for (int t = 0; t < KT; t++) acc[t] = make_float2(0.f, 0.f);
    const Chunk ch = chunks[c];
    spmm32_acc2<KT>(adj, S, k, lane, ch.e0, ch.e1, acc);
#pragma unroll
    for (int t = 0; t < KT; t++) {
      const int q = 2 * lane + 64 * t;
      if (q < k) *(float2 *)(part + c * k + q) = acc[t];
    }
  }
}

__device__ __forceinline__ void spmm32_acc(const uint32_t *adj, const float *S, int k, int lane, int64_t e0,
                                           int64_t e1, float (&acc)[MAXQ]) {
  int64_t e = e0;
  for (; e + 4 <= e1; e += 4) {
    const int64_t v0 = __ldg(adj + e), v1 = __ldg(adj + e + 1), v2 = __ldg(adj + e + 2), v3 = __ldg(adj + e + 3);
#pragma unroll
    for (int t = 0; t < MAXQ; t++) {
      const int q = lane + 32 * t;
      if (q < k) acc[t] -= (S[v0 * k + q] + S[v1 * k + q]) + (S[v2 * k + q] + S[v3 * k + q]);
    }
  }
  for (; e < e1; e++) {
    const int64_t v = __ldg(adj + e);
#pragma unroll
    for (int t = 0; t < MAXQ; t++) {
      const int q = lane + 32 * t;
      if (q < k) acc[t] -= S[v * k + q];
    }
  }
}

__global__ void spmm32_light_kernel(const int64_t *off, const uint32_t *adj, const double *deg, const float *S,
                                    float *LS, int64_t n, int k) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t gws = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = gw; i < n; i += gws) {
    const int64_t e0 = off[i], e1 = off[i + 1];
    if (e1 - e0 > SPMM_HEAVY) continue;
    const float di = (float)deg[i];
    float acc[MAXQ];
#pragma unroll
    for (int t = 0; t < MAXQ; t++) {
      const int q = lane + 32 * t;
      acc[t] = q < k ? di * S[i * k + q] : 0.f;
    }
    spmm32_acc(adj, S, k, lane, e0, e1, acc);
#pragma unroll
    for (int t = 0; t < MAXQ; t++) {
      const int q = lane + 32 * t;
      if (q < k) LS[i * k + q] = acc[t];
    }
  }
}

__global__ void spmm32_chunk_kernel(const uint32_t *adj, const float *S, const Chunk *chunks, int64_t nchunks,
                                    float *part, int k) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t gws = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = gw; c < nchunks; c += gws) {
    float acc[MAXQ];
#pragma unroll
    for (int t = 0; t < MAXQ; t++) acc[t] = 0.f;
    const Chunk ch = chunks[c];
    spmm32_acc(adj, S, k, lane, ch.e0, ch.e1, acc);
#pragma unroll
    for (int t = 0; t < MAXQ; t++) {
      const int q = lane + 32 * t;
      if (q < k) part[c * k + q] = acc[t];
    }
  }
}

__global__ void spmm32_fix_kernel(const HeavyRow *heavy, int64_t nheavy, const double *deg, const float *S,
                                  const float *part, float *LS, int k) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t gws = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t h = gw; h < nheavy; h += gws) {
    const HeavyRow hr = heavy[h];
    const int64_t i = hr.row;
    const float di = (float)deg[i];
#pragma unroll
    for (int t = 0; t < MAXQ; t++) {
      const int q = lane + 32 * t;
      if (q < k) {
        float s = di * S[i * k + q];
        for (int64_t c = 0; c < hr.nchunks; c++) s += part[(hr.first_chunk + c) * k + q];
        LS[i * k + q] = s;
      }
    }
  }
}

// ---- Gram A^T B with FP32 inputs: 64x64 tile per block, 16-row staged slabs, FP32 over 128 rows, FP64 beyond ----
constexpr int GT = 64, GR = 16;
__global__ void __launch_bounds__(256) gram32_kernel(const float *A, const float *B, int64_t n, int k, double *part) {
  __shared__ float sA[GR][GT + 1];
  __shared__ float sB[GR][GT + 1];
  const int tiles = (k + GT - 1) / GT;
  const int tp = blockIdx.x / tiles, tq = blockIdx.x % tiles;
  const int p0 = tp * GT, q0 = tq * GT;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t rows_per = (n + gridDim.y - 1) / gridDim.y;
  const int64_t r0 = (int64_t)blockIdx.y * rows_per;
  const int64_t r1 = min(n, r0 + rows_per);
  double accd[4][4] = {};
  float acc[4][4] = {};
  int slab = 0;
  for (int64_t rb = r0; rb < r1; rb += GR, slab++) {
    for (int idx = threadIdx.x; idx < GR * GT; idx += 256) {
      const int rr = idx / GT, cc = idx % GT;
      const int64_t r = rb + rr;
      sA[rr][cc] = (r < r1 && p0 + cc < k) ? A[r * k + p0 + cc] : 0.f;
      sB[rr][cc] = (r < r1 && q0 + cc < k) ? B[r * k + q0 + cc] : 0.f;
    }
    __syncthreads();
#pragma unroll 4
    for (int rr = 0; rr < GR; rr++) {
      float av[4], bv[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        av[u] = sA[rr][ty + 16 * u];
        bv[u] = sB[rr][tx + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) acc[u][v] = fmaf(av[u], bv[v], acc[u][v]);
    }
    // FP32 sums over 128 rows, then into FP64: GB300's FP64 adds are 1/64-rate, so not after every slab
    if ((slab & 7) == 7 || rb + GR >= r1) {
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int v = 0; v < 4; v++) {
          accd[u][v] += (double)acc[u][v];
          acc[u][v] = 0.f;
        }
    }
    __syncthreads();
  }
  double *out = part + (int64_t)blockIdx.y * k * k;
#pragma unroll
  for (int u = 0; u < 4; u++)
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const int p = p0 + ty + 16 * u, q = q0 + tx + 16 * v;
      if (p < k && q < k) out[q + (int64_t)p * k] = accd[u][v];
    }
}

// out[i] = sum over splits of part[b][i]: a block per 32 outputs, its 8 warps over interleaved splits (two
// chains each), combined in warp order -- deterministic, and short FP64 dependency chains.
__global__ void __launch_bounds__(256) sum_parts32_kernel(const double *part, int splits, int64_t len, double *out) {
  __shared__ double red[8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t i = (int64_t)blockIdx.x * 32 + lane;
  double s0 = 0, s1 = 0;
  if (i < len) {
    int b = warp;
    for (; b + 8 < splits; b += 16) {
      s0 += part[(int64_t)b * len + i];
      s1 += part[(int64_t)(b + 8) * len + i];
    }
    if (b < splits) s0 += part[(int64_t)b * len + i];
  }
  red[warp][lane] = s0 + s1;
  __syncthreads();
  if (warp == 0 && i < len) {
    double t = 0;
    for (int w = 0; w < 8; w++) t += red[w][lane];
    out[i] = t;
  }
}

// X[i + t*n] = sum_q S[i,q] * Y[q + t*k] (FP32 basis, FP64 eigenvectors and accumulation)
// X[:, t] = S Y[:, t] for c <= COORD_MAXC coordinates: a block stages COORD_ROWS consecutive rows of S (one
// contiguous range of memory, read coalesced) into shared memory, then a thread per row forms its c FP32 dot
// products over the row's k entries; per-block FP64 sums of squares for the column norms.
constexpr int COORD_ROWS = 128;
__global__ void __launch_bounds__(COORD_ROWS) coords32_kernel(const float *S, const double *Y, int64_t n, int k, int c,
                                                              double *X, double *part) {
  extern __shared__ float smc[];  // [COORD_ROWS * k] rows of S, then Ys[q * c + t]
  __shared__ double red[32];
  float *rows = smc, *Ys = smc + COORD_ROWS * k;
  for (int idx = threadIdx.x; idx < k * c; idx += blockDim.x) {
    const int q = idx / c, t = idx % c;
    Ys[idx] = (float)Y[q + (int64_t)t * k];
  }
  double ss[COORD_MAXC];
#pragma unroll
  for (int t = 0; t < COORD_MAXC; t++) ss[t] = 0;
  for (int64_t i0 = (int64_t)blockIdx.x * COORD_ROWS; i0 < n; i0 += (int64_t)gridDim.x * COORD_ROWS) {
    const int nr = (int)min((int64_t)COORD_ROWS, n - i0);
    __syncthreads();  // Ys written (first tile), or the previous tile's rows read
    const float *src = S + i0 * k;
    for (int e = threadIdx.x; e < nr * k; e += blockDim.x) rows[e] = src[e];
    __syncthreads();
    if ((int)threadIdx.x < nr) {
      float acc[COORD_MAXC];
#pragma unroll
      for (int t = 0; t < COORD_MAXC; t++) acc[t] = 0.f;
      const float *row = rows + threadIdx.x * k;
      for (int q = 0; q < k; q++) {
        const float sv = row[q];
#pragma unroll
        for (int t = 0; t < COORD_MAXC; t++)
          if (t < c) acc[t] = fmaf(sv, Ys[q * c + t], acc[t]);
      }
#pragma unroll
      for (int t = 0; t < COORD_MAXC; t++) {
        if (t >= c) break;
        X[i0 + threadIdx.x + (int64_t)t * n] = (double)acc[t];
        ss[t] = fma((double)acc[t], (double)acc[t], ss[t]);
      }
    }
  }
  for (int t = 0; t < c; t++) {  // c is uniform: every thread takes part in each block sum
    const double s = block_sum(ss[t], red);
    if (threadIdx.x == 0) part[(int64_t)blockIdx.x * c + t] = s;
  }
}

// X[:, t] /= ||X[:, t]||: each block sums the per-block partials itself (a block-wide reduction, the same
// fixed order in every block), then scales its share.
__global__ void scale32_kernel(double *X, int64_t n, int c, const double *part, int nparts, double *norm2) {
  __shared__ double inv[COORD_MAXC];
  __shared__ double red[32];
  for (int t = 0; t < c; t++) {
    double s = 0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) s += part[(int64_t)b * c + t];
    s = block_sum(s, red);
    if (threadIdx.x == 0) inv[t] = 1.0 / sqrt(s);
    if (norm2 && blockIdx.x == 0 && threadIdx.x == 0) norm2[t] = s;  // ||X[:, t]||^2 before the scaling
  }
  __syncthreads();
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n * c;
       idx += (int64_t)gridDim.x * blockDim.x)
    X[idx] *= inv[idx / n];
}

int grid_of(phde_ctx *ctx, int64_t work, int threads, int per_sm) {
  int64_t b = (work + threads - 1) / threads;
  b = std::min<int64_t>(b, (int64_t)ctx->nsm * per_sm);
  return (int)std::max<int64_t>(b, 1);
}

}  // namespace

int phde_cgs2_mixed(phde_ctx *ctx, const int32_t *D, int P, const ull *sumsq, const double *deg, float *S, int k,
                    int *h_state, double *h_dlog) {
  const int64_t n = ctx->n;
  const size_t smem = sizeof(double) * (C2_THREADS / 32) * (size_t)(k + 2) + sizeof(float) * (C2_THREADS / 32) * 32 * TILE_LD;
  int per_sm = 0;
  PHDE_CK(ctx, cudaFuncSetAttribute(cgs2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  PHDE_CK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cgs2_kernel, C2_THREADS, smem));
  if (per_sm < 1) return phde_fail(ctx, PHDE_ERR_CUDA, "cgs2 kernel cannot be resident");
  per_sm = std::min(per_sm, 4);
  const int grid = ctx->nsm * per_sm;
  float *X = (float *)phde_buf(ctx, "cgs2.X", sizeof(float) * n);
  double *part = (double *)phde_buf(ctx, "cgs2.part", sizeof(double) * grid * (size_t)(k + 2));
  double *part2 = (double *)phde_buf(ctx, "cgs2.part2", sizeof(double) * grid);
  double *coef = (double *)phde_buf(ctx, "cgs2.coef", sizeof(double) * (k + 1));
  double *inv_den = (double *)phde_buf(ctx, "cgs2.inv_den", sizeof(double) * (k + 1));
  int *state = (int *)phde_buf(ctx, "cgs2.state", sizeof(int) * 4);
  double *dlog = (double *)phde_buf(ctx, "cgs2.dlog", sizeof(double) * P);
  if (!X || !part || !part2 || !coef || !inv_den || !state || !dlog) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(dlog, 0xff, sizeof(double) * P, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(state, 0, sizeof(int) * 4, ctx->stream));
  int rc = phde_reset_sync(ctx);
  if (rc) return rc;
  Cgs2Args a;
  a.D = D;
  a.n = n;
  a.P = P;
  a.sumsq = sumsq;
  a.deg = deg;
  a.S = S;
  a.k = k;
  a.X = X;
  a.part = part;
  a.part2 = part2;
  a.coef = coef;
  a.inv_den = inv_den;
  a.state = state;
  a.dlog = dlog;
  a.gs = ctx->d_sync;
  a.err = ctx->d_err;
  a.timeout_ns = ctx->timeout_ns;
  void *args[] = {&a};
  PHDE_CK(ctx, cudaLaunchCooperativeKernel((const void *)cgs2_kernel, dim3(grid), dim3(C2_THREADS), args, smem,
                                           ctx->stream));
  PHDE_LAUNCHED(ctx);
  PHDE_CK(ctx, cudaMemcpyAsync(h_state, state, sizeof(int) * 4, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaMemcpyAsync(h_dlog, dlog, sizeof(double) * P, cudaMemcpyDeviceToHost, ctx->stream));
  return PHDE_OK;
}

int phde_lap_spmm_mixed(phde_ctx *ctx, const double *deg, const float *S, float *LS, int k) {
  HeavyRow *heavy;
  Chunk *chunks;
  int64_t nheavy, nchunks;
  int rc = phde_spmm_plan(ctx, &heavy, &chunks, &nheavy, &nchunks);
  if (rc) return rc;
  const int threads = 256;
  // float2 gathers for even k on unweighted graphs (the degree is the row length), else the scalar kernels
  const int KT = (k + 63) / 64;
  const bool v2 = k % 2 == 0 && !ctx->weighted && KT <= 4;
  const int gl = grid_of(ctx, ctx->n * 32, threads, 8);
#define PHDE_SPMM_LIGHT(T) \
  spmm32_light2_kernel<T><<<gl, threads, 0, ctx->stream>>>(ctx->d_off, ctx->d_adj, deg, S, LS, ctx->n, k)
  if (v2) {
    if (KT == 1) PHDE_SPMM_LIGHT(1);
    else if (KT == 2) PHDE_SPMM_LIGHT(2);
    else if (KT == 3) PHDE_SPMM_LIGHT(3);
    else PHDE_SPMM_LIGHT(4);
  } else {
    spmm32_light_kernel<<<gl, threads, 0, ctx->stream>>>(ctx->d_off, ctx->d_adj, deg, S, LS, ctx->n, k);
  }
#undef PHDE_SPMM_LIGHT
  PHDE_LAUNCHED(ctx);
  if (nheavy > 0) {
    float *part = (float *)phde_buf(ctx, "spmm32.part", sizeof(float) * nchunks * k);
    if (!part) return PHDE_ERR_OOM;
    const int gc = grid_of(ctx, nchunks * 32, threads, 8);
#define PHDE_SPMM_CHUNK(T) spmm32_chunk2_kernel<T><<<gc, threads, 0, ctx->stream>>>(ctx->d_adj, S, chunks, nchunks, part, k)
    if (v2) {
      if (KT == 1) PHDE_SPMM_CHUNK(1);
      else if (KT == 2) PHDE_SPMM_CHUNK(2);
      else if (KT == 3) PHDE_SPMM_CHUNK(3);
      else PHDE_SPMM_CHUNK(4);
    } else {
      spmm32_chunk_kernel<<<gc, threads, 0, ctx->stream>>>(ctx->d_adj, S, chunks, nchunks, part, k);
    }
#undef PHDE_SPMM_CHUNK
    PHDE_LAUNCHED(ctx);
    spmm32_fix_kernel<<<grid_of(ctx, nheavy * 32, threads, 8), threads, 0, ctx->stream>>>(heavy, nheavy, deg, S, part,
                                                                                          LS, k);
    PHDE_LAUNCHED(ctx);
  }
  return PHDE_OK;
}

int phde_gram_mixed(phde_ctx *ctx, const float *A, const float *B, int k, double *M) {
  const int tiles = (k + GT - 1) / GT;
  if (ctx->tc_gram) {  // tensor cores (tcgram.cu): 2 CTAs per SM, rows split evenly
    const int splits =
        (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->nsm * 2 / (tiles * tiles), (ctx->n + 1023) / 1024));
    double *part = (double *)phde_buf(ctx, "gram32.part", sizeof(double) * (size_t)splits * k * k);
    if (!part) return PHDE_ERR_OOM;
    int rc = phde_tc_gram64(ctx, A, k, k, B, k, k, nullptr, ctx->n, splits, part);
    if (rc) return rc;
    sum_parts32_kernel<<<(int)(((int64_t)k * k + 31) / 32), 256, 0, ctx->stream>>>(part, splits, (int64_t)k * k, M);
    PHDE_LAUNCHED(ctx);
    return PHDE_OK;
  }
  const int splits =
      (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->nsm * 8 / (tiles * tiles), (ctx->n + 255) / 256));
  double *part = (double *)phde_buf(ctx, "gram32.part", sizeof(double) * (size_t)splits * k * k);
  if (!part) return PHDE_ERR_OOM;
  gram32_kernel<<<dim3(tiles * tiles, splits), 256, 0, ctx->stream>>>(A, B, ctx->n, k, part);
  PHDE_LAUNCHED(ctx);
  sum_parts32_kernel<<<(int)(((int64_t)k * k + 31) / 32), 256, 0, ctx->stream>>>(part, splits, (int64_t)k * k, M);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

int phde_coords_mixed(phde_ctx *ctx, const float *S, const double *Y, int k, int c, double *X, double *norm2) {
  const int grid = grid_of(ctx, ctx->n, COORD_ROWS, 8);
  double *part = (double *)phde_buf(ctx, "coords32.part", sizeof(double) * grid * (size_t)COORD_MAXC);
  if (!part) return PHDE_ERR_OOM;
  const size_t smem_max = sizeof(float) * ((size_t)COORD_ROWS * k + (size_t)k * COORD_MAXC);
  PHDE_CK(ctx, cudaFuncSetAttribute(coords32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)std::max<size_t>(smem_max, 48 * 1024)));
  for (int t0 = 0; t0 < c; t0 += COORD_MAXC) {  // coordinates in groups of COORD_MAXC
    const int cg = std::min(COORD_MAXC, c - t0);
    const size_t smem = sizeof(float) * ((size_t)COORD_ROWS * k + (size_t)k * cg);
    coords32_kernel<<<grid, COORD_ROWS, smem, ctx->stream>>>(S, Y + (int64_t)t0 * k, ctx->n, k, cg,
                                                             X + (int64_t)t0 * ctx->n, part);
    PHDE_LAUNCHED(ctx);
    scale32_kernel<<<grid_of(ctx, ctx->n * cg, 256, 8), 256, 0, ctx->stream>>>(X + (int64_t)t0 * ctx->n, ctx->n, cg,
                                                                               part, grid, norm2 ? norm2 + t0 : nullptr);
    PHDE_LAUNCHED(ctx);
  }
  return PHDE_OK;
}
