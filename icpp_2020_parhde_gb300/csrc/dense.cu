// dense.cu -- the dense stages of the layout pipeline in FP64 (the reference's arithmetic).
//
//   cgs_kernel        ParHDE D-orthogonalisation (ParHDE.cpp:190-285): one persistent cooperative launch
//                     runs the whole candidate loop -- coefficient dots, projection update, norm test and
//                     acceptance -- with device-side control, so no host round trip per candidate.
//   mgs kernels       WParHDE modified Gram-Schmidt (WParHDE.cpp:164-213) in its one-reduction form: a dot
//                     sweep, a one-warp coefficient solve and an update sweep per distance column.
//   spmm kernels      LS = D*S - A*S (ParHDE.cpp:288-300, WParHDE.cpp:229-241): one warp per row, lanes
//                     across the k columns of a row-major S, neighbours in CSR order.
//   gram kernels      C = A^T B for row-major n x k operands (matrixTransMultiplication,
//                     DrawingBase.cpp:221-244), C symmetric: the upper triangle, split over row ranges,
//                     partials summed in a fixed order and mirrored.
//   centring kernels  PivotMDS double centring (PivotMDS.cpp:30-66) and PHDE column centring
//                     (PHDE.cpp:30-47) from exact integer sums.
//   coords kernels    X = M * Y (DrawingBase.cpp:207-219) and the unit-norm scaling of getCoordinates
//                     (DrawingBase.cpp:196-205).
// Layout: S, LS and C are row-major n x k (a row is one vertex's k values, so the SpMM's neighbour
// gathers are contiguous k-vectors); distance columns are column-major n x P int32.
#include <vector>

#include "ctx.h"
#include "spmm_plan.cuh"

namespace {

constexpr int CGS_THREADS = 256;
constexpr int MAXQ = 8;  // columns per lane: k <= 256

// ------------------------------------------------------------------------------------------------
struct CgsArgs {
  const int32_t *D;
  int64_t n;
  int P;
  const ull *sumsq;
  const double *deg;
  double *S;  // row-major n x k
  int k;
  double *X;       // [n] projected candidate
  double *part;    // [gridDim][k+2]
  double *part2;   // [gridDim]
  double *coef;    // [k+1]
  double *inv_den; // [k+1], slot k = the constant column
  int *state;      // [0] accepted, [1] discarded, [2] candidates examined
  double *dlog;    // [P] norm of every discarded candidate (NaN otherwise)
  GridSync *gs;
  int *err;
  uint64_t timeout_ns;
};

// Sum of one value per block (written before a grid barrier), in a fixed order for a given grid size;
// the result is valid in every thread of the calling block.
__device__ __forceinline__ double grid_partials_sum(const double *part, double *red) {
  double s = 0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s += __ldcg(part + b);
  return block_sum(s, red);
}

// Stage rows [i0, i0+rows) x columns [c0, c0+nc) of a row-major n x k matrix into a warp's tile
// (row r at tile[r*TILE_LD]); every load is independent and coalesced along the row.
constexpr int TILE_LD = 33;
template <typename T>
__device__ __forceinline__ void stage_tile(const T *S, int64_t i0, int rows, int k, int c0, int nc, T *tile, int lane) {
  __syncwarp();
  if (lane < nc) {
    const T *src = S + i0 * k + c0 + lane;
#pragma unroll 8
    for (int r = 0; r < rows; r++) tile[r * TILE_LD + lane] = src[(int64_t)r * k];
  }
  __syncwarp();
}

__global__ void __launch_bounds__(CGS_THREADS) cgs_kernel(CgsArgs a) {
  extern __shared__ double sm[];  // [nwarps][k+2] reduction scratch (coefficients in phase E), then tiles
  __shared__ double red[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int64_t n = a.n;
  const int k = a.k, ld = k + 2;
  double *tile = sm + nw * ld + warp * 32 * TILE_LD;
  const int64_t gw = (int64_t)blockIdx.x * nw + warp, gws = (int64_t)gridDim.x * nw;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, gts = (int64_t)gridDim.x * blockDim.x;
  const double inv0 = 1.0 / sqrt((double)n);  // the constant column: 1 * (1/||1||), ParHDE.cpp:96-108

  // denominator of the constant column, sum_i u0*u0*d_i
  double acc = 0;
  const double u02 = inv0 * inv0;
  for (int64_t i = gt; i < n; i += gts) acc = fma(u02, a.deg[i], acc);
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) a.part2[blockIdx.x] = acc;
  if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
  const double inv_den0 = 1.0 / grid_partials_sum(a.part2, red);
  if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;

  int j = 1, ndisc = 0, ncand = 0;
  bool newcol = false;
  for (int rc = 0; rc < a.P; rc++) {
    if (j > k) break;
    ncand++;
    const int32_t *Dc = a.D + (int64_t)rc * n;
    const double inv_rc = 1.0 / sqrt((double)__ldcg(a.sumsq + rc));  // ParHDE.cpp:179-184
    const int jm1 = j - 1;
    // ---- A: dots <x, D S_q> for the accepted columns q < j-1 (lanes across q), and <x, D u0> ----
    // A warp takes 32 rows at a time and stages them 32 columns at a time in shared memory (coalesced,
    // independent loads); lane r forms row r's x_i*d_i once and the warp broadcasts it.  The constant
    // column's dot is inv0 * sum_i x_i d_i.
    double accq[MAXQ];
#pragma unroll
    for (int t = 0; t < MAXQ; t++) accq[t] = 0;
    double xsum = 0;
    for (int64_t i0 = gw * 32; i0 < n; i0 += gws * 32) {
      const int64_t il = i0 + lane;
      const double xdl = il < n ? (double)Dc[il] * inv_rc * a.deg[il] : 0.0;
      xsum += xdl;
      const int rows = n - i0 < 32 ? (int)(n - i0) : 32;
#pragma unroll
      for (int t = 0; t < MAXQ; t++) {
        const int c0 = 32 * t;
        if (c0 >= jm1) break;
        const int nc = jm1 - c0 < 32 ? jm1 - c0 : 32;
        stage_tile(a.S, i0, rows, k, c0, nc, tile, lane);
        double acc = accq[t];
        for (int rr = 0; rr < rows; rr++) {
          const double xd = __shfl_sync(PHDE_FULL_MASK, xdl, rr);
          if (lane < nc) acc = fma(xd, tile[rr * TILE_LD + lane], acc);
        }
        accq[t] = acc;
        __syncwarp();
      }
    }
    xsum = warp_sum(xsum);
#pragma unroll
    for (int t = 0; t < MAXQ; t++) {
      const int q = lane + 32 * t;
      if (q < jm1) sm[warp * ld + q] = accq[t];
    }
    if (lane == 0) sm[warp * ld + k] = xsum * inv0;
    __syncthreads();
    for (int q = threadIdx.x; q < k + 1; q += blockDim.x) {
      if (q < jm1 || q == k) {
        double s = 0;
        for (int w = 0; w < nw; w++) s += sm[w * ld + q];
        a.part[(int64_t)blockIdx.x * ld + q] = s;
      }
    }
    if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
    // ---- C: one block per coefficient sums the block partials in a fixed order ----
    for (int q = blockIdx.x; q < j; q += gridDim.x) {
      const int slot = q == jm1 ? k : q;  // q == j-1 stands for the constant column
      const bool fresh = newcol && q == j - 2;  // column accepted by the previous candidate
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
    // ---- E: x' = x - (sum_q coef_q S_q + coef_0 u0), one lane per row of a staged tile; ||x'||^2 ----
    __syncthreads();
    for (int q = threadIdx.x; q < jm1; q += blockDim.x) sm[q] = __ldcg(a.coef + q);
    __syncthreads();
    const double c0u0 = __ldcg(a.coef + k) * inv0;
    double ssq = 0;
    for (int64_t i0 = gw * 32; i0 < n; i0 += gws * 32) {
      const int rows = n - i0 < 32 ? (int)(n - i0) : 32;
      double p = 0;
      for (int c0 = 0; c0 < jm1; c0 += 32) {
        const int nc = jm1 - c0 < 32 ? jm1 - c0 : 32;
        stage_tile(a.S, i0, rows, k, c0, nc, tile, lane);
        if (lane < rows)
          for (int q = 0; q < nc; q++) p = fma(sm[c0 + q], tile[lane * TILE_LD + q], p);
        __syncwarp();
      }
      if (lane < rows) {
        const int64_t i = i0 + lane;
        const double xp = (double)Dc[i] * inv_rc - (p + c0u0);
        a.X[i] = xp;
        ssq = fma(xp, xp, ssq);
      }
    }
    ssq = block_sum(ssq, red);
    if (threadIdx.x == 0) a.part2[blockIdx.x] = ssq;
    if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
    // ---- G: norm test (ParHDE.cpp:267) and acceptance; the new column's D-norm partials ----
    const double nrm = sqrt(grid_partials_sum(a.part2, red));
    if (nrm < 0.001) {
      ndisc++;
      if (blockIdx.x == 0 && threadIdx.x == 0) a.dlog[rc] = nrm;
      newcol = false;
    } else {
      const double scale = 1.0 / nrm;
      double dd = 0;
      for (int64_t i = gt; i < n; i += gts) {
        const double v = __ldcg(a.X + i) * scale;
        a.S[i * k + (j - 1)] = v;
        dd = fma(v * v, a.deg[i], dd);
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

// ------------------------------------------------------------------------------------------------
// WParHDE coupled D-orthogonalisation (WParHDE.cpp:164-213): the new distance column x0 (normalised) is
// projected against the accepted columns y_0 .. y_{j-1} of U (column-major n x (k+1), y_0 the constant
// column) by modified Gram-Schmidt: c_q = <x_q, D y_q> / <y_q, D y_q>, x_{q+1} = x_q - c_q y_q.  MGS's j
// sweeps over memory are replaced by two, with the same coefficients in exact arithmetic:
//   <x_q, D y_q> = <x0, D y_q> - sum_{p<q} c_p <y_p, D y_q>,
// so one sweep forms r_q = <x0, D y_q> for every q (and, once per accepted column g, the Gram entries
// G[p][g] = <y_p, D y_g>, p <= g), a one-warp kernel solves the recurrence for the c_q, and a second sweep
// forms x = x0 - sum_q c_q y_q with its squared L2 norm (the discard test, WParHDE.cpp:194-204).  This is
// the one-reduction form of MGS (Swirydowicz, Langou, Ananthan, Yang and Thomas, "Low synchronization
// Gram-Schmidt and GMRES algorithms", 2020), whose loss of orthogonality is MGS's; GB300 runs FP64 at 1/64
// of the FP32 rate, and it needs about half of MGS's FP64 instructions and a fifth of its memory traffic.
constexpr int MGS_TP = 8;  // columns per thread in the dot sweep

// Column p of U (p < j) gives r_p = sum_i y_p[i] * (x0[i] * d[i]) (product p) and, when g >= 0 (then g = j - 1),
// G[p][g] = sum_i y_p[i] * (y_g[i] * d[i]) (product j + p), from one load of y_p[i].  x0 = col * (1/sqrt(sumsq))
// as WParHDE.cpp:154-162.  blockIdx.y picks MGS_TP columns; part[blockIdx.x * np + product] = the block's sum.
__global__ void __launch_bounds__(256) mgs_dots_kernel(const int32_t *col, const ull *sumsq, const double *U,
                                                       const double *deg, int64_t n, int j, int g, double *part) {
  __shared__ double red[8][2 * MGS_TP];
  const bool gr = g >= 0;
  const int np = j + (gr ? j : 0);
  const int p0 = blockIdx.y * MGS_TP;
  const double inv = 1.0 / sqrt((double)*sumsq);
  const double *yg = U + (int64_t)(gr ? g : 0) * n;
  double ar[MGS_TP], ag[MGS_TP];
#pragma unroll
  for (int t = 0; t < MGS_TP; t++) ar[t] = ag[t] = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double d = deg[i];
    const double z0 = __dmul_rn(__dmul_rn((double)col[i], inv), d);
    const double z1 = gr ? __dmul_rn(yg[i], d) : 0.0;
#pragma unroll
    for (int t = 0; t < MGS_TP; t++)
      if (p0 + t < j) {
        const double y = U[(int64_t)(p0 + t) * n + i];
        ar[t] = fma(y, z0, ar[t]);
        if (gr) ag[t] = fma(y, z1, ag[t]);
      }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < MGS_TP; t++) {
    const double vr = warp_sum(ar[t]);
    const double vg = warp_sum(ag[t]);
    if (lane == 0) {
      red[warp][t] = vr;
      red[warp][MGS_TP + t] = vg;
    }
  }
  __syncthreads();
  if (threadIdx.x < 2 * MGS_TP) {
    const int t = threadIdx.x % MGS_TP, p = p0 + t;
    const bool isg = threadIdx.x >= MGS_TP;
    if (p < j && (!isg || gr)) {
      double v = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += red[w][threadIdx.x];
      part[(int64_t)blockIdx.x * np + (isg ? j + p : p)] = v;
    }
  }
}

// One warp: sums the dot sweep's partials (block order), stores the new Gram entries G[p][g] (row-major
// (k+1) x (k+1), p <= g), then solves c_q = (r_q - sum_{p<q} c_p G[p][q]) / G[q][q] for q = 0 .. j-1.
__global__ void mgs_solve_kernel(const double *part, int nparts, int j, int g, int ldg, double *G, double *coef) {
  __shared__ double r[PHDE_MAX_K + 1], c[PHDE_MAX_K + 1];
  const int lane = threadIdx.x;
  const int np = j + (g >= 0 ? g + 1 : 0);
  for (int p = lane; p < np; p += 32) {
    double v = 0;
    for (int b = 0; b < nparts; b++) v += part[(int64_t)b * np + p];
    if (p < j)
      r[p] = v;
    else
      G[(int64_t)(p - j) * ldg + g] = v;
  }
  __threadfence_block();
  __syncwarp();
  for (int q = 0; q < j; q++) {
    double s = 0;
    for (int p = lane; p < q; p += 32) s = fma(c[p], G[(int64_t)p * ldg + q], s);
    s = warp_sum(s);
    if (lane == 0) c[q] = __dmul_rn(r[q] - s, 1.0 / G[(int64_t)q * ldg + q]);
    __syncwarp();
  }
  for (int q = lane; q < j; q += 32) coef[q] = c[q];
}

// x = x0 - sum_q c_q y_q into U column j; part[block] = the block's sum of x^2.
__global__ void __launch_bounds__(256) mgs_apply_kernel(const int32_t *col, const ull *sumsq, double *U, int64_t n,
                                                        int j, const double *coef, double *part) {
  __shared__ double cs[PHDE_MAX_K + 1];
  __shared__ double red[32];
  for (int q = threadIdx.x; q < j; q += blockDim.x) cs[q] = coef[q];
  __syncthreads();
  const double inv = 1.0 / sqrt((double)*sumsq);
  double *x = U + (int64_t)j * n;
  double ss = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double xi = __dmul_rn((double)col[i], inv);
#pragma unroll 4
    for (int q = 0; q < j; q++) xi = fma(-cs[q], U[(int64_t)q * n + i], xi);
    x[i] = xi;
    ss = fma(xi, xi, ss);
  }
  ss = block_sum(ss, red);
  if (threadIdx.x == 0) part[blockIdx.x] = ss;
}

// Accept: x *= 1/nrm in place (WParHDE.cpp:205-208).
__global__ void scale_col_kernel(double *x, int64_t n, double scale) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = __dmul_rn(x[i], scale);
}

// S (row-major n x k) from U's accepted columns 1 .. k (the distMatrix copy, WParHDE.cpp:210-213): a block
// transposes 32 rows x k columns through shared memory.
__global__ void __launch_bounds__(256) basis_rows_kernel(const double *U, int64_t n, int k, double *S) {
  __shared__ double t[32][33];
  for (int64_t i0 = (int64_t)blockIdx.x * 32; i0 < n; i0 += (int64_t)gridDim.x * 32) {
    for (int q0 = 0; q0 < k; q0 += 32) {
      const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
      for (int qq = w; qq < 32; qq += 8) {
        const int q = q0 + qq;
        if (q < k && i0 + lane < n) t[qq][lane] = U[(int64_t)(q + 1) * n + i0 + lane];
      }
      __syncthreads();
      for (int rr = w; rr < 32; rr += 8) {
        const int q = q0 + lane;
        if (q < k && i0 + rr < n) S[(i0 + rr) * k + q] = t[lane][rr];
      }
      __syncthreads();
    }
  }
}

__global__ void const_col_kernel(double *U, int64_t n) {
  const double inv0 = 1.0 / sqrt((double)n);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    U[i] = inv0;
}

// ------------------------------------------------------------------------------------------------
__global__ void degrees_kernel(const int64_t *off, const int32_t *w, int64_t n, double *deg) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (w == nullptr) {
      deg[i] = (double)(off[i + 1] - off[i]);  // ParHDE.cpp:58-59
    } else {
      double d = 0;  // WParHDE.cpp:53-58: summed in CSR order
      for (int64_t e = off[i]; e < off[i + 1]; e++) d = __dadd_rn(d, (double)w[e]);
      deg[i] = d;
    }
  }
}

// ---- Laplacian SpMM, load balanced ----
// Rows of degree <= SPMM_HEAVY are done by one warp each, neighbours in CSR order (the reference's
// subtraction sequence, ParHDE.cpp:293-298), four neighbour rows in flight.  Weighted rows subtract
// w*S[j] with one fused multiply-add, the weights read as FP64 (converted once per uploaded graph): GB300
// runs FP64 at 1/64 of the FP32 rate, so one FP64 instruction per edge and column instead of three.  Heavier rows (R-MAT
// hubs) are cut into chunks of SPMM_CHUNK neighbours; one warp sums each chunk, and a fix-up pass forms
// LS = d*S - (sum of the chunk partials in chunk order), so the result is deterministic.
__global__ void widen_weights_kernel(const int32_t *w, int64_t nnz, double *w64) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x)
    w64[e] = (double)w[e];
}

__global__ void spmm_plan_kernel(const int64_t *off, int64_t n, HeavyRow *heavy, Chunk *chunks, ull *counts) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e0 = off[i], e1 = off[i + 1], deg = e1 - e0;
    if (deg <= SPMM_HEAVY) continue;
    const int64_t nch = (deg + SPMM_CHUNK - 1) / SPMM_CHUNK;
    const int64_t base = (int64_t)atomicAdd(counts + 1, (ull)nch);
    const int64_t h = (int64_t)atomicAdd(counts, 1ull);
    heavy[h] = HeavyRow{i, base, nch};
    for (int64_t c = 0; c < nch; c++) chunks[base + c] = Chunk{e0 + c * SPMM_CHUNK, min(e1, e0 + (c + 1) * SPMM_CHUNK)};
  }
}

template <bool W, int KT>
__device__ __forceinline__ void spmm_accumulate(const uint32_t *adj, const double *w, const double *S, int k,
                                                int lane, int64_t e0, int64_t e1, double (&acc)[KT]) {
  int64_t e = e0;
  for (; e + 4 <= e1; e += 4) {
    const int64_t v0 = __ldg(adj + e), v1 = __ldg(adj + e + 1), v2 = __ldg(adj + e + 2), v3 = __ldg(adj + e + 3);
    double w0 = 1, w1 = 1, w2 = 1, w3 = 1;
    if (W) {
      w0 = __ldg(w + e);
      w1 = __ldg(w + e + 1);
      w2 = __ldg(w + e + 2);
      w3 = __ldg(w + e + 3);
    }
#pragma unroll
    for (int t = 0; t < KT; t++) {
      const int q = lane + 32 * t;
      if (q < k) {
        const double s0 = S[v0 * k + q], s1 = S[v1 * k + q], s2 = S[v2 * k + q], s3 = S[v3 * k + q];
        if (W) {
          acc[t] = fma(-w0, s0, acc[t]);
          acc[t] = fma(-w1, s1, acc[t]);
          acc[t] = fma(-w2, s2, acc[t]);
          acc[t] = fma(-w3, s3, acc[t]);
        } else {
          acc[t] = __dsub_rn(__dsub_rn(__dsub_rn(__dsub_rn(acc[t], s0), s1), s2), s3);
        }
      }
    }
  }
  for (; e < e1; e++) {
    const int64_t v = __ldg(adj + e);
    const double we = W ? __ldg(w + e) : 1.0;
#pragma unroll
    for (int t = 0; t < KT; t++) {
      const int q = lane + 32 * t;
      if (q < k) acc[t] = W ? fma(-we, S[v * k + q], acc[t]) : __dsub_rn(acc[t], S[v * k + q]);
    }
  }
}

// Light rows: LS[i,q] = d_i*S[i,q] - sum_e w_e*S[adj_e,q].  Heavy rows are skipped here.
template <bool W, int KT>
__global__ void spmm_light_kernel(const int64_t *off, const uint32_t *adj, const double *w, const double *deg,
                                  const double *S, double *LS, int64_t n, int k) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t gws = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = gw; i < n; i += gws) {
    const int64_t e0 = off[i], e1 = off[i + 1];
    if (e1 - e0 > SPMM_HEAVY) continue;
    const double di = deg[i];
    double acc[KT];
#pragma unroll
    for (int t = 0; t < KT; t++) {
      const int q = lane + 32 * t;
      acc[t] = q < k ? __dmul_rn(di, S[i * k + q]) : 0.0;
    }
    spmm_accumulate<W, KT>(adj, w, S, k, lane, e0, e1, acc);
#pragma unroll
    for (int t = 0; t < KT; t++) {
      const int q = lane + 32 * t;
      if (q < k) LS[i * k + q] = acc[t];
    }
  }
}

// Heavy-row chunks: part[c, q] = sum over the chunk of w_e*S[adj_e,q].
template <bool W, int KT>
__global__ void spmm_chunk_kernel(const uint32_t *adj, const double *w, const double *S, const Chunk *chunks,
                                  int64_t nchunks, double *part, int k) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t gws = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = gw; c < nchunks; c += gws) {
    double acc[KT];
#pragma unroll
    for (int t = 0; t < KT; t++) acc[t] = 0.0;
    const Chunk ch = chunks[c];
    spmm_accumulate<W, KT>(adj, w, S, k, lane, ch.e0, ch.e1, acc);  // accumulates -sum
#pragma unroll
    for (int t = 0; t < KT; t++) {
      const int q = lane + 32 * t;
      if (q < k) part[c * k + q] = acc[t];
    }
  }
}

__global__ void spmm_heavy_fix_kernel(const HeavyRow *heavy, int64_t nheavy, const double *deg, const double *S,
                                      const double *part, double *LS, int k) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t gws = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t h = gw; h < nheavy; h += gws) {
    const HeavyRow hr = heavy[h];
    const int64_t i = hr.row;
    const double di = deg[i];
#pragma unroll
    for (int t = 0; t < MAXQ; t++) {
      const int q = lane + 32 * t;
      if (q < k) {
        double a = __dmul_rn(di, S[i * k + q]);
        for (int64_t c = 0; c < hr.nchunks; c++) a = __dadd_rn(a, part[(hr.first_chunk + c) * k + q]);
        LS[i * k + q] = a;
      }
    }
  }
}

// Partial C = A^T B over one row range, for C symmetric (A^T B = S^T L S with L symmetric): only the
// entries p <= q are summed, the rest are mirrored when the partials are added (sum_parts_sym_kernel).
// part: [splits][k*k] column-major (entry (p,q) at q + p*k, the reference's C[k + i*mdim] layout).
//
// gram_list_kernel (k(k+1)/2 <= 8192): thread t of the block owns upper-triangle outputs t, t + T, ... (NO
// of them, T threads), each summed over the block's rows in order from row slabs staged in shared memory.
// FP64 runs at 1/64 of the FP32 rate on GB300, so no FMA is spent on padding or on the lower triangle.
// gram_kernel (larger k): 16 x 16 threads, U x U accumulators each, on the tiles at or above the diagonal.
constexpr int GT = 64, GR = 16;
template <int U>
__global__ void __launch_bounds__(256) gram_kernel(const double *A, const double *B, int64_t n, int k,
                                                   double *part) {
  constexpr int TS = 16 * U;
  __shared__ double sA[GR][TS + 1];
  __shared__ double sB[GR][TS + 1];
  const int tiles = (k + TS - 1) / TS;
  int tp = 0, rest = blockIdx.x;  // blockIdx.x enumerates the tile pairs tp <= tq row by row
  while (rest >= tiles - tp) {
    rest -= tiles - tp;
    tp++;
  }
  const int tq = tp + rest;
  const int p0 = tp * TS, q0 = tq * TS;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t rows_per = (n + gridDim.y - 1) / gridDim.y;
  const int64_t r0 = (int64_t)blockIdx.y * rows_per;
  const int64_t r1 = min(n, r0 + rows_per);
  double acc[U][U] = {};
  for (int64_t rb = r0; rb < r1; rb += GR) {
    for (int idx = threadIdx.x; idx < GR * TS; idx += 256) {
      const int rr = idx / TS, cc = idx % TS;
      const int64_t r = rb + rr;
      sA[rr][cc] = (r < r1 && p0 + cc < k) ? A[r * k + p0 + cc] : 0.0;
      sB[rr][cc] = (r < r1 && q0 + cc < k) ? B[r * k + q0 + cc] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int rr = 0; rr < GR; rr++) {
      double av[U], bv[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        av[u] = sA[rr][ty + 16 * u];
        bv[u] = sB[rr][tx + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < U; u++)
#pragma unroll
        for (int v = 0; v < U; v++) acc[u][v] = fma(av[u], bv[v], acc[u][v]);
    }
    __syncthreads();
  }
  double *out = part + (int64_t)blockIdx.y * k * k;
#pragma unroll
  for (int u = 0; u < U; u++)
#pragma unroll
    for (int v = 0; v < U; v++) {
      const int p = p0 + ty + 16 * u, q = q0 + tx + 16 * v;
      if (p <= q && q < k) out[q + (int64_t)p * k] = acc[u][v];
    }
}

template <int NO>
__global__ void __launch_bounds__(1024) gram_list_kernel(const double *A, const double *B, int64_t n, int k,
                                                         double *part) {
  extern __shared__ double gsm[];  // sA[GR][k + 1], sB[GR][k + 1]
  double *sA = gsm, *sB = gsm + GR * (k + 1);
  const int kp = k + 1;
  const int64_t rows_per = (n + gridDim.y - 1) / gridDim.y;
  const int64_t r0 = (int64_t)blockIdx.y * rows_per;
  const int64_t r1 = min(n, r0 + rows_per);
  const int nout = k * (k + 1) / 2;
  int op[NO], oq[NO];
#pragma unroll
  for (int u = 0; u < NO; u++) {
    int o = threadIdx.x + (int)blockDim.x * u, p = 0;
    if (o >= nout) o = 0;  // a spare slot repeats output 0 and is not stored
    while (o >= k - p) {   // row p of the upper triangle holds k - p outputs
      o -= k - p;
      p++;
    }
    op[u] = p;
    oq[u] = p + o;
  }
  double acc[NO] = {};
  for (int64_t rb = r0; rb < r1; rb += GR) {
    for (int idx = threadIdx.x; idx < GR * k; idx += blockDim.x) {
      const int rr = idx / k, cc = idx % k;
      const int64_t r = rb + rr;
      sA[rr * kp + cc] = r < r1 ? A[r * k + cc] : 0.0;
      sB[rr * kp + cc] = r < r1 ? B[r * k + cc] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int rr = 0; rr < GR; rr++)
#pragma unroll
      for (int u = 0; u < NO; u++) acc[u] = fma(sA[rr * kp + op[u]], sB[rr * kp + oq[u]], acc[u]);
    __syncthreads();
  }
  double *out = part + (int64_t)blockIdx.y * k * k;
#pragma unroll
  for (int u = 0; u < NO; u++)
    if (threadIdx.x + (int)blockDim.x * u < nout) out[oq[u] + (int64_t)op[u] * k] = acc[u];
}

// M[i] = sum over splits of the partials, in split order; for a symmetric product the entries below the
// diagonal take the partials of their mirror.
__global__ void sum_parts_sym_kernel(const double *part, int splits, int k, double *out) {
  const int64_t len = (int64_t)k * k;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(i / k), q = (int)(i % k);
    const int64_t src = p <= q ? i : (int64_t)p + (int64_t)q * k;
    double s = 0;
    for (int b = 0; b < splits; b++) s += part[(int64_t)b * len + src];
    out[i] = s;
  }
}

// ---- reference-order kernels (PivotMDS / PHDE) ----
// The centred matrix C of PivotMDS/PHDE is bit-identical to the reference's (exact integer sums), so
// when every later sum follows the reference's one-thread order -- C^T C entry by entry over rows in
// order (DrawingBase.cpp:226-237), X = C*Y over pivots in order (DrawingBase.cpp:212-217), the norm of
// each coordinate over vertices in order (ParallelComponents.cpp:13-20) -- the coordinates are too.
__global__ void gram_seq_kernel(const double *C, int64_t n, int k, double *M) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= k * k) return;
  const int p = idx / k, q = idx % k;
  double s = 0;
  for (int64_t i = 0; i < n; i++) s = __dadd_rn(s, __dmul_rn(C[i * k + p], C[i * k + q]));
  M[q + (int64_t)p * k] = s;
}

__global__ void coords_seq_kernel(const double *M, const double *Y, int64_t n, int k, int c, double *X) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n * c;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx % n;
    const int t = (int)(idx / n);
    double s = 0;
    for (int j = 0; j < k; j++) s = __dadd_rn(s, __dmul_rn(M[i * k + j], Y[j + (int64_t)t * k]));
    X[idx] = s;
  }
}

// one block per coordinate; lane 0 sums the squares in vertex order
__global__ void colnorm_seq_kernel(const double *X, int64_t n, double *part) {
  if (threadIdx.x != 0) return;
  const double *x = X + (int64_t)blockIdx.x * n;
  double s = 0;
  for (int64_t i = 0; i < n; i++) s = __dadd_rn(s, __dmul_rn(x[i], x[i]));
  part[blockIdx.x] = s;
}

// ------------------------------------------------------------------------------------------------
// Exact integer sums of the raw distance columns: colsq[q] = sum_i d^2, colsum[q] = sum_i d, and
// rowsq[i] = sum_q d^2 (exact in FP64 for BFS distances).
__global__ void dist_sums_kernel(const int32_t *D, int64_t n, int k, ull *colsq, ull *colsum, double *rowsq) {
  __shared__ ull red[32];
  for (int q = 0; q < k; q++) {
    ull s2 = 0, s1 = 0;
    const int32_t *col = D + (int64_t)q * n;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      const ull d = (ull)col[i];
      s2 += d * d;
      s1 += d;
    }
    s2 = block_sum(s2, red);
    s1 = block_sum(s1, red);
    if (threadIdx.x == 0) {
      atomicAdd(colsq + q, s2);
      atomicAdd(colsum + q, s1);
    }
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double r = 0;
    for (int q = 0; q < k; q++) {
      const double d = (double)D[i + (int64_t)q * n];
      r = __dadd_rn(r, __dmul_rn(d, d));
    }
    rowsq[i] = r;
  }
}

// C[i,q] = -0.5*(d^2 - rN*colsum_q - rK*rowsum_i + rK*rN*total) (PivotMDS.cpp:42-53), or for PHDE
// C[i,q] = d - colsum_q/n (PHDE.cpp:32-46).  Row-major output.
__global__ void centre_kernel(const int32_t *D, int64_t n, int k, const ull *colsq, const ull *colsum,
                              const double *rowsq, int pivotmds, double *C) {
  double total = 0;
  for (int q = 0; q < k; q++) total = __dadd_rn(total, (double)colsq[q]);
  const double rN = 1.0 / (double)n, rK = 1.0 / (double)k;
  const double t4 = __dmul_rn(__dmul_rn(rK, rN), total);
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n * k;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / k;
    const int q = (int)(idx % k);
    const double d = (double)D[i + (int64_t)q * n];
    double v;
    if (pivotmds) {
      const double t = __dadd_rn(__dsub_rn(__dsub_rn(__dmul_rn(d, d), __dmul_rn(rN, (double)colsq[q])),
                                           __dmul_rn(rK, rowsq[i])),
                                 t4);
      v = __dmul_rn(-0.5, t);
    } else {
      v = __dsub_rn(d, __ddiv_rn((double)colsum[q], (double)n));
    }
    C[idx] = v;
  }
}

// X[i + t*n] = sum_q M[i,q] * Y[q + t*k]; per-block partial sums of squares per coordinate.
// X[:, t] = S Y[:, t], FP64: a block stages blockDim.x consecutive rows of S (one contiguous range, read
// coalesced) into shared memory at a padded stride, then a thread per row forms up to CO_MAXC coordinates,
// each summed over the row's k entries in order with fused multiply-adds (more coordinates run in groups).
constexpr int CO_MAXC = 8;
__global__ void __launch_bounds__(128) coords_kernel(const double *M, const double *Y, int64_t n, int k, int c,
                                                     double *X, double *part) {
  extern __shared__ double csm[];  // the group's Ys[q + t * k], then the row tile [blockDim.x][k + 1]
  __shared__ double red[32];
  const int rows = blockDim.x, kp = k + 1;
  double *Ys = csm, *tile = csm + (size_t)k * CO_MAXC;
  for (int t0 = 0; t0 < c; t0 += CO_MAXC) {
    const int cg = min(CO_MAXC, c - t0);
    __syncthreads();  // the previous group's last tile read
    for (int i = threadIdx.x; i < k * cg; i += blockDim.x) Ys[i] = Y[(int64_t)t0 * k + i];
    double ss[CO_MAXC];
#pragma unroll
    for (int t = 0; t < CO_MAXC; t++) ss[t] = 0;
    for (int64_t i0 = (int64_t)blockIdx.x * rows; i0 < n; i0 += (int64_t)gridDim.x * rows) {
      const int nr = (int)min((int64_t)rows, n - i0);
      __syncthreads();  // Ys written (first tile), or the previous tile read
      const double *src = M + i0 * k;
      for (int e = threadIdx.x; e < nr * k; e += blockDim.x) tile[(e / k) * kp + e % k] = src[e];
      __syncthreads();
      if ((int)threadIdx.x < nr) {
        const double *row = tile + threadIdx.x * kp;
        double sv[CO_MAXC];
#pragma unroll
        for (int t = 0; t < CO_MAXC; t++) sv[t] = 0;
        for (int q = 0; q < k; q++) {
          const double m = row[q];
#pragma unroll
          for (int t = 0; t < CO_MAXC; t++)
            if (t < cg) sv[t] = fma(m, Ys[q + t * k], sv[t]);
        }
#pragma unroll
        for (int t = 0; t < CO_MAXC; t++)
          if (t < cg) {
            X[i0 + threadIdx.x + (int64_t)(t0 + t) * n] = sv[t];
            ss[t] = fma(sv[t], sv[t], ss[t]);
          }
      }
    }
    for (int t = 0; t < cg; t++) {  // cg is uniform: every thread takes part in each block sum
      const double tot = block_sum(ss[t], red);
      if (threadIdx.x == 0) part[(int64_t)blockIdx.x * c + t0 + t] = tot;
    }
  }
}

// X[:, t] /= ||X[:, t]||: each block sums the per-block partials itself (block-wide, fixed order), then scales;
// block 0 also reports ||X[:, t]||^2 before the scaling (norm2, optional).
__global__ void scale_coords_kernel(double *X, int64_t n, int c, const double *part, int nparts, double *norm2) {
  __shared__ double inv[PHDE_MAX_K];
  __shared__ double red[32];
  for (int t = 0; t < c; t++) {
    double s = 0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) s += part[(int64_t)b * c + t];
    s = block_sum(s, red);
    if (threadIdx.x == 0) inv[t] = 1.0 / sqrt(s);
    if (norm2 && blockIdx.x == 0 && threadIdx.x == 0) norm2[t] = s;
  }
  __syncthreads();
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n * c;
       idx += (int64_t)gridDim.x * blockDim.x)
    X[idx] = __dmul_rn(X[idx], inv[idx / n]);
}

}  // namespace

// ==================================================================================================
// host launchers
int phde_reset_sync(phde_ctx *ctx);

static int grid_for(phde_ctx *ctx, int64_t work, int threads, int per_sm = 8) {
  int64_t b = (work + threads - 1) / threads;
  b = std::min<int64_t>(b, (int64_t)ctx->nsm * per_sm);
  return (int)std::max<int64_t>(b, 1);
}

int phde_degrees(phde_ctx *ctx, double *deg) {
  degrees_kernel<<<grid_for(ctx, ctx->n, 256), 256, 0, ctx->stream>>>(ctx->d_off, ctx->weighted ? ctx->d_w : nullptr,
                                                                      ctx->n, deg);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

// ParHDE CGS: candidates are the P distance columns of D; accepted vectors go to row-major S.
int phde_cgs(phde_ctx *ctx, const int32_t *D, int P, const ull *sumsq, const double *deg, double *S, int k,
             int *h_state, double *h_dlog) {
  const int64_t n = ctx->n;
  int per_sm = 0;
  const size_t smem = sizeof(double) * (CGS_THREADS / 32) * ((size_t)(k + 2) + 32 * TILE_LD);
  PHDE_CK(ctx, cudaFuncSetAttribute(cgs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  PHDE_CK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cgs_kernel, CGS_THREADS, smem));
  if (per_sm < 1) return phde_fail(ctx, PHDE_ERR_CUDA, "cgs kernel cannot be resident");
  per_sm = std::min(per_sm, 4);
  const int grid = ctx->nsm * per_sm;
  double *X = (double *)phde_buf(ctx, "cgs.X", sizeof(double) * n);
  double *part = (double *)phde_buf(ctx, "cgs.part", sizeof(double) * grid * (size_t)(k + 2));
  double *part2 = (double *)phde_buf(ctx, "cgs.part2", sizeof(double) * grid);
  double *coef = (double *)phde_buf(ctx, "cgs.coef", sizeof(double) * (k + 1));
  double *inv_den = (double *)phde_buf(ctx, "cgs.inv_den", sizeof(double) * (k + 1));
  int *state = (int *)phde_buf(ctx, "cgs.state", sizeof(int) * 4);
  double *dlog = (double *)phde_buf(ctx, "cgs.dlog", sizeof(double) * P);
  if (!X || !part || !part2 || !coef || !inv_den || !state || !dlog) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(dlog, 0xff, sizeof(double) * P, ctx->stream));  // NaN: not discarded
  PHDE_CK(ctx, cudaMemsetAsync(state, 0, sizeof(int) * 4, ctx->stream));
  int rc = phde_reset_sync(ctx);
  if (rc) return rc;
  CgsArgs a;
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
  PHDE_CK(ctx, cudaLaunchCooperativeKernel((const void *)cgs_kernel, dim3(grid), dim3(CGS_THREADS), args, smem,
                                           ctx->stream));
  PHDE_LAUNCHED(ctx);
  PHDE_CK(ctx, cudaMemcpyAsync(h_state, state, sizeof(int) * 4, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaMemcpyAsync(h_dlog, dlog, sizeof(double) * P, cudaMemcpyDeviceToHost, ctx->stream));
  return PHDE_OK;
}

// WParHDE: project the new distance column (normalised) against U's columns 0 .. j-1 into column j; g >= 0
// names the column accepted since the last call, whose Gram entries the dot sweep adds.  Returns the
// squared norm of the projected vector in *h_nrm2 (synchronises).
int phde_mgs_pass(phde_ctx *ctx, const int32_t *col, const ull *sumsq, double *U, int j, int g, int k,
                  const double *deg, double *h_nrm2) {
  const int64_t n = ctx->n;
  const int threads = 256;
  const int np = j + (g >= 0 ? g + 1 : 0);
  const int ty = (j + MGS_TP - 1) / MGS_TP;
  const int gx = (int)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, (int64_t)ctx->nsm * 8 / ty));
  const int ga = grid_for(ctx, n, threads, 8);
  double *part = (double *)phde_buf(ctx, "mgs.part", sizeof(double) * (size_t)gx * (2 * PHDE_MAX_K + 2));
  double *G = (double *)phde_buf(ctx, "mgs.G", sizeof(double) * (size_t)(PHDE_MAX_K + 1) * (PHDE_MAX_K + 1));
  double *coef = (double *)phde_buf(ctx, "mgs.coef", sizeof(double) * (PHDE_MAX_K + 1));
  double *pn = (double *)phde_buf(ctx, "mgs.norm", sizeof(double) * ga);
  if (!part || !G || !coef || !pn) return PHDE_ERR_OOM;
  mgs_dots_kernel<<<dim3(gx, ty), threads, 0, ctx->stream>>>(col, sumsq, U, deg, n, j, g, part);
  PHDE_LAUNCHED(ctx);
  mgs_solve_kernel<<<1, 32, 0, ctx->stream>>>(part, gx, j, g, k + 1, G, coef);
  PHDE_LAUNCHED(ctx);
  mgs_apply_kernel<<<ga, threads, 0, ctx->stream>>>(col, sumsq, U, n, j, coef, pn);
  PHDE_LAUNCHED(ctx);
  std::vector<double> h(ga);
  PHDE_CK(ctx, cudaMemcpyAsync(h.data(), pn, sizeof(double) * ga, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  double s = 0;
  for (int b = 0; b < ga; b++) s += h[b];
  *h_nrm2 = s;
  return PHDE_OK;
}

int phde_const_col(phde_ctx *ctx, double *U) {
  const_col_kernel<<<grid_for(ctx, ctx->n, 256), 256, 0, ctx->stream>>>(U, ctx->n);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

int phde_accept_col(phde_ctx *ctx, double *U, int xcol, double scale) {
  scale_col_kernel<<<grid_for(ctx, ctx->n, 256), 256, 0, ctx->stream>>>(U + (int64_t)xcol * ctx->n, ctx->n, scale);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

int phde_basis_rows(phde_ctx *ctx, const double *U, int k, double *S) {
  basis_rows_kernel<<<grid_for(ctx, (ctx->n + 31) / 32 * 256, 256, 4), 256, 0, ctx->stream>>>(U, ctx->n, k, S);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

// Heavy-row chunk plan, built once per uploaded graph (ctx->spmm_plan_epoch tracks which graph).
int phde_spmm_plan(phde_ctx *ctx, HeavyRow **heavy, Chunk **chunks, int64_t *nheavy, int64_t *nchunks) {
  const int64_t cap_h = ctx->nnz / SPMM_HEAVY + 1, cap_c = ctx->nnz / SPMM_CHUNK + cap_h + 1;
  *heavy = (HeavyRow *)phde_buf(ctx, "spmm.heavy", sizeof(HeavyRow) * cap_h);
  *chunks = (Chunk *)phde_buf(ctx, "spmm.chunks", sizeof(Chunk) * cap_c);
  ull *counts = (ull *)phde_buf(ctx, "spmm.counts", sizeof(ull) * 2);
  if (!*heavy || !*chunks || !counts) return PHDE_ERR_OOM;
  if (ctx->spmm_plan_epoch != ctx->graph_epoch) {
    PHDE_CK(ctx, cudaMemsetAsync(counts, 0, sizeof(ull) * 2, ctx->stream));
    spmm_plan_kernel<<<grid_for(ctx, ctx->n, 256), 256, 0, ctx->stream>>>(ctx->d_off, ctx->n, *heavy, *chunks, counts);
    PHDE_LAUNCHED(ctx);
    ull h[2];
    PHDE_CK(ctx, cudaMemcpyAsync(h, counts, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->spmm_nheavy = (int64_t)h[0];
    ctx->spmm_nchunks = (int64_t)h[1];
    ctx->spmm_plan_epoch = ctx->graph_epoch;
  }
  *nheavy = ctx->spmm_nheavy;
  *nchunks = ctx->spmm_nchunks;
  return PHDE_OK;
}

int phde_lap_spmm(phde_ctx *ctx, const double *deg, const double *S, double *LS, int k) {
  HeavyRow *heavy;
  Chunk *chunks;
  int64_t nheavy, nchunks;
  int rc = phde_spmm_plan(ctx, &heavy, &chunks, &nheavy, &nchunks);
  if (rc) return rc;
  const int threads = 256;
  const double *w = nullptr;
  if (ctx->weighted) {
    double *w64 = (double *)phde_buf(ctx, "spmm.w64", sizeof(double) * ctx->nnz);
    if (!w64) return PHDE_ERR_OOM;
    if (ctx->w64_epoch != ctx->graph_epoch || ctx->w64_buf != w64) {
      widen_weights_kernel<<<grid_for(ctx, ctx->nnz, 256), 256, 0, ctx->stream>>>(ctx->d_w, ctx->nnz, w64);
      PHDE_LAUNCHED(ctx);
      ctx->w64_epoch = ctx->graph_epoch;
      ctx->w64_buf = w64;
    }
    w = w64;
  }
  const int grid = grid_for(ctx, ctx->n * 32, threads, 8);
  // column tiles of 32 per lane, a compile-time count (1, 2, 4 or 8): the FP64 instructions of empty tiles
  // are not issued at all
  const int kt = k <= 32 ? 1 : (k <= 64 ? 2 : (k <= 128 ? 4 : 8));
#define PHDE_SPMM64(WW, T) \
  spmm_light_kernel<WW, T><<<grid, threads, 0, ctx->stream>>>(ctx->d_off, ctx->d_adj, w, deg, S, LS, ctx->n, k)
#define PHDE_SPMM64_KT(WW) \
  do {                    \
    if (kt == 1) PHDE_SPMM64(WW, 1); \
    else if (kt == 2) PHDE_SPMM64(WW, 2); \
    else if (kt == 4) PHDE_SPMM64(WW, 4); \
    else PHDE_SPMM64(WW, 8); \
  } while (0)
  if (w)
    PHDE_SPMM64_KT(true);
  else
    PHDE_SPMM64_KT(false);
#undef PHDE_SPMM64_KT
#undef PHDE_SPMM64
  PHDE_LAUNCHED(ctx);
  if (nheavy > 0) {
    double *part = (double *)phde_buf(ctx, "spmm.part", sizeof(double) * nchunks * k);
    if (!part) return PHDE_ERR_OOM;
    const int g2 = grid_for(ctx, nchunks * 32, threads, 8);
#define PHDE_CHUNK64(WW, T) \
  spmm_chunk_kernel<WW, T><<<g2, threads, 0, ctx->stream>>>(ctx->d_adj, w, S, chunks, nchunks, part, k)
#define PHDE_CHUNK64_KT(WW) \
  do {                     \
    if (kt == 1) PHDE_CHUNK64(WW, 1); \
    else if (kt == 2) PHDE_CHUNK64(WW, 2); \
    else if (kt == 4) PHDE_CHUNK64(WW, 4); \
    else PHDE_CHUNK64(WW, 8); \
  } while (0)
    if (w)
      PHDE_CHUNK64_KT(true);
    else
      PHDE_CHUNK64_KT(false);
#undef PHDE_CHUNK64_KT
#undef PHDE_CHUNK64
    PHDE_LAUNCHED(ctx);
    spmm_heavy_fix_kernel<<<grid_for(ctx, nheavy * 32, threads, 8), threads, 0, ctx->stream>>>(heavy, nheavy, deg, S,
                                                                                              part, LS, k);
    PHDE_LAUNCHED(ctx);
  }
  return PHDE_OK;
}

// M (k x k, column-major as the reference stores it) = A^T B.
int phde_gram(phde_ctx *ctx, const double *A, const double *B, int k, double *M) {
  // C = S^T L S is symmetric: the entries p <= q are summed and mirrored
  const int nout = k * (k + 1) / 2;
  const int no = nout <= 1024 ? 1 : (nout <= 2048 ? 2 : (nout <= 4096 ? 4 : (nout <= 8192 ? 8 : 0)));
  int blocks_x, threads, splits;
  size_t smem = 0;
  if (no) {
    threads = (int)(((nout + no - 1) / no + 31) / 32 * 32);
    blocks_x = 1;
    smem = sizeof(double) * 2 * GR * (k + 1);
    const int per_sm = std::max(1, 2048 / threads);
    splits = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->nsm * per_sm, (ctx->n + 255) / 256));
  } else {
    const int tiles = (k + GT - 1) / GT;
    threads = 256;
    blocks_x = tiles * (tiles + 1) / 2;
    splits = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->nsm * 4 / blocks_x, (ctx->n + 255) / 256));
  }
  double *part = (double *)phde_buf(ctx, "gram.part", sizeof(double) * (size_t)splits * k * k);
  if (!part) return PHDE_ERR_OOM;
  const dim3 grid(blocks_x, splits);
  if (no == 1)
    gram_list_kernel<1><<<grid, threads, smem, ctx->stream>>>(A, B, ctx->n, k, part);
  else if (no == 2)
    gram_list_kernel<2><<<grid, threads, smem, ctx->stream>>>(A, B, ctx->n, k, part);
  else if (no == 4)
    gram_list_kernel<4><<<grid, threads, smem, ctx->stream>>>(A, B, ctx->n, k, part);
  else if (no == 8)
    gram_list_kernel<8><<<grid, threads, smem, ctx->stream>>>(A, B, ctx->n, k, part);
  else
    gram_kernel<4><<<grid, threads, 0, ctx->stream>>>(A, B, ctx->n, k, part);
  PHDE_LAUNCHED(ctx);
  sum_parts_sym_kernel<<<grid_for(ctx, (int64_t)k * k, 256), 256, 0, ctx->stream>>>(part, splits, k, M);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

int phde_centre(phde_ctx *ctx, const int32_t *D, int k, int pivotmds, double *C) {
  const int64_t n = ctx->n;
  ull *colsq = (ull *)phde_buf(ctx, "ctr.colsq", sizeof(ull) * k);
  ull *colsum = (ull *)phde_buf(ctx, "ctr.colsum", sizeof(ull) * k);
  double *rowsq = (double *)phde_buf(ctx, "ctr.rowsq", sizeof(double) * n);
  if (!colsq || !colsum || !rowsq) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(colsq, 0, sizeof(ull) * k, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(colsum, 0, sizeof(ull) * k, ctx->stream));
  dist_sums_kernel<<<grid_for(ctx, n, 256, 4), 256, 0, ctx->stream>>>(D, n, k, colsq, colsum, rowsq);
  PHDE_LAUNCHED(ctx);
  centre_kernel<<<grid_for(ctx, n * k, 256), 256, 0, ctx->stream>>>(D, n, k, colsq, colsum, rowsq, pivotmds, C);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

int phde_coords(phde_ctx *ctx, const double *M, const double *Y, int k, int c, double *X, int seq, double *norm2) {
  const int threads = 256;
  if (seq) {
    double *part = (double *)phde_buf(ctx, "coords.part", sizeof(double) * c);
    if (!part) return PHDE_ERR_OOM;
    coords_seq_kernel<<<grid_for(ctx, ctx->n * c, threads), threads, 0, ctx->stream>>>(M, Y, ctx->n, k, c, X);
    PHDE_LAUNCHED(ctx);
    colnorm_seq_kernel<<<c, 32, 0, ctx->stream>>>(X, ctx->n, part);
    PHDE_LAUNCHED(ctx);
    scale_coords_kernel<<<grid_for(ctx, ctx->n * c, 256), 256, 0, ctx->stream>>>(X, ctx->n, c, part, 1, norm2);
    PHDE_LAUNCHED(ctx);
    return PHDE_OK;
  }
  // row tiles of 128 rows (64 for k > 100): at most (256 * 8 + 64 * 257) * 8 bytes of shared memory
  const int rows = k <= 100 ? 128 : 64;
  const int grid = grid_for(ctx, ctx->n, rows, 8);
  double *part = (double *)phde_buf(ctx, "coords.part", sizeof(double) * grid * (size_t)c);
  if (!part) return PHDE_ERR_OOM;
  const size_t smem = sizeof(double) * ((size_t)k * CO_MAXC + (size_t)rows * (k + 1));
  PHDE_CK(ctx, cudaFuncSetAttribute(coords_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)std::max<size_t>(smem, 48 * 1024)));
  coords_kernel<<<grid, rows, smem, ctx->stream>>>(M, Y, ctx->n, k, c, X, part);
  PHDE_LAUNCHED(ctx);
  scale_coords_kernel<<<grid_for(ctx, ctx->n * c, 256), 256, 0, ctx->stream>>>(X, ctx->n, c, part, grid, norm2);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

// M = C^T C in the reference's summation order (one thread per entry).
int phde_gram_seq(phde_ctx *ctx, const double *C, int k, double *M) {
  gram_seq_kernel<<<(k * k + 127) / 128, 128, 0, ctx->stream>>>(C, ctx->n, k, M);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}
