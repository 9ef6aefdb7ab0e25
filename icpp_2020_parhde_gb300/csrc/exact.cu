// exact.cu -- ParHDE's dense stages from exact integer Gram matrices of the distance columns
//             (PHDE_PREC_EXACT).
//
// The reference turns the integer BFS columns into FP64 vectors and works on those vectors: it normalises
// them, D-orthogonalises them by classical Gram-Schmidt (ParHDE.cpp:176-285), forms LS = D S - A S
// (ParHDE.cpp:288-300) and S^T LS (DrawingBase.cpp:221-244), and finally X = S Y (DrawingBase.cpp:207-219).
// Every vector it builds is a linear combination of the integer columns Z = [1, d_1, ..., d_P] (1 = the
// constant column before its 1/sqrt(n) scaling).  So S = Z A for a small coefficient matrix A, and every
// n-sized product the reference needs is a small integer matrix of Z:
//     <x, D q>, <q, D q>   from  G_D = Z^T D Z         ||x - sum c q||_2   from  G_I = Z^T Z
//     S^T L S = A^T (Z_acc^T L Z_acc) A_acc            X = Z (A Y)
// Here those integer matrices are formed EXACTLY (64-bit sums of integer products of distances and
// degrees, order-free), and the reference's candidate loop -- the same coefficients, the same ||x|| < 1e-3
// discard rule, the same acceptance order -- runs in FP64 on (P+1)-dimensional coefficient vectors.
// GB300 issues FP64 at 1/64 of its FP32 rate; this path keeps FP64 out of every n-sized loop, and the
// n-sized sums themselves carry no rounding at all.
//
//   zgram_kernel     G_I, G_D for a block of candidate columns (upper triangle, 4x4 register tiles,
//                    32-bit partial sums flushed to 64-bit atomics under a per-row magnitude bound)
//   coef_kernel      the candidate loop in coefficient space (one CTA, FP64)
//   pack_kernel      the accepted columns as a row-major uint8 / uint16 matrix Z_acc (n x kp)
//   lgram_kernel     Z_acc^T A Z_acc from each undirected edge once: per row (or heavy-row chunk) the sum of
//                    the neighbours above it gathered by a warp (16-bit lanes packed two to a register for uint8
//                    rows), then the outer product with z_i accumulated in register tiles -- the adjacency
//                    product never reaches memory; lfin_kernel subtracts it from G_D's accepted entries
//   mgram_kernel     M = A_acc^T (Z_acc^T L Z_acc) A_acc (FP64, k x k)
//   coords kernels   X = Z (A Y) in fixed point: A Y scaled to 62-bit integers per coordinate, exact
//                    integer row sums, one rounding to FP64; then the unit-norm scaling of getCoordinates
//                    (DrawingBase.cpp:196-205)
#include <cmath>
#include <cstring>
#include <vector>

#include "ctx.h"

namespace {

constexpr int ZG_THREADS = 256;
constexpr int ZG_ROWS = 32;   // rows per staged slab
constexpr int LG_THREADS = 256;
constexpr int LG_ITEMS = 64;  // rows / chunks per slab
constexpr int64_t LG_LIGHT = 16;  // rows of at most this many neighbours are gathered by one lane group
constexpr int CF_THREADS = 256;
constexpr uint64_t B32 = 1ull << 32;
constexpr uint64_t B31 = 1ull << 31;

// Upper-triangle tile (pb, qb), pb <= qb, qb in [qb0, qb1): tiles are numbered qb-major.
__device__ __forceinline__ void tile_of(int t, int qb0, int qb1, int &pb, int &qb) {
  pb = -1;
  qb = -1;
  for (int b = qb0; b < qb1; b++) {
    if (t <= b) {
      pb = t;
      qb = b;
      return;
    }
    t -= b + 1;
  }
}

__device__ __forceinline__ double gsym(const ull *G, int ld, int p, int q) {
  return (double)(long long)(p <= q ? G[(int64_t)p * ld + q] : G[(int64_t)q * ld + p]);
}

// ------------------------------------------------------------------------------------------------
// G_I = Z^T Z and G_D = Z^T D Z for the Z columns p in [0, c1), q in [c0, c1), p <= q.
struct ZgArgs {
  ZSrc src;          // Z column 0 is all ones, columns 1..P the candidates (ZSrc)
  const int64_t *off;
  int64_t n;
  int P;
  int c0, c1;        // multiples of 4
  int ntiles;        // tiles of the block, CTA y takes [y * ZG_THREADS, ...)
  ull *GI, *GD;
  int ld;
  unsigned *maxz;    // [0] largest distance, [1] largest degree
  const unsigned *wide_only;  // non-null: run only when *wide_only > 255 (the byte kernel did not apply)
};

// A slab whose distances all fit a byte goes through byte dot products: zs4[q][col] packs rows 4q .. 4q+3 of a
// column into one word (dp4a: four rows of Z^T Z per instruction) and ys2[h][col] packs deg * z of rows 2h, 2h+1
// as two 16-bit halves (dp2a against the bytes of zs4: two rows of Z^T D Z per instruction).  Rows whose
// deg * z does not fit 16 bits take the one-row 32-bit path.  Every sum is still exact.
__global__ void __launch_bounds__(ZG_THREADS) zgram_kernel(ZgArgs a) {
  if (a.wide_only && __ldg(a.wide_only) <= 255u) return;  // uniform: the quad-layout kernel formed them
  extern __shared__ int zsm[];  // [ZG_ROWS][S], zs4[ZG_ROWS/4][S], ys2[ZG_ROWS/2][S], then the record columns
  __shared__ unsigned s_deg[ZG_ROWS];
  __shared__ ull red[32];
  const int S = a.c1 + 4;
  uint32_t *zs4 = (uint32_t *)zsm + ZG_ROWS * S, *ys2 = zs4 + (ZG_ROWS / 4) * S;
  int *s_rmap = (int *)(ys2 + (ZG_ROWS / 2) * S);
  const int P0 = a.src.P0;
  // Z columns [0, nd) are the ones column and D columns; [nd, c1) record columns (or padding beyond P)
  const int nd = min(a.c1, P0 + 1), nr = a.c1 - nd;
  for (int j = threadIdx.x; j < nr; j += ZG_THREADS) s_rmap[j] = nd + j <= a.P ? a.src.rmap[nd + j - 1 - P0] : -1;
  const int t = blockIdx.y * ZG_THREADS + threadIdx.x;
  int pb, qb;
  tile_of(t, a.c0 / 4, a.c1 / 4, pb, qb);
  const bool active = t < a.ntiles && pb >= 0;
  uint32_t aI[4][4], aD[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) aI[i][j] = aD[i][j] = 0;
  auto flush = [&]() {
    if (!active) return;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int p = 4 * pb + i, q = 4 * qb + j;
        if (p <= q && q < a.c1) {
          if (aI[i][j]) atomicAdd(a.GI + (int64_t)p * a.ld + q, (ull)aI[i][j]);
          if (aD[i][j]) atomicAdd(a.GD + (int64_t)p * a.ld + q, (ull)aD[i][j]);
        }
        aI[i][j] = aD[i][j] = 0;
      }
  };
  const int64_t per = ((a.n + gridDim.x - 1) / gridDim.x + ZG_ROWS - 1) / ZG_ROWS * ZG_ROWS;
  const int64_t r0 = (int64_t)blockIdx.x * per, r1 = min(a.n, r0 + per);
  ull run = 0;  // bound on every partial sum since the last flush (uniform across the block)
  for (int64_t i0 = r0; i0 < r1; i0 += ZG_ROWS) {
    const int rows = (int)min((int64_t)ZG_ROWS, r1 - i0);
    __syncthreads();  // previous slab consumed
    unsigned mz = 0, md = 0;
    for (int e = threadIdx.x; e < ZG_ROWS * nd; e += ZG_THREADS) {  // consecutive threads: rows of a column
      const int col = e / ZG_ROWS, r = e - col * ZG_ROWS;
      int v = 0;
      if (r < rows) v = col == 0 ? 1 : (col - 1 < a.P ? a.src.D[(int64_t)(col - 1) * a.n + i0 + r] : 0);
      zsm[r * S + col] = v;
      mz = max(mz, (unsigned)v);
    }
    for (int e = threadIdx.x; e < ZG_ROWS * nr; e += ZG_THREADS) {  // consecutive threads: columns of a row
      const int r = e / nr, j = e - r * nr;
      const int rc = s_rmap[j];
      const int v = r < rows && rc >= 0 ? (int)a.src.R[(i0 + r) * a.src.RW + rc] - 1 : 0;
      zsm[r * S + nd + j] = v;
      mz = max(mz, (unsigned)v);
    }
    if (threadIdx.x < ZG_ROWS) {
      const int r = threadIdx.x;
      const unsigned d = r < rows ? (unsigned)(a.off[i0 + r + 1] - a.off[i0 + r]) : 0u;
      s_deg[r] = d;
      md = d;
    }
    const ull mzs = block_max_u64((ull)mz, red);
    const ull mds = block_max_u64((ull)md, red);
    if (threadIdx.x == 0) {
      atomicMax(a.maxz, (unsigned)mzs);
      atomicMax(a.maxz + 1, (unsigned)mds);
    }
    const ull mz2 = mzs * mzs;
    const bool bytes = mzs <= 255;  // uniform: the slab's distances fit a byte
    if (bytes) {
      // pack (rows past the end and rows for the 32-bit path pack as zeros)
      for (int e = threadIdx.x; e < (ZG_ROWS / 4) * a.c1; e += ZG_THREADS) {
        const int q = e / a.c1, col = e - q * a.c1;
        uint32_t w = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int r = 4 * q + j;
          if ((ull)max(s_deg[r], 1u) * mzs <= 65535ull) w |= (uint32_t)zsm[r * S + col] << (8 * j);
        }
        zs4[q * S + col] = w;
      }
      for (int e = threadIdx.x; e < (ZG_ROWS / 2) * a.c1; e += ZG_THREADS) {
        const int h = e / a.c1, col = e - h * a.c1;
        uint32_t w = 0;
#pragma unroll
        for (int j = 0; j < 2; j++) {
          const int r = 2 * h + j;
          const unsigned d = s_deg[r];
          if ((ull)max(d, 1u) * mzs <= 65535ull) w |= ((uint32_t)zsm[r * S + col] * d) << (16 * j);
        }
        ys2[h * S + col] = w;
      }
      __syncthreads();
      for (int q = 0; q < ZG_ROWS / 4; q++) {
        ull b = 0;  // bound of the quad's light rows
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int r = 4 * q + j;
          const unsigned d = s_deg[r];
          if (r < rows && (ull)max(d, 1u) * mzs <= 65535ull) b += (ull)max(d, 1u) * mz2;
        }
        if (b == 0) continue;
        if (run + b >= B32) {
          flush();
          run = 0;
        }
        run += b;
        if (active) {
          const uint4 zp = *(const uint4 *)(zs4 + q * S + 4 * pb);
          const uint4 zq = *(const uint4 *)(zs4 + q * S + 4 * qb);
          const uint4 y0 = *(const uint4 *)(ys2 + (2 * q) * S + 4 * pb);
          const uint4 y1 = *(const uint4 *)(ys2 + (2 * q + 1) * S + 4 * pb);
          const uint32_t p4[4] = {zp.x, zp.y, zp.z, zp.w}, q4[4] = {zq.x, zq.y, zq.z, zq.w};
          const uint32_t ya[4] = {y0.x, y0.y, y0.z, y0.w}, yb[4] = {y1.x, y1.y, y1.z, y1.w};
#pragma unroll
          for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
              aI[i][j] = __dp4a(p4[i], q4[j], aI[i][j]);
              aD[i][j] = __dp2a_lo(ya[i], q4[j], aD[i][j]);
              aD[i][j] = __dp2a_hi(yb[i], q4[j], aD[i][j]);
            }
        }
      }
    }
    for (int r = 0; r < rows; r++) {
      const unsigned d = s_deg[r];
      if (bytes && (ull)max(d, 1u) * mzs <= 65535ull) continue;  // done above
      const ull b = (ull)max(d, 1u) * mz2;  // every product of this row is at most b
      const int *zr = zsm + r * S;
      if (b >= B32) {  // a row whose products may not fit 32 bits: 64-bit atomics directly (rare hubs)
        if (active) {
#pragma unroll
          for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
              const int p = 4 * pb + i, q = 4 * qb + j;
              if (p <= q && q < a.c1) {
                const ull zz = (ull)(unsigned)zr[p] * (ull)(unsigned)zr[q];
                if (zz) {
                  atomicAdd(a.GI + (int64_t)p * a.ld + q, zz);
                  atomicAdd(a.GD + (int64_t)p * a.ld + q, zz * d);
                }
              }
            }
        }
        continue;
      }
      if (run + b >= B32) {
        flush();
        run = 0;
      }
      run += b;
      if (active) {
        const int4 zp = *(const int4 *)(zr + 4 * pb);
        const int4 zq = *(const int4 *)(zr + 4 * qb);
        const uint32_t p4[4] = {(uint32_t)zp.x, (uint32_t)zp.y, (uint32_t)zp.z, (uint32_t)zp.w};
        const uint32_t q4[4] = {(uint32_t)zq.x, (uint32_t)zq.y, (uint32_t)zq.z, (uint32_t)zq.w};
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const uint32_t y = p4[i] * d;
#pragma unroll
          for (int j = 0; j < 4; j++) {
            aI[i][j] += p4[i] * q4[j];
            aD[i][j] += y * q4[j];
          }
        }
      }
    }
  }
  flush();
}

// ------------------------------------------------------------------------------------------------
// The byte path of G_I, G_D from a quad layout of Z, when every distance fits a byte.
//
// zq_pack_kernel writes Z columns [c0, c1) as Zq[(i / 4) * ldq + t]: byte j of that word is Z[4 (i / 4) + j][t],
// the four rows a dp4a consumes at once, so the Gram kernel stages a slab with plain coalesced word loads and
// no repacking.  It also keeps, per slab of ZQ_ROWS rows, the largest value of every column packed so far
// (smaxz, atomicMax over the calls of one orthogonalisation) and the largest distance and degree overall
// (maxz[0], maxz[1]).  Rows past n pack as zeros.
constexpr int ZQ_ROWS = 128;
constexpr int ZQ_QUADS = ZQ_ROWS / 4;
constexpr int ZQ_PACK_COLS = 160;  // columns staged per pass of the pack kernel (the first block of k <= 140 in one)
constexpr int ZQ_THREADS = 256;
constexpr int ZQ_GRAM_THREADS = 192;  // the Gram kernel's largest block (190 tiles at 76 columns); three per SM

// Level mode of zq_pack_kernel: thread per (row, source word), the 128 rows of a word on four whole warps (one
// chosen-bit mask per warp: no divergence).  The levels fold into NB bit planes (plane k = OR of the arrays
// whose level has bit k set) and every chosen source's distance is read off the planes; chosen sources that
// never reached the row give -1 (the exact path then refuses the basis), rows past n pack as zeros.
template <int NB>
__device__ __forceinline__ void zq_level_fill(const ZSrc &src, int64_t n, int64_t i0, const ull *s_cmask,
                                              const int *s_cmap, uint8_t (*zb)[ZQ_PACK_COLS + 4], unsigned &m) {
  constexpr int U = 8;
  const int W = src.W;
  for (int e = threadIdx.x; e < ZQ_ROWS * W; e += blockDim.x) {
    const int w = e / ZQ_ROWS, r = e - w * ZQ_ROWS;
    const int64_t i = i0 + r;
    const ull want = s_cmask[w];
    if (!want) continue;
    ull pl[NB], seen = 0;
#pragma unroll
    for (int k = 0; k < NB; k++) pl[k] = 0ull;
    if (i < n) {
      for (int L0 = 0; L0 < src.nlev; L0 += U) {
        ull x[U];
#pragma unroll
        for (int u = 0; u < U; u++)
          x[u] = L0 + u < src.nlev ? __ldg(src.lvl + ((int64_t)(L0 + u) * n + i) * W + w) & want : 0ull;
#pragma unroll
        for (int u = 0; u < U; u++) {
          seen |= x[u];
#pragma unroll
          for (int k = 0; k < NB; k++)
            if (((L0 + u) >> k) & 1) pl[k] |= x[u];
        }
      }
    }
    for (ull y = want; y; y &= y - 1) {
      const int b = __ffsll((long long)y) - 1;
      unsigned d = 0;
#pragma unroll
      for (int k = 0; k < NB; k++) d |= (unsigned)((pl[k] >> b) & 1ull) << k;
      const bool reached = (seen >> b) & 1ull;
      zb[r][s_cmap[64 * w + b]] = i >= n ? (uint8_t)0 : reached ? (uint8_t)d : (uint8_t)0xff;
      if (i < n) m = max(m, reached ? d : 0xffffffffu);
    }
  }
}

__global__ void __launch_bounds__(ZQ_THREADS) zq_pack_kernel(ZSrc src, const int64_t *off, int64_t n, int P, int c0,
                                                             int c1, int ldq, uint32_t *Zq, unsigned *smaxz,
                                                             unsigned *maxz) {
  __shared__ uint8_t zb[ZQ_ROWS][ZQ_PACK_COLS + 4];
  __shared__ unsigned s_m;
  __shared__ int s_cmap[64 * 4];  // level mode: source -> column of the pass (-1: not chosen)
  __shared__ ull s_cmask[4];      // level mode: chosen sources of the pass, per source word
  const int64_t nslab = (n + ZQ_ROWS - 1) / ZQ_ROWS;
  const int P0 = src.P0;
  for (int64_t s = blockIdx.x; s < nslab; s += gridDim.x) {
    const int64_t i0 = s * ZQ_ROWS;
    unsigned m = 0, md = 0;
    if (c0 == 0)
      for (int r = threadIdx.x; r < ZQ_ROWS; r += blockDim.x)
        if (i0 + r < n) md = max(md, (unsigned)(off[i0 + r + 1] - off[i0 + r]));
    for (int t0 = c0; t0 < c1; t0 += ZQ_PACK_COLS) {
      const int nc = min(ZQ_PACK_COLS, c1 - t0);
      __syncthreads();  // zb of the previous pass consumed
      // ones, distance (D) and padding columns -- the pass's prefix up to Z index P0 and its suffix past P (the
      // record columns lie between): consecutive threads take consecutive rows of a column; eight loads in
      // flight per thread
      constexpr int U = 8;
      const int nd1 = max(0, min(t0 + nc, P0 + 1) - t0);
      const int ts = max(t0, P + 1), nd = nd1 + max(0, t0 + nc - ts);
      for (int e0 = threadIdx.x; e0 < ZQ_ROWS * nd; e0 += U * blockDim.x) {
        int v[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int e = e0 + u * blockDim.x;
          const int jj = e / ZQ_ROWS, r = e - jj * ZQ_ROWS;
          const int t = jj < nd1 ? t0 + jj : ts + (jj - nd1);
          const int64_t i = i0 + r;
          v[u] = -2;  // nothing to store here
          if (e < ZQ_ROWS * nd) v[u] = i >= n ? 0 : (t == 0 ? 1 : (t <= P ? __ldg(src.D + (int64_t)(t - 1) * n + i) : 0));
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int e = e0 + u * blockDim.x;
          if (v[u] == -2) continue;
          const int jj = e / ZQ_ROWS, r = e - jj * ZQ_ROWS;
          const int j = jj < nd1 ? jj : (ts - t0) + (jj - nd1);
          m = max(m, (unsigned)v[u]);
          zb[r][j] = (uint8_t)v[u];
        }
      }
      if (src.lvl) {
        // level mode: thread per (row, source word), the 128 rows of a word on four whole warps (one chosen-bit
        // mask per warp: no divergence).  The levels fold into bit planes (plane k = OR of the arrays whose
        // level has bit k) and every chosen source's distance is read off the planes; chosen sources that
        // never reached the row give -1 (the exact path then refuses the basis), rows past n pack as zeros
        const int W = src.W, nb = 64 * W;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) s_cmap[b] = -1;
        if (threadIdx.x < W) s_cmask[threadIdx.x] = 0ull;
        __syncthreads();
        for (int j = threadIdx.x; j < nc; j += blockDim.x) {
          const int t = t0 + j;
          if (t >= 1 && t <= P && t > P0) {
            const int b = src.rmap[t - 1 - P0];
            s_cmap[b] = j;
            atomicOr(s_cmask + (b >> 6), 1ull << (b & 63));
          }
        }
        __syncthreads();
        const int nbits = src.nlev > 1 ? 32 - __clz(src.nlev - 1) : 0;  // planes for levels 0 .. nlev - 1 (<= 8)
        if (nbits <= 4)
          zq_level_fill<4>(src, n, i0, s_cmask, s_cmap, zb, m);
        else
          zq_level_fill<8>(src, n, i0, s_cmask, s_cmap, zb, m);
      } else
      // record columns: consecutive threads take consecutive chosen columns of a row
      for (int e0 = threadIdx.x; e0 < ZQ_ROWS * nc; e0 += U * blockDim.x) {
        int v[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int e = e0 + u * blockDim.x;
          const int r = e / nc, j = e - r * nc, t = t0 + j;
          const int64_t i = i0 + r;
          v[u] = -2;
          if (e < ZQ_ROWS * nc && t >= 1 && t <= P && t > P0)
            v[u] = i >= n ? 0 : (int)__ldg(src.R + i * src.RW + src.rmap[t - 1 - P0]) - 1;
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int e = e0 + u * blockDim.x;
          if (v[u] == -2) continue;
          const int r = e / nc, j = e - r * nc;
          m = max(m, (unsigned)v[u]);
          zb[r][j] = (uint8_t)v[u];
        }
      }
      __syncthreads();
      for (int e = threadIdx.x; e < ZQ_QUADS * nc; e += blockDim.x) {
        const int q = e / nc, j = e - q * nc;
        const uint32_t w = (uint32_t)zb[4 * q][j] | ((uint32_t)zb[4 * q + 1][j] << 8) |
                           ((uint32_t)zb[4 * q + 2][j] << 16) | ((uint32_t)zb[4 * q + 3][j] << 24);
        Zq[(s * ZQ_QUADS + q) * ldq + t0 + j] = w;
      }
    }
    if (threadIdx.x == 0) s_m = 0;
    __syncthreads();
    m = warp_max_u32(m);
    md = warp_max_u32(md);
    if ((threadIdx.x & 31) == 0) {
      atomicMax(&s_m, m);
      if (md) atomicMax(maxz + 1, md);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      atomicMax(smaxz + s, s_m);
      atomicMax(maxz, s_m);
    }
  }
}

// G_I, G_D (upper triangle, Z columns p < c1 against q in [c0, c1)) from the quad layout.  Per slab: the rows'
// degrees, the rows whose deg * (slab's largest value) exceeds 16 bits (heavy: the one-row 32-bit path, their
// bytes masked out of the quads), then the staged quads zs4 and the deg * z pairs ys (two 16-bit halves per
// word: rows 4q, 4q+1 in ys[2q], rows 4q+2, 4q+3 in ys[2q+1]).  Thread t owns the 4 x 4 tile tile_of(t):
// per quad 16 dp4a (Z^T Z) and 32 dp2a (Z^T D Z).  32-bit partial sums, flushed to the 64-bit Grams before a
// slab's bound (sum of its light rows' max(deg, 1) times the square of its largest value; below 2^32 since
// 128 * 65535 * 255 is) could carry them past 2^32.  Every sum is exact.
struct ZqArgs {
  const uint32_t *Zq;
  int ldq;
  const int64_t *off;
  int64_t n;
  int c0, c1;  // multiples of 4
  int ntiles;
  ull *GI, *GD;
  int ld;
  const unsigned *smaxz, *maxz;
};

// Copies of slab s (its quad words and its rows' offsets) into one staging buffer, as one cp.async group.
__device__ __forceinline__ void zq_stage(const ZqArgs &a, int64_t s, uint32_t *raw, int64_t *soff) {
  const int C = a.c1, c4 = C / 4;
  const int64_t i0 = s * ZQ_ROWS;
  for (int e = threadIdx.x; e < ZQ_QUADS * c4; e += blockDim.x) {
    const int q = e / c4, w = e - q * c4;
    cp_async16(raw + q * C + 4 * w, a.Zq + (s * ZQ_QUADS + q) * a.ldq + 4 * w);
  }
  for (int r = threadIdx.x; r <= ZQ_ROWS; r += blockDim.x)
    if (i0 + r <= a.n) cp_async8(soff + r, a.off + i0 + r);
  cp_async_commit();
}

__global__ void __launch_bounds__(ZQ_GRAM_THREADS, 3) zgram_q_kernel(ZqArgs a) {
  if (__ldg(a.maxz) > 255u) return;  // uniform: a distance wider than a byte, the 32-bit kernel forms them
  // raw[2][ZQ_QUADS][c1] (the slabs in flight), zs4[ZQ_QUADS][c1], ys[2 * ZQ_QUADS][c1], soff[2][ZQ_ROWS + 2]
  extern __shared__ __align__(16) uint32_t zqs[];
  __shared__ unsigned s_deg[ZQ_ROWS];  // light rows: degree; heavy rows: ~0u
  __shared__ int s_hv[ZQ_ROWS];
  __shared__ int s_nh;
  __shared__ ull s_dsum;
  const int C = a.c1;
  uint32_t *raw0 = zqs, *raw1 = zqs + ZQ_QUADS * C, *zs4 = zqs + 2 * ZQ_QUADS * C, *ys = zs4 + ZQ_QUADS * C;
  int64_t *soff0 = (int64_t *)(ys + 2 * ZQ_QUADS * C), *soff1 = soff0 + (ZQ_ROWS + 2);
  const int t = blockIdx.y * blockDim.x + threadIdx.x;
  int pb, qb;
  tile_of(t, a.c0 / 4, a.c1 / 4, pb, qb);
  const bool active = t < a.ntiles && pb >= 0;
  uint32_t aI[4][4], aD[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) aI[i][j] = aD[i][j] = 0;
  auto flush = [&]() {
    if (!active) return;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int p = 4 * pb + i, q = 4 * qb + j;
        if (p <= q) {
          if (aI[i][j]) atomicAdd(a.GI + (int64_t)p * a.ld + q, (ull)aI[i][j]);
          if (aD[i][j]) atomicAdd(a.GD + (int64_t)p * a.ld + q, (ull)aD[i][j]);
        }
        aI[i][j] = aD[i][j] = 0;
      }
  };
  const int64_t nslab = (a.n + ZQ_ROWS - 1) / ZQ_ROWS;
  ull run = 0;  // bound on every partial sum since the last flush (uniform across the block)
  if ((int64_t)blockIdx.x < nslab) zq_stage(a, blockIdx.x, raw0, soff0);
  int buf = 0;
  for (int64_t s = blockIdx.x; s < nslab; s += gridDim.x, buf ^= 1) {
    const int64_t i0 = s * ZQ_ROWS;
    uint32_t *raw = buf ? raw1 : raw0;
    const int64_t *soff = buf ? soff1 : soff0;
    cp_async_wait<0>();  // this thread's copies of slab s
    const unsigned mz = __ldg(a.smaxz + s);
    const ull mz2 = (ull)mz * mz;
    __syncthreads();  // slab s visible; the last slab (its buffer, zs4, ys, s_deg, s_hv) consumed
    // the next slab's copies fly while this one is transformed and multiplied
    if (s + gridDim.x < nslab) zq_stage(a, s + gridDim.x, buf ? raw0 : raw1, buf ? soff0 : soff1);
    if (threadIdx.x == 0) {
      s_nh = 0;
      s_dsum = 0;
    }
    __syncthreads();
    ull dsum = 0;
    for (int r = threadIdx.x; r < ZQ_ROWS; r += blockDim.x) {
      const int64_t i = i0 + r;
      const unsigned d = i < a.n ? (unsigned)(soff[r + 1] - soff[r]) : 0u;
      const bool light = (ull)max(d, 1u) * mz <= 65535ull;
      s_deg[r] = light ? d : ~0u;
      if (!light) s_hv[atomicAdd(&s_nh, 1)] = r;
      else if (i < a.n) dsum += max(d, 1u);
    }
    dsum = warp_sum(dsum);
    if ((threadIdx.x & 31) == 0 && dsum) atomicAdd(&s_dsum, dsum);
    __syncthreads();
    for (int e = threadIdx.x; e < ZQ_QUADS * C; e += blockDim.x) {
      const int q = e / C;
      const uint32_t w = raw[e];
      uint32_t mask = 0, lo = 0, hi = 0;
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const unsigned d = s_deg[4 * q + j];
        if (d != ~0u) {
          mask |= 0xffu << (8 * j);
          const uint32_t y = ((w >> (8 * j)) & 0xffu) * d;  // <= 65535
          if (j < 2) lo |= y << (16 * j);
          else hi |= y << (16 * (j - 2));
        }
      }
      const int col = e - q * C;
      zs4[e] = w & mask;
      ys[(2 * q) * C + col] = lo;
      ys[(2 * q + 1) * C + col] = hi;
    }
    __syncthreads();
    const ull b = s_dsum * mz2;
    if (run + b >= B32) {
      flush();
      run = 0;
    }
    run += b;
    if (active) {
#pragma unroll 1
      for (int q = 0; q < ZQ_QUADS; q++) {
        const uint4 zp = *(const uint4 *)(zs4 + q * C + 4 * pb);
        const uint4 zq = *(const uint4 *)(zs4 + q * C + 4 * qb);
        const uint4 y0 = *(const uint4 *)(ys + (2 * q) * C + 4 * pb);
        const uint4 y1 = *(const uint4 *)(ys + (2 * q + 1) * C + 4 * pb);
        const uint32_t p4[4] = {zp.x, zp.y, zp.z, zp.w}, q4[4] = {zq.x, zq.y, zq.z, zq.w};
        const uint32_t ya[4] = {y0.x, y0.y, y0.z, y0.w}, yb[4] = {y1.x, y1.y, y1.z, y1.w};
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < 4; j++) {
            aI[i][j] = __dp4a(p4[i], q4[j], aI[i][j]);
            aD[i][j] = __dp2a_lo(ya[i], q4[j], aD[i][j]);
            aD[i][j] = __dp2a_hi(yb[i], q4[j], aD[i][j]);
          }
      }
    }
    // heavy rows of the slab, one at a time (their bytes from the staged words, their degree from the offsets)
    const int nh = s_nh;
    for (int h = 0; h < nh; h++) {
      const int r = s_hv[h];
      const unsigned d = (unsigned)(soff[r + 1] - soff[r]);
      const ull bh = (ull)max(d, 1u) * mz2;  // every product of this row is at most bh
      uint32_t p4[4] = {0, 0, 0, 0}, q4[4] = {0, 0, 0, 0};
      if (active) {
        const int sh = 8 * (r & 3);
        const uint32_t *rq = raw + (r >> 2) * C;
#pragma unroll
        for (int ii = 0; ii < 4; ii++) {
          p4[ii] = (rq[4 * pb + ii] >> sh) & 0xffu;
          q4[ii] = (rq[4 * qb + ii] >> sh) & 0xffu;
        }
      }
      if (bh >= B32) {  // products that may not fit 32 bits: 64-bit atomics directly (rare hubs)
        if (active) {
#pragma unroll
          for (int ii = 0; ii < 4; ii++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
              const int p = 4 * pb + ii, q = 4 * qb + j;
              const ull zz = (ull)p4[ii] * q4[j];
              if (p <= q && zz) {
                atomicAdd(a.GI + (int64_t)p * a.ld + q, zz);
                atomicAdd(a.GD + (int64_t)p * a.ld + q, zz * d);
              }
            }
        }
        continue;
      }
      if (run + bh >= B32) {
        flush();
        run = 0;
      }
      run += bh;
      if (active) {
#pragma unroll
        for (int ii = 0; ii < 4; ii++) {
          const uint32_t y = p4[ii] * d;
#pragma unroll
          for (int j = 0; j < 4; j++) {
            aI[ii][j] += p4[ii] * q4[j];
            aD[ii][j] += y * q4[j];
          }
        }
      }
    }
  }
  flush();
}

// Z_acc (row-major bytes, n x kp) from the quad layout: thread per (quad, 16 accepted columns); row 4q + r,
// column t is byte r of Zq[q * ldq + acc_idx[t]]; columns t >= k are zero.
__global__ void pack_from_zq_kernel(const uint32_t *Zq, int ldq, int64_t n, const int *acc_idx, int k, int kp,
                                    uint8_t *Z) {
  __shared__ int s_idx[PHDE_MAX_K];
  for (int t = threadIdx.x; t < kp; t += blockDim.x) s_idx[t] = t < k ? acc_idx[t] : -1;
  __syncthreads();
  const int ng = kp / 16;
  const int64_t nq = (n + 3) / 4;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nq * ng; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = e / ng;
    const int g = (int)(e - q * ng);
    uint32_t w[16];
#pragma unroll
    for (int j = 0; j < 16; j++) {
      const int z = s_idx[16 * g + j];
      w[j] = z >= 0 ? __ldg(Zq + q * ldq + z) : 0u;
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int64_t i = 4 * q + r;
      if (i >= n) break;
      const unsigned sel = (unsigned)r | ((unsigned)(r + 4) << 4);  // byte r of x, byte r of y
      uint32_t o[4];
#pragma unroll
      for (int c = 0; c < 4; c++)
        o[c] = __byte_perm(__byte_perm(w[4 * c], w[4 * c + 1], sel), __byte_perm(w[4 * c + 2], w[4 * c + 3], sel),
                           0x5410);
      *(uint4 *)(Z + i * kp + 16 * g) = make_uint4(o[0], o[1], o[2], o[3]);
    }
  }
}

// ------------------------------------------------------------------------------------------------
// The reference's candidate loop (ParHDE.cpp:190-285) on coefficient vectors over Z.  Accepted vector q
// is S_q = Z A[q][*] (A[q][i] = 0 for i > acc_idx[q]); the candidate with Z index r is x = d_r / ||d_r||,
// i.e. the vector inv * e_r with inv = 1 / sqrt(G_I[r][r]).  Per candidate:
//   num_q = <x, D S_q> = inv * sum_i G_D[r][i] A[q][i],   den_q = <S_q, D S_q> (kept from acceptance)
//   c_q = num_q * (1 / den_q); the constant column u0 = e_0 / sqrt(n) likewise
//   t = inv e_r - sum c_q A[q] - c_0 e_0 / sqrt(n),   ||x - sum c q||^2 = t^T G_I t
//   discard when the norm is below 1e-3, else A[nacc] = t * (1 / norm).
struct CoefArgs {
  const ull *GI, *GD;
  int ld;
  int nc;         // > 0: the leading nc x nc blocks of G_I and G_D are staged in shared memory as FP64
  int64_t n;
  int r_end;      // examine Z indices [state[3], r_end)
  int k;
  double *A;      // [k][ld]
  double *den;    // [k]
  int *acc_idx;   // [k]
  int *state;     // [0] accepted, [1] discarded, [2] examined, [3] next Z index
  double *dlog;   // [P]: norm of each discarded candidate (by candidate index = Z index - 1); NaN otherwise
  int sa;         // the accepted rows of A are staged in shared memory too
  // [0] largest distance, [1] largest degree (the Gram kernels': launched before this one with no host
  // round trip, so the range check is repeated here); nmax = max(nnz, n)
  const unsigned *maxz;
  double nmax;
};

// GB300 issues FP64 at two lanes per clock per SM: a warp-wide FP64 instruction holds the pipe for 16 clocks
// whatever it computes, so the loop keeps FP64 work in full warps and leaves the scalars (square roots,
// reciprocals, the final sums) to one thread, broadcast through shared memory.
__global__ void __launch_bounds__(CF_THREADS, 1) coef_kernel(CoefArgs a) {
  // rr[ld], gdr[ld], cq[k], rden[k], part[CF_THREADS], then (nc > 0) GIs[nc][nc], GDs[nc][nc], then (sa) As[k][ld]
  extern __shared__ double cs[];
  __shared__ int s_idx[PHDE_MAX_K];
  __shared__ double s_inv, s_c0, s_nrm;
  {  // out of the exact path's range (the host reads the same words and takes the FP64 vector kernels)
    const double mz = (double)__ldg(a.maxz), md = (double)__ldg(a.maxz + 1);
    if (mz > 65535.0 || a.nmax * mz * mz >= 9007199254740992.0 || md * mz >= 2147483647.0) return;
  }
  const int ld = a.ld;
  double *rr = cs, *gdr = cs + ld, *cq = cs + 2 * ld, *rden = cq + a.k, *part = rden + a.k;
  double *GIs = part + CF_THREADS, *GDs = GIs + (size_t)a.nc * a.nc;
  const int nc = a.nc;
  for (int e = threadIdx.x; e < nc * nc; e += CF_THREADS) {
    const int i = e / nc, j = e - i * nc;
    GIs[e] = gsym(a.GI, ld, i, j);
    GDs[e] = gsym(a.GD, ld, i, j);
  }
  int nacc = a.state[0], ndisc = a.state[1], nexam = a.state[2];
  // the accepted coefficient rows (zero past each row's own Z index), staged when they fit
  double *As = a.sa ? GDs + (size_t)nc * nc : a.A;
  if (a.sa)
    for (int e = threadIdx.x; e < a.k * ld; e += CF_THREADS) As[e] = e < nacc * ld ? a.A[e] : 0.0;
  for (int q = threadIdx.x; q < nacc; q += CF_THREADS) {
    s_idx[q] = a.acc_idx[q];
    rden[q] = 1.0 / a.den[q];
  }
  __syncthreads();
  // G_I / G_D entry (i, j): from shared memory when staged (every index the loop reads is below r_end <= nc)
  auto gi = [&](int i, int j) { return nc ? GIs[i * nc + j] : gsym(a.GI, ld, i, j); };
  auto gd = [&](int i, int j) { return nc ? GDs[i * nc + j] : gsym(a.GD, ld, i, j); };
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double rsn = 1.0 / sqrt((double)a.n);
  const double den0 = gsym(a.GD, ld, 0, 0) * rsn * rsn;  // <u0, D u0> = nnz / n
  int r = a.state[3];
  // the per-thread partials in part[] summed by warp 0 in a fixed order; the total lands in thread 0
  auto total0 = [&](double v) -> double {
    part[threadIdx.x] = v;
    __syncthreads();
    double t = 0;
    if (warp == 0) {
      for (int w = lane; w < CF_THREADS; w += 32) t += part[w];
      t = warp_sum(t);
    }
    return t;
  };
  // rr^T G rr over the upper triangle: thread (p, sub) takes the rows p and r - p (the middle row once), so
  // every thread has r + 1 terms, and the columns j > i with j = i + 1 + sub (mod 4)
  auto quad = [&](auto g) -> double {
    const int np = (r + 2) / 2;
    double s = 0;
    for (int t = threadIdx.x; t < 4 * np; t += CF_THREADS) {
      const int p = t >> 2, sub = t & 3;
      for (int h = 0; h < 2; h++) {
        const int i = h ? r - p : p;
        if (h && i == p) break;
        double acc = 0;
        for (int j = i + 1 + sub; j <= r; j += 4) acc = fma(g(i, j), rr[j], acc);
        const double ri = rr[i];
        s += fma(2.0 * ri, acc, sub == 0 ? ri * g(i, i) * ri : 0.0);
      }
    }
    return total0(s);
  };
  for (; r < a.r_end && nacc < a.k; r++) {
    __syncthreads();
    for (int i = threadIdx.x; i <= r; i += CF_THREADS) gdr[i] = gd(i, r);
    if (threadIdx.x == 0) {
      const double inv = 1.0 / sqrt(gi(r, r));
      s_inv = inv;
      s_c0 = (inv * gd(0, r) * rsn) * (1.0 / den0);
    }
    __syncthreads();
    const double inv = s_inv, c0 = s_c0;
    // cq[q] = inv <G_D[r], A[q]> / den[q]: four threads per accepted vector
    for (int base = 0; base < nacc; base += CF_THREADS / 4) {
      const int q = base + (threadIdx.x >> 2), sub = threadIdx.x & 3;
      double v = 0;
      if (q < nacc) {
        const int top = s_idx[q];
        const double *Aq = As + (int64_t)q * ld;
        for (int i = sub; i <= top; i += 4) v = fma(gdr[i], Aq[i], v);
      }
      v += __shfl_xor_sync(PHDE_FULL_MASK, v, 1);
      v += __shfl_xor_sync(PHDE_FULL_MASK, v, 2);
      if (q < nacc && sub == 0) cq[q] = (inv * v) * rden[q];
    }
    __syncthreads();
    // rr = inv e_r - c0 e_0 / sqrt(n) - sum_q cq[q] A[q]: four threads per index i, the terms q of accepted index
    // >= i (the accepted indices increase with q: a binary search finds the first)
    for (int base = 0; base <= r; base += CF_THREADS / 4) {
      const int i = base + (threadIdx.x >> 2), sub = threadIdx.x & 3;
      double v = 0;
      if (i <= r) {
        int lo = 0, hi = nacc;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (s_idx[mid] < i) lo = mid + 1;
          else hi = mid;
        }
        for (int q = lo + sub; q < nacc; q += 4) v = fma(cq[q], As[(int64_t)q * ld + i], v);
      }
      v += __shfl_xor_sync(PHDE_FULL_MASK, v, 1);
      v += __shfl_xor_sync(PHDE_FULL_MASK, v, 2);
      if (i <= r && sub == 0) {
        double b = i == r ? inv : 0.0;
        if (i == 0) b -= c0 * rsn;
        rr[i] = b - v;
      }
    }
    __syncthreads();
    const double n2 = quad(gi);
    if (threadIdx.x == 0) s_nrm = sqrt(fmax(n2, 0.0));
    __syncthreads();
    const double nrm = s_nrm;
    nexam++;
    if (nrm < 0.001) {
      if (threadIdx.x == 0) a.dlog[r - 1] = nrm;
      ndisc++;
      continue;
    }
    if (threadIdx.x == 0) s_inv = 1.0 / nrm;
    __syncthreads();
    const double sc = s_inv;
    double *An = a.A + (int64_t)nacc * ld;
    for (int i = threadIdx.x; i <= r; i += CF_THREADS) {
      const double v = rr[i] * sc;
      rr[i] = v;
      An[i] = v;
      if (a.sa) As[(int64_t)nacc * ld + i] = v;
    }
    __syncthreads();
    const double dsum = quad(gd);
    if (threadIdx.x == 0) {
      a.den[nacc] = dsum;
      a.acc_idx[nacc] = r;
      rden[nacc] = 1.0 / dsum;
    }
    s_idx[nacc] = r;  // every thread writes the same value
    nacc++;
  }
  if (threadIdx.x == 0) {
    a.state[0] = nacc;
    a.state[1] = ndisc;
    a.state[2] = nexam;
    a.state[3] = r;
  }
}

// ------------------------------------------------------------------------------------------------
// Z_acc[i][t] = D[acc_idx[t] - 1][i] for t < k, 0 for k <= t < kp; 16 bytes per store.
template <typename T>
__global__ void pack_kernel(ZSrc src, int64_t n, const int *acc_idx, int k, int kp, T *Z) {
  __shared__ int s_col[PHDE_MAX_K];
  __shared__ bool s_rec[PHDE_MAX_K];
  for (int t = threadIdx.x; t < kp; t += blockDim.x) {
    const int z = t < k ? acc_idx[t] : 0;  // Z index of accepted column t
    s_rec[t] = z > src.P0;
    s_col[t] = t >= k ? -1 : (z > src.P0 ? src.rmap[z - 1 - src.P0] : z - 1);
  }
  __syncthreads();
  constexpr int V = 16 / sizeof(T);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    for (int t0 = 0; t0 < kp; t0 += V) {
      union {
        uint4 u;
        T v[V];
      } w;
#pragma unroll
      for (int j = 0; j < V; j++) {
        const int col = s_col[t0 + j];
        w.v[j] = col < 0 ? (T)0 : s_rec[t0 + j] ? (T)(src.R[i * src.RW + col] - 1) : (T)src.D[(int64_t)col * n + i];
      }
      *(uint4 *)(Z + i * kp + t0) = w.u;
    }
  }
}

// ------------------------------------------------------------------------------------------------
// Z_acc^T L Z_acc = Z_acc^T D Z_acc - Z_acc^T A Z_acc, the first term read off G_D (the candidates' exact
// Z^T D Z), the second from each undirected edge once: with T2 = sum over items of z (x) u, item u of row i
// having z = Z_acc[i] and u = 2 * (sum of Z_acc[j] over its edges with j > i) + (its self-loops) * z,
// Z^T A Z = (T2 + T2^T) / 2 for a symmetric adjacency (lfin_kernel forms the difference).  Items: rows
// 0..n-1 (rows of degree > heavy contribute nothing as rows) and the heavy rows' chunks of at most `chunk`
// (<= 256) edges.  Only half the neighbour rows are gathered, at the price of the full (not symmetric) T2.
//
// Gathers: a row of Z_acc is KP values; LPR lanes read it with one 16-byte load each, so a warp is
// G = 32 / LPR lane groups, each on its own neighbour, and one load instruction fetches G neighbour rows.
// Sums: for uint8 rows two columns share a 32-bit register as 16-bit halves (bytes moved apart by one byte
// permute; an item has at most 256 neighbours of at most 255, so no half ever carries into the next, also
// after the groups are added together); uint16 rows sum each column in its own register.
template <typename T>
struct Sum16 {  // the sums of one 16-byte slice of a row: 16 uint8 or 8 uint16 columns, in 8 registers
  uint32_t s[8];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int i = 0; i < 8; i++) s[i] = 0;
  }
  __device__ __forceinline__ void add(const uint4 &v) {
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int i = 0; i < 4; i++) {
      if (sizeof(T) == 1) {
        s[2 * i] += __byte_perm(w[i], 0u, 0x4140);
        s[2 * i + 1] += __byte_perm(w[i], 0u, 0x4342);
      } else {
        s[2 * i] += w[i] & 0xffffu;
        s[2 * i + 1] += w[i] >> 16;
      }
    }
  }
  __device__ __forceinline__ void add_from(int lane_mask) {  // add the sums of lane ^ lane_mask
#pragma unroll
    for (int i = 0; i < 8; i++) s[i] += __shfl_xor_sync(PHDE_FULL_MASK, s[i], lane_mask);
  }
  __device__ __forceinline__ int get(int c) const {  // column c of the slice
    if (sizeof(T) == 1) return (int)((s[c / 2] >> (16 * (c % 2))) & 0xffffu);
    return (int)s[c];
  }
};

template <typename T>
__device__ __forceinline__ int slice_val(const uint4 &v, int c) {
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
  if (sizeof(T) == 1) return (int)((w[c / 4] >> (8 * (c % 4))) & 0xffu);
  return (int)((w[c / 2] >> (16 * (c % 2))) & 0xffffu);
}

struct LgArgs {
  const int64_t *off;
  const uint32_t *adj;
  int64_t n;
  const void *Z;  // row-major n x kp
  int kp;
  int64_t heavy;  // rows of degree > heavy are done as chunks
  const int64_t *chunk_row, *chunk_e0;
  int64_t nchunks, chunk;
  ull *GL;        // T2 [kp x kp], every entry (p, q) at p * kp + q, two's complement
  int ntiles;
};

template <typename T, int KP, int TS>
__global__ void __launch_bounds__(LG_THREADS, KP == 64 ? 4 : 2) lgram_kernel(LgArgs a) {
  constexpr int V = 16 / (int)sizeof(T);  // columns per 16-byte slice
  constexpr int LPR = KP / V;             // lanes per row
  constexpr int G = 32 / LPR;             // neighbour rows per load instruction
  constexpr int CPL = V / G;              // columns of a slice each lane finishes (2, 4 or 8)
  constexpr int RPL = sizeof(T) == 1 ? CPL / 2 : CPL;  // sum registers those columns sit in
  constexpr int SL = KP + 4;
  // uint8 rows (PK): the items' z bytes and neighbour sums s (< 2^16: at most 256 neighbours of at most 255) are
  // staged four items to a word -- Zb[quad][col] = the z bytes of items 4 quad .. +3, Sh[quad][h][col] = the s
  // of items 4 quad + 2h, +1 as 16-bit halves -- and the outer products go by dp2a, four items in two
  // instructions; T = sum z (x) s is accumulated and flushed doubled, self-loops (c z (x) z) go to T2 directly.
  // uint16 rows: zs[LG_ITEMS][SL], rs[LG_ITEMS][SL] as ints, u = 2 s + c z, one IMAD per item.
  constexpr bool PK = sizeof(T) == 1;
  extern __shared__ int lsm[];
  __shared__ ull s_bnd[LG_ITEMS];
  __shared__ int s_self[LG_ITEMS];
  __shared__ int s_list[LG_ITEMS];  // phase 2 items of the slab
  __shared__ int s_next, s_nlist, s_lnext;
  int *zs = lsm, *rs = lsm + LG_ITEMS * SL;
  // Zb and Sh rows are ZR = KP + 4 words apart: the rows of a store instruction's items fall in different banks
  constexpr int ZR = KP + 4;
  uint8_t *Zb = (uint8_t *)lsm;
  uint16_t *Sh = (uint16_t *)(Zb + (LG_ITEMS / 4) * ZR * 4);
  const int lane = threadIdx.x & 31;
  const int gi = lane / LPR, pi = lane % LPR;  // lane group (neighbour) and slice within the row
  const T *Z = (const T *)a.Z;
  const int t = blockIdx.y * LG_THREADS + threadIdx.x;
  constexpr int NBK = KP / TS;
  const int pb = t / NBK, qb = t - (t / NBK) * NBK;  // every tile of the (not symmetric) T2
  const bool active = t < a.ntiles;
  uint32_t acc[TS][TS];  // PK: T (unsigned); uint16 rows: T2 (signed, two's complement)
#pragma unroll
  for (int i = 0; i < TS; i++)
#pragma unroll
    for (int j = 0; j < TS; j++) acc[i][j] = 0;
  auto flush = [&]() {
    if (!active) return;
#pragma unroll
    for (int i = 0; i < TS; i++)
#pragma unroll
      for (int j = 0; j < TS; j++) {
        const int p = TS * pb + i, q = TS * qb + j;
        if (acc[i][j])
          atomicAdd(a.GL + (int64_t)p * KP + q, PK ? 2ull * (ull)acc[i][j] : (ull)(long long)(int)acc[i][j]);
        acc[i][j] = 0;
      }
  };
  const int64_t items = a.n + a.nchunks;
  const int64_t nslab = (items + LG_ITEMS - 1) / LG_ITEMS;
  ull run = 0;
  for (int64_t s = blockIdx.x; s < nslab; s += gridDim.x) {
    const int64_t u0 = s * LG_ITEMS;
    __syncthreads();  // previous slab consumed
    if (threadIdx.x == 0) s_next = s_nlist = s_lnext = 0;
    __syncthreads();
    // phase 1: the warps take G of the slab's items at a time; a light row (at most LG_LIGHT neighbours) is
    // done by its LPR-lane group alone (lane pi sums slice pi of the neighbours' rows, no cross-group
    // reduction), as are the empty slots; the other items are listed for phase 2
    for (;;) {
      int sbase = 0;
      if (lane == 0) sbase = atomicAdd(&s_next, G);
      sbase = __shfl_sync(PHDE_FULL_MASK, sbase, 0);
      if (sbase >= LG_ITEMS) break;
      const int gslot = sbase + gi;  // LG_ITEMS is a multiple of G
      const int64_t u = u0 + gslot;
      int64_t row = -1, e0 = 0, e1 = 0;
      bool listed = false;
      if (u < a.n) {
        e0 = a.off[u];
        e1 = a.off[u + 1];
        if (e1 - e0 <= LG_LIGHT)
          row = u;
        else if (e1 - e0 <= a.heavy)
          listed = true;  // (heavier rows are done as chunks: their own slot stays empty)
      } else if (u < items) {
        listed = true;
      }
      unsigned zm = 0, rm = 0;
      if (!listed) {
        Sum16<T> nb;
        nb.zero();
        int selfc = 0;
        uint4 own = make_uint4(0, 0, 0, 0);
        if (row >= 0) {
          const uint64_t keep = l2_policy_evict_last(), stream = l2_policy_evict_first();
          for (int64_t e = e0; e < e1; e += 4) {  // four neighbour rows in flight per lane
            int64_t vv[4];
            uint4 x[4];
#pragma unroll
            for (int j = 0; j < 4; j++) vv[j] = e + j < e1 ? (int64_t)ld_nc_hint(a.adj + e + j, stream) : -1;
#pragma unroll
            for (int j = 0; j < 4; j++) {
              x[j] = make_uint4(0, 0, 0, 0);
              if (vv[j] > row) x[j] = ld_nc_hint16((const uint4 *)(Z + vv[j] * KP) + pi, keep);
              selfc += vv[j] == row;
            }
#pragma unroll
            for (int j = 0; j < 4; j++) nb.add(x[j]);
          }
          own = __ldg((const uint4 *)(Z + row * KP) + pi);
        }
        if constexpr (PK) {
#pragma unroll
          for (int c = 0; c < V; c++) {
            const int col = pi * V + c;
            const int z = slice_val<T>(own, c), sum = nb.get(c);
            Zb[((gslot >> 2) * ZR + col) * 4 + (gslot & 3)] = (uint8_t)z;
            Sh[(((gslot >> 2) * 2 + ((gslot & 3) >> 1)) * ZR + col) * 2 + (gslot & 1)] = (uint16_t)sum;
            zm = max(zm, (unsigned)z);
            rm = max(rm, (unsigned)sum);
          }
          if (pi == 0) s_self[gslot] = selfc;
        } else {
          int *zd = zs + gslot * SL + pi * V, *rd = rs + gslot * SL + pi * V;
#pragma unroll
          for (int c = 0; c < V; c += 2) {
            const int z0 = slice_val<T>(own, c), z1 = slice_val<T>(own, c + 1);
            const int r0 = 2 * nb.get(c) + selfc * z0, r1 = 2 * nb.get(c + 1) + selfc * z1;
            *(int2 *)(zd + c) = make_int2(z0, z1);
            *(int2 *)(rd + c) = make_int2(r0, r1);
            zm = max(zm, (unsigned)max(z0, z1));
            rm = max(rm, (unsigned)max(abs(r0), abs(r1)));
          }
        }
      }
#pragma unroll
      for (int m = 1; m < LPR; m <<= 1) {  // the group's maxima
        zm = max(zm, __shfl_xor_sync(PHDE_FULL_MASK, zm, m));
        rm = max(rm, __shfl_xor_sync(PHDE_FULL_MASK, rm, m));
      }
      if (pi == 0) {
        if (listed)
          s_list[atomicAdd(&s_nlist, 1)] = gslot;
        else
          s_bnd[gslot] = (ull)zm * (ull)rm;
      }
    }
    __syncthreads();
    // phase 2: the listed items (longer rows, hub-row chunks), one at a time per warp, all lanes on one row
    const int nlist = s_nlist;
    for (;;) {
      int li = 0;
      if (lane == 0) li = atomicAdd(&s_lnext, 1);
      li = __shfl_sync(PHDE_FULL_MASK, li, 0);
      if (li >= nlist) break;
      const int slot = s_list[li];
      const int64_t u = u0 + slot;
      int64_t row = -1, e0 = 0, e1 = 0;
      if (u < a.n) {
        e0 = a.off[u];
        e1 = a.off[u + 1];
        if (e1 - e0 <= a.heavy) row = u;
      } else if (u < items) {
        const int64_t c = u - a.n;
        row = a.chunk_row[c];
        e0 = a.chunk_e0[c];
        e1 = min(e0 + a.chunk, a.off[row + 1]);
      }
      unsigned zm = 0, rm = 0;
      if (row >= 0) {
        Sum16<T> nb;
        nb.zero();
        // the packed rows are gathered again and again (evict-last in L2), the adjacency streams by once
        const uint64_t keep = l2_policy_evict_last(), stream = l2_policy_evict_first();
        // only the neighbours above the row: every undirected edge once (ZtAZ = T + T^T, T = sum_i z_i (x)
        // sum_{j > i} z_j); self-loops counted (their z_i z_i^T goes in once)
        int selfc = 0;
        int64_t e = e0 + gi;
        for (; e + G < e1; e += 2 * G) {
          const int64_t v0 = ld_nc_hint(a.adj + e, stream), v1 = ld_nc_hint(a.adj + e + G, stream);
          uint4 x0 = make_uint4(0, 0, 0, 0), x1 = make_uint4(0, 0, 0, 0);
          if (v0 > row) x0 = ld_nc_hint16((const uint4 *)(Z + v0 * KP) + pi, keep);
          if (v1 > row) x1 = ld_nc_hint16((const uint4 *)(Z + v1 * KP) + pi, keep);
          selfc += (v0 == row) + (v1 == row);
          nb.add(x0);
          nb.add(x1);
        }
        if (e < e1) {
          const int64_t v0 = ld_nc_hint(a.adj + e, stream);
          if (v0 > row) nb.add(ld_nc_hint16((const uint4 *)(Z + v0 * KP) + pi, keep));
          selfc += v0 == row;
        }
#pragma unroll
        for (int m = LPR; m < 32; m <<= 1) {
          nb.add_from(m);
          selfc += __shfl_xor_sync(PHDE_FULL_MASK, selfc, m);
        }
        // every group of the warp now holds the row's sums: lane (gi, pi) finishes columns gi * CPL .. + CPL of
        // slice pi (sum registers gi * RPL .. + RPL, picked by selects: no indexed register arrays)
        const uint4 own = __ldg((const uint4 *)(Z + row * KP) + pi);
        int zi[CPL], r[CPL];
#pragma unroll
        for (int k2 = 0; k2 < RPL; k2++) {
          const int want = gi * RPL + k2;
          uint32_t sv = nb.s[0];
#pragma unroll
          for (int j = 1; j < 8; j++) sv = want == j ? nb.s[j] : sv;
          // the own row's word holding these columns
          const int c0 = gi * CPL + k2 * (CPL / RPL);
          const int wi = sizeof(T) == 1 ? c0 >> 2 : c0 >> 1;
          const uint32_t ow = wi == 0 ? own.x : wi == 1 ? own.y : wi == 2 ? own.z : own.w;
#pragma unroll
          for (int h = 0; h < CPL / RPL; h++) {
            const int c = k2 * (CPL / RPL) + h;
            const int z = sizeof(T) == 1 ? (int)((ow >> (8 * ((c0 + h) & 3))) & 0xffu)
                                         : (int)((ow >> (16 * ((c0 + h) & 1))) & 0xffffu);
            const int sum = sizeof(T) == 1 ? (int)((sv >> (16 * h)) & 0xffffu) : (int)sv;
            zi[c] = z;
            // uint8 rows stage s itself; uint16 rows the row's u = 2 sum_{j > i} z_j + (self-loops) z_i
            r[c] = PK ? sum : 2 * sum + selfc * z;
            zm = max(zm, (unsigned)z);
            rm = max(rm, (unsigned)abs(r[c]));
          }
        }
        if constexpr (PK) {
#pragma unroll
          for (int c = 0; c < CPL; c++) {
            const int col = pi * V + gi * CPL + c;
            Zb[((slot >> 2) * ZR + col) * 4 + (slot & 3)] = (uint8_t)zi[c];
            Sh[(((slot >> 2) * 2 + ((slot & 3) >> 1)) * ZR + col) * 2 + (slot & 1)] = (uint16_t)r[c];
          }
          if (lane == 0) s_self[slot] = selfc;
        } else {
          int *zd = zs + slot * SL + pi * V + gi * CPL, *rd = rs + slot * SL + pi * V + gi * CPL;
#pragma unroll
          for (int c = 0; c < CPL; c += 2) {
            *(int2 *)(zd + c) = make_int2(zi[c], zi[c + 1]);
            *(int2 *)(rd + c) = make_int2(r[c], r[c + 1]);
          }
        }
      } else {
        if constexpr (PK) {
#pragma unroll
          for (int c = 0; c < CPL; c++) {
            const int col = pi * V + gi * CPL + c;
            Zb[((slot >> 2) * ZR + col) * 4 + (slot & 3)] = 0;
            Sh[(((slot >> 2) * 2 + ((slot & 3) >> 1)) * ZR + col) * 2 + (slot & 1)] = 0;
          }
          if (lane == 0) s_self[slot] = 0;
        } else {
          int *zd = zs + slot * SL + pi * V + gi * CPL, *rd = rs + slot * SL + pi * V + gi * CPL;
#pragma unroll
          for (int c = 0; c < CPL; c += 2) {
            *(int2 *)(zd + c) = make_int2(0, 0);
            *(int2 *)(rd + c) = make_int2(0, 0);
          }
        }
      }
      zm = __reduce_max_sync(PHDE_FULL_MASK, zm);
      rm = __reduce_max_sync(PHDE_FULL_MASK, rm);
      if (lane == 0) s_bnd[slot] = (ull)zm * (ull)rm;
    }
    __syncthreads();
    const int nit = active ? (int)min((int64_t)LG_ITEMS, items - u0) : 0;  // threads without a tile skip it
    if constexpr (PK) {
      const uint32_t *Zw = (const uint32_t *)Zb, *Sw = (const uint32_t *)Sh;
      for (int q4 = 0; q4 < (nit + 3) / 4; q4++) {
        // every product is at most z_max * s_max of its item (< 2^24), the quad's sum below 2^26
        const ull b = s_bnd[4 * q4] + s_bnd[4 * q4 + 1] + s_bnd[4 * q4 + 2] + s_bnd[4 * q4 + 3];
        if (b == 0) continue;
        if (run + b >= B32) {
          flush();
          run = 0;
        }
        run += b;
        uint32_t zq[TS], alo[TS], ahi[TS];
#pragma unroll
        for (int i = 0; i < TS; i += 4) {
          const uint4 x = *(const uint4 *)(Zw + q4 * ZR + TS * pb + i);
          const uint4 y0 = *(const uint4 *)(Sw + (2 * q4) * ZR + TS * qb + i);
          const uint4 y1 = *(const uint4 *)(Sw + (2 * q4 + 1) * ZR + TS * qb + i);
          zq[i] = x.x, zq[i + 1] = x.y, zq[i + 2] = x.z, zq[i + 3] = x.w;
          alo[i] = y0.x, alo[i + 1] = y0.y, alo[i + 2] = y0.z, alo[i + 3] = y0.w;
          ahi[i] = y1.x, ahi[i + 1] = y1.y, ahi[i + 2] = y1.z, ahi[i + 3] = y1.w;
        }
#pragma unroll
        for (int i = 0; i < TS; i++)
#pragma unroll
          for (int j = 0; j < TS; j++) {
            acc[i][j] = __dp2a_lo(alo[j], zq[i], acc[i][j]);
            acc[i][j] = __dp2a_hi(ahi[j], zq[i], acc[i][j]);
          }
      }
      // self-loops (rare): c z (x) z straight into T2
      for (int slot = 0; slot < nit; slot++) {
        const int c = s_self[slot];
        if (c == 0) continue;
#pragma unroll
        for (int i = 0; i < TS; i++)
#pragma unroll
          for (int j = 0; j < TS; j++) {
            const int p = TS * pb + i, q = TS * qb + j;
            const ull v = (ull)c * Zb[((slot >> 2) * ZR + p) * 4 + (slot & 3)] * Zb[((slot >> 2) * ZR + q) * 4 + (slot & 3)];
            if (v) atomicAdd(a.GL + (int64_t)p * KP + q, v);
          }
      }
      continue;
    }
    for (int slot = 0; slot < nit; slot++) {
      const ull b = s_bnd[slot];
      if (b == 0) continue;
      const int *zr = zs + slot * SL, *rr = rs + slot * SL;
      if (b >= B31) {  // products of this item may not fit 32 bits: 64-bit atomics directly
        if (active) {
#pragma unroll
          for (int i = 0; i < TS; i++)
#pragma unroll
            for (int j = 0; j < TS; j++) {
              const int p = TS * pb + i, q = TS * qb + j;
              const long long v = (long long)zr[p] * (long long)rr[q];
              if (v) atomicAdd(a.GL + (int64_t)p * KP + q, (ull)v);
            }
        }
        continue;
      }
      if (run + b >= B31) {
        flush();
        run = 0;
      }
      run += b;
      if (active) {
        int zp[TS], rq[TS];
#pragma unroll
        for (int i = 0; i < TS; i += 4) {
          const int4 x = *(const int4 *)(zr + TS * pb + i);
          const int4 y = *(const int4 *)(rr + TS * qb + i);
          zp[i] = x.x, zp[i + 1] = x.y, zp[i + 2] = x.z, zp[i + 3] = x.w;
          rq[i] = y.x, rq[i + 1] = y.y, rq[i + 2] = y.z, rq[i + 3] = y.w;
        }
#pragma unroll
        for (int i = 0; i < TS; i++)
#pragma unroll
          for (int j = 0; j < TS; j++) acc[i][j] += (uint32_t)(zp[i] * rq[j]);
      }
    }
  }
  flush();
}

// G_L (upper triangle, p <= q < k) = G_D[acc_idx[p]][acc_idx[q]] - (T2[p][q] + T2[q][p]) / 2 (the sum is even:
// it is twice Z^T A Z).  acc_idx increases, so the G_D entry is in G_D's upper triangle.
__global__ void lfin_kernel(const ull *T2, int kp, const ull *GD, int ld, const int *acc_idx, int k, ull *GL) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < k * k; e += gridDim.x * blockDim.x) {
    const int p = e / k, q = e - p * k;
    if (p > q) continue;
    const long long t = (long long)T2[(int64_t)p * kp + q] + (long long)T2[(int64_t)q * kp + p];
    const long long d = (long long)GD[(int64_t)acc_idx[p] * ld + acc_idx[q]];
    GL[(int64_t)p * kp + q] = (ull)(d - t / 2);
  }
}

// ------------------------------------------------------------------------------------------------
// M = A_acc^T G_L A_acc, A_acc[t][q] = A[q][acc_idx[t]] (zero for t > q).  CTA q forms B = G_L A_acc[:, q]
// and the entries M[p][q] = M[q][p], p <= q (each written once: M is exactly symmetric).
__global__ void __launch_bounds__(256) mgram_kernel(const ull *GL, int kp, const double *A, int ld, const int *acc_idx,
                                                     int k, double *M) {
  __shared__ double aq[PHDE_MAX_K], bq[PHDE_MAX_K];
  __shared__ int idx[PHDE_MAX_K];
  const int q = blockIdx.x;
  for (int t = threadIdx.x; t < k; t += blockDim.x) {
    idx[t] = acc_idx[t];
    aq[t] = A[(int64_t)q * ld + acc_idx[t]];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < k; t += blockDim.x) {
    double s = 0;
    for (int u = 0; u <= q; u++) s = fma(gsym(GL, kp, t, u), aq[u], s);
    bq[t] = s;
  }
  __syncthreads();
  for (int p = threadIdx.x; p <= q; p += blockDim.x) {
    const double *Ap = A + (int64_t)p * ld;
    double s = 0;
    for (int t = 0; t <= p; t++) s = fma(Ap[idx[t]], bq[t], s);
    M[p + (int64_t)q * k] = s;
    M[q + (int64_t)p * k] = s;
  }
}

// S (row-major n x k) = Z A^T restricted to the accepted columns, for callers that ask for the basis.
// S from the packed accepted columns Z_acc (row-major n x kp, uint8 or uint16): column t of Z_acc is Z index
// acc_idx[t].
template <typename T>
__global__ void basis_packed_kernel(const T *Z, int kp, int64_t n, const double *A, int ld, const int *acc_idx, int k,
                                    double *S) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * k; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / k;
    const int q = (int)(e - i * k);
    const double *Aq = A + (int64_t)q * ld;
    double s = Aq[0];
    for (int t = 0; t <= q; t++) s = fma(Aq[acc_idx[t]], (double)Z[i * kp + t], s);
    S[e] = s;
  }
}

__global__ void basis_kernel(ZSrc src, int64_t n, const double *A, int ld, const int *acc_idx, int k,
                             double *S) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * k; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / k;
    const int q = (int)(e - i * k);
    const double *Aq = A + (int64_t)q * ld;
    double s = Aq[0];
    for (int t = 0; t <= q; t++) {
      const int z = acc_idx[t];
      const int d = z <= src.P0 ? src.D[(int64_t)(z - 1) * n + i] : (int)src.R[i * src.RW + src.rmap[z - 1 - src.P0]] - 1;
      s = fma(Aq[z], (double)d, s);
    }
    S[e] = s;
  }
}

// ------------------------------------------------------------------------------------------------
// Coordinates X = Z W, W = A Y (W[0] on the constant column, W[1 + t] on accepted column t).  Per
// coordinate, W is scaled by 2^s to 62-bit integers (s the largest with |W_0| + maxz sum |W_t| < 2^61 / 2^s),
// stored as signed high and unsigned low 32-bit words; a row's sum is then exact in 64-bit integers and
// rounded once to FP64.  The scaling error is below 2^-62 of the row's largest possible magnitude.
// Also the Rayleigh quotient of each coordinate: x = Z w is S y, so x^T L x = y^T M y (M = S^T L S, the
// matrix handed to the eigensolver) and x^T x = w^T G_I w over the constant and accepted columns.
__global__ void coords_prep_kernel(const double *A, int ld, const int *acc_idx, int k, const double *Y, int c,
                                   unsigned maxz, int kp, int32_t *whi, uint32_t *wlo, long long *w0fix,
                                   double *sinv, const double *M, const ull *GI, double *rq) {
  __shared__ double W[PHDE_MAX_K + 1];
  __shared__ double red[32];
  for (int j = 0; j < c; j++) {
    __syncthreads();
    for (int t = threadIdx.x; t <= k; t += blockDim.x) {
      // t == 0: the constant column; t >= 1: accepted column t - 1
      double s = 0;
      for (int q = 0; q < k; q++) {
        const double aqt = t == 0 ? A[(int64_t)q * ld] : (q >= t - 1 ? A[(int64_t)q * ld + acc_idx[t - 1]] : 0.0);
        s = fma(aqt, Y[q + (int64_t)j * k], s);
      }
      W[t] = s;
    }
    __syncthreads();
    double b = 0;
    for (int t = threadIdx.x; t <= k; t += blockDim.x) b += fabs(W[t]) * (t == 0 ? 1.0 : (double)maxz);
    b = block_sum(b, red);
    int e = 0;
    frexp(b, &e);  // b < 2^e
    const int sh = b > 0 ? 61 - e : 0;
    for (int t = threadIdx.x; t < kp + 1; t += blockDim.x) {
      const long long f = t <= k ? llrint(ldexp(W[t], sh)) : 0ll;
      if (t == 0) {
        w0fix[j] = f;
      } else {
        whi[(int64_t)j * kp + t - 1] = (int32_t)(f >> 32);
        wlo[(int64_t)j * kp + t - 1] = (uint32_t)(f & 0xffffffffll);
      }
    }
    if (threadIdx.x == 0) sinv[j] = ldexp(1.0, -sh);
    if (j < PHDE_RQ_MAX) {
      double num = 0, den = 0;
      for (int p = threadIdx.x; p < k; p += blockDim.x) {
        double t = 0;
        for (int q = 0; q < k; q++) t = fma(M[p + (int64_t)q * k], Y[q + (int64_t)j * k], t);
        num = fma(Y[p + (int64_t)j * k], t, num);
      }
      for (int s = threadIdx.x; s <= k; s += blockDim.x) {
        const int is = s == 0 ? 0 : acc_idx[s - 1];
        double t = 0;
        for (int u = 0; u <= k; u++) t = fma(gsym(GI, ld, is, u == 0 ? 0 : acc_idx[u - 1]), W[u], t);
        den = fma(W[s], t, den);
      }
      num = block_sum(num, red);
      den = block_sum(den, red);
      if (threadIdx.x == 0) rq[j] = num / den;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(128) coords_fix_kernel(const T *Z, int64_t n, int kp, int c, const int32_t *whi,
                                                         const uint32_t *wlo, const long long *w0fix,
                                                         const double *sinv, double *X, double *part) {
  extern __shared__ uint32_t wsm[];  // per coordinate: hi[kp], lo[kp]
  __shared__ double red[32];
  for (int e = threadIdx.x; e < c * kp; e += blockDim.x) {
    wsm[2 * e] = (uint32_t)whi[e];
    wsm[2 * e + 1] = wlo[e];
  }
  __syncthreads();
  constexpr int V = 16 / sizeof(T);
  double ss[4] = {0, 0, 0, 0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    for (int j0 = 0; j0 < c; j0 += 4) {
      long long hi[4];
      ull lo[4];
#pragma unroll
      for (int j = 0; j < 4; j++) {
        hi[j] = 0;
        lo[j] = 0;
      }
      for (int t0 = 0; t0 < kp; t0 += V) {
        union {
          uint4 u;
          T v[V];
        } w;
        w.u = *(const uint4 *)(Z + i * kp + t0);
#pragma unroll
        for (int x = 0; x < V; x++) {
          const uint32_t z = (uint32_t)w.v[x];
#pragma unroll
          for (int j = 0; j < 4; j++)
            if (j0 + j < c) {
              const uint32_t *wp = wsm + 2 * ((int64_t)(j0 + j) * kp + t0 + x);
              hi[j] += (long long)(int32_t)wp[0] * (long long)z;
              lo[j] += (ull)wp[1] * (ull)z;
            }
        }
      }
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (j0 + j < c) {
          const long long tot = (long long)((ull)hi[j] << 32) + (long long)lo[j] + w0fix[j0 + j];
          const double x = (double)tot * sinv[j0 + j];
          X[i + (int64_t)(j0 + j) * n] = x;
          if (j0 + j < 4) ss[j] = fma(x, x, ss[j]);
        }
    }
  }
  // column sums of squares for the first four coordinates here; more coordinates use norm_part_kernel
  for (int j = 0; j < 4 && j < c; j++) {
    const double tot = block_sum(ss[j], red);
    if (threadIdx.x == 0) part[(int64_t)blockIdx.x * c + j] = tot;
  }
}

__global__ void norm_part_kernel(const double *X, int64_t n, int c, int j0, double *part) {
  __shared__ double red[32];
  for (int j = j0; j < c; j++) {
    double s = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
      s = fma(X[i + (int64_t)j * n], X[i + (int64_t)j * n], s);
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[(int64_t)blockIdx.x * c + j] = s;
  }
}

// X[:, j] *= 1 / ||X[:, j]|| (getCoordinates, DrawingBase.cpp:196-205): each block sums the per-block
// partials itself in a fixed order, then scales its share.
__global__ void unit_scale_kernel(double *X, int64_t n, int c, const double *part, int nparts) {
  __shared__ double inv[PHDE_MAX_K];
  __shared__ double red[32];
  for (int j = 0; j < c; j++) {
    double s = 0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) s += part[(int64_t)b * c + j];
    s = block_sum(s, red);
    if (threadIdx.x == 0) inv[j] = 1.0 / sqrt(s);
  }
  __syncthreads();
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * c; e += (int64_t)gridDim.x * blockDim.x)
    X[e] = X[e] * inv[e / n];
}

// Rayleigh quotients of the coordinates X = S Y (before their unit scaling): x_j^T L x_j = y_j^T M y_j with
// M = S^T L S (the matrix handed to the eigensolver), over ||x_j||^2 (the coordinate kernels' own sum).
__global__ void rq_gram_kernel(const double *M, const double *Y, int k, int c, const double *norm2, double *rq) {
  __shared__ double red[32];
  for (int j = 0; j < c && j < PHDE_RQ_MAX; j++) {
    double num = 0;
    for (int p = threadIdx.x; p < k; p += blockDim.x) {
      double t = 0;
      for (int q = 0; q < k; q++) t = fma(M[p + (int64_t)q * k], Y[q + (int64_t)j * k], t);
      num = fma(Y[p + (int64_t)j * k], t, num);
    }
    num = block_sum(num, red);
    if (threadIdx.x == 0) rq[j] = num / norm2[j];
  }
}

int grid_n(phde_ctx *ctx, int64_t work, int threads, int per_sm) {
  int64_t b = (work + threads - 1) / threads;
  b = std::min<int64_t>(b, (int64_t)ctx->nsm * per_sm);
  return (int)std::max<int64_t>(b, 1);
}

}  // namespace

// ==================================================================================================
// host side

// G_I, G_D for Z columns p < c1, q in [c0, c1).  byte_state: 1 every distance fits a byte (the quad layout:
// pack Z columns [c0, c1), then the byte kernel), 0 some does not (the 32-bit kernel), -1 not known yet (both
// are launched; each checks maxz, which the pack kernel completes first, and one returns at once).
static int exact_zgram(phde_ctx *ctx, const ZSrc &src, int P, int c0, int c1, ull *GI, ull *GD, int ld,
                       unsigned *maxz, uint32_t *Zq, unsigned *smaxz, int byte_state) {
  const int nq = (c1 - c0) / 4;
  const int ntiles = nq * (c0 / 4) + nq * (nq + 1) / 2;
  if (byte_state != 0) {
    const int64_t nslab = (ctx->n + ZQ_ROWS - 1) / ZQ_ROWS;
    int pk_sm = 0;
    PHDE_CK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pk_sm, zq_pack_kernel, ZQ_THREADS, 0));
    const int gp = (int)std::max<int64_t>(1, std::min<int64_t>(nslab, (int64_t)ctx->nsm * std::max(pk_sm, 1)));
    zq_pack_kernel<<<gp, ZQ_THREADS, 0, ctx->stream>>>(src, ctx->d_off, ctx->n, P, c0, c1, ld, Zq, smaxz, maxz);
    PHDE_LAUNCHED(ctx);
    const int threads = std::min(ZQ_GRAM_THREADS, (ntiles + 31) / 32 * 32);
    const int gy = (ntiles + threads - 1) / threads;
    const size_t smem = sizeof(uint32_t) * 5 * ZQ_QUADS * (size_t)c1 + sizeof(int64_t) * 2 * (ZQ_ROWS + 2);
    PHDE_CK(ctx, cudaFuncSetAttribute(zgram_q_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    PHDE_CK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, zgram_q_kernel, threads, smem));
    per_sm = std::max(1, std::min(per_sm, 4));
    // every CTA resident at once: the slabs are dealt out evenly, so a partial second wave would double the time
    const int gx = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->nsm * per_sm / gy, nslab));
    ZqArgs q;
    q.Zq = Zq;
    q.ldq = ld;
    q.off = ctx->d_off;
    q.n = ctx->n;
    q.c0 = c0;
    q.c1 = c1;
    q.ntiles = ntiles;
    q.GI = GI;
    q.GD = GD;
    q.ld = ld;
    q.smaxz = smaxz;
    q.maxz = maxz;
    zgram_q_kernel<<<dim3(gx, gy), threads, smem, ctx->stream>>>(q);
    PHDE_LAUNCHED(ctx);
    if (byte_state == 1) return PHDE_OK;
  }
  if (src.lvl) return PHDE_OK;  // level mode: distances above 254 cannot occur; an unreached one (maxz) is refused
  const int gy = (ntiles + ZG_THREADS - 1) / ZG_THREADS;
  const size_t smem = sizeof(int) * ((ZG_ROWS + ZG_ROWS / 4 + ZG_ROWS / 2) * (size_t)(c1 + 4) + c1);
  PHDE_CK(ctx, cudaFuncSetAttribute(zgram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  PHDE_CK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, zgram_kernel, ZG_THREADS, smem));
  per_sm = std::max(1, std::min(per_sm, 4));
  const int gx = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->nsm * per_sm / gy,
                                                              (ctx->n + ZG_ROWS - 1) / ZG_ROWS));
  ZgArgs a;
  a.src = src;
  a.off = ctx->d_off;
  a.n = ctx->n;
  a.P = P;
  a.c0 = c0;
  a.c1 = c1;
  a.ntiles = ntiles;
  a.GI = GI;
  a.GD = GD;
  a.ld = ld;
  a.maxz = maxz;
  a.wide_only = byte_state < 0 ? maxz : nullptr;
  zgram_kernel<<<dim3(gx, gy), ZG_THREADS, smem, ctx->stream>>>(a);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

// The D-orthogonalisation of the P candidate columns of D (ParHDE.cpp:190-285) in coefficient space.
// Candidates go in blocks: the first block holds k + max(4, k/8) of them (discards are rare), later blocks
// 16; each block adds its rows and columns to G_I and G_D and runs the candidate loop until k are accepted.
// h_state: accepted, discarded, examined; h_dlog[i]: norm of discarded candidate i (NaN otherwise).
// Returns PHDE_ERR_TOO_LARGE when the distances or degrees are too large for exact 64-bit sums that
// convert exactly to FP64 (the caller then takes the FP64 vector path).
int phde_exact_orth(phde_ctx *ctx, const ZSrc &src, int P, int k, ExactBasis *eb, int *h_state, double *h_dlog) {
  const int64_t n = ctx->n;
  const int ld = ((P + 1) + 3) / 4 * 4;
  ull *GI = (ull *)phde_buf(ctx, "ex.GI", sizeof(ull) * ld * ld);
  ull *GD = (ull *)phde_buf(ctx, "ex.GD", sizeof(ull) * ld * ld);
  double *A = (double *)phde_buf(ctx, "ex.A", sizeof(double) * (size_t)k * ld);
  double *den = (double *)phde_buf(ctx, "ex.den", sizeof(double) * k);
  int *acc_idx = (int *)phde_buf(ctx, "ex.acc", sizeof(int) * k);
  int *state = (int *)phde_buf(ctx, "ex.state", sizeof(int) * 4);
  unsigned *maxz = (unsigned *)phde_buf(ctx, "ex.maxz", sizeof(unsigned) * 2);
  double *dlog = (double *)phde_buf(ctx, "ex.dlog", sizeof(double) * P);
  const int64_t nslab = (n + ZQ_ROWS - 1) / ZQ_ROWS;
  uint32_t *Zq = (uint32_t *)phde_buf(ctx, "ex.Zq", sizeof(uint32_t) * (size_t)nslab * ZQ_QUADS * ld);
  unsigned *smaxz = (unsigned *)phde_buf(ctx, "ex.smaxz", sizeof(unsigned) * nslab);
  if (!GI || !GD || !A || !den || !acc_idx || !state || !maxz || !dlog || !Zq || !smaxz) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(smaxz, 0, sizeof(unsigned) * nslab, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(GI, 0, sizeof(ull) * ld * ld, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(GD, 0, sizeof(ull) * ld * ld, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(A, 0, sizeof(double) * (size_t)k * ld, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(dlog, 0xff, sizeof(double) * P, ctx->stream));  // NaN: not discarded
  PHDE_CK(ctx, cudaMemsetAsync(maxz, 0, sizeof(unsigned) * 2, ctx->stream));
  const int st0[4] = {0, 0, 0, 1};
  PHDE_CK(ctx, cudaMemcpyAsync(state, st0, sizeof(st0), cudaMemcpyHostToDevice, ctx->stream));
  const size_t csmem0 = sizeof(double) * (2 * (size_t)ld + 2 * (size_t)k + CF_THREADS);
  constexpr size_t CF_SMEM_MAX = 200 * 1024;
  PHDE_CK(ctx, cudaFuncSetAttribute(coef_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CF_SMEM_MAX));
  int c0 = 0, c1 = std::min(ld, (1 + std::min(P, k + std::max(4, k / 8)) + 3) / 4 * 4);
  int hs[4] = {0, 0, 0, 1};
  unsigned hm[2] = {0, 0};
  int byte_state = -1;
  for (;;) {
    int rc = exact_zgram(ctx, src, P, c0, c1, GI, GD, ld, maxz, Zq, smaxz, byte_state);
    if (rc) return rc;
    CoefArgs ca;
    ca.maxz = maxz;
    ca.nmax = (double)std::max<int64_t>(ctx->nnz, n);
    ca.GI = GI;
    ca.GD = GD;
    ca.ld = ld;
    // stage the Gram blocks the loop reads when both fit next to the vectors
    const int rend = std::min(c1, P + 1);
    ca.nc = csmem0 + sizeof(double) * 2 * (size_t)rend * rend <= CF_SMEM_MAX ? rend : 0;
    size_t csmem = csmem0 + sizeof(double) * 2 * (size_t)ca.nc * ca.nc;
    ca.sa = csmem + sizeof(double) * (size_t)k * ld <= CF_SMEM_MAX;
    if (ca.sa) csmem += sizeof(double) * (size_t)k * ld;
    ca.n = n;
    ca.r_end = std::min(c1, P + 1);
    ca.k = k;
    ca.A = A;
    ca.den = den;
    ca.acc_idx = acc_idx;
    ca.state = state;
    ca.dlog = dlog;
    coef_kernel<<<1, CF_THREADS, csmem, ctx->stream>>>(ca);
    PHDE_LAUNCHED(ctx);
    PHDE_CK(ctx, cudaMemcpyAsync(hm, maxz, sizeof(hm), cudaMemcpyDeviceToHost, ctx->stream));
    PHDE_CK(ctx, cudaMemcpyAsync(hs, state, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream));
    PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    byte_state = hm[0] <= 255u ? 1 : 0;
    // G_I, G_D, Z^T L Z entries are at most nnz * maxz^2 (and n * maxz^2): exact in FP64 below 2^53; the
    // Laplacian sums stay in 32 bits; distances fit 16 bits (coef_kernel made the same check and did nothing)
    const double mz = (double)hm[0];
    if (hm[0] > 65535u || (double)std::max<int64_t>(ctx->nnz, n) * mz * mz >= 9007199254740992.0 ||
        (double)hm[1] * mz >= 2147483647.0)
      return phde_fail(ctx, PHDE_ERR_TOO_LARGE, "exact path: distances or degrees too large");
    if (hs[0] >= k || c1 >= P + 1) break;
    c0 = c1;
    c1 = std::min(ld, c1 + 16);
  }
  h_state[0] = hs[0];
  h_state[1] = hs[1];
  h_state[2] = hs[2];
  PHDE_CK(ctx, cudaMemcpyAsync(h_dlog, dlog, sizeof(double) * P, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  eb->A = A;
  eb->GI = GI;
  eb->GD = GD;
  eb->acc_idx = acc_idx;
  eb->ld = ld;
  eb->maxz = hm[0];
  eb->maxdeg = hm[1];
  eb->Z = nullptr;
  eb->Zq = byte_state == 1 ? Zq : nullptr;  // every accepted column is packed (examined blocks only)
  return PHDE_OK;
}

// Pack the accepted columns, form Z_acc^T L Z_acc exactly and M = A_acc^T (Z_acc^T L Z_acc) A_acc.
int phde_exact_lap(phde_ctx *ctx, const ZSrc &src, int k, ExactBasis *eb, double *M) {
  const int64_t n = ctx->n;
  const bool z16 = eb->maxz > 255u;
  const int kp = k <= 64 ? 64 : k <= 128 ? 128 : 256;
  void *Z = phde_buf(ctx, "ex.Z", (size_t)n * kp * (z16 ? 2 : 1));
  ull *T2 = (ull *)phde_buf(ctx, "ex.T2", sizeof(ull) * kp * kp);
  ull *GL = (ull *)phde_buf(ctx, "ex.GL", sizeof(ull) * kp * kp);
  if (!Z || !T2 || !GL) return PHDE_ERR_OOM;
  const int gp = grid_n(ctx, n, 256, 8);
  if (src.lvl && !eb->Zq)  // level-mode columns exist only in the quad layout (distances below 255)
    return phde_fail(ctx, PHDE_ERR_INVALID, "exact path: level-mode columns without the byte layout");
  if (z16)
    pack_kernel<uint16_t><<<gp, 256, 0, ctx->stream>>>(src, n, eb->acc_idx, k, kp, (uint16_t *)Z);
  else if (eb->Zq)
    pack_from_zq_kernel<<<grid_n(ctx, (n + 3) / 4 * (kp / 16), 256, 8), 256, 0, ctx->stream>>>(
        eb->Zq, eb->ld, n, eb->acc_idx, k, kp, (uint8_t *)Z);
  else
    pack_kernel<uint8_t><<<gp, 256, 0, ctx->stream>>>(src, n, eb->acc_idx, k, kp, (uint8_t *)Z);
  PHDE_LAUNCHED(ctx);
  eb->Z = Z;
  eb->z16 = z16;
  eb->kp = kp;
  const int64_t *crow, *ce0;
  int64_t nch, chunk;
  int rc = phde_heavy_chunks(ctx, &crow, &ce0, &nch, &chunk);
  if (rc) return rc;
  PHDE_CK(ctx, cudaMemsetAsync(T2, 0, sizeof(ull) * kp * kp, ctx->stream));
  LgArgs a;
  a.off = ctx->d_off;
  a.adj = ctx->d_adj;
  a.n = n;
  a.Z = Z;
  a.kp = kp;
  a.heavy = chunk;  // rows above the chunk length are the ones the plan cut into chunks
  a.chunk_row = crow;
  a.chunk_e0 = ce0;
  a.nchunks = nch;
  a.chunk = chunk;
  a.GL = T2;
  const int TS = kp <= 64 ? 4 : 8;
  const int nb = kp / TS;
  a.ntiles = nb * nb;
  const int gy = (a.ntiles + LG_THREADS - 1) / LG_THREADS;
  const size_t smem = sizeof(int) * 2 * LG_ITEMS * (size_t)(kp + 4);
  const int64_t nslab = (n + nch + LG_ITEMS - 1) / LG_ITEMS;
  auto launch = [&](auto kern) -> int {
    PHDE_CK(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    PHDE_CK(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, LG_THREADS, smem));
    per_sm = std::max(1, per_sm);
    const int gx = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->nsm * per_sm / gy, nslab));
    cudaEventRecord(ctx->lev[0], ctx->stream);
    kern<<<dim3(gx, gy), LG_THREADS, smem, ctx->stream>>>(a);
    PHDE_LAUNCHED(ctx);
    cudaEventRecord(ctx->lev[1], ctx->stream);
    ctx->lev_pending = true;
    return PHDE_OK;
  };
  if (z16) {
    if (kp == 64) rc = launch(lgram_kernel<uint16_t, 64, 4>);
    else if (kp == 128) rc = launch(lgram_kernel<uint16_t, 128, 8>);
    else rc = launch(lgram_kernel<uint16_t, 256, 8>);
  } else {
    if (kp == 64) rc = launch(lgram_kernel<uint8_t, 64, 4>);
    else if (kp == 128) rc = launch(lgram_kernel<uint8_t, 128, 8>);
    else rc = launch(lgram_kernel<uint8_t, 256, 8>);
  }
  if (rc) return rc;
  lfin_kernel<<<(k * k + 255) / 256, 256, 0, ctx->stream>>>(T2, kp, eb->GD, eb->ld, eb->acc_idx, k, GL);
  PHDE_LAUNCHED(ctx);
  mgram_kernel<<<k, 256, 0, ctx->stream>>>(GL, kp, eb->A, eb->ld, eb->acc_idx, k, M);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

// X (column-major n x c, unit columns) = Z (A Y).
int phde_exact_coords(phde_ctx *ctx, const double *M, const double *Y, int k, int c, ExactBasis *eb, double *X,
                      double *rq) {
  const int64_t n = ctx->n;
  const int kp = eb->kp;
  int32_t *whi = (int32_t *)phde_buf(ctx, "ex.whi", sizeof(int32_t) * (size_t)c * kp);
  uint32_t *wlo = (uint32_t *)phde_buf(ctx, "ex.wlo", sizeof(uint32_t) * (size_t)c * kp);
  long long *w0 = (long long *)phde_buf(ctx, "ex.w0", sizeof(long long) * c);
  double *sinv = (double *)phde_buf(ctx, "ex.sinv", sizeof(double) * c);
  const int grid = grid_n(ctx, n, 128, 8);
  double *part = (double *)phde_buf(ctx, "ex.part", sizeof(double) * (size_t)grid * c);
  if (!whi || !wlo || !w0 || !sinv || !part) return PHDE_ERR_OOM;
  coords_prep_kernel<<<1, 256, 0, ctx->stream>>>(eb->A, eb->ld, eb->acc_idx, k, Y, c, eb->maxz, kp, whi, wlo, w0,
                                                 sinv, M, eb->GI, rq);
  PHDE_LAUNCHED(ctx);
  const size_t smem = sizeof(uint32_t) * 2 * (size_t)c * kp;
  if (eb->z16) {
    PHDE_CK(ctx, cudaFuncSetAttribute(coords_fix_kernel<uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)std::max<size_t>(smem, 48 * 1024)));
    coords_fix_kernel<uint16_t><<<grid, 128, smem, ctx->stream>>>((const uint16_t *)eb->Z, n, kp, c, whi, wlo, w0,
                                                                  sinv, X, part);
  } else {
    PHDE_CK(ctx, cudaFuncSetAttribute(coords_fix_kernel<uint8_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)std::max<size_t>(smem, 48 * 1024)));
    coords_fix_kernel<uint8_t><<<grid, 128, smem, ctx->stream>>>((const uint8_t *)eb->Z, n, kp, c, whi, wlo, w0,
                                                                 sinv, X, part);
  }
  PHDE_LAUNCHED(ctx);
  if (c > 4) {
    norm_part_kernel<<<grid, 128, 0, ctx->stream>>>(X, n, c, 4, part);
    PHDE_LAUNCHED(ctx);
  }
  unit_scale_kernel<<<grid_n(ctx, n * c, 256, 8), 256, 0, ctx->stream>>>(X, n, c, part, grid);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

// The basis S = Z A (row-major n x k FP64), only for callers that ask for it.
int phde_exact_basis(phde_ctx *ctx, const ZSrc &src, int k, const ExactBasis *eb, double *S) {
  const int g = grid_n(ctx, ctx->n * k, 256, 8);
  if (eb->Z && eb->z16)
    basis_packed_kernel<uint16_t><<<g, 256, 0, ctx->stream>>>((const uint16_t *)eb->Z, eb->kp, ctx->n, eb->A, eb->ld,
                                                               eb->acc_idx, k, S);
  else if (eb->Z)
    basis_packed_kernel<uint8_t><<<g, 256, 0, ctx->stream>>>((const uint8_t *)eb->Z, eb->kp, ctx->n, eb->A, eb->ld,
                                                              eb->acc_idx, k, S);
  else if (src.lvl)
    return phde_fail(ctx, PHDE_ERR_INVALID, "exact basis: level-mode columns need the packed accepted columns");
  else
    basis_kernel<<<g, 256, 0, ctx->stream>>>(src, ctx->n, eb->A, eb->ld, eb->acc_idx, k, S);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

// Rayleigh quotients of the first min(c, PHDE_RQ_MAX) coordinates from M, Y and the pre-scaling column norms
// (device arrays), into rq (device).
int phde_rayleigh(phde_ctx *ctx, const double *M, const double *Y, int k, int c, const double *norm2, double *rq) {
  rq_gram_kernel<<<1, 256, 0, ctx->stream>>>(M, Y, k, c, norm2, rq);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}
