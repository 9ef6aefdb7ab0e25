// draw.cu -- the reference's `draw` tool (draw_graph.c) on the GPU: a CSR graph and two vertex coordinates to
// the edge image, pixel for pixel the image the reference draws in its serial order.
//
// The reference walks the CSR entries in order, draws each as a Bresenham line from u to v (later lines
// overwrite earlier pixels) and colours it by its length bin and four running counters (draw_graph.c:49-128,
// 282-326).  Here that order is made explicit so that all entries and all pixels are processed at once:
//   1. the bounds of the coordinates (one reduction); the image size on the host, in the reference's
//      arithmetic; every vertex scaled and clamped to its pixel (draw_graph.c:201-268);
//   2. the longest entry: FP64 square root of the integer squared length, rounded to float, as the
//      reference computes it (draw_graph.c:130-133, 282-298);
//   3. the rasteriser: each CTA takes a tile of entries, computes their bins in float arithmetic
//      (draw_graph.c:322-323) and per-tile counts of the four bins that have counters, splits the tile's
//      pixels into equal chunks and plots them with a closed form of the reference's Bresenham loop -- on a
//      line of major extent M and minor extent m the minor coordinate after i major steps is
//      floor((i m + M - floor(M / 2) - 1) / M) -- so a thread can start anywhere on any line.  Every pixel
//      gets atomicMax(owner, entry + 1): the last entry in CSR order covering a pixel owns it, as the
//      reference's overwrite order decides.  Tiles run from the last to the first, and an owner that a
//      cached read already shows to be later needs no atomic (owners only grow);
//   4. the counters only grow and each grants its colour to the first entries that reach it, so the
//      entries given each counted colour are exactly those before a cut position.  One CTA finds the four
//      cuts from the tile counts: entries of bin 0 past the first counter's limit reach the second counter,
//      entries of bin 6 past theirs reach the third -- the reference's case fall-throughs;
//   5. every pixel's colour from its owner's bin and the cuts, written as 4-bit palette indices in PNG
//      scanline layout (filter byte 0, two pixels per byte), which the host deflates into the PNG file.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ctx.h"
#include "png.h"

namespace {

constexpr int RT = 2048;          // CSR entries per raster tile
constexpr int RT_THREADS = 512;   // threads per raster CTA
constexpr int RCHUNK = 32;        // pixels per raster chunk
constexpr int RGROUP = 8;         // pixels whose owner reads a thread issues together
constexpr int SEL_THREADS = 1024; // the cut-selection CTA
constexpr uint32_t BG_INDEX = 8;  // palette index of the background
// The owner image is stored in 8 x 8-pixel tiles (256 bytes, tiles in row-major order): a line of any
// direction stays inside one tile for about eight steps, so more of its owner reads hit L1.
__host__ __device__ __forceinline__ uint32_t tile_index(unsigned x, unsigned y, unsigned tiles_w) {
  return (((y >> 3) * tiles_w + (x >> 3)) << 6) + ((y & 7u) << 3) + (x & 7u);  // < 2^31: the size cap
}
constexpr uint32_t MAX_SIDE = 1u << 20;

// colour codes 0..7 (draw_line's colours, draw_graph.c:57-102) and 8 (the background, draw_graph.c:273-277),
// as 0xAABBGGRR
__constant__ uint32_t c_palette[9] = {
    0xff4953fbu,  // 0 red-orange   251, 83, 73
    0xff04a5fbu,  // 1 orange       251, 165, 4
    0xff42aefbu,  // 2 yellow-orange 251, 174, 66
    0xff04fbfbu,  // 3 yellow       251, 251, 4
    0xff32fb9au,  // 4 yellow-green 154, 251, 50
    0xff04fb04u,  // 5 green        4, 251, 4
    0xffba980du,  // 6 blue-green   13, 152, 186
    0xff000000u,  // 7 black: the longest bin, which no case names
    0xff040404u,  // 8 background   4, 4, 4
};

__device__ __forceinline__ ull order_key(double v) {
  const ull b = (ull)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
double key_value(ull k) {
  const ull b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double v;
  memcpy(&v, &b, sizeof v);
  return v;
}

__device__ __forceinline__ ull warp_min_u64(ull v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const ull w = __shfl_xor_sync(PHDE_FULL_MASK, v, o);
    v = w < v ? w : v;
  }
  return v;
}

// keys: {min x, min y, max x, max y} as order keys; bad: a coordinate that is not finite.
__global__ void draw_bounds_kernel(const double *x, const double *y, int64_t n, ull *keys, int *bad) {
  ull xlo = ~0ull, ylo = ~0ull, xhi = 0, yhi = 0;
  int nonfinite = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double a = x[i], b = y[i];
    if (!isfinite(a) || !isfinite(b)) {
      nonfinite = 1;
      continue;
    }
    const ull ka = order_key(a), kb = order_key(b);
    xlo = ka < xlo ? ka : xlo;
    xhi = ka > xhi ? ka : xhi;
    ylo = kb < ylo ? kb : ylo;
    yhi = kb > yhi ? kb : yhi;
  }
  xlo = warp_min_u64(xlo);
  ylo = warp_min_u64(ylo);
  xhi = warp_max_u64(xhi);
  yhi = warp_max_u64(yhi);
  nonfinite = __any_sync(PHDE_FULL_MASK, nonfinite);
  if ((threadIdx.x & 31) == 0) {
    if (xlo != ~0ull) {
      atomicMin(&keys[0], xlo);
      atomicMin(&keys[1], ylo);
      atomicMax(&keys[2], xhi);
      atomicMax(&keys[3], yhi);
    }
    if (nonfinite) atomicOr(bad, 1);
  }
}

// Pixel of every vertex: ((-min + v) * (1 / range)) * size, clamped to [0, size - 1], floored
// (draw_graph.c:259-268); the explicit roundings keep the reference's operation order.
__global__ void draw_scale_kernel(const double *x, const double *y, int64_t n, double xmin, double ymin, double xri,
                                  double yri, unsigned W, unsigned H, int2 *pix) {
  const double wd = (double)W, hd = (double)H, wmax = (double)(W - 1u), hmax = (double)(H - 1u);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double vx = __dmul_rn(__dmul_rn(__dadd_rn(-xmin, x[i]), xri), wd);
    double vy = __dmul_rn(__dmul_rn(__dadd_rn(-ymin, y[i]), yri), hd);
    if (vx < 0) vx = 0;
    if (vy < 0) vy = 0;
    if (vx > wmax) vx = wmax;
    if (vy > hmax) vy = hmax;
    pix[i] = make_int2((int)floor(vx), (int)floor(vy));
  }
}

// Row of every CSR entry, one warp per vertex.
__global__ void draw_rows_kernel(const int64_t *off, int64_t n, uint32_t *erow) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n; u += nw) {
    const int64_t e1 = off[u + 1];
    for (int64_t e = off[u] + lane; e < e1; e += 32) erow[e] = (uint32_t)u;
  }
}

// length(floor(u), floor(v)) of draw_graph.c:130-133 as float: the squared length is an exact integer below
// 2^53 for images below 2^26 pixels a side, so only the square root and the float conversion round.
__device__ __forceinline__ float entry_length(int2 p, int2 q) {
  const double dx = (double)(q.x - p.x), dy = (double)(q.y - p.y);
  return __double2float_rn(__dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy))));
}

// bin = (int) floor((len / max) * 7) in float (draw_graph.c:323); 0 / 0 (every entry of length 0) is not a
// number, whose conversion gives INT_MIN on x86-64, a bin no case names: drawn black like bin 7.
__device__ __forceinline__ int entry_bin(float len, float mx) {
  const float q = __fmul_rn(__fdiv_rn(len, mx), 7.0f);
  if (q != q) return 7;
  return (int)floorf(q);
}

__global__ void draw_maxlen_kernel(const uint32_t *erow, const uint32_t *adj, const int2 *pix, int64_t nnz,
                                   unsigned *maxbits) {
  float mx = 0.f;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x)
    mx = fmaxf(mx, entry_length(pix[erow[e]], pix[adj[e]]));
  // non-negative floats order like their bit patterns
  unsigned b = __float_as_uint(mx);
  b = __reduce_max_sync(PHDE_FULL_MASK, b);
  if ((threadIdx.x & 31) == 0 && b) atomicMax(maxbits, b);
}

// The Bresenham state of one line at major step k.
struct Line {
  int cx, cy;        // current pixel
  int smaj_x, smaj_y;  // major step (one of them 0)
  int smin_x, smin_y;  // minor step
  uint32_t M, m, r;  // major and minor extents, remainder of (k m + M - floor(M/2) - 1) mod M
};

__device__ __forceinline__ void line_at(Line &L, int2 p, int2 q, uint32_t k) {
  const int dx = q.x - p.x, dy = q.y - p.y;
  const uint32_t adx = (uint32_t)abs(dx), ady = (uint32_t)abs(dy);
  const int sx = p.x < q.x ? 1 : -1, sy = p.y < q.y ? 1 : -1;
  const bool xmajor = adx > ady;  // a tie steps both ways every time: either form gives the same pixels
  L.M = xmajor ? adx : ady;
  L.m = xmajor ? ady : adx;
  L.smaj_x = xmajor ? sx : 0;
  L.smaj_y = xmajor ? 0 : sy;
  L.smin_x = xmajor ? 0 : sx;
  L.smin_y = xmajor ? sy : 0;
  uint32_t kk = 0;
  L.r = 0;
  if (L.M > 0) {
    const ull num = (ull)k * L.m + (L.M - L.M / 2u - 1u);
    kk = (uint32_t)(num / L.M);
    L.r = (uint32_t)(num % L.M);
  }
  L.cx = p.x + L.smaj_x * (int)k + L.smin_x * (int)kk;
  L.cy = p.y + L.smaj_y * (int)k + L.smin_y * (int)kk;
}

__device__ __forceinline__ void line_step(Line &L) {
  L.cx += L.smaj_x;
  L.cy += L.smaj_y;
  L.r += L.m;
  if (L.r >= L.M) {
    L.r -= L.M;
    L.cx += L.smin_x;
    L.cy += L.smin_y;
  }
}

// One CTA per tile of RT entries: bins and per-tile counts of bins 0, 1, 5, 6 (tcnt[tile * 4 + j]), then
// every pixel of the tile's lines.  SKIP: tiles run from the last to the first, and a pixel whose owner (read
// through L1, possibly stale) is already a later entry needs no atomic -- owners only grow, so a stale value
// that is already larger is still larger.
template <bool SKIP>
__global__ void __launch_bounds__(RT_THREADS) draw_raster_kernel(const uint32_t *erow, const uint32_t *adj,
                                                                 const int2 *pix, int64_t nnz,
                                                                 const unsigned *maxbits, unsigned W, unsigned H,
                                                                 uint32_t *owner, uint8_t *bin, uint32_t *tcnt,
                                                                 ull *pixels) {
  __shared__ int2 s_a[RT], s_b[RT];
  __shared__ uint32_t s_pre[RT + 1];
  __shared__ uint32_t s_warp[RT_THREADS / 32];
  __shared__ uint32_t s_cnt[4];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t tile = SKIP ? (int64_t)gridDim.x - 1 - blockIdx.x : (int64_t)blockIdx.x;
  const int64_t e0 = tile * RT;
  const int cnt = (int)min((int64_t)RT, nnz - e0);
  const float mx = __uint_as_float(*maxbits);
  if (tid < 4) s_cnt[tid] = 0;
  uint32_t c0 = 0, c1 = 0, c5 = 0, c6 = 0;
  for (int i = tid; i < RT; i += RT_THREADS) {
    uint32_t len = 0;
    if (i < cnt) {
      const int64_t e = e0 + i;
      const int2 p = pix[erow[e]], q = pix[adj[e]];
      s_a[i] = p;
      s_b[i] = q;
      len = (uint32_t)max(abs(q.x - p.x), abs(q.y - p.y)) + 1u;
      const int b = entry_bin(entry_length(p, q), mx);
      bin[e] = (uint8_t)b;
      c0 += b == 0;
      c1 += b == 1;
      c5 += b == 5;
      c6 += b == 6;
    }
    s_pre[i] = len;
  }
  c0 = __reduce_add_sync(PHDE_FULL_MASK, c0);
  c1 = __reduce_add_sync(PHDE_FULL_MASK, c1);
  c5 = __reduce_add_sync(PHDE_FULL_MASK, c5);
  c6 = __reduce_add_sync(PHDE_FULL_MASK, c6);
  __syncthreads();
  if (lane == 0) {
    atomicAdd(&s_cnt[0], c0);
    atomicAdd(&s_cnt[1], c1);
    atomicAdd(&s_cnt[2], c5);
    atomicAdd(&s_cnt[3], c6);
  }
  // exclusive prefix of the pixel counts: 4 consecutive entries per thread
  constexpr int PER = RT / RT_THREADS;
  uint32_t v[PER], sum = 0;
#pragma unroll
  for (int j = 0; j < PER; j++) {
    v[j] = s_pre[tid * PER + j];
    sum += v[j];
  }
  uint32_t incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(PHDE_FULL_MASK, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < RT_THREADS / 32 ? s_warp[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(PHDE_FULL_MASK, w, o);
      if (lane >= o) w += t;
    }
    if (lane < RT_THREADS / 32) s_warp[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  uint32_t run = incl - sum + (warp > 0 ? s_warp[warp - 1] : 0u);
#pragma unroll
  for (int j = 0; j < PER; j++) {
    s_pre[tid * PER + j] = run;
    run += v[j];
  }
  if (tid == RT_THREADS - 1) s_pre[RT] = run;
  __syncthreads();
  if (tid < 4) tcnt[tile * 4 + tid] = s_cnt[tid];
  const uint32_t P = s_pre[RT];
  if (tid == 0) atomicAdd(pixels, (ull)P);
  const uint32_t nch = (P + RCHUNK - 1) / RCHUNK;
  const unsigned tiles_w = (W + 7) >> 3;
  for (uint32_t c = tid; c < nch; c += RT_THREADS) {
    const uint32_t p0 = c * RCHUNK, pend = min(p0 + RCHUNK, P);
    int lo = 0, hi = cnt;  // s_pre[lo] <= p0 < s_pre[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (s_pre[mid] <= p0) lo = mid;
      else hi = mid;
    }
    int i = lo;
    uint32_t k = p0 - s_pre[i];
    uint32_t left = s_pre[i + 1] - p0;  // pixels of line i from step k on
    Line L;
    line_at(L, s_a[i], s_b[i], k);
    uint32_t tag = (uint32_t)(e0 + i + 1);
    // RGROUP pixels at a time: their positions first, then all their owner reads, then the atomics, so a
    // thread has RGROUP independent reads in flight instead of one read-compare-atomic chain per pixel
    for (uint32_t p = p0; p < pend; p += RGROUP) {
      uint32_t at[RGROUP];
      uint32_t tg[RGROUP];
#pragma unroll
      for (int q = 0; q < RGROUP; q++) {
        tg[q] = 0;  // 0: no pixel (past the chunk, or outside the image)
        if (p + q < pend) {
          if ((unsigned)L.cx < W && (unsigned)L.cy < H) {
            at[q] = tile_index((unsigned)L.cx, (unsigned)L.cy, tiles_w);
            tg[q] = tag;
          }
          if (--left == 0) {
            if (p + q + 1 < pend) {
              i++;
              left = s_pre[i + 1] - s_pre[i];
              line_at(L, s_a[i], s_b[i], 0);
              tag++;
            }
          } else {
            line_step(L);
          }
        }
      }
      uint32_t cur[RGROUP];
#pragma unroll
      for (int q = 0; q < RGROUP; q++) cur[q] = (SKIP && tg[q]) ? __ldca(&owner[at[q]]) : 0u;
#pragma unroll
      for (int q = 0; q < RGROUP; q++)
        if (tg[q] && cur[q] < tg[q]) atomicMax(&owner[at[q]], tg[q]);
    }
  }
}

// Inclusive block scan of one int64 per thread (SEL_THREADS threads); returns the block total too.
__device__ __forceinline__ int64_t sel_scan(int64_t x, int64_t *s_w, int64_t &total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t t = __shfl_up_sync(PHDE_FULL_MASK, x, o);
    if (lane >= o) x += t;
  }
  __syncthreads();
  if (lane == 31) s_w[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int64_t w = s_w[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t t = __shfl_up_sync(PHDE_FULL_MASK, w, o);
      if (lane >= o) w += t;
    }
    s_w[lane] = w;
  }
  __syncthreads();
  const int64_t r = x + (warp > 0 ? s_w[warp - 1] : 0);
  total = s_w[SEL_THREADS / 32 - 1];
  __syncthreads();
  return r;
}

struct SelShared {
  int64_t w[SEL_THREADS / 32];
  int64_t tile, before, idx;
};

// Entry classes for the counters: 0 = bin 0; 1 = reaches the second counter (bin 1, or bin 0 at or past
// cut0); 2 = bin 6; 3 = reaches the fourth counter (bin 5, or bin 6 at or past cut6).
__device__ __forceinline__ bool in_class(int cls, int b, int64_t e, int64_t cut0, int64_t cut6) {
  switch (cls) {
    case 0: return b == 0;
    case 1: return b == 1 || (b == 0 && e >= cut0);
    case 2: return b == 6;
    default: return b == 5 || (b == 6 && e >= cut6);
  }
}

// Count of class `cls` entries in tile t.  Classes 1 and 3 add the bin-0 (bin-6) entries at or past the cut,
// which splits at most one tile; that tile is counted entry by entry (every thread must call).
__device__ int64_t tile_class_count(int cls, int64_t t, int64_t ntiles, const uint32_t *tcnt, int64_t cut0,
                                    int64_t cut6, int64_t nnz, int64_t split_cnt, int64_t split_tile) {
  if (t >= ntiles) return 0;
  const uint32_t *c = tcnt + t * 4;
  if (cls == 0) return c[0];
  if (cls == 2) return c[3];
  const int64_t cut = cls == 1 ? cut0 : cut6;
  const int64_t base = cls == 1 ? c[1] : c[2];
  const int64_t spill = cls == 1 ? c[0] : c[3];
  const int64_t t0 = t * RT, t1 = min(t0 + RT, nnz);
  if (t1 <= cut) return base;
  if (t0 >= cut) return base + spill;
  return t == split_tile ? base + split_cnt : base;
}

// Index + 1 of the K-th entry of class `cls` in CSR order (K >= 1), or nnz when the class has fewer.
__device__ int64_t kth_entry(int cls, int64_t K, const uint8_t *bin, const uint32_t *tcnt, int64_t ntiles,
                             int64_t nnz, int64_t cut0, int64_t cut6, SelShared &S) {
  if (K <= 0) return 0;
  // the tile a cut splits, and its entries of the spilling bin at or past the cut
  int64_t split_tile = -1, split_cnt = 0;
  if (cls == 1 || cls == 3) {
    const int64_t cut = cls == 1 ? cut0 : cut6;
    const int spill_bin = cls == 1 ? 0 : 6;
    if (cut % RT != 0 && cut < nnz) {
      split_tile = cut / RT;
      const int64_t t1 = min(split_tile * RT + RT, nnz);
      int64_t mine = 0;
      for (int64_t e = cut + threadIdx.x; e < t1; e += SEL_THREADS) mine += bin[e] == spill_bin;
      int64_t tot;
      sel_scan(mine, S.w, tot);
      split_cnt = tot;
    }
  }
  int64_t acc = 0;
  for (int64_t t0 = 0; t0 < ntiles; t0 += SEL_THREADS) {
    const int64_t t = t0 + threadIdx.x;
    const int64_t c = tile_class_count(cls, t, ntiles, tcnt, cut0, cut6, nnz, split_cnt, split_tile);
    int64_t tot;
    const int64_t incl = sel_scan(c, S.w, tot);
    if (acc + tot >= K) {
      if (t < ntiles && acc + incl - c < K && acc + incl >= K) {
        S.tile = t;
        S.before = acc + incl - c;
      }
      __syncthreads();
      const int64_t tile = S.tile, need = K - S.before;  // the need-th class entry of this tile
      const int64_t b0 = tile * RT, b1 = min(b0 + RT, nnz);
      int64_t seen = 0;
      for (int64_t s0 = b0; s0 < b1; s0 += SEL_THREADS) {
        const int64_t e = s0 + threadIdx.x;
        const int64_t f = e < b1 && in_class(cls, bin[e], e, cut0, cut6) ? 1 : 0;
        int64_t ftot;
        const int64_t fi = sel_scan(f, S.w, ftot);
        if (f && seen + fi == need) S.idx = e;
        __syncthreads();
        if (seen + ftot >= need) break;
        seen += ftot;
      }
      __syncthreads();
      const int64_t r = S.idx + 1;
      __syncthreads();
      return r;
    }
    acc += tot;
  }
  return nnz;
}

// cuts[0]: entries of bin 0 below it take the first colour; cuts[1]: second-counter entries below it take
// the second; cuts[2]: bin-6 entries below it take the third; cuts[3]: fourth-counter entries below it take
// the fourth.  G = m (the first counter's integer-division limit), T = the others' limit.
__global__ void __launch_bounds__(SEL_THREADS) draw_cuts_kernel(const uint8_t *bin, const uint32_t *tcnt,
                                                                int64_t ntiles, int64_t nnz, int64_t G, int64_t T,
                                                                int64_t *cuts) {
  __shared__ SelShared S;
  const int64_t cut0 = kth_entry(0, G, bin, tcnt, ntiles, nnz, 0, 0, S);
  const int64_t cut2 = kth_entry(1, T, bin, tcnt, ntiles, nnz, cut0, 0, S);
  const int64_t cut6 = kth_entry(2, T, bin, tcnt, ntiles, nnz, 0, 0, S);
  const int64_t cut5 = kth_entry(3, T, bin, tcnt, ntiles, nnz, 0, cut6, S);
  if (threadIdx.x == 0) {
    cuts[0] = cut0;
    cuts[1] = cut2;
    cuts[2] = cut6;
    cuts[3] = cut5;
  }
}

__device__ __forceinline__ uint32_t pixel_code(uint32_t o, const uint8_t *bin, int64_t cut0, int64_t cut2,
                                               int64_t cut6, int64_t cut5) {
  if (o == 0) return BG_INDEX;
  const int64_t e = (int64_t)o - 1;
  const uint32_t b = bin[e];
  switch (b) {
    case 0: return e < cut0 ? 0u : (e < cut2 ? 1u : 2u);
    case 1: return e < cut2 ? 1u : 3u;
    case 5: return e < cut5 ? 5u : 3u;
    case 6: return e < cut6 ? 6u : (e < cut5 ? 5u : 4u);
    default: return b;  // 2, 3, 4 and the black bin 7
  }
}

// 4-bit palette scanlines: row y at y * S, filter byte 0, then pixels 2j (high nibble) and 2j + 1.
__global__ void draw_pack_kernel(const uint32_t *owner, const uint8_t *bin, const int64_t *cuts, unsigned W,
                                 unsigned H, size_t S, uint8_t *packed) {
  const int64_t cut0 = cuts[0], cut2 = cuts[1], cut6 = cuts[2], cut5 = cuts[3];
  const unsigned tiles_w = (W + 7) >> 3;
  for (unsigned y = blockIdx.x; y < H; y += gridDim.x) {
    uint8_t *out = packed + (size_t)y * S;
    for (size_t j = threadIdx.x; j < S; j += blockDim.x) {
      if (j == 0) {
        out[0] = 0;
        continue;
      }
      const unsigned x = 2 * (unsigned)(j - 1);  // even: x and x + 1 share a tile row
      const uint32_t t = tile_index(x, y, tiles_w);
      const uint32_t hi = pixel_code(owner[t], bin, cut0, cut2, cut6, cut5);
      const uint32_t lo = x + 1 < W ? pixel_code(owner[t + 1], bin, cut0, cut2, cut6, cut5) : 0u;
      out[j] = (uint8_t)((hi << 4) | lo);
    }
  }
}

// RGBA (0xAABBGGRR per pixel) from the packed scanlines.
__global__ void draw_expand_kernel(const uint8_t *packed, unsigned W, unsigned H, size_t S, uint32_t *rgba) {
  const size_t npix = (size_t)W * H;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (size_t)gridDim.x * blockDim.x) {
    const size_t y = p / W, x = p - y * W;
    const uint8_t b = packed[y * S + 1 + x / 2];
    const uint32_t code = (x & 1) ? (b & 15u) : (b >> 4);
    rgba[p] = c_palette[code < 9 ? code : BG_INDEX];
  }
}

int grid_of(phde_ctx *ctx, int64_t work, int threads) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((work + threads - 1) / threads, (int64_t)ctx->nsm * 16));
}

// Entries c >= 0 with (double) c / (double) m <= 0.05: the limit of draw_line's floating-point counters
// (draw_graph.c:64, 71, 79), found from the test itself.
int64_t counter_limit(int64_t m) {
  if (m <= 0) return 0;  // 0 / 0 and c / 0 both fail the test
  int64_t c = (int64_t)(0.05 * (double)m) + 4;
  while (c >= 0 && !((double)c / (double)m <= 0.05)) c--;
  while ((double)(c + 1) / (double)m <= 0.05) c++;
  return c + 1;
}

}  // namespace

extern "C" int phde_draw(phde_ctx *ctx, const double *x, const double *y, phde_draw_info *info) {
  if (!ctx) return PHDE_ERR_INVALID;
  if (!x || !y) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_draw: null coordinates");
  if (ctx->n <= 0) return phde_fail(ctx, PHDE_ERR_NO_GRAPH, "phde_draw: no graph uploaded");
  PHDE_CK(ctx, cudaSetDevice(ctx->device));
  const auto t_host0 = std::chrono::steady_clock::now();
  const int64_t n = ctx->n, nnz = ctx->nnz;
  const long long launches0 = ctx->launches;
  double *d_x = (double *)phde_buf(ctx, "draw.x", sizeof(double) * n);
  double *d_y = (double *)phde_buf(ctx, "draw.y", sizeof(double) * n);
  ull *keys = (ull *)phde_buf(ctx, "draw.keys", sizeof(ull) * 4 + sizeof(int) * 2);
  int2 *pix = (int2 *)phde_buf(ctx, "draw.pix", sizeof(int2) * n);
  if (!d_x || !d_y || !keys || !pix) return PHDE_ERR_OOM;
  int *bad = (int *)(keys + 4);
  cudaEventRecord(ctx->ev[0], ctx->stream);
  PHDE_CK(ctx, cudaMemcpyAsync(d_x, x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  PHDE_CK(ctx, cudaMemcpyAsync(d_y, y, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(keys, 0xff, sizeof(ull) * 2, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(keys + 2, 0, sizeof(ull) * 2 + sizeof(int) * 2, ctx->stream));
  draw_bounds_kernel<<<grid_of(ctx, n, 256), 256, 0, ctx->stream>>>(d_x, d_y, n, keys, bad);
  PHDE_LAUNCHED(ctx);
  ull hk[5];
  PHDE_CK(ctx, cudaMemcpyAsync(hk, keys, sizeof(ull) * 4 + sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  cudaEventRecord(ctx->ev[1], ctx->stream);
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  int hbad = 0;
  memcpy(&hbad, &hk[4], sizeof(int));
  if (hbad) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_draw: a coordinate is not finite");

  // bounds start at 1 and -1 (draw_graph.c:201-204, 223-226); size as draw_graph.c:233-249
  const double dxlo = key_value(hk[0]), dylo = key_value(hk[1]), dxhi = key_value(hk[2]), dyhi = key_value(hk[3]);
  const double xmin = dxlo < 1.0 ? dxlo : 1.0, ymin = dylo < 1.0 ? dylo : 1.0;
  const double xmax = dxhi > -1.0 ? dxhi : -1.0, ymax = dyhi > -1.0 ? dyhi : -1.0;
  const double aspect = (xmax - xmin) / (ymax - ymin);
  const double wd = std::sqrt((double)(100 * n) / aspect);
  if (!(wd >= 1.0 && wd < 4294967296.0))
    return phde_fail(ctx, PHDE_ERR_INVALID, "phde_draw: the image width is not a positive 32-bit number (degenerate "
                                            "coordinate range)");
  const unsigned w0 = (unsigned)wd;
  const double hd = aspect * (double)w0;
  if (!(hd >= 1.0 && hd < 4294967296.0))
    return phde_fail(ctx, PHDE_ERR_INVALID, "phde_draw: the image height is not a positive 32-bit number");
  const unsigned h0 = (unsigned)hd;
  unsigned W = w0, H = h0;
  if (W > 100000 || H > 100000) {
    W /= 10;
    H /= 10;
  } else if (W > 20000 || H > 20000) {
    W /= 5;
    H /= 5;
  }
  if (W == 0 || H == 0) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_draw: the corrected image size is 0");
  if (W > MAX_SIDE || H > MAX_SIDE || (uint64_t)((W + 7) >> 3) * ((H + 7) >> 3) * 64 > (1ull << 31))
    return phde_fail(ctx, PHDE_ERR_TOO_LARGE, "phde_draw: the image exceeds 2^20 pixels a side or 2^31 pixels");
  const double xri = 1.0 / (xmax - xmin), yri = 1.0 / (ymax - ymin);

  const size_t S = 1 + ((size_t)W + 1) / 2;
  const size_t npix_tiled = (size_t)((W + 7) >> 3) * ((H + 7) >> 3) * 64;  // >= W * H
  const int64_t ntiles = (nnz + RT - 1) / RT;
  uint32_t *owner = (uint32_t *)phde_buf(ctx, "draw.owner", sizeof(uint32_t) * npix_tiled);
  uint8_t *packed = (uint8_t *)phde_buf(ctx, "draw.packed", S * H);
  uint32_t *erow = (uint32_t *)phde_buf(ctx, "draw.erow", sizeof(uint32_t) * std::max<int64_t>(nnz, 1));
  uint8_t *bin = (uint8_t *)phde_buf(ctx, "draw.bin", std::max<int64_t>(nnz, 1));
  uint32_t *tcnt = (uint32_t *)phde_buf(ctx, "draw.tcnt", sizeof(uint32_t) * 4 * std::max<int64_t>(ntiles, 1));
  ull *misc = (ull *)phde_buf(ctx, "draw.misc", sizeof(ull) * 8);
  if (!owner || !packed || !erow || !bin || !tcnt || !misc) return PHDE_ERR_OOM;
  unsigned *maxbits = (unsigned *)misc;        // misc[0] low word
  ull *pixels = misc + 1;
  int64_t *cuts = (int64_t *)(misc + 2);       // misc[2..5]
  cudaEventRecord(ctx->ev[2], ctx->stream);
  if (ctx->draw_rows_epoch != ctx->graph_epoch || ctx->draw_rows_buf != (void *)erow) {
    if (nnz > 0) {
      draw_rows_kernel<<<grid_of(ctx, n * 32, 256), 256, 0, ctx->stream>>>(ctx->d_off, n, erow);
      PHDE_LAUNCHED(ctx);
    }
    ctx->draw_rows_epoch = ctx->graph_epoch;
    ctx->draw_rows_buf = erow;
  }
  draw_scale_kernel<<<grid_of(ctx, n, 256), 256, 0, ctx->stream>>>(d_x, d_y, n, xmin, ymin, xri, yri, W, H, pix);
  PHDE_LAUNCHED(ctx);
  PHDE_CK(ctx, cudaMemsetAsync(misc, 0, sizeof(ull) * 8, ctx->stream));
  PHDE_CK(ctx, cudaMemsetAsync(owner, 0, sizeof(uint32_t) * npix_tiled, ctx->stream));
  if (nnz > 0) {
    draw_maxlen_kernel<<<grid_of(ctx, nnz, 256), 256, 0, ctx->stream>>>(erow, ctx->d_adj, pix, nnz, maxbits);
    PHDE_LAUNCHED(ctx);
    cudaEventRecord(ctx->ev[3], ctx->stream);
    const char *rv = getenv("PHDE_DRAW_RASTER");
    if (rv && strcmp(rv, "plain") == 0)
      draw_raster_kernel<false><<<(unsigned)ntiles, RT_THREADS, 0, ctx->stream>>>(erow, ctx->d_adj, pix, nnz, maxbits,
                                                                                  W, H, owner, bin, tcnt, pixels);
    else
      draw_raster_kernel<true><<<(unsigned)ntiles, RT_THREADS, 0, ctx->stream>>>(erow, ctx->d_adj, pix, nnz, maxbits,
                                                                                 W, H, owner, bin, tcnt, pixels);
    PHDE_LAUNCHED(ctx);
    cudaEventRecord(ctx->ev[4], ctx->stream);
    const int64_t m = nnz / 2;  // g.m = m / 2 (draw_graph.c:181), handed to draw_line
    draw_cuts_kernel<<<1, SEL_THREADS, 0, ctx->stream>>>(bin, tcnt, ntiles, nnz, m, counter_limit(m), cuts);
    PHDE_LAUNCHED(ctx);
  } else {
    cudaEventRecord(ctx->ev[3], ctx->stream);
    cudaEventRecord(ctx->ev[4], ctx->stream);
  }
  draw_pack_kernel<<<(unsigned)std::min<size_t>(H, (size_t)ctx->nsm * 16), 256, 0, ctx->stream>>>(owner, bin, cuts, W,
                                                                                                 H, S, packed);
  PHDE_LAUNCHED(ctx);
  ull hm[2] = {0, 0};
  PHDE_CK(ctx, cudaMemcpyAsync(hm, misc, sizeof(ull) * 2, cudaMemcpyDeviceToHost, ctx->stream));
  cudaEventRecord(ctx->ev[5], ctx->stream);
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->draw_W = W;
  ctx->draw_H = H;
  ctx->draw_epoch = ctx->graph_epoch;
  if (info) {
    memset(info, 0, sizeof(*info));
    info->width = W;
    info->height = H;
    info->width_computed = w0;
    info->height_computed = h0;
    info->xmin = xmin;
    info->xmax = xmax;
    info->ymin = ymin;
    info->ymax = ymax;
    info->aspect = aspect;
    unsigned mb = (unsigned)(hm[0] & 0xffffffffu);
    memcpy(&info->max_edge_length, &mb, sizeof(float));
    info->pixels = (int64_t)hm[1];
    float t01 = 0, t25 = 0, t34 = 0;
    cudaEventElapsedTime(&t01, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&t25, ctx->ev[2], ctx->ev[5]);
    cudaEventElapsedTime(&t34, ctx->ev[3], ctx->ev[4]);
    info->ms_device = (double)t01 + (double)t25;
    info->ms_raster = t34;
    info->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_host0).count();
    info->gpu_launches = (int)(ctx->launches - launches0);
  }
  return PHDE_OK;
}

extern "C" int phde_draw_download(phde_ctx *ctx, uint8_t *rgba, size_t bytes) {
  if (!ctx) return PHDE_ERR_INVALID;
  if (ctx->draw_W == 0) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_draw_download: nothing drawn");
  const unsigned W = ctx->draw_W, H = ctx->draw_H;
  const size_t npix = (size_t)W * H, S = 1 + ((size_t)W + 1) / 2;
  if (!rgba || bytes < npix * 4) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_draw_download: buffer too small");
  PHDE_CK(ctx, cudaSetDevice(ctx->device));
  uint8_t *packed = (uint8_t *)phde_buf(ctx, "draw.packed", S * H);
  uint32_t *out = (uint32_t *)phde_buf(ctx, "draw.owner", sizeof(uint32_t) * npix);  // owners are spent
  if (!packed || !out) return PHDE_ERR_OOM;
  draw_expand_kernel<<<grid_of(ctx, (int64_t)npix, 256), 256, 0, ctx->stream>>>(packed, W, H, S, out);
  PHDE_LAUNCHED(ctx);
  PHDE_CK(ctx, cudaMemcpyAsync(rgba, out, npix * 4, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return PHDE_OK;
}

// The packed scanlines (H rows of 1 + ceil(W / 2) bytes) on the host; used by the PNG writer.
int phde_draw_scanlines(phde_ctx *ctx, std::vector<uint8_t> &out, unsigned &W, unsigned &H) {
  if (ctx->draw_W == 0) return phde_fail(ctx, PHDE_ERR_INVALID, "nothing drawn");
  W = ctx->draw_W;
  H = ctx->draw_H;
  const size_t S = 1 + ((size_t)W + 1) / 2;
  uint8_t *packed = (uint8_t *)phde_buf(ctx, "draw.packed", S * H);
  if (!packed) return PHDE_ERR_OOM;
  out.resize(S * H);
  PHDE_CK(ctx, cudaSetDevice(ctx->device));
  PHDE_CK(ctx, cudaMemcpyAsync(out.data(), packed, S * H, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return PHDE_OK;
}

// The drawn image as a PNG file: 4-bit palette (the nine colours above, in code order).
extern "C" int phde_draw_write_png(phde_ctx *ctx, const char *path, int nthreads) {
  if (!ctx) return PHDE_ERR_INVALID;
  if (!path) return phde_fail(ctx, PHDE_ERR_INVALID, "phde_draw_write_png: null path");
  std::vector<uint8_t> rows;
  unsigned W = 0, H = 0;
  int rc = phde_draw_scanlines(ctx, rows, W, H);
  if (rc) return rc;
  uint32_t pal[9];
  PHDE_CK(ctx, cudaMemcpyFromSymbol(pal, c_palette, sizeof(pal)));
  if (phde_png_write_rows(path, rows.data(), W, H, 4, 3, pal, 9, nthreads) != 0)
    return phde_fail(ctx, PHDE_ERR_INVALID, std::string("phde_draw_write_png: cannot write ") + path);
  return PHDE_OK;
}
