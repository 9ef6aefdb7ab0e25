/*
 * parhde_oracle.c -- CPU restatement of the ParHDE layout pipeline.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU product and the CPU baseline
 * that bench.py times.  Only tests/, __graft_entry__.smoke() and bench.py load it; nothing in the
 * product (the icpp_2020_parhde_gb300 package, libparhde_gb300.so, the embed binary) links or calls it.
 *
 * Each routine restates, in code of its own, the algorithm of the reference file:line it cites
 * (paths are relative to the ParHDE source tree).  The restatement is pinned against the reference
 * itself: oracle/build_ref.sh compiles the reference sources into oracle/_ref/, and
 * tests/golden/make_golden.py records its outputs (distance columns, Kcenters pivot order, final
 * coordinates at one OpenMP thread) as fixtures that tests/test_oracle.py compares against.
 *
 * Two distance back ends are provided for every pipeline:
 *   dist_algo = 0  the reference's parallel algorithms (direction-optimising BFS, gapbs/bfs.cc:43-185;
 *                  delta-stepping SSSP, gapbs/sssp.cc:53-140) restated with OpenMP -- the timed baseline;
 *   dist_algo = 1  textbook serial BFS / Dijkstra -- the simplest possible checker.
 * Both produce identical integer distances (shortest-path lengths are unique), which the tests assert.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <math.h>
#include <limits.h>
#include <omp.h>

#define ORC_OK 0
#define ORC_ERR_INVALID (-1)
#define ORC_ERR_CSR (-2)
#define ORC_ERR_DISCONNECTED (-3)
#define ORC_ERR_K_RANGE (-4)
#define ORC_ERR_TOO_FEW_PIVOTS (-5)
#define ORC_ERR_OOM (-6)
#define ORC_ERR_NOCONVERGE (-7)
#define ORC_ERR_WEIGHTS (-10)

/* algorithm ids: spectralDrawing.cpp:101-109 */
#define ALGO_PIVOTMDS 0
#define ALGO_PHDE 1
#define ALGO_WPARHDE 2
#define ALGO_PARHDE 3
/* pivot strategies (doRand): spectralDrawing.cpp:88-94 */
#define STRAT_RANDCOARSE 0
#define STRAT_RANDFINE 1
#define STRAT_KCENTERS 2

#define SSSP_INF ((int32_t)(INT32_MAX / 2)) /* kDistInf, gapbs/sssp.cc:50 */

typedef struct {
  int algo, strategy, k, c;
  int eig;       /* 0: subspace power iteration (ParallelComponents.cpp:48-158); 1: exact (Jacobi) */
  int dist_algo; /* 0: reference-structured parallel; 1: serial textbook */
  int nthreads;  /* 0: OpenMP default */
  int verbose;
  uint64_t seed; /* random pivot strategies */
} orc_opts;

typedef struct {
  int status;
  int npasses;   /* distance passes (BFS/SSSP) executed */
  int naccepted; /* vectors accepted by the D-orthogonalisation */
  int ndiscarded;
  int eig_iters;
  double t_dist, t_orth, t_mmult, t_eig, t_coords, t_total; /* seconds */
} orc_stats;

int orc_abi_version(void) { return 3; }

static double now_s(void) { return omp_get_wtime(); }

/* ------------------------------------------------------------------------------------------ */
/* glibc rand() stream.  The reference seeds its eigensolver with srand(1) and draws rand()/RAND_MAX
 * (ParallelComponents.cpp:56-63) and draws random pivots with rand() % n (ParHDE.cpp:160-162,
 * DrawingBase.cpp:175-177).  This is the published TYPE_3 additive-feedback generator glibc uses
 * (degree 31, separation 3, Park-Miller seeding, 310 discarded outputs), restated so that the
 * oracle does not disturb the process-wide rand() state.  tests/test_oracle.py checks it against
 * libc's own rand(). */
void orc_glibc_rand(uint32_t seed, int count, int32_t *out) {
  int total = count + 344;
  int32_t *r = (int32_t *)malloc(sizeof(int32_t) * (size_t)total);
  if (seed == 0) seed = 1;
  r[0] = (int32_t)seed;
  for (int i = 1; i < 31; i++) {
    int32_t hi = r[i - 1] / 127773, lo = r[i - 1] % 127773;
    int32_t word = 16807 * lo - 2836 * hi;
    if (word < 0) word += 2147483647;
    r[i] = word;
  }
  for (int i = 31; i < 34; i++) r[i] = r[i - 31];
  for (int i = 34; i < total; i++) r[i] = (int32_t)((uint32_t)r[i - 31] + (uint32_t)r[i - 3]);
  for (int i = 0; i < count; i++) out[i] = (int32_t)(((uint32_t)r[i + 344]) >> 1);
  free(r);
}

/* ------------------------------------------------------------------------------------------ */
/* CSR validation: offsets start at 0, are monotone and end at m; every neighbour is < n. */
int orc_check_csr(const uint32_t *off, const uint32_t *adj, int64_t n, int64_t m) {
  if (n <= 0 || m < 0) return ORC_ERR_INVALID;
  if (off[0] != 0 || (int64_t)off[n] != m) return ORC_ERR_CSR;
  for (int64_t i = 0; i < n; i++)
    if (off[i + 1] < off[i]) return ORC_ERR_CSR;
  for (int64_t j = 0; j < m; j++)
    if ((int64_t)adj[j] >= n) return ORC_ERR_CSR;
  return ORC_OK;
}

/* ------------------------------------------------------------------------------------------ */
/* Serial textbook BFS (checker).  dist[v] = hop count, -1 when unreachable. */
void orc_bfs_serial(const uint32_t *off, const uint32_t *adj, int64_t n, int64_t src, int32_t *dist) {
  uint32_t *q = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n);
  for (int64_t i = 0; i < n; i++) dist[i] = -1;
  int64_t head = 0, tail = 0;
  q[tail++] = (uint32_t)src;
  dist[src] = 0;
  while (head < tail) {
    uint32_t u = q[head++];
    int32_t du = dist[u];
    for (uint32_t j = off[u]; j < off[u + 1]; j++) {
      uint32_t v = adj[j];
      if (dist[v] < 0) {
        dist[v] = du + 1;
        q[tail++] = v;
      }
    }
  }
  free(q);
}

/* ------------------------------------------------------------------------------------------ */
/* Direction-optimising BFS with OpenMP, restating gapbs/bfs.cc:43-185 (Beamer et al., SC'12):
 * parent[] holds -degree for unvisited vertices (InitParent, bfs.cc:134-141); top-down steps claim
 * vertices by compare-and-swap on parent (TDStep, bfs.cc:76-106) and report the edges leaving the new
 * frontier; bottom-up steps let every unvisited vertex look for a parent in the frontier bitmap
 * (BUStep, bfs.cc:48-73); the switch rule is scout > edges_to_check/alpha, and bottom-up continues
 * while the frontier grows or stays above n/beta (DOBFS, bfs.cc:144-185).  Output: hop counts in dist
 * (-1 when unreachable; the reference leaves those entries unwritten). */
typedef struct {
  int64_t *buf;
  int64_t in, out_start, out_end;
} orc_queue;

static inline int bm_get(const uint64_t *bm, int64_t i) { return (int)((bm[i >> 6] >> (i & 63)) & 1ull); }

void orc_dobfs(const uint32_t *off, const uint32_t *adj, int64_t n, int64_t m, int64_t src, int32_t *dist,
               int alpha, int beta) {
  int64_t *parent = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
  int64_t words = (n + 63) / 64;
  uint64_t *front = (uint64_t *)calloc((size_t)words, 8);
  uint64_t *next = (uint64_t *)calloc((size_t)words, 8);
  orc_queue q;
  q.buf = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
  q.in = q.out_start = q.out_end = 0;

#pragma omp parallel for
  for (int64_t v = 0; v < n; v++) {
    int64_t d = (int64_t)(off[v + 1] - off[v]);
    parent[v] = d != 0 ? -d : -1;
    dist[v] = -1;
  }
  parent[src] = src;
  dist[src] = 0;
  q.buf[q.in++] = src;
  q.out_start = q.out_end;
  q.out_end = q.in;

  int64_t edges_to_check = m;
  int64_t scout = (int64_t)(off[src + 1] - off[src]);
  int32_t level = 0;
  while (q.out_start != q.out_end) {
    if (scout > edges_to_check / alpha) {
      /* queue -> bitmap */
      memset(front, 0, (size_t)words * 8);
#pragma omp parallel for
      for (int64_t e = q.out_start; e < q.out_end; e++) {
        int64_t u = q.buf[e];
        __atomic_fetch_or(&front[u >> 6], 1ull << (u & 63), __ATOMIC_RELAXED);
      }
      int64_t awake = q.out_end - q.out_start, old_awake;
      q.out_start = q.out_end;
      q.out_end = q.in;
      do {
        old_awake = awake;
        awake = 0;
        memset(next, 0, (size_t)words * 8);
        int32_t lv = level;
#pragma omp parallel for reduction(+ : awake) schedule(dynamic, 1024)
        for (int64_t u = 0; u < n; u++) {
          if (parent[u] < 0) {
            for (uint32_t j = off[u]; j < off[u + 1]; j++) {
              int64_t v = adj[j];
              if (bm_get(front, v)) {
                parent[u] = v;
                dist[u] = lv + 1;
                awake++;
                __atomic_fetch_or(&next[u >> 6], 1ull << (u & 63), __ATOMIC_RELAXED);
                break;
              }
            }
          }
        }
        level++;
        uint64_t *t = front;
        front = next;
        next = t;
      } while (awake >= old_awake || awake > n / (int64_t)beta);
      /* bitmap -> queue */
      int64_t base = q.in;
      int64_t cnt = 0;
      for (int64_t u = 0; u < n; u++)
        if (bm_get(front, u)) q.buf[base + cnt++] = u;
      q.in = base + cnt;
      q.out_start = q.out_end;
      q.out_end = q.in;
      scout = 1;
    } else {
      edges_to_check -= scout;
      int64_t sc = 0;
      int32_t lv = level;
      int64_t qb = q.out_start, qe = q.out_end;
#pragma omp parallel reduction(+ : sc)
      {
        int64_t cap = 1024, len = 0;
        int64_t *local = (int64_t *)malloc(sizeof(int64_t) * (size_t)cap);
#pragma omp for schedule(dynamic, 64)
        for (int64_t e = qb; e < qe; e++) {
          int64_t u = q.buf[e];
          for (uint32_t j = off[u]; j < off[u + 1]; j++) {
            int64_t v = adj[j];
            int64_t cur = __atomic_load_n(&parent[v], __ATOMIC_RELAXED);
            if (cur < 0) {
              if (__atomic_compare_exchange_n(&parent[v], &cur, u, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
                if (len == cap) {
                  cap *= 2;
                  local = (int64_t *)realloc(local, sizeof(int64_t) * (size_t)cap);
                }
                local[len++] = v;
                sc += -cur;
                dist[v] = lv + 1;
              }
            }
          }
        }
        int64_t at = __atomic_fetch_add(&q.in, len, __ATOMIC_RELAXED);
        memcpy(q.buf + at, local, sizeof(int64_t) * (size_t)len);
        free(local);
      }
      scout = sc;
      level++;
      q.out_start = q.out_end;
      q.out_end = q.in;
    }
    /* the queue buffer is a sliding window over at most n pushes per BFS */
  }
  free(parent);
  free(front);
  free(next);
  free(q.buf);
}

/* ------------------------------------------------------------------------------------------ */
/* Serial Dijkstra with a binary heap (checker).  dist[v] = weighted distance, SSSP_INF when unreachable. */
void orc_dijkstra(const uint32_t *off, const uint32_t *adj, const int32_t *w, int64_t n, int64_t src,
                  int32_t *dist) {
  typedef struct {
    int64_t d;
    int64_t v;
  } hent;
  int64_t cap = 1024, sz = 0;
  hent *h = (hent *)malloc(sizeof(hent) * (size_t)cap);
  int64_t *best = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
  for (int64_t i = 0; i < n; i++) best[i] = INT64_MAX;
  best[src] = 0;
  h[sz++] = (hent){0, src};
  while (sz) {
    hent top = h[0];
    h[0] = h[--sz];
    for (int64_t i = 0;;) { /* sift down */
      int64_t l = 2 * i + 1, r = l + 1, s = i;
      if (l < sz && h[l].d < h[s].d) s = l;
      if (r < sz && h[r].d < h[s].d) s = r;
      if (s == i) break;
      hent t = h[i];
      h[i] = h[s];
      h[s] = t;
      i = s;
    }
    if (top.d > best[top.v]) continue;
    for (uint32_t j = off[top.v]; j < off[top.v + 1]; j++) {
      int64_t v = adj[j];
      int64_t nd = top.d + w[j];
      if (nd < best[v]) {
        best[v] = nd;
        if (sz == cap) {
          cap *= 2;
          h = (hent *)realloc(h, sizeof(hent) * (size_t)cap);
        }
        int64_t i = sz++;
        h[i] = (hent){nd, v};
        while (i > 0) { /* sift up */
          int64_t p = (i - 1) / 2;
          if (h[p].d <= h[i].d) break;
          hent t = h[p];
          h[p] = h[i];
          h[i] = t;
          i = p;
        }
      }
    }
  }
  for (int64_t i = 0; i < n; i++) dist[i] = best[i] == INT64_MAX ? SSSP_INF : (int32_t)best[i];
  free(h);
  free(best);
}

/* ------------------------------------------------------------------------------------------ */
/* Delta-stepping SSSP with OpenMP, restating gapbs/sssp.cc:53-140 (Meyer & Sanders 2003): thread-local
 * bins of width delta, CAS-min relaxation of every out-edge of a frontier vertex whose distance is
 * still inside the current bin, a vote for the smallest non-empty bin, and a shared frontier that
 * every thread refills from its copy of that bin.  Vertices are never removed from older bins; stale
 * entries are skipped by the dist >= delta*bin test (sssp.cc:60-62). */
typedef struct {
  int64_t *v;
  int64_t len, cap;
} orc_vec;

static void vec_push(orc_vec *b, int64_t x) {
  if (b->len == b->cap) {
    b->cap = b->cap ? 2 * b->cap : 64;
    b->v = (int64_t *)realloc(b->v, sizeof(int64_t) * (size_t)b->cap);
  }
  b->v[b->len++] = x;
}

void orc_deltastep(const uint32_t *off, const uint32_t *adj, const int32_t *w, int64_t n, int64_t m, int64_t src,
                   int32_t *dist, int32_t delta) {
  const size_t kMaxBin = SIZE_MAX / 2;
  for (int64_t i = 0; i < n; i++) dist[i] = SSSP_INF;
  dist[src] = 0;
  int64_t *frontier = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m > 1 ? m : 1));
  size_t shared_idx[2] = {0, kMaxBin};
  size_t tails[2] = {1, 0};
  frontier[0] = src;
#pragma omp parallel
  {
    orc_vec *bins = NULL;
    size_t nbins = 0;
    size_t iter = 0;
    while (__atomic_load_n(&shared_idx[iter & 1], __ATOMIC_SEQ_CST) != kMaxBin) {
      size_t *cur_bin = &shared_idx[iter & 1];
      size_t *next_bin = &shared_idx[(iter + 1) & 1];
      size_t *cur_tail = &tails[iter & 1];
      size_t *next_tail = &tails[(iter + 1) & 1];
      size_t cb = *cur_bin;
      size_t ct = *cur_tail;
#pragma omp for nowait schedule(dynamic, 64)
      for (size_t i = 0; i < ct; i++) {
        int64_t u = frontier[i];
        int32_t du = __atomic_load_n(&dist[u], __ATOMIC_RELAXED);
        if ((int64_t)du >= (int64_t)delta * (int64_t)cb) {
          for (uint32_t j = off[u]; j < off[u + 1]; j++) {
            int64_t v = adj[j];
            int32_t old = __atomic_load_n(&dist[v], __ATOMIC_RELAXED);
            int32_t nd = du + w[j];
            if (nd < old) {
              int changed = 1;
              while (!__atomic_compare_exchange_n(&dist[v], &old, nd, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
                if (old <= nd) {
                  changed = 0;
                  break;
                }
              }
              if (changed) {
                size_t b = (size_t)(nd / delta);
                if (b >= nbins) {
                  bins = (orc_vec *)realloc(bins, sizeof(orc_vec) * (b + 1));
                  memset(bins + nbins, 0, sizeof(orc_vec) * (b + 1 - nbins));
                  nbins = b + 1;
                }
                vec_push(&bins[b], v);
              }
            }
          }
        }
      }
      for (size_t i = cb; i < nbins; i++) {
        if (bins[i].len) {
#pragma omp critical
          {
            if (i < *next_bin) *next_bin = i;
          }
          break;
        }
      }
#pragma omp barrier
#pragma omp single nowait
      {
        *cur_bin = kMaxBin;
        *cur_tail = 0;
      }
      size_t nb = *next_bin;
      if (nb < nbins) {
        size_t at = __atomic_fetch_add(next_tail, (size_t)bins[nb].len, __ATOMIC_SEQ_CST);
        memcpy(frontier + at, bins[nb].v, sizeof(int64_t) * (size_t)bins[nb].len);
        bins[nb].len = 0;
      }
      iter++;
#pragma omp barrier
    }
    for (size_t i = 0; i < nbins; i++) free(bins[i].v);
    free(bins);
  }
  free(frontier);
}

/* ------------------------------------------------------------------------------------------ */
/* One distance pass from src into dist (int32). */
static void distance_pass(const orc_opts *o, const uint32_t *off, const uint32_t *adj, const int32_t *w, int64_t n,
                          int64_t m, int64_t src, int32_t *dist) {
  if (w == NULL) {
    if (o->dist_algo == 1)
      orc_bfs_serial(off, adj, n, src, dist);
    else
      orc_dobfs(off, adj, n, m, src, dist, 15, 18); /* beta forced to 18: DrawingBase.cpp:114 */
  } else {
    if (o->dist_algo == 1)
      orc_dijkstra(off, adj, w, n, src, dist);
    else
      orc_deltastep(off, adj, w, n, m, src, dist, 10000); /* delta: WParHDE.cpp:104 */
  }
}

static int reached_all(const int32_t *dist, int64_t n, int weighted) {
  for (int64_t i = 0; i < n; i++)
    if (weighted ? dist[i] >= SSSP_INF : dist[i] < 0) return 0;
  return 1;
}

/* ------------------------------------------------------------------------------------------ */
/* Kcenters selection step.  Folds one distance column into min_d (the running minimum over all
 * pivots so far) and returns the vertex farthest from the pivot set, lowest index first: the strict
 * '>' scan of ParHDE.cpp:130-139 / WParHDE.cpp:123-134 / DrawingBase.cpp:415-424 run by one thread.
 * If that vertex is already in `hist` and check_fix is set, the duplicate fix-up of ParHDE.cpp:144-154
 * (and its twins WParHDE.cpp:139-151, DrawingBase.cpp:428-438) picks, as one thread does, the LAST
 * vertex with the same minimum distance that is not in `hist`.  *raw receives the unadjusted argmax. */
static int in_hist(const int64_t *hist, int nh, int64_t v) {
  for (int i = 0; i < nh; i++)
    if (hist[i] == v) return 1;
  return 0;
}

static int64_t kcenters_step(int64_t *min_d, const int32_t *col, int64_t n, int check_fix, const int64_t *hist,
                             int nh, int64_t *raw) {
  int64_t best_val = -1, best_idx = 0;
#pragma omp parallel
  {
    int64_t bv = -1, bi = 0;
#pragma omp for schedule(static)
    for (int64_t i = 0; i < n; i++) {
      int64_t d = col[i];
      if (d < min_d[i]) min_d[i] = d;
      if (min_d[i] > bv) {
        bv = min_d[i];
        bi = i;
      }
    }
#pragma omp critical
    {
      if (bv > best_val || (bv == best_val && bi < best_idx)) {
        best_val = bv;
        best_idx = bi;
      }
    }
  }
  *raw = best_idx;
  int64_t next = best_idx;
  if (check_fix && in_hist(hist, nh, best_idx)) {
    for (int64_t i = 0; i < n; i++)
      if (min_d[i] == best_val && !in_hist(hist, nh, i)) next = i;
  }
  return next;
}

/* Pivot sources for the random strategies.  The reference draws rand() % n after srand(time(NULL))
 * (ParHDE.cpp:113,160-162) or without seeding (DrawingBase.cpp:175-177), writes P entries into an
 * array of k, and reads index run_count-1 at run_count = 0 (DrawingBase.cpp:182,187).  Here the glibc
 * stream is seeded with opts.seed (1 reproduces an unseeded process) and exactly `count` sources are
 * drawn in order. */
static void random_sources(uint64_t seed, int64_t n, int count, int64_t *src) {
  int32_t *r = (int32_t *)malloc(sizeof(int32_t) * (size_t)count);
  orc_glibc_rand((uint32_t)seed, count, r);
  for (int i = 0; i < count; i++) src[i] = (int64_t)r[i] % n;
  free(r);
}

/* ------------------------------------------------------------------------------------------ */
/* Dense helpers (FP64).  Sums use a fixed static schedule so a given thread count is deterministic. */
static double sum_sq(const double *x, int64_t n) { /* ParallelComponents::normL2 without the sqrt */
  double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t i = 0; i < n; i++) s += x[i] * x[i];
  return s;
}

/* C[q + p*k] = sum_i A[i + p*n] * B[i + q*n]: matrixTransMultiplication, DrawingBase.cpp:221-244. */
static void gram_t(const double *A, const double *B, double *C, int64_t n, int k) {
#pragma omp parallel for collapse(2) schedule(guided)
  for (int p = 0; p < k; p++)
    for (int q = 0; q < k; q++) {
      double s = 0;
      const double *a = A + (int64_t)p * n, *b = B + (int64_t)q * n;
      for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
      C[q + (int64_t)p * k] = s;
    }
}

/* X[i + t*n] = sum_j M[i + j*n] * Y[j + t*k]: computeCoordinates, DrawingBase.cpp:207-219. */
static void coords_from(const double *M, const double *Y, double *X, int64_t n, int k, int c) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++)
    for (int t = 0; t < c; t++) {
      double s = 0;
      for (int j = 0; j < k; j++) s += M[i + (int64_t)j * n] * Y[j + (int64_t)t * k];
      X[i + (int64_t)t * n] = s;
    }
}

/* getCoordinates: every coordinate column scaled to unit L2 norm, DrawingBase.cpp:196-205. */
static void normalise_coords(double *X, int64_t n, int c) {
  for (int t = 0; t < c; t++) {
    double inv = 1.0 / sqrt(sum_sq(X + (int64_t)t * n, n));
    for (int64_t i = 0; i < n; i++) X[i + (int64_t)t * n] *= inv;
  }
}

/* ------------------------------------------------------------------------------------------ */
/* Subspace power iteration, restating ParallelComponents.cpp:48-158: s = N random start vectors from
 * srand(1)/rand()/RAND_MAX, each sweep multiplies by K, Gram-Schmidts every vector against the ones
 * before it, renormalises, and stops when every vector moved by less than |cos| = 0.999.  On exit
 * the columns of K are overwritten with the vectors in ascending order of |eigenvalue| (vector i goes
 * to column N-1-i, negated when the first entry of eVecs column N-1-i is negative -- the reference's
 * sign rule, ParallelComponents.cpp:140-153).  evals receives the norms in ascending order. */
static int power_method(double *K, double *evals, int N, int *iters_out) {
  const int s = N;
  double *E = (double *)malloc(sizeof(double) * (size_t)N * N);
  double *T = (double *)malloc(sizeof(double) * (size_t)N * N);
  int32_t *r = (int32_t *)malloc(sizeof(int32_t) * (size_t)N * N);
  orc_glibc_rand(1, N * N, r);
  for (int i = 0; i < s; i++)
    for (int j = 0; j < N; j++) E[j + i * N] = (double)r[i * N + j] / 2147483647.0;
  free(r);
  for (int i = 0; i < s; i++) {
    double nv = 0;
    for (int j = 0; j < N; j++) nv += E[j + i * N] * E[j + i * N];
    evals[i] = sqrt(nv);
    for (int j = 0; j < N; j++) E[j + i * N] /= evals[i];
  }
  double rr = 0;
  int it = 0, status = ORC_OK;
  while (rr < 1.0 - 1e-3) {
    it++;
    if (isnan(rr) || isinf(rr) || it > 20000) {
      status = ORC_ERR_NOCONVERGE;
      break;
    }
    memcpy(T, E, sizeof(double) * (size_t)N * N);
    memset(E, 0, sizeof(double) * (size_t)N * N);
    for (int i = 0; i < s; i++)
      for (int j = 0; j < N; j++) {
        double t = T[j + i * N];
        for (int kk = 0; kk < N; kk++) E[kk + i * N] += K[kk + j * N] * t;
      }
    for (int i = 0; i < s; i++)
      for (int j = 0; j < i; j++) {
        double a = 0, b = 0;
        for (int kk = 0; kk < N; kk++) a += E[kk + j * N] * E[kk + i * N];
        for (int kk = 0; kk < N; kk++) b += E[kk + j * N] * E[kk + j * N];
        double fac = a / b;
        for (int kk = 0; kk < N; kk++) E[kk + i * N] -= fac * E[kk + j * N];
      }
    for (int i = 0; i < s; i++) {
      double nv = 0;
      for (int j = 0; j < N; j++) nv += E[j + i * N] * E[j + i * N];
      evals[i] = sqrt(nv);
      for (int j = 0; j < N; j++) E[j + i * N] /= evals[i];
    }
    rr = 1;
    for (int i = 0; i < s; i++) {
      double d = 0;
      for (int j = 0; j < N; j++) d += E[j + i * N] * T[j + i * N];
      if (d < 0) d = -d;
      if (d < rr) rr = d;
    }
  }
  for (int a = 0, b = s - 1; a < b; a++, b--) {
    double t = evals[a];
    evals[a] = evals[b];
    evals[b] = t;
  }
  for (int i = 0; i < s; i++) {
    int neg = E[(s - i - 1) * N] < 0;
    for (int j = 0; j < N; j++) K[j + (s - i - 1) * N] = neg ? -E[j + i * N] : E[j + i * N];
  }
  free(E);
  free(T);
  *iters_out = it;
  return status;
}

/* Exact symmetric eigensolve (the role LAPACKE_dsyev plays in the MKL build, DrawingBase.cpp:62,91):
 * cyclic Jacobi on the symmetric part of K.  On exit the columns of K hold eigenvectors in ascending
 * eigenvalue order, each signed so that its largest-magnitude entry (lowest index on ties) is
 * positive; evals ascending. */
static int jacobi_eig(double *K, double *evals, int N, int *sweeps_out) {
  double *A = (double *)malloc(sizeof(double) * (size_t)N * N);
  double *V = (double *)calloc((size_t)N * N, sizeof(double));
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) A[i + j * N] = 0.5 * (K[i + j * N] + K[j + i * N]);
  for (int i = 0; i < N; i++) V[i + i * N] = 1.0;
  int sweep = 0;
  for (; sweep < 100; sweep++) {
    double off = 0, tot = 0;
    for (int j = 0; j < N; j++)
      for (int i = 0; i < N; i++) {
        double a = A[i + j * N] * A[i + j * N];
        tot += a;
        if (i != j) off += a;
      }
    if (off <= 1e-28 * tot || off == 0) break;
    for (int p = 0; p < N - 1; p++)
      for (int q = p + 1; q < N; q++) {
        double apq = A[p + q * N];
        if (apq == 0) continue;
        double app = A[p + p * N], aqq = A[q + q * N];
        double theta = (aqq - app) / (2 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
        double cs = 1 / sqrt(t * t + 1), sn = t * cs;
        for (int kk = 0; kk < N; kk++) { /* columns p,q */
          double akp = A[kk + p * N], akq = A[kk + q * N];
          A[kk + p * N] = cs * akp - sn * akq;
          A[kk + q * N] = sn * akp + cs * akq;
        }
        for (int kk = 0; kk < N; kk++) { /* rows p,q */
          double apk = A[p + kk * N], aqk = A[q + kk * N];
          A[p + kk * N] = cs * apk - sn * aqk;
          A[q + kk * N] = sn * apk + cs * aqk;
        }
        for (int kk = 0; kk < N; kk++) {
          double vkp = V[kk + p * N], vkq = V[kk + q * N];
          V[kk + p * N] = cs * vkp - sn * vkq;
          V[kk + q * N] = sn * vkp + cs * vkq;
        }
      }
  }
  /* sort ascending (selection sort, stable on ties by index) */
  int *ord = (int *)malloc(sizeof(int) * (size_t)N);
  for (int i = 0; i < N; i++) ord[i] = i;
  for (int i = 0; i < N; i++) {
    int b = i;
    for (int j = i + 1; j < N; j++)
      if (A[ord[j] + ord[j] * N] < A[ord[b] + ord[b] * N]) b = j;
    int t = ord[i];
    ord[i] = ord[b];
    ord[b] = t;
  }
  for (int c = 0; c < N; c++) {
    int src = ord[c];
    evals[c] = A[src + src * N];
    int arg = 0;
    for (int i = 1; i < N; i++)
      if (fabs(V[i + src * N]) > fabs(V[arg + src * N])) arg = i;
    double sg = V[arg + src * N] < 0 ? -1.0 : 1.0;
    for (int i = 0; i < N; i++) K[i + c * N] = sg * V[i + src * N];
  }
  free(ord);
  free(A);
  free(V);
  *sweeps_out = sweep;
  return ORC_OK;
}

/* compute_eigens (DrawingBase.cpp:39-108): eigensolve M in place, then pick c eigenvectors into Y.
 * First (ParHDE, WParHDE): columns 0..c-1 (smallest).  Largest (PivotMDS, PHDE): column N-1-j. */
static int eigen_pick(const orc_opts *o, double *M, int N, int c, int largest, double *Y, double *evals,
                      int *iters) {
  int st = o->eig == 1 ? jacobi_eig(M, evals, N, iters) : power_method(M, evals, N, iters);
  if (st) return st;
  for (int j = 0; j < c; j++) {
    int col = largest ? N - 1 - j : j;
    for (int i = 0; i < N; i++) Y[i + (int64_t)j * N] = M[i + (int64_t)col * N];
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------------------------------ */
/* ParHDE pipeline, ParHDE.cpp:45-352 (decoupled: all 3k distance passes first, then one pass of
 * classical Gram-Schmidt in the degree inner product). */
static int run_parhde(const orc_opts *o, const uint32_t *off, const uint32_t *adj, int64_t n, int64_t m,
                      double *coords, int64_t *sources, double *S_out, double *M_out, double *evec_out,
                      double *eval_out, orc_stats *st) {
  const int k = o->k, c = o->c, P = 3 * k;
  double t0 = now_s();
  double *deg = (double *)malloc(sizeof(double) * (size_t)n);
  for (int64_t i = 0; i < n; i++) deg[i] = (double)(off[i + 1] - off[i]); /* ParHDE.cpp:58-59 */
  int32_t *D = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * (size_t)P);
  double *U = (double *)malloc(sizeof(double) * (size_t)n * (size_t)(P + 1));
  double *S = (double *)malloc(sizeof(double) * (size_t)n * (size_t)k);
  int64_t *min_d = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
  int64_t *hist = (int64_t *)malloc(sizeof(int64_t) * (size_t)P);
  if (!deg || !D || !U || !S || !min_d || !hist) return ORC_ERR_OOM;

  /* column 0: the constant vector, L2-normalised (ParHDE.cpp:94-108) */
  for (int64_t i = 0; i < n; i++) {
    U[i] = 1.0;
    min_d[i] = INT_MAX;
  }
  {
    double inv = 1.0 / sqrt(sum_sq(U, n));
    for (int64_t i = 0; i < n; i++) U[i] = U[i] * inv;
  }
  /* distance passes (ParHDE.cpp:118-175) */
  if (o->strategy == STRAT_KCENTERS) {
    int64_t src = 0;
    for (int rc = 1; rc <= P; rc++) {
      int32_t *col = D + (int64_t)(rc - 1) * n;
      distance_pass(o, off, adj, NULL, n, m, src, col);
      sources[rc - 1] = src;
      if (rc == 1 && !reached_all(col, n, 0)) return ORC_ERR_DISCONNECTED;
      int64_t raw;
      int64_t nxt = kcenters_step(min_d, col, n, rc != 1, hist, rc - 1, &raw);
      hist[rc - 1] = raw; /* sources.insert(old_idx) inserts the unadjusted argmax, ParHDE.cpp:143,155 */
      src = nxt;
    }
  } else {
    random_sources(o->seed, n, P, sources);
    for (int rc = 1; rc <= P; rc++) {
      int32_t *col = D + (int64_t)(rc - 1) * n;
      distance_pass(o, off, adj, NULL, n, m, sources[rc - 1], col);
      if (!reached_all(col, n, 0)) return ORC_ERR_DISCONNECTED;
    }
  }
  st->npasses = P;
  /* normalise every distance column to unit L2 norm (ParHDE.cpp:176-185) */
#pragma omp parallel for schedule(static)
  for (int rc = 1; rc <= P; rc++) {
    const int32_t *col = D + (int64_t)(rc - 1) * n;
    double s = 0;
    for (int64_t i = 0; i < n; i++) s += (double)col[i] * (double)col[i];
    s = 1.0 / sqrt(s);
    double *u = U + (int64_t)rc * n;
    for (int64_t i = 0; i < n; i++) u[i] = (double)col[i] * s;
  }
  double t1 = now_s();
  st->t_dist = t1 - t0;

  /* classical Gram-Schmidt in the D inner product (ParHDE.cpp:190-285) */
  int correct = 1;
  double *num = (double *)malloc(sizeof(double) * (size_t)(k + 1));
  double *den = (double *)malloc(sizeof(double) * (size_t)(k + 1));
  for (int rc = 1; rc <= P; rc++) {
    if (correct > k) break;
    int j = correct;
    double *x = U + (int64_t)rc * n;
    for (int q = 0; q <= k; q++) num[q] = den[q] = 0;
    /* slot k holds the constant column (the reference keeps it in slot S_MAX-1) */
#pragma omp parallel
    {
      double ln[257], ld[257];
      for (int q = 0; q <= k; q++) ln[q] = ld[q] = 0;
#pragma omp for schedule(static)
      for (int64_t i = 0; i < n; i++) {
        double xi = x[i], di = deg[i];
        for (int q = 0; q < j - 1; q++) {
          double s = S[i + (int64_t)q * n];
          ln[q] += xi * s * di;
          ld[q] += s * s * di;
        }
        ln[k] += xi * U[i] * di;
        ld[k] += U[i] * U[i] * di;
      }
#pragma omp critical
      {
        for (int q = 0; q < j - 1; q++) {
          num[q] += ln[q];
          den[q] += ld[q];
        }
        num[k] += ln[k];
        den[k] += ld[k];
      }
    }
    for (int q = 0; q < j - 1; q++) den[q] = 1.0 / den[q];
    den[k] = 1.0 / den[k];
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
      double acc = 0;
      for (int q = 0; q < j - 1; q++) acc += num[q] * den[q] * S[i + (int64_t)q * n];
      acc += num[k] * den[k] * U[i];
      x[i] -= acc;
    }
    double nrm = sqrt(sum_sq(x, n));
    if (nrm < 0.001) { /* ParHDE.cpp:267-268 */
      st->ndiscarded++;
      if (o->verbose) printf("discarding vec %d, normdist %g\n", j, nrm);
    } else {
      double inv = 1.0 / nrm;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; i++) S[i + (int64_t)(j - 1) * n] = x[i] * inv;
      correct++;
    }
  }
  free(num);
  free(den);
  st->naccepted = correct - 1;
  double t2 = now_s();
  st->t_orth = t2 - t1;
  /* exact pivot-count check; the reference's check is off by one (ParHDE.cpp:192,281) */
  if (correct - 1 < k) return ORC_ERR_TOO_FEW_PIVOTS;

  /* LS = D*S - A*S, one (row, column) pair at a time in CSR order (ParHDE.cpp:288-300) */
  double *LS = U; /* the candidate columns are no longer needed */
#pragma omp parallel for collapse(2) schedule(guided)
  for (int q = 0; q < k; q++)
    for (int64_t i = 0; i < n; i++) {
      double v = deg[i] * S[i + (int64_t)q * n];
      for (uint32_t e = off[i]; e < off[i + 1]; e++) v -= S[adj[e] + (int64_t)q * n];
      LS[i + (int64_t)q * n] = v;
    }
  double *M = (double *)malloc(sizeof(double) * (size_t)k * k);
  gram_t(S, LS, M, n, k); /* ParHDE.cpp:301 */
  if (M_out) memcpy(M_out, M, sizeof(double) * (size_t)k * k);
  double t3 = now_s();
  st->t_mmult = t3 - t2;

  double *Y = (double *)malloc(sizeof(double) * (size_t)k * c);
  double *ev = (double *)malloc(sizeof(double) * (size_t)k);
  int status = eigen_pick(o, M, k, c, 0, Y, ev, &st->eig_iters); /* First, ParHDE.cpp:306 */
  if (evec_out) memcpy(evec_out, M, sizeof(double) * (size_t)k * k);
  if (eval_out) memcpy(eval_out, ev, sizeof(double) * (size_t)k);
  double t4 = now_s();
  st->t_eig = t4 - t3;
  if (status == ORC_OK) {
    coords_from(S, Y, coords, n, k, c); /* ParHDE.cpp:308 */
    normalise_coords(coords, n, c);
  }
  st->t_coords = now_s() - t4;
  if (S_out) memcpy(S_out, S, sizeof(double) * (size_t)n * k);
  free(M);
  free(Y);
  free(ev);
  free(deg);
  free(D);
  free(U);
  free(S);
  free(min_d);
  free(hist);
  return status;
}

/* ------------------------------------------------------------------------------------------ */
/* WParHDE pipeline, WParHDE.cpp:40-292 (coupled: each SSSP pass is followed at once by modified
 * Gram-Schmidt against every column kept so far, the constant column included; weighted degrees). */
static int run_wparhde(const orc_opts *o, const uint32_t *off, const uint32_t *adj, const int32_t *w, int64_t n,
                       int64_t m, double *coords, int64_t *sources, double *S_out, double *M_out,
                       double *evec_out, double *eval_out, orc_stats *st) {
  const int k = o->k, c = o->c, P = 3 * k;
  double t0 = now_s();
  double *deg = (double *)malloc(sizeof(double) * (size_t)n);
  for (int64_t i = 0; i < n; i++) { /* WParHDE.cpp:53-58 */
    double d = 0;
    for (uint32_t e = off[i]; e < off[i + 1]; e++) d += (double)w[e];
    deg[i] = d;
  }
  double *U = (double *)malloc(sizeof(double) * (size_t)n * (size_t)(k + 1));
  double *S = (double *)malloc(sizeof(double) * (size_t)n * (size_t)k);
  int32_t *col = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
  int64_t *min_d = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
  int64_t *hist = (int64_t *)malloc(sizeof(int64_t) * (size_t)P);
  if (!deg || !U || !S || !col || !min_d || !hist) return ORC_ERR_OOM;
  for (int64_t i = 0; i < n; i++) {
    U[i] = 1.0;
    min_d[i] = INT_MAX;
  }
  {
    double inv = 1.0 / sqrt(sum_sq(U, n));
    for (int64_t i = 0; i < n; i++) U[i] *= inv;
  }
  int64_t src = 0;
  int correct = 1;
  double t_dist = 0, t_orth = 0;
  int npass = 0;
  int64_t *rsrc = NULL;
  if (o->strategy != STRAT_KCENTERS) {
    rsrc = (int64_t *)malloc(sizeof(int64_t) * (size_t)P);
    random_sources(o->seed, n, P, rsrc);
  }
  for (int rc = 1; rc <= P; rc++) {
    if (correct > k) break;
    double ta = now_s();
    if (rsrc) src = rsrc[rc - 1];
    distance_pass(o, off, adj, w, n, m, src, col);
    sources[rc - 1] = src;
    npass++;
    if (rc == 1 && !reached_all(col, n, 1)) return ORC_ERR_DISCONNECTED;
    if (!rsrc) {
      int64_t raw;
      int64_t nxt = kcenters_step(min_d, col, n, correct != 1, hist, rc - 1, &raw);
      hist[rc - 1] = raw; /* WParHDE.cpp:137-153 */
      src = nxt;
    }
    double *x = U + (int64_t)correct * n;
    {
      double s = 0;
      for (int64_t i = 0; i < n; i++) s += (double)col[i] * (double)col[i];
      double inv = 1.0 / sqrt(s); /* WParHDE.cpp:154-162 */
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; i++) x[i] = (double)col[i] * inv;
    }
    double tb = now_s();
    t_dist += tb - ta;
    /* modified Gram-Schmidt against columns 0..j-1 (WParHDE.cpp:167-190) */
    int j = correct;
    for (int q = 0; q < j; q++) {
      const double *y = U + (int64_t)q * n;
      double dn = 0, nm = 0;
#pragma omp parallel for reduction(+ : dn, nm) schedule(static)
      for (int64_t i = 0; i < n; i++) {
        double dy = y[i] * deg[i];
        dn += y[i] * dy;
        nm += x[i] * dy;
      }
      dn = 1.0 / dn;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; i++) x[i] -= nm * y[i] * dn;
    }
    double nrm = sqrt(sum_sq(x, n));
    if (nrm < 0.001) { /* WParHDE.cpp:197-202: the slot is reused by the next pass */
      st->ndiscarded++;
      if (o->verbose) printf("discarding vec %d, normdist %g\n", j, nrm);
    } else {
      double inv = 1.0 / nrm;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; i++) x[i] = x[i] * inv;
      memcpy(S + (int64_t)(j - 1) * n, x, sizeof(double) * (size_t)n);
      correct++;
    }
    t_orth += now_s() - tb;
  }
  free(rsrc);
  st->npasses = npass;
  st->naccepted = correct - 1;
  st->t_dist = t_dist;
  st->t_orth = t_orth;
  if (correct - 1 < k) return ORC_ERR_TOO_FEW_PIVOTS;
  double t2 = now_s();
  /* weighted LS (WParHDE.cpp:229-241) */
  double *LS = U;
#pragma omp parallel for collapse(2) schedule(guided)
  for (int q = 0; q < k; q++)
    for (int64_t i = 0; i < n; i++) {
      double v = deg[i] * S[i + (int64_t)q * n];
      for (uint32_t e = off[i]; e < off[i + 1]; e++) v -= (double)w[e] * S[adj[e] + (int64_t)q * n];
      LS[i + (int64_t)q * n] = v;
    }
  double *M = (double *)malloc(sizeof(double) * (size_t)k * k);
  gram_t(S, LS, M, n, k);
  if (M_out) memcpy(M_out, M, sizeof(double) * (size_t)k * k);
  double t3 = now_s();
  st->t_mmult = t3 - t2;
  double *Y = (double *)malloc(sizeof(double) * (size_t)k * c);
  double *ev = (double *)malloc(sizeof(double) * (size_t)k);
  int status = eigen_pick(o, M, k, c, 0, Y, ev, &st->eig_iters);
  if (evec_out) memcpy(evec_out, M, sizeof(double) * (size_t)k * k);
  if (eval_out) memcpy(eval_out, ev, sizeof(double) * (size_t)k);
  double t4 = now_s();
  st->t_eig = t4 - t3;
  if (status == ORC_OK) {
    coords_from(S, Y, coords, n, k, c);
    normalise_coords(coords, n, c);
  }
  st->t_coords = now_s() - t4;
  if (S_out) memcpy(S_out, S, sizeof(double) * (size_t)n * k);
  (void)t0;
  free(M);
  free(Y);
  free(ev);
  free(deg);
  free(U);
  free(S);
  free(col);
  free(min_d);
  free(hist);
  return status;
}

/* ------------------------------------------------------------------------------------------ */
/* PivotMDS (PivotMDS.cpp:30-152) and PHDE (PHDE.cpp:30-141).  Both take k raw distance columns from
 * distancePhaseComputation (DrawingBase.cpp:119-194: k passes, Kcenters history = the sources used),
 * centre them (double centring of squared distances for PivotMDS, column centring for PHDE), form
 * C^T C and keep the c eigenvectors of largest eigenvalue. */
static int run_mds(const orc_opts *o, const uint32_t *off, const uint32_t *adj, int64_t n, int64_t m,
                   double *coords, int64_t *sources, double *S_out, double *M_out, double *evec_out,
                   double *eval_out, orc_stats *st) {
  const int k = o->k, c = o->c;
  double t0 = now_s();
  int32_t *D = (int32_t *)malloc(sizeof(int32_t) * (size_t)n * k);
  double *C = (double *)malloc(sizeof(double) * (size_t)n * k);
  int64_t *min_d = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
  int64_t *hist = (int64_t *)malloc(sizeof(int64_t) * (size_t)k);
  if (!D || !C || !min_d || !hist) return ORC_ERR_OOM;
  if (o->strategy == STRAT_KCENTERS) {
    for (int64_t i = 0; i < n; i++) min_d[i] = INT_MAX;
    int64_t src = 0;
    for (int r = 0; r < k; r++) {
      int32_t *col = D + (int64_t)r * n;
      distance_pass(o, off, adj, NULL, n, m, src, col);
      sources[r] = src;
      if (r == 0 && !reached_all(col, n, 0)) return ORC_ERR_DISCONNECTED;
      int64_t raw;
      int64_t nxt = kcenters_step(min_d, col, n, r != 0, hist, r, &raw);
      hist[r] = src; /* DrawingBase.cpp:157,169: old_idx is the source just used */
      src = nxt;
    }
  } else {
    random_sources(o->seed, n, k, sources);
    for (int r = 0; r < k; r++) {
      distance_pass(o, off, adj, NULL, n, m, sources[r], D + (int64_t)r * n);
      if (!reached_all(D + (int64_t)r * n, n, 0)) return ORC_ERR_DISCONNECTED;
    }
  }
  st->npasses = k;
  double t1 = now_s();
  st->t_dist = t1 - t0;
  if (o->algo == ALGO_PIVOTMDS) { /* doubleCentering, PivotMDS.cpp:30-66 */
    double *colsum = (double *)calloc((size_t)k, sizeof(double));
    double *rowsum = (double *)calloc((size_t)n, sizeof(double));
    double total = 0;
    for (int q = 0; q < k; q++) {
      double s = 0;
      const int32_t *col = D + (int64_t)q * n;
#pragma omp parallel for reduction(+ : s) schedule(static)
      for (int64_t i = 0; i < n; i++) {
        double d2 = (double)col[i] * (double)col[i];
        s += d2;
        rowsum[i] += d2;
      }
      colsum[q] = s;
      total += s;
    }
    double rn = 1.0 / (double)n, rk = 1.0 / (double)k;
#pragma omp parallel for collapse(2) schedule(static)
    for (int q = 0; q < k; q++)
      for (int64_t i = 0; i < n; i++) {
        double d = (double)D[i + (int64_t)q * n];
        C[i + (int64_t)q * n] = -0.5 * (d * d - (rn * colsum[q]) - (rk * rowsum[i]) + (rk * rn * total));
      }
    free(colsum);
    free(rowsum);
  } else { /* columnCentering, PHDE.cpp:30-47 */
    for (int q = 0; q < k; q++) {
      const int32_t *col = D + (int64_t)q * n;
      double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
      for (int64_t i = 0; i < n; i++) s += (double)col[i];
      s /= (double)n;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; i++) C[i + (int64_t)q * n] = (double)col[i] - s;
    }
  }
  double t2 = now_s();
  st->t_orth = t2 - t1;
  double *M = (double *)malloc(sizeof(double) * (size_t)k * k);
  gram_t(C, C, M, n, k); /* cTransCmatrixComputation, PivotMDS.cpp:149-152 */
  if (M_out) memcpy(M_out, M, sizeof(double) * (size_t)k * k);
  double t3 = now_s();
  st->t_mmult = t3 - t2;
  double *Y = (double *)malloc(sizeof(double) * (size_t)k * c);
  double *ev = (double *)malloc(sizeof(double) * (size_t)k);
  int status = eigen_pick(o, M, k, c, 1, Y, ev, &st->eig_iters); /* Largest */
  if (evec_out) memcpy(evec_out, M, sizeof(double) * (size_t)k * k);
  if (eval_out) memcpy(eval_out, ev, sizeof(double) * (size_t)k);
  double t4 = now_s();
  st->t_eig = t4 - t3;
  if (status == ORC_OK) {
    coords_from(C, Y, coords, n, k, c);
    normalise_coords(coords, n, c);
  }
  st->t_coords = now_s() - t4;
  if (S_out) memcpy(S_out, C, sizeof(double) * (size_t)n * k);
  st->naccepted = k;
  free(M);
  free(Y);
  free(ev);
  free(D);
  free(C);
  free(min_d);
  free(hist);
  return status;
}

/* ------------------------------------------------------------------------------------------ */
/* Entry point.  coords: n*c column-major; sources: capacity 3k (the passes' source vertices in order);
 * S_out: n*k column-major (the D-orthogonal basis, or C for PivotMDS/PHDE), M_out: the k*k matrix
 * given to the eigensolver, evec_out: k*k eigenvector matrix after the solve, eval_out: k values.
 * Any of the optional outputs may be NULL. */
int orc_layout(const orc_opts *o, const uint32_t *off, const uint32_t *adj, const int32_t *w, int64_t n,
               int64_t m, double *coords, int64_t *sources, double *S_out, double *M_out, double *evec_out,
               double *eval_out, orc_stats *st) {
  orc_stats dummy;
  if (!st) st = &dummy;
  memset(st, 0, sizeof(*st));
  if (!o || !off || !adj || !coords || !sources) return st->status = ORC_ERR_INVALID;
  if (o->k < 1 || o->k > 256 || o->c < 1 || o->c > o->k) return st->status = ORC_ERR_K_RANGE;
  if (o->k >= n) return st->status = ORC_ERR_K_RANGE;
  int rc = orc_check_csr(off, adj, n, m);
  if (rc) return st->status = rc;
  int prev_threads = omp_get_max_threads();
  if (o->nthreads > 0) omp_set_num_threads(o->nthreads);
  double t0 = now_s();
  switch (o->algo) {
  case ALGO_PARHDE:
    rc = w ? ORC_ERR_WEIGHTS : run_parhde(o, off, adj, n, m, coords, sources, S_out, M_out, evec_out, eval_out, st);
    break;
  case ALGO_WPARHDE:
    rc = !w ? ORC_ERR_WEIGHTS
            : run_wparhde(o, off, adj, w, n, m, coords, sources, S_out, M_out, evec_out, eval_out, st);
    break;
  case ALGO_PIVOTMDS:
  case ALGO_PHDE:
    rc = run_mds(o, off, adj, n, m, coords, sources, S_out, M_out, evec_out, eval_out, st);
    break;
  default:
    rc = ORC_ERR_INVALID;
  }
  st->t_total = now_s() - t0;
  if (o->nthreads > 0) omp_set_num_threads(prev_threads);
  st->status = rc;
  return rc;
}

/* Kcenters distance columns only (the exact-parity hook): P passes of the ParHDE selection rule
 * (variant 0, ParHDE.cpp:118-157), the WParHDE rule (variant 1: history of raw argmaxes, fix-up from
 * the second pass; identical to variant 0 when no pass is discarded) or the DrawingBase rule
 * (variant 2: history of used sources, DrawingBase.cpp:119-172).  D: n*P int32 column-major. */
int orc_kcenters(const uint32_t *off, const uint32_t *adj, const int32_t *w, int64_t n, int64_t m, int P,
                 int variant, int dist_algo, int nthreads, int32_t *D, int64_t *sources) {
  orc_opts o;
  memset(&o, 0, sizeof(o));
  o.dist_algo = dist_algo;
  int prev = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
  int64_t *min_d = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
  int64_t *hist = (int64_t *)malloc(sizeof(int64_t) * (size_t)P);
  for (int64_t i = 0; i < n; i++) min_d[i] = INT_MAX;
  int64_t src = 0;
  int status = ORC_OK;
  for (int r = 0; r < P; r++) {
    int32_t *col = D + (int64_t)r * n;
    distance_pass(&o, off, adj, w, n, m, src, col);
    sources[r] = src;
    if (r == 0 && !reached_all(col, n, w != NULL)) {
      status = ORC_ERR_DISCONNECTED;
      break;
    }
    int64_t raw;
    int64_t nxt = kcenters_step(min_d, col, n, r != 0, hist, r, &raw);
    hist[r] = variant == 2 ? src : raw;
    src = nxt;
  }
  free(min_d);
  free(hist);
  if (nthreads > 0) omp_set_num_threads(prev);
  return status;
}
