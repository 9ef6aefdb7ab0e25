/*
 * parhde.h -- C ABI of the GB300 ParHDE layout library (libparhde_gb300.so).
 *
 * Plain pointers and sizes only.  Host buffers are owned by the caller; device buffers are owned
 * by the context.  Every call returns an int status (PHDE_OK == 0, negative on error); the message
 * of the last error is available from phde_last_error().  One context per host thread.
 *
 * Reference interfaces replaced (paths relative to the ParHDE source tree):
 *   - DrawingBase / ParHDE / WParHDE / PivotMDS / PHDE construction + run() + getCoordinates()
 *     (variants/DrawingBase.h:41-47, spectralDrawing.cpp:176-193)      -> phde_graph_upload + phde_layout
 *   - DOBFS (gapbs/bfs.cc:144-185, declared variants/DrawingBase.h:62-64) -> phde_DOBFS
 *   - DeltaStep (gapbs/sssp.cc:53-140, declared variants/DrawingBase.h:65-67) -> phde_DeltaStep
 *   - the Kcenters distance phase (variants/ParHDE.cpp:118-157, variants/DrawingBase.cpp:119-172)
 *                                                                        -> phde_kcenters
 *   - distance columns for given sources (the bit-exactness hook)         -> phde_distances
 */
#ifndef PARHDE_GB300_H_
#define PARHDE_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------------------------- */
#define PHDE_OK 0
#define PHDE_ERR_INVALID (-1)         /* bad argument (null pointer, unknown algorithm, ...)          */
#define PHDE_ERR_CSR (-2)             /* malformed CSR: offsets not monotone / not ending at nnz, ...  */
#define PHDE_ERR_DISCONNECTED (-3)    /* a distance pass did not reach every vertex                   */
#define PHDE_ERR_K_RANGE (-4)         /* k < 1, k > 256, k >= n, c < 1 or c > k                       */
#define PHDE_ERR_TOO_FEW_PIVOTS (-5)  /* fewer than k vectors survived D-orthogonalisation           */
#define PHDE_ERR_OOM (-6)             /* device allocation failed                                     */
#define PHDE_ERR_NOCONVERGE (-7)      /* eigensolver iteration cap reached                            */
#define PHDE_ERR_TIMEOUT (-8)         /* a bounded device-side wait gave up                           */
#define PHDE_ERR_CUDA (-9)            /* CUDA runtime error                                           */
#define PHDE_ERR_WEIGHTS (-10)        /* weighted algorithm without weights, or the reverse           */
#define PHDE_ERR_NO_GRAPH (-11)       /* no graph uploaded to the context                             */
#define PHDE_ERR_TOO_LARGE (-12)      /* input exceeds the fixed scratch capacity of phde_bfs_noalloc  */

/* ---- algorithm / strategy / precision / eigensolver ids ------------------------------------- */
/* algorithm numbering follows spectralDrawing.cpp:101-109 */
#define PHDE_ALGO_PIVOTMDS 0
#define PHDE_ALGO_PHDE 1
#define PHDE_ALGO_WPARHDE 2
#define PHDE_ALGO_PARHDE 3
/* pivot strategies follow the doRand values of spectralDrawing.cpp:88-94 */
#define PHDE_STRAT_RANDCOARSE 0
#define PHDE_STRAT_RANDFINE 1
#define PHDE_STRAT_KCENTERS 2
/* No counterpart in the reference: pivots proposed at once by a per-vertex MLP and ordered by
 * farthest-point selection on their exact pairwise distances; one multi-source BFS replaces the 3k
 * serial Kcenters passes (ParHDE only). */
#define PHDE_STRAT_LEARNED 3
/* PHDE_STRAT_LEARNED with its acceptance test in the same call: the Kcenters layout (same precision and
 * eigensolver) is computed too, and the learned layout is returned only when its Rayleigh quotients
 * x_i^T L x_i / x_i^T x_i are within the tolerance of the Kcenters layout's (phde_set_pivot_check: their sum,
 * by default, or every coordinate); otherwise the Kcenters layout is returned.  Costs one Kcenters layout more
 * than PHDE_STRAT_LEARNED.  Both learned strategies fall back to Kcenters by themselves when the proposal
 * cannot give a layout (the multi-source BFS's level limit, fewer than k vectors surviving the
 * D-orthogonalisation); phde_layout_stats.pivot_outcome says which layout came back. */
#define PHDE_STRAT_LEARNED_CHECKED 4
#define PHDE_LEARNED_CANDIDATES 256
#define PHDE_LEARNED_WARM 8 /* exact Kcenters passes before the learned candidates are scored */
/* precision of the dense stages (distances are always exact integers) */
#define PHDE_PREC_FP64 0  /* every dense stage in FP64, the reference's arithmetic            */
#define PHDE_PREC_MIXED 1 /* FP32 storage/SpMM, compensated Gram products; FP64 k x k solves  */
/* ParHDE only: every n-sized product the reference forms in FP64 (the D-orthogonalisation's dot products
 * and norms, L*S, S^T L S, S*Y) taken instead from exact integer Gram matrices of the distance columns
 * (int64 sums, no rounding); the Gram-Schmidt loop runs on FP64 coefficient vectors, k x k stages in FP64.
 * At least the reference's FP64 accuracy.  Distances above 65535, or degree * distance >= 2^31, take the
 * PHDE_PREC_FP64 kernels instead. */
#define PHDE_PREC_EXACT 2
/* eigensolver of the k x k problem */
#define PHDE_EIG_POWER 0  /* subspace power iteration, ParallelComponents.cpp:48-158 (non-MKL build) */
#define PHDE_EIG_EXACT 1  /* exact symmetric eigensolve, the LAPACKE_dsyev role (MKL build)          */

#define PHDE_MAX_K 256

typedef struct phde_ctx phde_ctx;

typedef struct {
  int algo;       /* PHDE_ALGO_*                                                                 */
  int strategy;   /* PHDE_STRAT_*  (WParHDE always uses Kcenters, as WParHDE.cpp:40-218 does)      */
  int k;          /* pivots (-r), 1..256                                                          */
  int c;          /* coordinates (-c), 1..k                                                       */
  int precision;  /* PHDE_PREC_*                                                                  */
  int eig;        /* PHDE_EIG_*                                                                   */
  uint64_t seed;  /* random strategies: glibc rand() stream seed (1 = an unseeded process)          */
  int verbose;    /* print the reference's progress lines ("discarding vec ...")                  */
} phde_layout_opts;

typedef struct {
  int status;
  int npasses;       /* distance passes (BFS / SSSP) executed                                       */
  int naccepted;     /* vectors accepted by the D-orthogonalisation                                 */
  int ndiscarded;    /* candidates discarded (norm < 1e-3 after projection)                         */
  int eig_iters;     /* power-method sweeps, or Jacobi sweeps                                        */
  int gpu_launches;  /* kernels this call launched                                                  */
  double ms_dist;    /* distance phase (device events): BFS/SSSP + Kcenters selection + normalisation */
  double ms_orth;    /* D-orthogonalisation (or centring for PivotMDS/PHDE)                         */
  double ms_mmult;   /* Laplacian SpMM + Gram product                                               */
  double ms_eig;     /* k x k eigensolve                                                             */
  double ms_coords;  /* coordinates, normalisation and the copy to the host                          */
  double ms_total;   /* whole call                                                                   */
  int64_t edges_examined; /* adjacency entries read by the distance passes                          */
  double ms_dist_kernel;  /* device time of the distance kernel launches alone (events around each launch) */
  int dist_kernel_launches; /* number of distance kernel launches (1 for the Kcenters BFS)           */
  double ms_msbfs_kernel;   /* of which multi-source BFS sweeps (learned and random strategies)          */
  int msbfs_levels;         /* levels of those sweeps, summed                                           */
  int batch_graph_replay;   /* phde_layout_batched: 1 when the pipeline ran as one CUDA graph launch     */
  int batch_seg_rows;       /* phde_layout_batched: rows per segment CTA picked by the autotuner         */
  double ms_batch_tune;     /* phde_layout_batched: the autotuner's best whole-batch time (first call)   */
  int64_t sssp_rounds;      /* WParHDE: synchronised relaxation rounds of the SSSP passes, summed        */
  /* learned strategies: PHDE_OUTCOME_*; 0 for the reference's strategies */
  int pivot_outcome;
  /* Rayleigh quotients x_i^T L x_i / x_i^T x_i of the first PHDE_RQ_MAX returned coordinates (learned
   * strategies and PHDE_PREC_EXACT; 0 otherwise), and for PHDE_STRAT_LEARNED_CHECKED the Kcenters layout's */
  double rayleigh[8];
  double rayleigh_kcenters[8];
  double ms_check;          /* PHDE_STRAT_LEARNED_CHECKED: the Kcenters layout's time (part of ms_total)  */
  double ms_lap_kernel;     /* PHDE_PREC_EXACT: device time of the fused Laplacian Gram kernel (Z^T L Z)   */
} phde_layout_stats;
#define PHDE_RQ_MAX 8
#define PHDE_OUTCOME_LEARNED 1        /* the learned proposal's layout                                      */
#define PHDE_OUTCOME_REJECTED 2       /* learned layout outside the Rayleigh tolerance: Kcenters layout      */
#define PHDE_OUTCOME_FAILED 3         /* learned proposal gave no layout (level limit, too few pivots): Kcenters */
#define PHDE_CHECK_SUM 0              /* sum of the c quotients within the tolerance of Kcenters' sum        */
#define PHDE_CHECK_EACH 1             /* every coordinate's quotient within the tolerance of Kcenters'       */

/* optional extra outputs of phde_layout (any member may be NULL) */
typedef struct {
  double *basis;   /* n*k column-major: the D-orthogonal basis S (ParHDE/WParHDE) or C (PivotMDS/PHDE) */
  double *gram;    /* k*k column-major: the matrix handed to the eigensolver (S^T L S or C^T C)         */
  double *evecs;   /* k*k column-major: eigenvector matrix after the solve                              */
  double *evals;   /* k: eigenvalues (|lambda| for the power method), ascending                         */
} phde_layout_extra;

/* ---- context -------------------------------------------------------------------------------- */
int phde_create(phde_ctx **out, int device);
void phde_destroy(phde_ctx *ctx);
const char *phde_last_error(const phde_ctx *ctx);
const char *phde_status_string(int status);
int phde_version(void);

/* Copy a CSR graph to the device (replaces the CSR arrays handed to the DrawingBase constructor,
 * variants/DrawingBase.cpp:16-26).  offsets: n+1 entries of offset_bytes (4: uint32 as in the .csr
 * file, 8: int64); adj: nnz uint32; weights: nnz int32 or NULL.  The offsets are widened to int64 on
 * the device.  Validates monotone offsets ending at nnz and neighbours < n. */
int phde_graph_upload(phde_ctx *ctx, const void *offsets, int offset_bytes, const uint32_t *adj,
                      const int32_t *weights, int64_t n, int64_t nnz);
int64_t phde_graph_n(const phde_ctx *ctx);
int64_t phde_graph_nnz(const phde_ctx *ctx);

/* The layout pipeline behind DrawingBase::run() + getCoordinates() (variants/ParHDE.cpp:45-352,
 * WParHDE.cpp:40-292, PivotMDS.cpp:68-147, PHDE.cpp:50-136, DrawingBase.cpp:196-219) on the uploaded
 * graph.  coords_out: n*c doubles, column-major (coordinate j of vertex i at i + j*n), each column of
 * unit L2 norm.  sources_out (optional): the source vertex of every distance pass, capacity 3k.
 * extra (optional): intermediate matrices.  stats (optional). */
int phde_layout(phde_ctx *ctx, const phde_layout_opts *opts, double *coords_out, int64_t *sources_out,
                phde_layout_extra *extra, phde_layout_stats *stats);

/* ---- batched layouts: many independent graphs in one call ----
 * Replaces a caller's loop of DrawingBase::run() + getCoordinates() over separate graphs
 * (variants/DrawingBase.h:41-60; spectralDrawing.cpp:186-197 per graph).  phde_batch_upload copies the
 * graphs (each its own CSR, local vertex ids; all with the same offset width) as one disjoint union;
 * phde_layout_batched lays every graph out (every graph connected with more than 3k vertices).  ParHDE with
 * Kcenters pivots or learned pivots (PHDE_STRAT_LEARNED: every graph above 256 vertices; each graph gets the
 * pivots a single-graph learned layout picks), opts->precision PHDE_PREC_MIXED, opts->eig PHDE_EIG_EXACT,
 * 2 <= k <= 32 and c <= 4 run as one fused pipeline over the union; any other options phde_layout accepts
 * (PHDE_PREC_FP64 -- the reference's arithmetic -- or PHDE_PREC_EXACT, k above 32, the power iteration, the
 * other algorithms) lay the graphs out one after another with the single-graph pipeline, each graph's CSR
 * cut out of the uploaded union on the device: the coordinates are those phde_layout gives that graph.
 * coords_out holds sum(n_b) * c doubles: graph b's coordinates, column-major (coordinate j of its local
 * vertex i at i + j * n_b), start at c * (n_0 + ... + n_{b-1}).  The first call on a batch autotunes and
 * captures the pipeline into a CUDA graph; later calls replay it. */
typedef struct {
  const void *offsets; /* n + 1 entries */
  int offset_bytes;    /* 4 (uint32) or 8 (int64) */
  const uint32_t *adj; /* nnz neighbour ids in 0..n-1 */
  int64_t n, nnz;
} phde_graph_desc;
/* ---- input conversion: Matrix Market entries to the layout's CSR (the reference's mtx2csr tool,
 * mtx2csr.cpp:117-296), on the GPU.  The result becomes the context's uploaded graph. ---- */
typedef struct {
  int64_t n_in;         /* vertices of the matrix graph (n1, or n1 + n2 for a bipartite reading) */
  int64_t nnz_dedup;    /* directed entries after self-loop removal and deduplication */
  int64_t ncomponents;  /* connected components */
  int64_t n;            /* vertices of the largest component (the graph kept) */
  int64_t nnz;          /* its directed entries */
} phde_csr_info;
/* u, v: 1-indexed row and column of each of `count` entries; w: their integer weights or NULL.
 * symmetric != 0: an n1 x n1 matrix read as an undirected graph (each entry both directions, self loops
 * dropped); symmetric == 0: an n1 x n2 matrix read as a bipartite graph (rows become vertices n2 .. n2+n1-1).
 * Parallel entries keep the smallest weight; the largest connected component (the one holding the smallest
 * vertex on ties) is kept and renumbered in increasing order, as the reference does. */
int phde_graph_from_entries(phde_ctx *ctx, const uint32_t *u, const uint32_t *v, const int32_t *w, int64_t count,
                            int64_t n1, int64_t n2, int symmetric, phde_csr_info *info);
/* Copy the uploaded graph to host memory: offsets as uint32 (n + 1), adjacency (nnz), weights (nnz, or NULL).
 * Sizes from phde_graph_n / phde_graph_nnz. */
int phde_graph_download(phde_ctx *ctx, uint32_t *offsets, uint32_t *adj, int32_t *weights);

/* Write coordinates (column-major n x c, the layout phde_layout returns) as a .nxyz text file: one line
 * per vertex, "x0,x1[,x2...]", each value formatted like std::ostream's default (%g, 6 significant digits)
 * -- byte-identical to the reference's writeCoords (spectralDrawing.cpp:42-65), formatted by `nthreads`
 * host threads (0: all cores).  Host only; needs no context. */
int phde_write_nxyz(const char *path, const double *coords, int64_t n, int c, int nthreads);

/* ---- drawing: the reference's draw tool (draw_graph.c:135-351), on the GPU ----
 * phde_draw rasterises the uploaded graph at the vertex positions (x[i], y[i]) (host arrays of n doubles: the
 * two coordinate columns the draw command line selects) into an image held by the context: the image size from
 * the coordinate bounds (draw_graph.c:201-249), one Bresenham line per CSR entry u -> v in CSR order, later lines
 * over earlier ones, coloured by length bin and draw_line's counters (draw_graph.c:49-128, 282-326), on the
 * (4, 4, 4) background.  The pixels are those of the reference run with one thread.  Coordinates that are not
 * finite, or a degenerate coordinate range (an image side that is not a positive 32-bit number), return
 * PHDE_ERR_INVALID; images above 2^20 pixels a side or 2^31 pixels return PHDE_ERR_TOO_LARGE.
 * phde_draw_download copies the image as RGBA bytes (width * height * 4, row-major, y down the rows as the
 * reference indexes it); phde_draw_write_png writes it as a PNG file (lodepng_encode32_file's role,
 * draw_graph.c:331) deflated by nthreads host threads (0: all cores).  phde_write_png writes any RGBA image
 * the same way (host only; needs no context). */
typedef struct {
  uint32_t width, height;                   /* image size, after the reference's size correction       */
  uint32_t width_computed, height_computed; /* sqrt(100 n / aspect) and aspect * width, before it      */
  double xmin, xmax, ymin, ymax;            /* coordinate bounds (starting from 1 and -1)               */
  double aspect;                            /* (xmax - xmin) / (ymax - ymin)                            */
  float max_edge_length;                    /* longest CSR entry, in pixels                             */
  int gpu_launches;                         /* kernels this call launched                               */
  int64_t pixels;                           /* pixel writes of all lines                                */
  double ms_device;                         /* device time: coordinate copy, bounds, raster, colours    */
  double ms_raster;                         /* of which the line rasteriser                             */
  double ms_total;                          /* the whole call, host clock                               */
} phde_draw_info;
int phde_draw(phde_ctx *ctx, const double *x, const double *y, phde_draw_info *info);
int phde_draw_download(phde_ctx *ctx, uint8_t *rgba, size_t bytes);
int phde_draw_write_png(phde_ctx *ctx, const char *path, int nthreads);
int phde_write_png(const char *path, const uint8_t *rgba, uint32_t width, uint32_t height, int nthreads);

int phde_batch_upload(phde_ctx *ctx, const phde_graph_desc *graphs, int count);
int phde_layout_batched(phde_ctx *ctx, const phde_layout_opts *opts, double *coords_out, phde_layout_stats *stats);
/* The Rayleigh quotients x^T L x / x^T x of every graph's coordinates from the last phde_layout_batched call:
 * graph b's coordinate t at rq_out[b * c + t] (count * c doubles).  No counterpart in the reference: the
 * per-graph quality figure by which a batch's learned pivots are compared with Kcenters'. */
int phde_batch_rayleigh(phde_ctx *ctx, double *rq_out);

/* Exact distance columns from the given sources on the uploaded graph: hop counts (unweighted graph)
 * or weighted shortest-path lengths (weighted graph).  out: n*nsrc int32, column-major; unreachable
 * vertices get -1 (BFS) or 1073741823 (SSSP, gapbs/sssp.cc:50). */
int phde_distances(phde_ctx *ctx, const int64_t *sources, int nsrc, int32_t *out);

/* Kcenters distance phase: `passes` distance passes, each starting from the vertex farthest from all
 * previous sources (lowest index on ties; ParHDE.cpp:118-157).  variant 0 = ParHDE/WParHDE history
 * rule, 2 = DrawingBase (PivotMDS/PHDE) history rule (DrawingBase.cpp:119-172).  dist_out: n*passes
 * int32 column-major (may be NULL); sources_out: passes entries. */
int phde_kcenters(phde_ctx *ctx, int passes, int variant, int32_t *dist_out, int64_t *sources_out);

/* Reference-shaped drop-ins for the two distance kernels (variants/DrawingBase.h:62-67), on host CSR
 * arrays.  They use a per-thread default context, upload the graph on every call (the reference
 * functions receive raw CSR pointers), and write only the entries of reached vertices, as the
 * reference does.  alpha/beta are accepted for signature compatibility; they tune the direction
 * switch and do not change the result. */
int phde_DOBFS(const uint32_t *row, const uint32_t *col, long source, long numNodes, long numEdges, double *dists,
               int alpha, int beta);
int phde_DeltaStep(const uint32_t *row, const uint32_t *col, const int32_t *weights, long source, long numNodes,
                   long numEdges, double *dist, int32_t delta);

/* Diagnostics used by the tests: run a grid barrier that can never complete (the kernel expects one
 * more block than it launches) with the given wait limit, and report the status the kernel returned.
 * Returns PHDE_ERR_TIMEOUT when the bounded wait gave up as designed. */
int phde_selftest_barrier_timeout(phde_ctx *ctx, int timeout_ms);

/* Diagnostics used by the tests: G = A^T diag(w) B through the tensor-core Gram kernel of the mixed path
 * (FP32 inputs split into three BF16 parts, FP32 accumulation in TMEM, FP64 across row blocks).  A: n rows of
 * acols FP32 (leading dimension lda), B: n rows of bcols (ldb), w: n doubles or NULL, all host arrays; G: acols
 * x bcols FP64 row-major.  nsplit: row blocks per output tile (0: one per 4096 rows). */
int phde_gram_f32(phde_ctx *ctx, const float *A, int lda, int acols, const float *B, int ldb, int bcols,
                  const double *w, int64_t n, int nsplit, double *G);

/* Diagnostics used by the tests: the exact eigensolver of the layouts (PHDE_EIG_EXACT: FP32 Jacobi sweeps, FP64
 * orthonormalisation and similarity, FP64 rotations of unseparated pairs, perturbation refinement; FP64 sweeps
 * when a wanted eigenvalue is not separated) on a symmetric k x k matrix M (column-major host array; the
 * symmetric part is used).  evals: the k eigenvalues ascending; Y: k x c column-major, the eigenvectors of the
 * c smallest eigenvalues (largest != 0: the c largest, largest first), each signed so that its entry of largest
 * magnitude is positive.  iters (may be NULL): FP32 plus FP64 sweeps.  The reference calls LAPACK's dsyev
 * for this step (DrawingBase.cpp). */
int phde_symeig(phde_ctx *ctx, const double *M, int k, int c, int largest, double *evals, double *Y, int *iters);

/* Replace the pivot-scoring MLP used by PHDE_STRAT_LEARNED (4 -> 64 -> 64 -> 1, ReLU): `count` floats,
 * W1[64][4], b1[64], W2[64][64], b2[64], w3[64], b3[1] (row-major).  The library starts with the
 * weights trained by train/train_pivot_mlp.py.  No counterpart in the reference. */
int phde_set_pivot_model(phde_ctx *ctx, const float *weights, int count);

/* Diagnostics used by the tests: the learned strategy's proposal step alone on the uploaded graph -- the
 * PHDE_LEARNED_WARM exact Kcenters passes, the per-vertex features and the pivot-scoring MLP -- returning
 * every vertex's score (scores: n floats), the warm start's minimum distance to its pivots (warm_dist: n int32)
 * and the `ncand` best-scored vertices the strategy takes as candidates (score descending, index ascending on
 * ties).  Any output may be NULL.  No counterpart in the reference. */
int phde_pivot_scores(phde_ctx *ctx, float *scores, int32_t *warm_dist, int64_t *candidates, int ncand);

/* The acceptance rule of PHDE_STRAT_LEARNED_CHECKED: rule PHDE_CHECK_SUM (default) or PHDE_CHECK_EACH, and
 * the tolerance (default 0.02: learned quotients at most 1.02 times Kcenters').  No counterpart in the
 * reference. */
int phde_set_pivot_check(phde_ctx *ctx, int rule, double tolerance);

/* Kernel launches issued through this context since it was created. */
int64_t phde_launch_count(const phde_ctx *ctx);

/* Hop distances from one source, for callers that must not allocate device memory.  This entry point
 * has no counterpart in the reference.  It is meant for host code that cannot call cudaMalloc -- code
 * whose device memory is owned by its own pool allocator, code on a latency-critical path where an
 * allocation would synchronise the device, or a plugin that is only handed pre-allocated buffers.
 * Inputs and output are DEVICE pointers: d_offsets (n+1 int64), d_adj (nnz uint32), d_dist (n int32,
 * overwritten: hop count, -1 when unreachable); stream is a cudaStream_t (NULL = the legacy default
 * stream).  The kernel's scratch is a fixed array inside the library (16 MiB, held by every GPU that
 * loads the library until the process exits), so n is limited to PHDE_NOALLOC_MAX_VERTICES; larger
 * inputs return PHDE_ERR_TOO_LARGE with a message on stderr.  The call allocates nothing, waits for
 * its own kernel on `stream`, and returns PHDE_OK or PHDE_ERR_TIMEOUT.  All calls share the scratch:
 * calls whose kernels overlap on the GPU race and must be serialised by the caller.  The first call on
 * a device looks up the scratch address (one-time set-up); make it before any stream capture.  The address
 * is kept for the life of the process: after a cudaDeviceReset of that device the module is loaded again
 * elsewhere, so a process that resets a device must not call this entry point on it afterwards. */
#define PHDE_NOALLOC_MAX_VERTICES 1048576
int phde_bfs_noalloc(const int64_t *d_offsets, const uint32_t *d_adj, int64_t n, int64_t nnz, int64_t source,
                     int32_t *d_dist, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PARHDE_GB300_H_ */
