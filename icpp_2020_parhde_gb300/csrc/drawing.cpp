// drawing.cpp -- the reference class interface (include/parhde_drawing.h) over the C ABI.
//
// run() prints the progress and timing lines of the reference variants (ParHDE.cpp:47-50,72-73,336-340;
// WParHDE.cpp:42-45,280-284; PivotMDS.cpp:70-76,428-432; PHDE.cpp:52-57,126-130) from the library's
// device-event phase times; error exits reproduce the reference's messages and exit codes.
#include "parhde_drawing.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>

static int env_eig() {
  const char *e = getenv("PHDE_EIG");
  return (e && !strcmp(e, "exact")) ? PHDE_EIG_EXACT : PHDE_EIG_POWER;
}

// PHDE_PRECISION=mixed|exact selects the ParHDE class's dense stages; the other classes keep FP64
static int env_precision(int algo) {
  const char *e = getenv("PHDE_PRECISION");
  if (!e || algo != PHDE_ALGO_PARHDE) return PHDE_PREC_FP64;
  if (!strcmp(e, "mixed")) return PHDE_PREC_MIXED;
  if (!strcmp(e, "exact")) return PHDE_PREC_EXACT;
  return PHDE_PREC_FP64;
}

DrawingBase::DrawingBase(unsigned int *rowPtrs_, unsigned int *adj_, int32_t *weights_, long n_, long m_,
                         int numSources_, int doRand_, int numCoord_)
    : rowPtrs(rowPtrs_), adj(adj_), weights(weights_), n(n_), m(m_), numSources(numSources_), numCoord(numCoord_),
      doRand(doRand_), coordinates(nullptr), ctx_(nullptr) {
  memset(&stats_, 0, sizeof(stats_));
  coordinates = (double *)calloc((size_t)n * (size_t)(numCoord > 0 ? numCoord : 1), sizeof(double));
  int dev = 0;
  if (const char *d = getenv("PHDE_DEVICE")) dev = atoi(d);
  int rc = phde_create(&ctx_, dev);
  if (rc != PHDE_OK) {
    fprintf(stderr, "Error: no usable CUDA device (%s)\n", phde_status_string(rc));
    exit(1);
  }
  rc = phde_graph_upload(ctx_, rowPtrs, 4, adj, weights, n, m);
  if (rc != PHDE_OK) {
    fprintf(stderr, "Error: %s\n", phde_last_error(ctx_));
    exit(1);
  }
}

DrawingBase::~DrawingBase() {
  free(coordinates);
  phde_destroy(ctx_);
}

double *DrawingBase::getCoordinates() { return coordinates; }

int DrawingBase::runAlgorithm(int algo, int strategy, int tries) {
  if (tries < 1) tries = 1;
  phde_layout_opts o;
  o.algo = algo;
  o.strategy = strategy;
  o.k = numSources;
  o.c = numCoord;
  o.precision = env_precision(algo);
  o.eig = env_eig();
  o.seed = 1;
  o.verbose = 1;
  double hde = 0, dist = 0, orth = 0, mm = 0, others = 0;
  for (int t = 0; t < tries; t++) {
    int rc = phde_layout(ctx_, &o, coordinates, nullptr, nullptr, &stats_);
    if (rc == PHDE_ERR_TOO_FEW_PIVOTS) {
      fprintf(stderr, "%s\n", phde_last_error(ctx_));
      exit(0);  // ParHDE.cpp:281-285
    }
    if (rc == PHDE_ERR_NOCONVERGE) {
      printf("The algorithm failed to compute eigenvalues.\n");
      exit(1);  // DrawingBase.cpp:65-69
    }
    if (rc != PHDE_OK) {
      fprintf(stderr, "Error: %s: %s\n", phde_status_string(rc), phde_last_error(ctx_));
      exit(1);
    }
    hde += stats_.ms_total * 1e-3;
    dist += stats_.ms_dist * 1e-3;
    orth += stats_.ms_orth * 1e-3;
    mm += stats_.ms_mmult * 1e-3;
    others += (stats_.ms_eig + stats_.ms_coords) * 1e-3;
  }
  const double inv = 1.0 / tries;
  if (algo == PHDE_ALGO_PARHDE || algo == PHDE_ALGO_WPARHDE) {
    printf("**** Means ******\n");
    printf("HDE mean time %g s.\n", hde * inv);
    printf("%s mean time %g s.\n", algo == PHDE_ALGO_PARHDE ? "BFS" : "SSSP", dist * inv);
    printf("DOrthogonalize mean time %g s.\n", orth * inv);
    printf("Matrix Multiply Mean time %g s.\n", mm * inv);
  } else {
    printf("**** %s Means ******\n", algo == PHDE_ALGO_PIVOTMDS ? "PivotMDS" : "PHDE");
    printf("Total mean time %g s.\n", hde * inv);
    printf("BFS mean time %g s.\n", dist * inv);
    printf("Matrix Multiply Mean time %g s.\n", mm * inv);
    printf("%s Mean time %g s.\n", algo == PHDE_ALGO_PIVOTMDS ? "Double Centering" : "ColumnCentering", orth * inv);
  }
  (void)others;
  return 0;
}

ParHDE::ParHDE(unsigned int *rowPtrs_, unsigned int *adj_, int32_t *weights_, long n_, long m_, int s, int r,
               int numCoord_)
    : DrawingBase(rowPtrs_, adj_, weights_, n_, m_, s, r, numCoord_) {
  if (weights_) {
    fprintf(stderr, "ParHDE code doesn't requires the weighted edges\n");  // ParHDE.cpp:27-31
    exit(0);
  }
}

int ParHDE::run(int tries, int, int, int32_t) {
  printf("Running ParHDE on the GPU\n");
  printf("Performing ParHDE with Number of sources: %d and Number of experiments: %d\n", numSources, tries);
  return runAlgorithm(PHDE_ALGO_PARHDE, doRand, tries);
}

WParHDE::WParHDE(unsigned int *rowPtrs_, unsigned int *adj_, int32_t *weights_, long n_, long m_, int s, int numCoord_)
    : DrawingBase(rowPtrs_, adj_, weights_, n_, m_, s, PHDE_STRAT_KCENTERS, numCoord_) {
  if (!weights_) {
    fprintf(stderr, "Weighted ParHDE code requires the weighted edges\n");  // WParHDE.cpp:22-26
    exit(0);
  }
}

int WParHDE::run(int tries, int, int, int32_t) {
  printf("Running Weighted ParHDE on the GPU\n");
  printf("Performing parHDE with Number of sources: %d and Number of experiments: %d\n", numSources, tries);
  return runAlgorithm(PHDE_ALGO_WPARHDE, PHDE_STRAT_KCENTERS, tries);
}

PivotMDS::PivotMDS(unsigned int *rowPtrs_, unsigned int *adj_, int32_t *weights_, long n_, long m_, int s, int r,
                   int numCoord_)
    : DrawingBase(rowPtrs_, adj_, weights_, n_, m_, s, r, numCoord_) {}

int PivotMDS::run(int tries, int, int, int32_t) {
  printf("Performing PivotMDS with %d tries and pivots: %d\n", tries, numSources);
  return runAlgorithm(PHDE_ALGO_PIVOTMDS, doRand, tries);
}

PHDE::PHDE(unsigned int *rowPtrs_, unsigned int *adj_, int32_t *weights_, long n_, long m_, int s, int r,
           int numCoord_)
    : DrawingBase(rowPtrs_, adj_, weights_, n_, m_, s, r, numCoord_) {}

int PHDE::run(int tries, int, int, int32_t) {
  printf("Performing PHDE with %d tries and pivots: %d\n", tries, numSources);
  return runAlgorithm(PHDE_ALGO_PHDE, doRand, tries);
}
