// ref_harness.cpp -- C ABI around the reference ParHDE sources, for pinning the oracle.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles the reference's own files (read in place
// from the ParHDE tree) together with this harness into oracle/_ref/libparhde_ref.so.  The harness
// calls the reference exactly as its driver does (spectralDrawing.cpp:176-193: construct the variant,
// run(1), getCoordinates()) and records which source vertex every distance pass used, by standing in
// for DOBFS/DeltaStep (the reference definitions are compiled under the names ref_impl_DOBFS /
// ref_impl_DeltaStep and called from here unchanged).
#include <cstdint>
#include <cstring>
#include <vector>
#include <omp.h>
#include "DrawingBase.h"
#include "PHDE.h"
#include "ParHDE.h"
#include "PivotMDS.h"
#include "WParHDE.h"

void ref_impl_DOBFS(unsigned int *row, unsigned int *col, long source, long numNodes, long numEdges, double *dists,
                    int alpha, int beta);
double *ref_impl_DeltaStep(const unsigned int *row, unsigned int *col, int32_t *weights, long source, long numNodes,
                           long numEdges, double *dist, int32_t delta);

static std::vector<long> g_sources;

void DOBFS(unsigned int *row, unsigned int *col, long source, long numNodes, long numEdges, double *dists, int alpha,
           int beta) {
  g_sources.push_back(source);
  ref_impl_DOBFS(row, col, source, numNodes, numEdges, dists, alpha, beta);
}

double *DeltaStep(const unsigned int *row, unsigned int *col, int32_t *weights, long source, long numNodes,
                  long numEdges, double *dist, int32_t delta) {
  g_sources.push_back(source);
  return ref_impl_DeltaStep(row, col, weights, source, numNodes, numEdges, dist, delta);
}

extern "C" {

int ref_abi_version(void) { return 1; }

// One reference DOBFS pass (gapbs/bfs.cc:144-185).  Entries the BFS does not reach are left as the
// caller initialised them.
void ref_dobfs(const uint32_t *row, const uint32_t *col, long src, long n, long m, double *dists, int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  ref_impl_DOBFS(const_cast<unsigned *>(row), const_cast<unsigned *>(col), src, n, m, dists, 15, 18);
}

// One reference DeltaStep pass (gapbs/sssp.cc:53-140).
void ref_deltastep(const uint32_t *row, const uint32_t *col, const int32_t *w, long src, long n, long m,
                   double *dists, int delta, int nthreads) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  ref_impl_DeltaStep(row, const_cast<unsigned *>(col), const_cast<int32_t *>(w), src, n, m, dists, delta);
}

// The whole reference pipeline.  algo: 0 PivotMDS, 1 PHDE, 2 WParHDE, 3 ParHDE (spectralDrawing.cpp:101-109);
// doRand: 0 RandCoarse, 1 RandFine, 2 Kcenters.  coords_out receives n*c values (column-major) from
// getCoordinates(); WParHDE always produces 2 columns (its constructor passes numCoord into the doRand
// slot, WParHDE.cpp:12-13).  sources_out receives up to cap pass sources in call order.
int ref_layout(int algo, int doRand, const uint32_t *row, const uint32_t *adj, const int32_t *w, long n, long m, int k,
               int c, int nthreads, double *coords_out, long *sources_out, int cap, int *nsources_out) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  unsigned *r = const_cast<unsigned *>(row), *a = const_cast<unsigned *>(adj);
  int32_t *ww = const_cast<int32_t *>(w);
  DrawingBase *d = nullptr;
  int ncoord = c;
  switch (algo) {
    case 0: d = new PivotMDS(r, a, nullptr, n, m, k, doRand, c); break;
    case 1: d = new PHDE(r, a, nullptr, n, m, k, doRand, c); break;
    case 2: d = new WParHDE(r, a, ww, n, m, k, c); ncoord = 2; break;
    case 3: d = new ParHDE(r, a, nullptr, n, m, k, doRand, c); break;
    default: return -1;
  }
  g_sources.clear();
  d->run(1, 15, 18, 1);
  double *x = d->getCoordinates();
  std::memcpy(coords_out, x, sizeof(double) * (size_t)n * (size_t)ncoord);
  int ns = (int)g_sources.size();
  for (int i = 0; i < ns && i < cap; i++) sources_out[i] = g_sources[i];
  *nsources_out = ns;
  delete d;
  return ncoord;
}
}
