/*
 * parhde_drawing.h -- the reference's C++ class interface (variants/DrawingBase.h:13-48, ParHDE.h,
 * WParHDE.h, PivotMDS.h, PHDE.h) implemented over the C ABI of parhde.h.  Code written against the
 * reference classes compiles against this header unchanged:
 *
 *   DrawingBase *d = new ParHDE(rowOffsets, adj, NULL, n, m, numSources, doRand, numCoord);
 *   d->run(1);
 *   double *xy = d->getCoordinates();   // column-major n x numCoord, unit-norm columns
 *
 * Ownership follows the reference: the caller owns the CSR arrays, the object owns the coordinate
 * buffer (freed in the destructor).  Where the reference prints a message and exits, so do these
 * classes (same messages).  Two environment variables select the library's options without changing
 * the interface: PHDE_EIG=exact (exact eigensolver instead of the power iteration) and
 * PHDE_PRECISION=mixed (FP32/compensated dense stages).
 */
#ifndef PARHDE_GB300_DRAWING_H_
#define PARHDE_GB300_DRAWING_H_

#include <cstdint>

#include "parhde.h"

enum EigenChoice { First, Largest };

class DrawingBase {
 public:
  DrawingBase(unsigned int *rowPtrs, unsigned int *adj, int32_t *weights, long n, long m, int numSources, int doRand,
              int numCoord = 2);
  virtual ~DrawingBase();
  DrawingBase(const DrawingBase &) = delete;
  DrawingBase &operator=(const DrawingBase &) = delete;

  /* unit-norm coordinates, column-major: coordinate j of vertex i at [i + j*n] (DrawingBase.cpp:196-205) */
  double *getCoordinates();
  virtual int run(int tries = 11, int alpha = 15, int beta = 18, int32_t delta = 1) = 0;

  /* statistics of the last run (device-event phase times, passes, launches) */
  const phde_layout_stats &lastStats() const { return stats_; }

 protected:
  int runAlgorithm(int algo, int strategy, int tries);
  unsigned int *rowPtrs;
  unsigned int *adj;
  int32_t *weights;
  long n;
  long m;
  int numSources;
  int numCoord;
  int doRand;
  double *coordinates;
  phde_ctx *ctx_;
  phde_layout_stats stats_;
};

class ParHDE : public DrawingBase {
 public:
  ParHDE(unsigned int *rowPtrs, unsigned int *adj, int32_t *weights, long n, long m, int s, int r, int numCoord);
  int run(int tries = 1, int alpha = 15, int beta = 18, int32_t delta = 1) override;
};

/* The reference constructor drops numCoord (WParHDE.cpp:12-13); this one honours it. */
class WParHDE : public DrawingBase {
 public:
  WParHDE(unsigned int *rowPtrs, unsigned int *adj, int32_t *weights, long n, long m, int s, int numCoord = 2);
  int run(int tries = 11, int alpha = 15, int beta = 18, int32_t delta = 1) override;
};

class PivotMDS : public DrawingBase {
 public:
  PivotMDS(unsigned int *rowPtrs, unsigned int *adj, int32_t *weights, long n, long m, int s, int r, int numCoord);
  int run(int tries = 1, int alpha = 15, int beta = 18, int32_t delta = 1) override;
};

class PHDE : public DrawingBase {
 public:
  PHDE(unsigned int *rowPtrs, unsigned int *adj, int32_t *weights, long n, long m, int s, int r, int numCoord);
  int run(int tries = 1, int alpha = 15, int beta = 18, int32_t delta = 1) override;
};

#endif /* PARHDE_GB300_DRAWING_H_ */
