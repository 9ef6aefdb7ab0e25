/* draw_oracle.c -- CPU restatement of the reference's `draw` tool (draw_graph.c): vertex coordinates and a CSR
 * graph to an RGBA edge image.  TEST INFRASTRUCTURE ONLY: the checker for the GPU rasteriser, never shipped.
 *
 * One thread, in the reference's order, so that its order-dependent parts are reproduced exactly:
 *   - bounds start at xmin = ymin = 1, xmax = ymax = -1 (draw_graph.c:201-204, 223-226);
 *   - width = sqrt(100 n / aspect), height = aspect * width, both truncated to unsigned, divided by 10 when
 *     either exceeds 100000, else by 5 when either exceeds 20000 (draw_graph.c:233-249);
 *   - vertex positions scaled as ((-xmin + v) * (1 / (xmax - xmin))) * width, clamped to [0, width - 1]
 *     (draw_graph.c:254-268); pixels are their floors;
 *   - edge length = (float) sqrt(dx^2 + dy^2) of the floored positions, longest edge = max over all CSR
 *     entries (draw_graph.c:282-298); bin = (int) floor((len / max) * 7) in float (draw_graph.c:323);
 *   - every CSR entry u -> v, in CSR order, draws a Bresenham line from u to v (draw_graph.c:112-126), later
 *     lines overwriting earlier pixels, with the colour chosen by draw_line's bin counters
 *     (draw_graph.c:53-103), m = nnz / 2 (draw_graph.c:181, 324), including its case fall-throughs and the
 *     integer division of the first counter;
 *   - background (4, 4, 4, 255) (draw_graph.c:273-277).
 * A quotient that is not a number (every edge of length 0: 0 / 0) gives bin INT_MIN on x86-64 (cvttsd2si),
 * which no case matches: the line is black.  That outcome is restated here explicitly.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  long lw1, lw2, hg1, hg2; /* the four colour counters of draw_line */
} orc_counters;

/* draw_line's colour choice (draw_graph.c:53-103); returns 0xAABBGGRR. */
static uint32_t orc_line_colour(int bin, int nan_bin, long m, orc_counters *c) {
  unsigned R = 0, G = 0, B = 0;
  int set = 0;
  if (nan_bin) return 0xff000000u; /* no case matches: black */
  if (bin == 0) {
    if (m != 0 && c->lw1 / m == 0) { /* integer division, as draw_graph.c:57 */
      R = 251; G = 83; B = 73;
      c->lw1++;
      set = 1;
    }
  }
  if (!set && (bin == 0 || bin == 1)) { /* case 0 falls through into case 1 */
    if ((double)c->lw2 / (double)m <= 0.05) {
      R = 251; G = 165; B = 4;
      c->lw2++;
      set = 1;
    }
  }
  if (bin == 6) {
    if ((double)c->hg2 / (double)m <= 0.05) {
      R = 13; G = 152; B = 186;
      c->hg2++;
      set = 1;
    }
  }
  if (!set && (bin == 6 || bin == 5)) { /* case 6 falls through into case 5 */
    if ((double)c->hg1 / (double)m <= 0.05) {
      R = 4; G = 251; B = 4;
      c->hg1++;
      set = 1;
    }
  }
  if (!set) {
    int b = bin;
    if (b == 0 || b == 1) b += 2;
    if (b == 5 || b == 6) b -= 2;
    switch (b) {
      case 2: R = 251; G = 174; B = 66; break;
      case 3: R = 251; G = 251; B = 4; break;
      case 4: R = 154; G = 251; B = 50; break;
      default: break; /* bin 7 (the longest edges): black */
    }
  }
  return (uint32_t)R | ((uint32_t)G << 8) | ((uint32_t)B << 16) | 0xff000000u;
}

/* Bounds, aspect ratio and image size.  bounds: xmin, xmax, ymin, ymax, aspect.  dims: width and height as
 * computed, then as corrected.  Returns 0, or -1 when the size is not a positive 32-bit number (the reference
 * has undefined behaviour there). */
int orc_draw_geometry(const double *x, const double *y, long n, double *bounds, unsigned *dims) {
  double xmax = -1, xmin = 1, ymax = -1, ymin = 1;
  for (long i = 0; i < n; i++) {
    if (x[i] > xmax) xmax = x[i];
    if (x[i] < xmin) xmin = x[i];
    if (y[i] > ymax) ymax = y[i];
    if (y[i] < ymin) ymin = y[i];
  }
  const double aspect = (xmax - xmin) / (ymax - ymin);
  bounds[0] = xmin;
  bounds[1] = xmax;
  bounds[2] = ymin;
  bounds[3] = ymax;
  bounds[4] = aspect;
  const double wd = sqrt((double)(100 * n) / aspect);
  if (!(wd >= 1.0 && wd < 4294967296.0)) return -1;
  const unsigned w = (unsigned)wd;
  const double hd = aspect * (double)w;
  if (!(hd >= 1.0 && hd < 4294967296.0)) return -1;
  const unsigned h = (unsigned)hd;
  dims[0] = w;
  dims[1] = h;
  unsigned W = w, H = h;
  if (W > 100000 || H > 100000) {
    W /= 10;
    H /= 10;
  } else if (W > 20000 || H > 20000) {
    W /= 5;
    H /= 5;
  }
  dims[2] = W;
  dims[3] = H;
  return (W == 0 || H == 0) ? -1 : 0;
}

/* The image: rgba (W * H * 4 bytes, row-major, y down the rows as the reference indexes it).  max_len_out:
 * the longest edge (float).  Returns 0, or -1 on a bad size. */
int orc_draw(const uint32_t *off, const uint32_t *adj, long n, long nnz, const double *x, const double *y,
             unsigned char *rgba, unsigned W_expect, unsigned H_expect, float *max_len_out) {
  double bounds[5];
  unsigned dims[4];
  if (orc_draw_geometry(x, y, n, bounds, dims) != 0) return -1;
  const unsigned W = dims[2], H = dims[3];
  if (W != W_expect || H != H_expect) return -1;
  const double xmin = bounds[0], xmax = bounds[1], ymin = bounds[2], ymax = bounds[3];
  const double xri = 1.0 / (xmax - xmin), yri = 1.0 / (ymax - ymin);
  int *px = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  int *py = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  if (!px || !py) {
    free(px);
    free(py);
    return -1;
  }
  for (long i = 0; i < n; i++) {
    double vx = (-xmin + x[i]) * xri * W;
    double vy = (-ymin + y[i]) * yri * H;
    if (vx < 0) vx = 0;
    if (vy < 0) vy = 0;
    if (vx > (double)(W - 1)) vx = W - 1;
    if (vy > (double)(H - 1)) vy = H - 1;
    px[i] = (int)floor(vx);
    py[i] = (int)floor(vy);
  }
  float maxlen = 0;
  for (long u = 0; u < n; u++)
    for (long j = off[u]; j < (long)off[u + 1]; j++) {
      const long v = adj[j];
      const double dx = (double)(px[v] - px[u]), dy = (double)(py[v] - py[u]);
      const float len = (float)sqrt(dx * dx + dy * dy);
      if (len > maxlen) maxlen = len;
    }
  *max_len_out = maxlen;
  uint32_t *img = (uint32_t *)rgba;
  const size_t npix = (size_t)W * H;
  for (size_t p = 0; p < npix; p++) img[p] = 4u | (4u << 8) | (4u << 16) | 0xff000000u;
  orc_counters cnt = {0, 0, 0, 0};
  const long m = nnz / 2;
  for (long u = 0; u < n; u++)
    for (long j = off[u]; j < (long)off[u + 1]; j++) {
      const long v = adj[j];
      int x0 = px[u], y0 = py[u];
      const int x1 = px[v], y1 = py[v];
      const double ddx = (double)(x1 - x0), ddy = (double)(y1 - y0);
      const float len = (float)sqrt(ddx * ddx + ddy * ddy);
      const float q = (len / maxlen) * 7;
      const int nan_bin = q != q;
      const int bin = nan_bin ? 0 : (int)floor(q);
      const uint32_t col = orc_line_colour(bin, nan_bin, m, &cnt);
      const int dx = abs(x1 - x0), sx = x0 < x1 ? 1 : -1;
      const int dy = abs(y1 - y0), sy = y0 < y1 ? 1 : -1;
      int err = (dx > dy ? dx : -dy) / 2;
      for (;;) {
        img[(size_t)W * (size_t)y0 + (size_t)x0] = col;
        if (x0 == x1 && y0 == y1) break;
        const int e2 = err;
        if (e2 > -dx) {
          err -= dy;
          x0 += sx;
        }
        if (e2 < dy) {
          err += dx;
          y0 += sy;
        }
      }
    }
  free(px);
  free(py);
  return 0;
}
