// nxyz.cpp -- parallel .nxyz writer (host code).
//
// The reference writes one line per vertex, "x0,x1[,x2]", through std::ostream's default floating-point
// formatting (spectralDrawing.cpp:42-65), i.e. printf's %g with 6 significant digits; at 646k vertices that
// single-threaded text write takes longer than the whole GPU layout.  Here row ranges are formatted by
// several threads with the same %g conversion into private buffers, then written in order, so the file is
// byte-identical to the reference's.
#include <algorithm>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

#include "parhde.h"

namespace {

void format_rows(const double *xy, int64_t n, int c, int64_t r0, int64_t r1, std::string &out) {
  char num[64];
  out.clear();
  out.reserve((size_t)(r1 - r0) * (size_t)c * 13);
  for (int64_t i = r0; i < r1; i++) {
    for (int j = 0; j < c; j++) {
      const int len = snprintf(num, sizeof(num), "%g", xy[i + (int64_t)j * n]);
      out.append(num, (size_t)len);
      out.push_back(j + 1 < c ? ',' : '\n');
    }
  }
}

}  // namespace

extern "C" int phde_write_nxyz(const char *path, const double *coords, int64_t n, int c, int nthreads) {
  if (!path || (!coords && n > 0) || n < 0 || c < 1) return PHDE_ERR_INVALID;
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  nthreads = (int)std::max<int64_t>(1, std::min<int64_t>(nthreads, (n + 4095) / 4096));
  std::vector<std::string> parts((size_t)nthreads);
  std::vector<std::thread> pool;
  const int64_t per = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    const int64_t r0 = std::min<int64_t>(n, t * per), r1 = std::min<int64_t>(n, r0 + per);
    pool.emplace_back(format_rows, coords, n, c, r0, r1, std::ref(parts[(size_t)t]));
  }
  for (auto &th : pool) th.join();
  FILE *f = fopen(path, "wb");
  if (!f) return PHDE_ERR_INVALID;
  bool ok = true;
  for (const auto &p : parts)
    if (!p.empty() && fwrite(p.data(), 1, p.size(), f) != p.size()) ok = false;
  if (fclose(f) != 0) ok = false;
  return ok ? PHDE_OK : PHDE_ERR_INVALID;
}
