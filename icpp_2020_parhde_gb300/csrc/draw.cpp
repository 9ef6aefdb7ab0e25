// draw.cpp -- drop-in for the reference's draw tool (draw_graph.c): the same command line, messages and image,
// with the rasterisation on the GPU (phde_draw) and the PNG deflated by host threads (phde_draw_write_png).
//
//   draw <binary csr filename> <vertex coords filename> <output png filename> <num coordinates>
//        <first coord> <second coord>
//
// The CSR file is read as the reference reads it (draw_graph.c:162-174: n, m, four more header words, n + 1
// uint32 offsets, m uint32 neighbours; anything after is ignored).  The coordinate file holds one vertex per
// line, <num coordinates> numbers separated by commas (draw_graph.c:208-227); it is parsed by host threads.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "parhde.h"

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Parse vertices [v0, v1) whose text starts at p: numbers separated by commas and blanks, `nc` per vertex.
bool parse_block(const char *p, const char *end, long v0, long v1, int nc, int first, int second, double *x,
                 double *y) {
  std::vector<double> vals((size_t)nc);
  for (long v = v0; v < v1; v++) {
    for (int j = 0; j < nc; j++) {
      while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++;
      char *q = nullptr;
      vals[(size_t)j] = strtod(p, &q);
      if (q == p) return false;
      p = q;
      while (p < end && (*p == ' ' || *p == '\t')) p++;
      if (j + 1 < nc && p < end && *p == ',') p++;
    }
    x[v] = vals[(size_t)first];
    y[v] = vals[(size_t)second];
  }
  return true;
}

// Coordinates of n vertices, one per line; threads take line-aligned byte ranges.
bool read_coords(const char *path, long n, int nc, int first, int second, std::vector<double> &x,
                 std::vector<double> &y) {
  FILE *f = fopen(path, "rb");
  if (!f) return false;
  std::vector<char> buf;
  fseek(f, 0, SEEK_END);
  const long len = ftell(f);
  fseek(f, 0, SEEK_SET);
  buf.resize((size_t)std::max(len, 0L) + 1);
  const bool ok = len <= 0 || fread(buf.data(), 1, (size_t)len, f) == (size_t)len;
  fclose(f);
  if (!ok) return false;
  buf[(size_t)std::max(len, 0L)] = '\0';
  const char *base = buf.data(), *end = base + std::max(len, 0L);
  x.assign((size_t)n, 0.0);
  y.assign((size_t)n, 0.0);
  const int nt = (int)std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
  // cut points at line starts, then the lines (vertices) before each cut
  std::vector<const char *> cut(nt + 1);
  cut[0] = base;
  cut[nt] = end;
  for (int t = 1; t < nt; t++) {
    const char *c = base + (size_t)(end - base) * (size_t)t / (size_t)nt;
    while (c < end && c > base && c[-1] != '\n') c++;
    cut[t] = std::max(c, cut[t - 1]);
  }
  std::vector<long> lines(nt + 1, 0);
  {
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; t++)
      pool.emplace_back([&, t]() {
        long c = 0;
        for (const char *p = cut[t]; p < cut[t + 1]; p++) c += *p == '\n';
        lines[t + 1] = c;
      });
    for (auto &th : pool) th.join();
  }
  for (int t = 0; t < nt; t++) lines[t + 1] += lines[t];
  std::vector<char> good(nt, 1);
  {
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; t++)
      pool.emplace_back([&, t]() {
        const long v0 = std::min(lines[t], n), v1 = t + 1 == nt ? n : std::min(lines[t + 1], n);
        if (v1 > v0) good[t] = parse_block(cut[t], end, v0, v1, nc, first, second, x.data(), y.data());
      });
    for (auto &th : pool) th.join();
  }
  return std::all_of(good.begin(), good.end(), [](char g) { return g != 0; });
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 7) {
    fprintf(stderr,
            "Usage: %s <binary csr filename> <vertex coords filename> <output png filename> <num coordinates> "
            "<first coord> <second coord>\n",
            argv[0]);
    return 1;
  }
  const int nc = atoi(argv[4]), first = atoi(argv[5]) - 1, second = atoi(argv[6]) - 1;
  if (nc < 1 || first < 0 || first >= nc || second < 0 || second >= nc) {
    fprintf(stderr, "Error: the coordinates to draw must lie in 1..%d. Exiting ...\n", nc);
    return 1;
  }
  double t0 = now_s();
  const double t_total = t0;
  FILE *in = fopen(argv[1], "rb");
  if (!in) {
    fprintf(stderr, "Error: Could not open CSR file. Exiting ...\n");
    return 1;
  }
  long hdr[6];
  if (fread(hdr, sizeof(long), 6, in) != 6 || hdr[0] <= 0 || hdr[1] < 0) {
    fprintf(stderr, "Error: bad CSR header. Exiting ...\n");
    fclose(in);
    return 1;
  }
  const long n = hdr[0], m = hdr[1];
  std::vector<uint32_t> off((size_t)n + 1), adj((size_t)std::max(m, 1L));
  const bool rd = fread(off.data(), sizeof(uint32_t), (size_t)n + 1, in) == (size_t)n + 1 &&
                  (m == 0 || fread(adj.data(), sizeof(uint32_t), (size_t)m, in) == (size_t)m);
  fclose(in);
  if (!rd) {
    fprintf(stderr, "Error: truncated CSR file. Exiting ...\n");
    return 1;
  }
  fprintf(stderr, "CSR file read time: %9.6lf s\n", now_s() - t0);
  fprintf(stderr, "Num edges: %ld, num vertices: %u\n", m / 2, (unsigned)n);
  t0 = now_s();
  std::vector<double> x, y;
  if (!read_coords(argv[2], n, nc, first, second, x, y)) {
    fprintf(stderr, "Error: Could not read vertex coords file. Exiting ...\n");
    return 1;
  }
  fprintf(stderr, "Coord file read time: %9.6lf s\n", now_s() - t0);

  phde_ctx *ctx = nullptr;
  int dev = 0;
  if (const char *d = getenv("PHDE_DEVICE")) dev = atoi(d);
  int rc = phde_create(&ctx, dev);
  if (rc == PHDE_OK) rc = phde_graph_upload(ctx, off.data(), 4, adj.data(), nullptr, n, m);
  phde_draw_info info;
  t0 = now_s();
  if (rc == PHDE_OK) rc = phde_draw(ctx, x.data(), y.data(), &info);
  if (rc != PHDE_OK) {
    fprintf(stderr, "Error: %s: %s\n", phde_status_string(rc), ctx ? phde_last_error(ctx) : "");
    phde_destroy(ctx);
    return 1;
  }
  fprintf(stderr, "xmin %lf xmax %lf ymin %lf ymax %lf, aspect ratio %3.4lf\n", info.xmin, info.xmax, info.ymin,
          info.ymax, info.aspect);
  fprintf(stderr, "Computed width %u, height %u\n", info.width_computed, info.height_computed);
  fprintf(stderr, "Corrected width %u, height %u\n", info.width, info.height);
  printf("Image generation\n");
  printf("Max edge length: %f\n", info.max_edge_length);
  fprintf(stderr, "Image array generation time: %9.6lf s\n", now_s() - t0);
  t0 = now_s();
  rc = phde_draw_write_png(ctx, argv[3], 0);
  fprintf(stderr, "Png file write time: %9.6lf s\n", now_s() - t0);
  if (rc != PHDE_OK) printf("error %d: %s\n", rc, phde_last_error(ctx));
  phde_destroy(ctx);
  fprintf(stderr, "Total Draw time: %9.6lf s\n", now_s() - t_total);
  return rc == PHDE_OK ? 0 : 1;
}
