// mtx2csr.cpp -- drop-in for the reference's mtx2csr tool (mtx2csr.cpp): the same command line, messages and
// binary CSR output, with the graph work (symmetrisation, deduplication, largest connected component,
// renumbering) on the GPU through phde_graph_from_entries.  The Matrix Market text is parsed here, on the
// host: header words as the reference reads them ("coordinate" required; "general" = not symmetric;
// "real" weights read and dropped, "integer" weights kept), then one entry per line.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "parhde.h"

namespace {

// The next unsigned integer at p (skipping blanks); false at the end of the line.
bool next_uint(const char *&p, const char *end, unsigned long long &x) {
  while (p < end && (*p == ' ' || *p == '\t')) p++;
  if (p >= end || *p < '0' || *p > '9') return false;
  x = 0;
  while (p < end && *p >= '0' && *p <= '9') x = x * 10 + (unsigned long long)(*p++ - '0');
  return true;
}

}  // namespace

int main(int argc, char *argv[]) {
  if (argc != 3) {
    std::cout << "Usage: " << argv[0] << " <MM filename> <binary CSR filename>\n";
    return 1;
  }
  FILE *in = fopen(argv[1], "rb");
  if (!in) {
    std::cout << "Error: could not open input file " << argv[1] << "! Exiting" << std::endl;
    return 1;
  }
  std::vector<char> buf;
  {
    fseek(in, 0, SEEK_END);
    const long len = ftell(in);
    fseek(in, 0, SEEK_SET);
    buf.resize((size_t)(len > 0 ? len : 0));
    if (len > 0 && fread(buf.data(), 1, (size_t)len, in) != (size_t)len) {
      std::cout << "Error: could not read input file " << argv[1] << "! Exiting" << std::endl;
      return 1;
    }
    fclose(in);
  }
  int symmetric = 1, pattern = 1;  // pattern: 1 pattern, 0 real (dropped), 2 integer (kept)
  long long n1 = 0, n2 = 0, m = 0, lines = 0;
  std::vector<uint32_t> u, v;
  std::vector<int32_t> w;
  const char *p = buf.data(), *end = buf.data() + buf.size();
  while (p < end) {
    const char *eol = (const char *)memchr(p, '\n', (size_t)(end - p));
    if (!eol) eol = end;
    if (*p == '%') {
      if (p + 1 < eol && p[1] == '%') {
        const std::string hdr(p, eol);
        if (hdr.find("coordinate") == std::string::npos) {
          std::cout << "Error: File is not in coordinate format! Exiting." << std::endl;
          return 1;
        }
        if (hdr.find("general") != std::string::npos) {
          std::cout << "Non-zero pattern is not symmetric." << std::endl;
          symmetric = 0;
        }
        if (hdr.find("pattern") == std::string::npos) {
          if (hdr.find("real") != std::string::npos) {
            std::cout << "Matrix has real weights, ignoring them." << std::endl;
            pattern = 0;
          }
          if (hdr.find("integer") != std::string::npos) {
            std::cout << "Matrix has integer weights, using them" << std::endl;
            pattern = 2;
          }
        }
      }
    } else if (eol > p) {
      lines++;
      if (lines == 1) {
        if (sscanf(std::string(p, eol).c_str(), "%lld %lld %lld", &n1, &n2, &m) != 3) {
          std::cout << "Error: bad size line! Exiting." << std::endl;
          return 1;
        }
        std::cout << "Matrix size: " << n1 << " " << n2 << " " << m << std::endl;
        if (!symmetric) {
          if (n1 == n2) {
            symmetric = 1;
            std::cout << "Reading general matrix as an undirected graph." << std::endl;
          } else {
            std::cout << "Reading general matrix as a bipartite graph." << std::endl;
          }
        } else if (n1 != n2) {
          std::cout << "Error: a symmetric matrix must be square! Exiting." << std::endl;
          return 1;
        }
        u.reserve((size_t)m);
        v.reserve((size_t)m);
        if (pattern == 2) w.reserve((size_t)m);
      } else {
        unsigned long long a = 0, b = 0;
        const char *q = p;
        if (!next_uint(q, eol, a) || !next_uint(q, eol, b)) {
          std::cout << "Error: bad entry on data line " << lines << "! Exiting." << std::endl;
          return 1;
        }
        u.push_back((uint32_t)a);
        v.push_back((uint32_t)b);
        if (pattern == 2) w.push_back((int32_t)strtol(q, nullptr, 10));
      }
    }
    p = eol + 1;
  }
  std::cout << lines - 1 << " lines read from file. Non-zero count is given to be " << m << "." << std::endl;

  phde_ctx *ctx = nullptr;
  int dev = 0;
  if (const char *d = getenv("PHDE_DEVICE")) dev = atoi(d);
  int rc = phde_create(&ctx, dev);
  if (rc) {
    std::cout << "Error: " << phde_status_string(rc) << std::endl;
    return 1;
  }
  phde_csr_info info;
  rc = phde_graph_from_entries(ctx, u.data(), v.data(), pattern == 2 ? w.data() : nullptr, (int64_t)u.size(), n1,
                               symmetric ? n1 : n2, symmetric, &info);
  if (rc) {
    std::cout << "Error: " << phde_status_string(rc) << ": " << phde_last_error(ctx) << std::endl;
    return 1;
  }
  std::cout << "After deduplication and self loop removal, n: " << info.n_in << ", m: " << info.nnz_dedup / 2
            << std::endl;
  if (info.ncomponents == 1)
    std::cout << "There is just one connected component." << std::endl;
  else
    std::cout << "There are " << info.ncomponents << " components and the largest component size is " << info.n
              << std::endl;
  std::cout << "Old edge count: " << info.nnz_dedup / 2 << ", new edge count: " << info.nnz / 2 << std::endl;
  long N = (long)info.n, M = (long)info.nnz;
  std::vector<uint32_t> off((size_t)N + 1), adj((size_t)std::max<long>(M, 1));
  std::vector<int32_t> wt(pattern == 2 ? (size_t)std::max<long>(M, 1) : 0);
  rc = phde_graph_download(ctx, off.data(), adj.data(), pattern == 2 ? wt.data() : nullptr);
  phde_destroy(ctx);
  if (rc) {
    std::cout << "Error: " << phde_status_string(rc) << std::endl;
    return 1;
  }
  std::cout << "Writing binary file to disk." << std::endl;
  FILE *out = fopen(argv[2], "wb");
  if (!out) {
    std::cout << "Error: could not open output CSR file " << argv[2] << "! Exiting" << std::endl;
    return 1;
  }
  // header {n, nnz, undirected, graph_type, one_indexed, verification} as the reference writes it
  const long hdr[6] = {N, M, 1, 0, 1, 0};
  fwrite(hdr, sizeof(long), 6, out);
  fwrite(off.data(), sizeof(uint32_t), (size_t)N + 1, out);
  if (M > 0) fwrite(adj.data(), sizeof(uint32_t), (size_t)M, out);
  if (pattern == 2 && M > 0) fwrite(wt.data(), sizeof(int32_t), (size_t)M, out);
  fclose(out);
  return 0;
}
