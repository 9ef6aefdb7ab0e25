// embed.cpp -- drop-in replacement for the reference driver (spectralDrawing.cpp:67-203).
//
// Same command line (getopt string "w:hc:a:p:r:", so -w takes an argument exactly as in the reference),
// same binary CSR input (6 int64 header words, uint32 offsets, uint32 adjacency, int32 weights with -w),
// same output file <input>_hde.nxyz written with the default ostream float format, same progress lines.
// The layout itself runs on the GPU through the C++ class interface (include/parhde_drawing.h).
#include <getopt.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "parhde_drawing.h"

static void write_coords(long n, const double *xy, int c, const char *input) {
  std::string name(input);
  name += "_hde.nxyz";
  std::cout << "Writing coordinates to file " << name << std::endl;
  // the library's parallel writer: the reference's ostream formatting, byte for byte
  if (phde_write_nxyz(name.c_str(), xy, n, c, 0) != PHDE_OK) std::cerr << "cannot write " << name << std::endl;
}

int main(int argc, char **argv) {
  if (argc < 2) {
    std::cerr << "Usage: " << argv[0] << " [csr filename] [-w x] [-c n] [-a algo] [-p strat] [-r k] [-h]" << std::endl;
    return 1;
  }
  char *input = argv[1];
  int weighted = 0, numCoord = 2, doRand = 2, algo = 3, numSources = 10, opt;
  while ((opt = getopt(argc, argv, "w:hc:a:p:r:")) != -1) {
    switch (opt) {
      case 'w': weighted = 1; break;
      case 'c': numCoord = atoi(optarg); break;
      case 'p':
        if (!strcmp(optarg, "RandFine")) doRand = 1;
        else if (!strcmp(optarg, "RandCoarse")) doRand = 0;
        else if (!strcmp(optarg, "Kcenters")) doRand = 2;
        // beyond the reference's strategies (ParHDE only; the help text stays the reference's)
        else if (!strcmp(optarg, "Learned")) doRand = PHDE_STRAT_LEARNED;
        else if (!strcmp(optarg, "LearnedChecked")) doRand = PHDE_STRAT_LEARNED_CHECKED;
        else { std::cerr << "Unrecognized Strategy" << std::endl; abort(); }
        break;
      case 'a':
        if (!strcmp(optarg, "PivotMDS")) algo = 0;
        else if (!strcmp(optarg, "PHDE")) algo = 1;
        else if (!strcmp(optarg, "wParHDE")) algo = 2;
        else if (!strcmp(optarg, "ParHDE")) algo = 3;
        else { std::cerr << "Unrecognized algorithm" << std::endl; abort(); }
        break;
      case 'r': numSources = atoi(optarg); break;
      case 'h':
        std::cout << "Usage: " << argv[0] << " [csr filename]\n"
                  << "-w         : Indicates if CSR file is weighted or unweighted (default)\n"
                  << "-c <value> : number of coordinates to generate( default=2)\n"
                  << "-a <algo>  : Indicate the algorithm to run (PivotMDS,PHDE, wParHDE, ParHDE(default))\n"
                  << "-p <strat> : Pivot picking strategy to use (RandFine,RandCoarse,Kcenters(default))\n"
                  << "-r <value> : Number of pivots (default=10)\n"
                  << "-h         : help" << std::endl;
        exit(1);
      default: abort();
    }
  }
  auto t0 = std::chrono::high_resolution_clock::now();
  FILE *f = fopen(input, "rb");
  if (!f) {
    std::cout << "Error: Could not open input file. Exiting ..." << std::endl;
    return 1;
  }
  long hdr[6];
  if (fread(hdr, sizeof(long), 6, f) != 6 || hdr[0] <= 0 || hdr[1] < 0) {
    std::cout << "Error: malformed CSR header. Exiting ..." << std::endl;
    fclose(f);
    return 1;
  }
  const long n = hdr[0], m = hdr[1];
  std::vector<unsigned> row((size_t)n + 1), adj((size_t)(m > 0 ? m : 1));
  std::vector<int32_t> w;
  bool ok = fread(row.data(), sizeof(unsigned), n + 1, f) == (size_t)(n + 1) &&
            fread(adj.data(), sizeof(unsigned), m, f) == (size_t)m;
  if (ok && weighted) {
    w.resize((size_t)(m > 0 ? m : 1));
    ok = fread(w.data(), sizeof(int32_t), m, f) == (size_t)m;
  }
  fclose(f);
  if (!ok) {
    std::cout << "Error: truncated CSR file. Exiting ..." << std::endl;
    return 1;
  }
  std::chrono::duration<double> el = std::chrono::high_resolution_clock::now() - t0;
  std::cout << "CSR read time: " << el.count() << " s." << std::endl;
  std::cout << "Num edges: " << m / 2 << ", vertices: " << n << ", nnz: " << m << std::endl;

  int32_t *wp = weighted ? w.data() : nullptr;
  DrawingBase *d = nullptr;
  switch (algo) {
    case 0: d = new PivotMDS(row.data(), adj.data(), nullptr, n, m, numSources, doRand, numCoord); break;
    case 1: d = new PHDE(row.data(), adj.data(), nullptr, n, m, numSources, doRand, numCoord); break;
    case 2: d = new WParHDE(row.data(), adj.data(), wp, n, m, numSources, numCoord); break;
    default: d = new ParHDE(row.data(), adj.data(), nullptr, n, m, numSources, doRand, numCoord); break;
  }
  d->run(1);
  write_coords(n, d->getCoordinates(), numCoord, input);
  delete d;
  el = std::chrono::high_resolution_clock::now() - t0;
  std::cout << "Overall time: " << el.count() << " s." << std::endl;
  return 0;
}
