#!/bin/sh
# Builds the reference ParHDE sources, read in place from the ParHDE tree (never copied), into
# oracle/_ref/: libparhde_ref.so (reference classes + ref_harness.cpp, for golden generation and
# oracle pinning), embed (the reference driver, for .nxyz comparisons and CPU timing), mtx2csr (the
# reference's Matrix Market converter, for the converter's golden files) and draw (the reference's
# edge-image tool, for the rasteriser's golden images).
# Test infrastructure only.  Usage: oracle/build_ref.sh [path-to-ParHDE-tree]
set -e
REF=${1:-${PARHDE_REF_SRC:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/variants/ParHDE.cpp" ]; then echo "reference tree not found at $REF" >&2; exit 2; fi
mkdir -p "$OUT"
CXX=${CXX:-g++}
# the reference's own flags (Makefile:6,29-30,43-52), plus -fPIC for the shared library
FLAGS="-O2 -fopenmp -fPIC -std=c++11 -Wno-attributes -w"
INC="-I$HERE/gapbs_shim -I$REF/gapbs -I$REF/variants"
cd "$OUT"
$CXX $FLAGS $INC -DDOBFS=ref_impl_DOBFS -c "$REF/gapbs/bfs.cc" -o bfs_h.o &
$CXX $FLAGS $INC -DDeltaStep=ref_impl_DeltaStep -c "$REF/gapbs/sssp.cc" -o sssp_h.o &
$CXX $FLAGS $INC -c "$REF/gapbs/bfs.cc" -o bfs.o &
$CXX $FLAGS $INC -c "$REF/gapbs/sssp.cc" -o sssp.o &
for f in DrawingBase ParallelComponents PivotMDS PHDE WParHDE; do
  $CXX $FLAGS $INC -c "$REF/variants/$f.cpp" -o "$f.o" &
done
# ParHDE.cpp sizes its per-vector scratch with '#define S_MAX 51' (k <= 50, ParHDE.cpp:15); the source
# is streamed to the compiler with that one constant raised to 257 so that k up to 256 can be pinned.
sed 's/^#define S_MAX 51$/#define S_MAX 257/' "$REF/variants/ParHDE.cpp" |
  $CXX $FLAGS $INC -x c++ -c - -o ParHDE.o &
$CXX $FLAGS $INC -c "$HERE/ref_harness.cpp" -o ref_harness.o &
wait
VAR="DrawingBase.o ParallelComponents.o PivotMDS.o PHDE.o WParHDE.o ParHDE.o"
$CXX -shared -fopenmp -o libparhde_ref.so bfs_h.o sssp_h.o $VAR ref_harness.o
$CXX $FLAGS $INC "$REF/spectralDrawing.cpp" bfs.o sssp.o $VAR -o embed -lm
$CXX -O2 -std=c++11 -w "$REF/mtx2csr.cpp" -o mtx2csr
# the reference's draw tool with its own flags (Makefile:6,37-38); run with OMP_NUM_THREADS=1 for its serial order
${CC:-gcc} -std=c99 -O2 -fopenmp -w "$REF/draw_graph.c" "$REF/lodepng.c" -o draw -lm
echo "built $OUT/libparhde_ref.so, $OUT/embed, $OUT/mtx2csr and $OUT/draw"
