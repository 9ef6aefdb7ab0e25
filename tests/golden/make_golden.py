"""Generate the golden fixtures in tests/golden/ by running the REFERENCE itself.

The reference ParHDE sources are compiled (oracle/build_ref.sh, in place, never copied) into
oracle/_ref/libparhde_ref.so and called through oracle/ref_harness.cpp exactly as the reference driver
calls them (spectralDrawing.cpp:176-193), at ONE OpenMP thread so that the Kcenters tie-breaking and
every floating-point reduction are deterministic.  Recorded per case:

  csr_offsets / csr_adj / csr_weights   the input graph (seeded synthetic, see graphs.py)
  bfs_src, bfs_dist                     reference DOBFS / DeltaStep distance columns (int32; -1 unreached)
  sources                               the source vertex of every distance pass, in call order
  coords                                the reference's getCoordinates() output, (n, c)

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from icpp_2020_parhde_gb300 import graphs  # noqa: E402
from oracle import oracle as orc  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

CASES = [
    # name, graph factory, [(algo, k, c)], bfs sources
    ("mesh125", lambda: graphs.mesh(125, 125, seed=1),
     [("ParHDE", 10, 2), ("PivotMDS", 10, 2), ("PHDE", 10, 2)], [0, 7777, 15624]),
    ("rmat13", lambda: graphs.rmat(13, seed=3),
     [("ParHDE", 10, 3), ("ParHDE", 50, 3), ("PivotMDS", 10, 2)], [0, 100, 4000]),
    ("grid12w", lambda: graphs.grid3d(12, seed=5), [("wParHDE", 10, 2)], [0, 1000, 1727]),
    ("rgg2d_3k", lambda: graphs.rgg(3000, dim=2, avg_degree=8, seed=7), [("ParHDE", 10, 2)], [0, 500]),
    # degenerate cases: more distance passes than vertices exercise the duplicate-source fix-up
    # (ParHDE.cpp:144-154, DrawingBase.cpp:428-438) and discarded vectors (ParHDE.cpp:267)
    ("path20", lambda: graphs.path_graph(20), [("ParHDE", 7, 2)], [0, 19]),
    ("complete12", lambda: graphs.complete_graph(12), [("ParHDE", 7, 2), ("PivotMDS", 7, 2)], [3]),
    ("star20", lambda: graphs.star_graph(20), [("ParHDE", 7, 2), ("PivotMDS", 7, 2)], [0, 5]),
]


def main() -> None:
    orc.build_reference()
    if not orc.ref_available():
        raise SystemExit("the reference build (oracle/_ref) is not available")
    for name, make, runs, bsrc in CASES:
        g = make()
        rec = {"csr_offsets": g.offsets.astype(np.uint32), "csr_adj": g.adj.astype(np.uint32)}
        if g.weights is not None:
            rec["csr_weights"] = g.weights.astype(np.int32)
        cols = []
        for s in bsrc:
            d = orc.ref_sssp(g, s, 1) if g.weights is not None else orc.ref_bfs(g, s, 1)
            cols.append(np.where(np.isfinite(d) & (d >= 0), d, -1).astype(np.int32))
        rec["bfs_src"] = np.array(bsrc, dtype=np.int64)
        rec["bfs_dist"] = np.stack(cols, axis=1)
        for algo, k, c in runs:
            coords, sources = orc.ref_layout(g, algo, "Kcenters", k, c, nthreads=1)
            rec[f"{algo}_k{k}_c{c}_sources"] = sources
            rec[f"{algo}_k{k}_c{c}_coords"] = coords
        path = os.path.join(OUT, f"{name}.npz")
        np.savez_compressed(path, **rec)
        print(f"{path}: n={g.n} nnz={g.nnz} runs={[r[:3] for r in runs]} {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
