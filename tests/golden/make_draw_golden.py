"""Writes the draw fixtures under tests/golden/draw/: a graph (.csr), vertex coordinates (.nxyz) and the
reference's image of them (.png, made by oracle/_ref/draw -- the reference's own draw_graph.c and lodepng.c
compiled by oracle/build_ref.sh -- run with one OpenMP thread, its serial order), plus cases.json with the
command-line coordinate choice of each case.

    python tests/golden/make_draw_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
OUT = os.path.join(HERE, "draw")

from icpp_2020_parhde_gb300 import graphs  # noqa: E402
from icpp_2020_parhde_gb300.csr_io import CSRGraph, write_csr  # noqa: E402
from oracle import oracle as orc  # noqa: E402


def csr(n, pairs):
    """Undirected simple graph from (a, b) pairs: both directions, sorted, deduplicated, no self loops."""
    p = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    p = p[p[:, 0] != p[:, 1]]
    d = np.concatenate([p, p[:, ::-1]])
    d = np.unique(d[:, 0] * n + d[:, 1])
    src, dst = d // n, d % n
    off = np.zeros(n + 1, dtype=np.uint32)
    np.add.at(off, src + 1, 1)
    return CSRGraph(np.cumsum(off).astype(np.uint32), dst.astype(np.uint32), None, "draw")


def cases():
    rng = np.random.default_rng(2020)
    # a ParHDE layout of a small triangulated mesh, coordinates in the embed tool's %g format
    g = graphs.mesh(12, 10, seed=5)
    L = orc.layout(g, "ParHDE", "Kcenters", 6, 2, nthreads=1)
    yield "mesh_hde", g, L.coords, "%g", (2, 1, 2)
    # a grid with one corner-to-corner edge: almost every edge in the shortest bin, past its counter
    nx, ny = 20, 15
    idx = np.arange(nx * ny).reshape(ny, nx)
    pairs = [(a, b) for a, b in zip(idx[:, :-1].ravel(), idx[:, 1:].ravel())]
    pairs += [(a, b) for a, b in zip(idx[:-1, :].ravel(), idx[1:, :].ravel())]
    pairs.append((0, nx * ny - 1))
    pos = np.stack([np.tile(np.arange(nx), ny), np.repeat(np.arange(ny), nx)], axis=1).astype(np.float64)
    pos += rng.uniform(-0.2, 0.2, pos.shape)
    yield "grid_long", csr(nx * ny, pairs), pos, "%.17g", (2, 1, 2)
    # a random graph at random positions: lengths in every bin, every counter exhausted; three columns
    n = 200
    pairs = rng.integers(0, n, (900, 2))
    pos = np.column_stack([rng.uniform(-3, 5, n), rng.uniform(-2, 2, n), rng.uniform(0, 9, n)])
    yield "random_spread", csr(n, pairs), pos, "%.17g", (3, 3, 1)
    # a star at random positions inside (-1, 1): the bounds keep their starting values 1 and -1
    n = 60
    pos = np.column_stack([rng.uniform(-0.4, 0.3, n), rng.uniform(-0.2, 0.5, n)])
    yield "star_box", csr(n, [(0, i) for i in range(1, n)]), pos, "%.17g", (2, 1, 2)
    # two far clusters joined by every cross pair: the longest bins far past their counters
    k = 18
    pairs = [(a, b) for a in range(k) for b in range(k, 2 * k)]
    pairs += [(i, i + 1) for i in range(k - 1)] + [(k + i, k + i + 1) for i in range(k - 1)]
    pos = np.concatenate([rng.normal(0, 0.4, (k, 2)), rng.normal(0, 0.4, (k, 2)) + [9.0, 4.0]])
    yield "two_clusters", csr(2 * k, pairs), pos, "%.17g", (2, 1, 2)
    # pairs of vertices at the same position joined by one edge: every edge of length 0 (0 / 0 bins)
    n = 80
    pairs = [(2 * i, 2 * i + 1) for i in range(n // 2)]
    base = rng.uniform(0, 10, (n // 2, 2))
    pos = np.repeat(base, 2, axis=0)
    yield "zero_length", csr(n, pairs), pos, "%.17g", (2, 1, 2)


def main():
    if not orc.ref_draw_available():
        sys.exit("oracle/_ref/draw is missing: run oracle/build_ref.sh first")
    os.makedirs(OUT, exist_ok=True)
    meta = {}
    for name, g, pos, fmt, (nc, first, second) in cases():
        base = os.path.join(OUT, name)
        write_csr(base + ".csr", g)
        with open(base + ".nxyz", "w") as f:
            for row in np.asarray(pos, dtype=np.float64):
                f.write(",".join(fmt % v for v in row) + "\n")
        orc.ref_draw(base + ".csr", base + ".nxyz", base + ".png", nc, first, second)
        meta[name] = {"ncoords": nc, "first": first, "second": second, "n": int(g.n), "nnz": int(g.nnz)}
        print(name, meta[name], os.path.getsize(base + ".png"), "bytes")
    with open(os.path.join(OUT, "cases.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
