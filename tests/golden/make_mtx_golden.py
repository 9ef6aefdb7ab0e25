"""Writes the Matrix Market fixtures under tests/golden/mtx/ and the reference converter's output for each
(oracle/_ref/mtx2csr, built from the reference's own mtx2csr.cpp by oracle/build_ref.sh).

    python tests/golden/make_mtx_golden.py
"""
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "mtx")
REF = os.path.join(ROOT, "oracle", "_ref", "mtx2csr")


def write(name, header, n1, n2, entries):
    path = os.path.join(OUT, name + ".mtx")
    with open(path, "w") as f:
        f.write(header + "\n% seeded fixture\n")
        f.write("%d %d %d\n" % (n1, n2, len(entries)))
        for e in entries:
            f.write(" ".join(str(x) for x in e) + "\n")
    return path


def cases():
    rng = np.random.default_rng(2020)
    # symmetric pattern: three components (sizes 40, 25, 25), self loops, repeated entries in both orders
    e = []
    for base, size in ((0, 40), (40, 25), (65, 25)):
        for _ in range(size * 3):
            a, b = rng.integers(base + 1, base + size + 1, 2)
            e.append((int(a), int(b)))
        for i in range(base + 1, base + size):
            e.append((i + 1, i))  # a path keeps each component connected
    e += [(5, 5), (3, 3), (7, 2), (2, 7), (7, 2)]
    yield "sym_pattern", "%%MatrixMarket matrix coordinate pattern symmetric", 90, 90, e
    # general real square: asymmetric entries, weights dropped
    e = [(int(a), int(b), float(rng.standard_normal())) for a, b in rng.integers(1, 61, (300, 2))]
    yield "general_real", "%%MatrixMarket matrix coordinate real general", 60, 60, e
    # general integer square: parallel entries with different weights (the smallest is kept)
    e = [(int(a), int(b), int(rng.integers(-50, 200))) for a, b in rng.integers(1, 51, (260, 2))]
    e += [(4, 9, 17), (9, 4, 3), (4, 9, -8)]
    yield "general_integer", "%%MatrixMarket matrix coordinate integer general", 50, 50, e
    # general pattern, not square: a bipartite graph
    e = [(int(a), int(b)) for a, b in zip(rng.integers(1, 31, 120), rng.integers(1, 46, 120))]
    yield "bipartite", "%%MatrixMarket matrix coordinate pattern general", 30, 45, e
    # symmetric integer with two equally large components: the one found first (lowest vertex) is kept
    e = []
    for base in (10, 0, 20):
        for i in range(1, 10):
            e.append((base + i, base + i + 1, int(rng.integers(1, 255))))
    yield "sym_integer_tie", "%%MatrixMarket matrix coordinate integer symmetric", 30, 30, e


def main():
    os.makedirs(OUT, exist_ok=True)
    for name, header, n1, n2, e in cases():
        path = write(name, header, n1, n2, e)
        subprocess.check_call([REF, path, os.path.join(OUT, name + ".csr")], stdout=subprocess.DEVNULL)
        print("wrote", name)


if __name__ == "__main__":
    main()
