"""Reference file formats: the binary ``.csr`` graph and the text ``.nxyz`` layout.

``.csr`` (written by ``mtx2csr.cpp:281-295``, read by ``spectralDrawing.cpp:136-168``):
six little-endian int64 header words ``{n, nnz, undirected=1, graph_type=0, one_indexed=1,
verification=0}``, then ``uint32 offsets[n+1]``, ``uint32 adj[nnz]`` and, for weighted graphs,
``int32 weights[nnz]``.  Whether weights are present is not recorded in the header: the reader is
told (the reference's ``-w`` flag).

``.nxyz`` (``spectralDrawing.cpp:42-65``): one line per vertex, the coordinates separated by commas,
printed with the default ``std::ostream`` float format (``%g``, 6 significant digits).  The file name
is ``<input>_hde.nxyz``.
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

HEADER_WORDS = 6


@dataclass
class CSRGraph:
    """An undirected graph in the reference's CSR layout (both directions stored)."""

    offsets: np.ndarray  # uint32 or int64 [n+1]
    adj: np.ndarray  # uint32 [nnz]
    weights: Optional[np.ndarray] = None  # int32 [nnz] or None
    name: str = ""

    @property
    def n(self) -> int:
        return int(self.offsets.shape[0] - 1)

    @property
    def nnz(self) -> int:
        return int(self.adj.shape[0])

    def degrees(self) -> np.ndarray:
        return np.diff(self.offsets.astype(np.int64))


def read_csr(path: str, weighted: bool = False) -> CSRGraph:
    """Read a reference ``.csr`` file (``spectralDrawing.cpp:138-164``)."""
    with open(path, "rb") as f:
        hdr = np.fromfile(f, dtype="<i8", count=HEADER_WORDS)
        if hdr.shape[0] != HEADER_WORDS:
            raise ValueError(f"{path}: truncated header")
        n, m = int(hdr[0]), int(hdr[1])
        if n <= 0 or m < 0:
            raise ValueError(f"{path}: bad header n={n} nnz={m}")
        off = np.fromfile(f, dtype="<u4", count=n + 1)
        adj = np.fromfile(f, dtype="<u4", count=m)
        if off.shape[0] != n + 1 or adj.shape[0] != m:
            raise ValueError(f"{path}: truncated CSR body")
        w = None
        if weighted:
            w = np.fromfile(f, dtype="<i4", count=m)
            if w.shape[0] != m:
                raise ValueError(f"{path}: truncated weights")
    return CSRGraph(off, adj, w, os.path.basename(path))


def write_csr(path: str, g: CSRGraph) -> None:
    """Write ``g`` in the reference ``.csr`` layout (``mtx2csr.cpp:281-295``)."""
    if g.nnz >= 2**32:
        raise ValueError("the .csr format stores uint32 offsets; nnz must be < 2^32")
    hdr = np.array([g.n, g.nnz, 1, 0, 1, 0], dtype="<i8")
    with open(path, "wb") as f:
        hdr.tofile(f)
        g.offsets.astype("<u4").tofile(f)
        g.adj.astype("<u4").tofile(f)
        if g.weights is not None:
            g.weights.astype("<i4").tofile(f)


def format_nxyz(coords: np.ndarray) -> str:
    """Format an ``(n, c)`` coordinate array like ``writeCoords`` (``spectralDrawing.cpp:55-62``)."""
    lines = [",".join("%g" % v for v in row) for row in np.asarray(coords, dtype=np.float64)]
    return "\n".join(lines) + ("\n" if lines else "")


def write_nxyz(path: str, coords: np.ndarray) -> None:
    with open(path, "w") as f:
        f.write(format_nxyz(coords))


def read_nxyz(path: str) -> np.ndarray:
    return np.loadtxt(path, delimiter=",", ndmin=2)
