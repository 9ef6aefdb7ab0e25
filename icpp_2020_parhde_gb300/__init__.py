"""GB300-native ParHDE layout pipeline.

Python mirror of the reference's operator interface (``variants/DrawingBase.h:41-47``): the classes
``ParHDE``, ``WParHDE``, ``PivotMDS`` and ``PHDE`` take the same constructor arguments as the C++
classes, ``run()`` computes the layout and ``getCoordinates()`` returns the unit-norm coordinates
as the reference's column-major ``double*`` (coordinate j of vertex i at ``i + j*n``).  ``DOBFS`` and
``DeltaStep`` mirror the two distance kernels (``variants/DrawingBase.h:62-67``).  Everything runs in
``libparhde_gb300.so`` on the GPU through the C ABI of ``include/parhde.h``; where the reference calls
``exit``/``abort`` these raise ``ParHDEError``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .csr_io import CSRGraph, read_csr, write_csr, format_nxyz, write_nxyz, read_nxyz  # noqa: F401

__all__ = ["Context", "ParHDEError", "LayoutResult", "DrawingBase", "ParHDE", "WParHDE", "PivotMDS", "PHDE",
           "DOBFS", "DeltaStep", "CSRGraph", "read_csr", "write_csr", "write_nxyz", "read_nxyz"]


class ParHDEError(RuntimeError):
    def __init__(self, status: int, message: str):
        self.status = status
        self.name = _lib.STATUS.get(status, str(status))
        super().__init__(f"{self.name}: {message}")


def _ptr(a, ct):
    return None if a is None else a.ctypes.data_as(C.POINTER(ct))


@dataclass
class LayoutResult:
    coords: np.ndarray  # (n, c)
    sources: np.ndarray
    stats: dict
    basis: np.ndarray | None = None  # (n, k)
    gram: np.ndarray | None = None  # (k, k): entry (p, q) = <S_p, (L S)_q>
    evecs: np.ndarray | None = None  # (k, k) eigenvectors in columns
    evals: np.ndarray | None = None  # (k,)
    extra: dict = field(default_factory=dict)


class Context:
    """One device context: a CUDA stream, the uploaded graph and the device workspace."""

    def __init__(self, device: int = 0):
        self._L = _lib.load()
        h = C.c_void_p()
        rc = self._L.phde_create(C.byref(h), device)
        if rc != 0:
            raise ParHDEError(rc, "could not create a context on device %d (CUDA missing or no GPU)" % device)
        self._h = h
        self.n = 0
        self.nnz = 0
        self.weighted = False

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.phde_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int) -> None:
        if rc != 0:
            raise ParHDEError(rc, self._L.phde_last_error(self._h).decode())

    @property
    def launch_count(self) -> int:
        return int(self._L.phde_launch_count(self._h))

    def upload(self, g: CSRGraph) -> None:
        off = np.ascontiguousarray(g.offsets)
        width = 8 if off.dtype in (np.int64, np.uint64) else 4
        off = off.astype(np.int64 if width == 8 else np.uint32, copy=False)
        adj = np.ascontiguousarray(g.adj, dtype=np.uint32)
        w = None if g.weights is None else np.ascontiguousarray(g.weights, dtype=np.int32)
        self._check(self._L.phde_graph_upload(self._h, off.ctypes.data_as(C.c_void_p), width, _ptr(adj, C.c_uint32),
                                              _ptr(w, C.c_int32), g.n, g.nnz))
        self.n, self.nnz, self.weighted = g.n, g.nnz, w is not None

    def layout(self, algo: str = "ParHDE", strategy: str = "Kcenters", k: int = 10, c: int = 2,
               precision: str = "fp64", eig: str = "power", seed: int = 1, verbose: bool = False,
               extra: bool = False, coords_out: np.ndarray | None = None) -> LayoutResult:
        o = _lib.LayoutOpts(_lib.ALGOS[algo], _lib.STRATEGIES[strategy], k, c, _lib.PRECISIONS[precision],
                            _lib.EIGS[eig], seed, 1 if verbose else 0)
        n = self.n
        coords = coords_out if coords_out is not None else np.empty(n * c, dtype=np.float64)
        sources = np.full(3 * k, -1, dtype=np.int64)
        st = _lib.LayoutStats()
        ex = None
        bufs = {}
        if extra:
            bufs = {"basis": np.empty(n * k), "gram": np.empty(k * k), "evecs": np.empty(k * k),
                    "evals": np.empty(k)}
            ex = _lib.LayoutExtra(*(_ptr(bufs[f], C.c_double) for f in ("basis", "gram", "evecs", "evals")))
        rc = self._L.phde_layout(self._h, C.byref(o), _ptr(coords, C.c_double), _ptr(sources, C.c_int64),
                                 C.byref(ex) if ex is not None else None, C.byref(st))
        self._check(rc)
        res = LayoutResult(coords.reshape(c, n).T, sources[: st.npasses].copy(), st.as_dict())
        if extra:
            res.basis = bufs["basis"].reshape(k, n).T.copy()
            res.gram = bufs["gram"].reshape(k, k).T.copy()
            res.evecs = bufs["evecs"].reshape(k, k).T.copy()
            res.evals = bufs["evals"]
        return res

    def set_pivot_model(self, weights) -> None:
        """phde_set_pivot_model: replace the learned strategy's MLP weights (4 -> 64 -> 64 -> 1, ReLU)."""
        w = np.ascontiguousarray(weights, dtype=np.float32)
        self._check(self._L.phde_set_pivot_model(self._h, _ptr(w, C.c_float), w.size))

    def pivot_scores(self, ncand: int = 256):
        """phde_pivot_scores: the learned strategy's proposal step alone -- (scores (n,), warm-start minimum
        distances (n,), the ncand candidates it takes)."""
        sc = np.empty(self.n, dtype=np.float32)
        d0 = np.empty(self.n, dtype=np.int32)
        cand = np.empty(ncand, dtype=np.int64)
        self._check(self._L.phde_pivot_scores(self._h, _ptr(sc, C.c_float), _ptr(d0, C.c_int32),
                                              _ptr(cand, C.c_int64), ncand))
        return sc, d0, cand

    def set_pivot_check(self, rule: str = "sum", tolerance: float = 0.02) -> None:
        """phde_set_pivot_check: the acceptance rule of the "LearnedChecked" strategy ("sum" of the quotients,
        or "each" coordinate) and its tolerance."""
        self._check(self._L.phde_set_pivot_check(self._h, {"sum": 0, "each": 1}[rule], float(tolerance)))

    def distances(self, sources) -> np.ndarray:
        src = np.ascontiguousarray(np.atleast_1d(sources), dtype=np.int64)
        out = np.empty(self.n * src.shape[0], dtype=np.int32)
        self._check(self._L.phde_distances(self._h, _ptr(src, C.c_int64), src.shape[0], _ptr(out, C.c_int32)))
        return out.reshape(src.shape[0], self.n).T

    def kcenters(self, passes: int, variant: int = 0, want_dist: bool = True):
        D = np.empty(self.n * passes, dtype=np.int32) if want_dist else None
        src = np.empty(passes, dtype=np.int64)
        self._check(self._L.phde_kcenters(self._h, passes, variant, _ptr(D, C.c_int32), _ptr(src, C.c_int64)))
        return (D.reshape(passes, self.n).T if D is not None else None), src

    def graph_from_entries(self, u, v, w, n1: int, n2: int, symmetric: bool) -> dict:
        """phde_graph_from_entries: Matrix Market entries (1-indexed) -> the uploaded graph, on the GPU (the
        reference's mtx2csr).  Returns the conversion counts."""
        u = np.ascontiguousarray(u, dtype=np.uint32)
        v = np.ascontiguousarray(v, dtype=np.uint32)
        wa = None if w is None else np.ascontiguousarray(w, dtype=np.int32)
        info = _lib.CsrInfo()
        self._check(self._L.phde_graph_from_entries(self._h, _ptr(u, C.c_uint32), _ptr(v, C.c_uint32),
                                                    _ptr(wa, C.c_int32), u.shape[0], n1, n2, 1 if symmetric else 0,
                                                    C.byref(info)))
        self.n, self.nnz, self.weighted = info.n, info.nnz, wa is not None
        return {f: getattr(info, f) for f, _ in info._fields_}

    def download(self) -> CSRGraph:
        """phde_graph_download: the uploaded graph as host arrays (uint32 offsets)."""
        off = np.empty(self.n + 1, dtype=np.uint32)
        adj = np.empty(max(self.nnz, 1), dtype=np.uint32)
        w = np.empty(max(self.nnz, 1), dtype=np.int32) if self.weighted else None
        self._check(self._L.phde_graph_download(self._h, _ptr(off, C.c_uint32), _ptr(adj, C.c_uint32),
                                                _ptr(w, C.c_int32)))
        return CSRGraph(off, adj[: self.nnz], None if w is None else w[: self.nnz])

    def upload_batch(self, graphs) -> None:
        """Upload many graphs as one batch (phde_batch_upload); they keep their own local vertex ids."""
        keep, descs = [], []
        wide = any(np.asarray(g.offsets).dtype in (np.int64, np.uint64) for g in graphs)
        for g in graphs:
            off = np.ascontiguousarray(g.offsets, dtype=np.int64 if wide else np.uint32)
            adj = np.ascontiguousarray(g.adj, dtype=np.uint32)
            keep += [off, adj]
            descs.append(_lib.GraphDesc(off.ctypes.data, 8 if wide else 4, adj.ctypes.data, g.n, g.nnz))
        arr = (_lib.GraphDesc * len(descs))(*descs)
        self._check(self._L.phde_batch_upload(self._h, arr, len(descs)))
        self.batch_sizes = [g.n for g in graphs]
        self.n, self.nnz, self.weighted = sum(self.batch_sizes), sum(g.nnz for g in graphs), False

    def layout_batched(self, k: int = 10, c: int = 2, coords_out: np.ndarray | None = None,
                       strategy: str = "Kcenters", precision: str = "mixed", eig: str = "exact",
                       algo: str = "ParHDE"):
        """phde_layout_batched: (list of per-graph (n_b, c) coordinate arrays, stats dict).  ParHDE with strategy
        "Kcenters" or "Learned", precision "mixed", eig "exact", k <= 32 and c <= 4 run the fused batched
        pipeline; other options lay the graphs out one by one with the single-graph pipeline."""
        o = _lib.LayoutOpts(_lib.ALGOS[algo], _lib.STRATEGIES[strategy], k, c, _lib.PRECISIONS[precision],
                            _lib.EIGS[eig], 1, 0)
        total = sum(self.batch_sizes)
        out = coords_out if coords_out is not None else np.empty(total * c, dtype=np.float64)
        st = _lib.LayoutStats()
        self._check(self._L.phde_layout_batched(self._h, C.byref(o), _ptr(out, C.c_double), C.byref(st)))
        self._last_batch_c = c
        res, base = [], 0
        for nb in self.batch_sizes:
            res.append(out[c * base: c * (base + nb)].reshape(c, nb).T)
            base += nb
        return res, st.as_dict()

    def batch_rayleigh(self) -> np.ndarray:
        """phde_batch_rayleigh: (graphs, c) Rayleigh quotients of the last batched layout."""
        c = self._last_batch_c
        rq = np.empty(len(self.batch_sizes) * c, dtype=np.float64)
        self._check(self._L.phde_batch_rayleigh(self._h, _ptr(rq, C.c_double)))
        return rq.reshape(-1, c)

    def gram_f32(self, A, B, w=None, nsplit: int = 0) -> np.ndarray:
        """phde_gram_f32: A^T diag(w) B (FP64 result) on the tensor cores, for FP32 row-major A (n, p), B (n, q)."""
        A = np.ascontiguousarray(A, dtype=np.float32)
        B = np.ascontiguousarray(B, dtype=np.float32)
        n, p = A.shape
        q = B.shape[1]
        if B.shape[0] != n:
            raise ValueError("A and B need the same rows")
        wa = None if w is None else np.ascontiguousarray(w, dtype=np.float64)
        G = np.empty((p, q), dtype=np.float64)
        self._check(self._L.phde_gram_f32(self._h, _ptr(A, C.c_float), p, p, _ptr(B, C.c_float), q, q,
                                          _ptr(wa, C.c_double), n, nsplit, _ptr(G, C.c_double)))
        return G

    def symeig(self, M, c: int, largest: bool = False):
        """phde_symeig: the layouts' exact eigensolver on a symmetric k x k matrix.  Returns (evals ascending,
        Y (k, c): the eigenvectors of the c smallest -- or largest, largest first -- eigenvalues, sweeps)."""
        Mf = np.asfortranarray(M, dtype=np.float64)
        k = Mf.shape[0]
        if Mf.shape != (k, k):
            raise ValueError("M must be square")
        ev = np.empty(k, dtype=np.float64)
        Y = np.empty((c, k), dtype=np.float64)  # column-major k x c
        it = C.c_int(0)
        self._check(self._L.phde_symeig(self._h, Mf.ctypes.data_as(C.POINTER(C.c_double)), k, c, int(largest),
                                        _ptr(ev, C.c_double), _ptr(Y, C.c_double), C.byref(it)))
        return ev, Y.T.copy(), it.value

    def draw(self, x, y) -> dict:
        """phde_draw: rasterise the uploaded graph at vertex positions (x, y) on the GPU (the reference's draw
        tool).  Returns the image geometry and timings; the image stays on the device."""
        xa = np.ascontiguousarray(x, dtype=np.float64)
        ya = np.ascontiguousarray(y, dtype=np.float64)
        if xa.shape != (self.n,) or ya.shape != (self.n,):
            raise ValueError("x and y need one value per vertex (%d)" % self.n)
        info = _lib.DrawInfo()
        self._check(self._L.phde_draw(self._h, _ptr(xa, C.c_double), _ptr(ya, C.c_double), C.byref(info)))
        self.draw_size = (int(info.width), int(info.height))
        return info.as_dict()

    def draw_image(self, out: np.ndarray | None = None) -> np.ndarray:
        """phde_draw_download: the drawn image as an (height, width, 4) RGBA uint8 array."""
        W, H = self.draw_size
        img = out if out is not None else np.empty((H, W, 4), dtype=np.uint8)
        self._check(self._L.phde_draw_download(self._h, img.ctypes.data_as(C.POINTER(C.c_uint8)), img.nbytes))
        return img

    def draw_png(self, path: str, nthreads: int = 0) -> None:
        """phde_draw_write_png: the drawn image as a PNG file."""
        self._check(self._L.phde_draw_write_png(self._h, path.encode(), nthreads))

    def selftest_barrier_timeout(self, timeout_ms: int = 50) -> int:
        return int(self._L.phde_selftest_barrier_timeout(self._h, timeout_ms))


def write_nxyz_fast(path: str, coords: np.ndarray, nthreads: int = 0) -> None:
    """phde_write_nxyz: the .nxyz file of an (n, c) coordinate array, formatted by host threads in the
    library -- byte-identical to ``csr_io.write_nxyz`` and the reference's writeCoords."""
    X = np.asarray(coords, dtype=np.float64)
    n, c = X.shape
    colmajor = np.ascontiguousarray(X.T).ravel()
    rc = _lib.load().phde_write_nxyz(path.encode(), _ptr(colmajor, C.c_double), n, c, nthreads)
    if rc != 0:
        raise ParHDEError(rc, "phde_write_nxyz failed for " + path)


def write_png(path: str, rgba: np.ndarray, nthreads: int = 0) -> None:
    """phde_write_png: an (height, width, 4) RGBA uint8 image as a PNG file (palette when it has at most 256
    colours), deflated by host threads in the library."""
    img = np.ascontiguousarray(rgba, dtype=np.uint8)
    if img.ndim != 3 or img.shape[2] != 4:
        raise ValueError("rgba must be (height, width, 4)")
    H, W = img.shape[:2]
    rc = _lib.load().phde_write_png(path.encode(), img.ctypes.data_as(C.POINTER(C.c_uint8)), W, H, nthreads)
    if rc != 0:
        raise ParHDEError(rc, "phde_write_png failed for " + path)


# ---------------------------------------------------------------------------------------------
# The reference's class interface (variants/DrawingBase.h:41-47, ParHDE.h, WParHDE.h, PivotMDS.h, PHDE.h).

class DrawingBase:
    """``DrawingBase(rowPtrs, adj, weights, n, m, numSources, doRand, numCoord=2)``."""

    _algo = "ParHDE"

    def __init__(self, rowPtrs, adj, weights, n, m, numSources, doRand, numCoord=2, *, precision="fp64",
                 eig="power", seed=1, device=0, verbose=True):
        self.g = CSRGraph(np.asarray(rowPtrs), np.asarray(adj), None if weights is None else np.asarray(weights))
        if self.g.n != n or self.g.nnz != m:
            raise ParHDEError(-1, "n/m do not match the CSR arrays")
        self.numSources, self.doRand, self.numCoord = int(numSources), int(doRand), int(numCoord)
        self.precision, self.eig, self.seed, self.verbose = precision, eig, seed, verbose
        self.ctx = Context(device)
        self.ctx.upload(self.g)
        self.result: LayoutResult | None = None
        self.coordinates = np.zeros(n * self.numCoord)

    def run(self, tries: int = 11, alpha: int = 15, beta: int = 18, delta: int = 1) -> int:
        strategy = {0: "RandCoarse", 1: "RandFine", 2: "Kcenters"}[self.doRand]
        for _ in range(max(1, tries)):
            self.result = self.ctx.layout(self._algo, strategy, self.numSources, self.numCoord, self.precision,
                                          self.eig, self.seed, self.verbose)
        self.coordinates = np.asfortranarray(self.result.coords).ravel(order="F")
        return 0

    def getCoordinates(self) -> np.ndarray:
        """Unit-norm coordinates, column-major: coordinate j of vertex i at index i + j*n."""
        return self.coordinates


class ParHDE(DrawingBase):
    _algo = "ParHDE"

    def __init__(self, rowPtrs, adj, weights, n, m, s, r, numCoord, **kw):
        if weights is not None:
            raise ParHDEError(-10, "ParHDE code doesn't requires the weighted edges")
        super().__init__(rowPtrs, adj, None, n, m, s, r, numCoord, **kw)


class WParHDE(DrawingBase):
    """``WParHDE(rowPtrs, adj, weights, n, m, s, numCoord)``: always Kcenters (WParHDE.cpp:40-218).
    Unlike the reference (whose constructor drops numCoord, WParHDE.cpp:12-13), numCoord is honoured."""

    _algo = "wParHDE"

    def __init__(self, rowPtrs, adj, weights, n, m, s, numCoord=2, **kw):
        if weights is None:
            raise ParHDEError(-10, "Weighted ParHDE code requires the weighted edges")
        super().__init__(rowPtrs, adj, weights, n, m, s, 2, numCoord, **kw)


class PivotMDS(DrawingBase):
    _algo = "PivotMDS"


class PHDE(DrawingBase):
    _algo = "PHDE"


def DOBFS(row, col, source, numNodes, numEdges, dists, alpha=15, beta=18) -> None:
    """Hop distances from ``source`` into ``dists`` (float64, only reached entries written; bfs.cc:144-185)."""
    L = _lib.load()
    row = np.ascontiguousarray(row, dtype=np.uint32)
    col = np.ascontiguousarray(col, dtype=np.uint32)
    rc = L.phde_DOBFS(_ptr(row, C.c_uint32), _ptr(col, C.c_uint32), source, numNodes, numEdges,
                      _ptr(dists, C.c_double), alpha, beta)
    if rc != 0:
        raise ParHDEError(rc, "DOBFS failed")


def DeltaStep(row, col, weights, source, numNodes, numEdges, dist, delta) -> np.ndarray:
    """Weighted distances from ``source`` into ``dist`` (float64; kDistInf when unreached; sssp.cc:53-140)."""
    L = _lib.load()
    row = np.ascontiguousarray(row, dtype=np.uint32)
    col = np.ascontiguousarray(col, dtype=np.uint32)
    w = np.ascontiguousarray(weights, dtype=np.int32)
    rc = L.phde_DeltaStep(_ptr(row, C.c_uint32), _ptr(col, C.c_uint32), _ptr(w, C.c_int32), source, numNodes,
                          numEdges, _ptr(dist, C.c_double), delta)
    if rc != 0:
        raise ParHDEError(rc, "DeltaStep failed")
    return dist
