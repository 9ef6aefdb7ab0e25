"""ctypes bindings for the oracle (``parhde_oracle.c``) and for the reference build (``_ref/``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``
(its ``cpu_baseline`` leg and the ``--impl reference`` arm), never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB_PATH = os.path.join(REF_DIR, "libparhde_ref.so")
REF_EMBED_PATH = os.path.join(REF_DIR, "embed")

ALGOS = {"PivotMDS": 0, "PHDE": 1, "wParHDE": 2, "ParHDE": 3}
STRATEGIES = {"RandCoarse": 0, "RandFine": 1, "Kcenters": 2}
SSSP_INF = (2**31 - 1) // 2


def build_oracle(force: bool = False) -> str:
    """Compile parhde_oracle.c with the reference's optimisation level (-O2) and OpenMP.  No FMA contraction:
    the reference is built in ISO C++ mode, where gcc keeps a*b+c as two roundings on every architecture."""
    srcs = [os.path.join(HERE, f) for f in ("parhde_oracle.c", "draw_oracle.c")]
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(map(os.path.getmtime, srcs)):
        tmp = LIB_PATH + ".tmp"
        subprocess.check_call(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", *srcs,
                               "-o", tmp, "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_reference(ref_tree: str | None = None) -> str | None:
    """Build oracle/_ref from the reference sources when the tree is present.  The tree is `ref_tree`, else the
    recipe's own choice (build_ref.sh: $PARHDE_REF_SRC, else its default location); None when there is no tree
    (the recipe exits 2), as on a machine that only has this repository."""
    r = subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")] + ([ref_tree] if ref_tree else []),
                       stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)
    if r.returncode == 2:
        return None
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stderr[-2000:])
    return REF_LIB_PATH


class Opts(C.Structure):
    _fields_ = [
        ("algo", C.c_int), ("strategy", C.c_int), ("k", C.c_int), ("c", C.c_int), ("eig", C.c_int),
        ("dist_algo", C.c_int), ("nthreads", C.c_int), ("verbose", C.c_int), ("seed", C.c_uint64),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("status", C.c_int), ("npasses", C.c_int), ("naccepted", C.c_int), ("ndiscarded", C.c_int),
        ("eig_iters", C.c_int), ("t_dist", C.c_double), ("t_orth", C.c_double), ("t_mmult", C.c_double),
        ("t_eig", C.c_double), ("t_coords", C.c_double), ("t_total", C.c_double),
    ]


_lib = None
_ref = None


def _p(a, ct):
    return None if a is None else a.ctypes.data_as(C.POINTER(ct))


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = C.CDLL(LIB_PATH)
        u32p, i32p, i64p, f64p = C.POINTER(C.c_uint32), C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_double)
        L.orc_bfs_serial.argtypes = [u32p, u32p, C.c_int64, C.c_int64, i32p]
        L.orc_dobfs.argtypes = [u32p, u32p, C.c_int64, C.c_int64, C.c_int64, i32p, C.c_int, C.c_int]
        L.orc_dijkstra.argtypes = [u32p, u32p, i32p, C.c_int64, C.c_int64, i32p]
        L.orc_deltastep.argtypes = [u32p, u32p, i32p, C.c_int64, C.c_int64, C.c_int64, i32p, C.c_int32]
        L.orc_layout.argtypes = [C.POINTER(Opts), u32p, u32p, i32p, C.c_int64, C.c_int64, f64p, i64p, f64p, f64p,
                                 f64p, f64p, C.POINTER(Stats)]
        L.orc_kcenters.argtypes = [u32p, u32p, i32p, C.c_int64, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, i32p,
                                   i64p]
        L.orc_glibc_rand.argtypes = [C.c_uint32, C.c_int, i32p]
        L.orc_check_csr.argtypes = [u32p, u32p, C.c_int64, C.c_int64]
        L.orc_draw_geometry.argtypes = [f64p, f64p, C.c_long, f64p, C.POINTER(C.c_uint)]
        L.orc_draw.argtypes = [u32p, u32p, C.c_long, C.c_long, f64p, f64p, C.POINTER(C.c_ubyte), C.c_uint, C.c_uint,
                               C.POINTER(C.c_float)]
        _lib = L
    return _lib


def _csr_args(g):
    off = np.ascontiguousarray(g.offsets, dtype=np.uint32)
    adj = np.ascontiguousarray(g.adj, dtype=np.uint32)
    w = None if g.weights is None else np.ascontiguousarray(g.weights, dtype=np.int32)
    return off, adj, w


def bfs(g, src: int, parallel: bool = False) -> np.ndarray:
    off, adj, _ = _csr_args(g)
    d = np.empty(g.n, dtype=np.int32)
    if parallel:
        lib().orc_dobfs(_p(off, C.c_uint32), _p(adj, C.c_uint32), g.n, g.nnz, src, _p(d, C.c_int32), 15, 18)
    else:
        lib().orc_bfs_serial(_p(off, C.c_uint32), _p(adj, C.c_uint32), g.n, src, _p(d, C.c_int32))
    return d


def sssp(g, src: int, parallel: bool = False, delta: int = 10000) -> np.ndarray:
    off, adj, w = _csr_args(g)
    d = np.empty(g.n, dtype=np.int32)
    if parallel:
        lib().orc_deltastep(_p(off, C.c_uint32), _p(adj, C.c_uint32), _p(w, C.c_int32), g.n, g.nnz, src,
                            _p(d, C.c_int32), delta)
    else:
        lib().orc_dijkstra(_p(off, C.c_uint32), _p(adj, C.c_uint32), _p(w, C.c_int32), g.n, src, _p(d, C.c_int32))
    return d


def glibc_rand(seed: int, count: int) -> np.ndarray:
    out = np.empty(count, dtype=np.int32)
    lib().orc_glibc_rand(seed, count, _p(out, C.c_int32))
    return out


@dataclass
class Layout:
    status: int
    coords: np.ndarray  # (n, c)
    sources: np.ndarray  # pass sources in order
    S: np.ndarray | None  # (n, k) basis (or centred matrix for PivotMDS/PHDE)
    M: np.ndarray | None  # (k, k) matrix handed to the eigensolver (row-major view of the column-major buffer)
    evecs: np.ndarray | None
    evals: np.ndarray | None
    stats: Stats


def layout(g, algo: str = "ParHDE", strategy: str = "Kcenters", k: int = 10, c: int = 2, eig: str = "power",
           dist_algo: str = "parallel", nthreads: int = 0, seed: int = 1, want_S: bool = True,
           verbose: bool = False) -> Layout:
    off, adj, w = _csr_args(g)
    if algo in ("wParHDE",) and w is None:
        raise ValueError("wParHDE needs weights")
    if algo != "wParHDE":
        w = None
    o = Opts(ALGOS[algo], STRATEGIES[strategy], k, c, 1 if eig == "exact" else 0,
             0 if dist_algo == "parallel" else 1, nthreads, 1 if verbose else 0, seed)
    n = g.n
    coords = np.zeros(n * c, dtype=np.float64)
    sources = np.full(3 * k, -1, dtype=np.int64)
    S = np.zeros(n * k, dtype=np.float64) if want_S else None
    M = np.zeros(k * k, dtype=np.float64)
    E = np.zeros(k * k, dtype=np.float64)
    ev = np.zeros(k, dtype=np.float64)
    st = Stats()
    rc = lib().orc_layout(C.byref(o), _p(off, C.c_uint32), _p(adj, C.c_uint32), _p(w, C.c_int32), n, g.nnz,
                          _p(coords, C.c_double), _p(sources, C.c_int64), _p(S, C.c_double), _p(M, C.c_double),
                          _p(E, C.c_double), _p(ev, C.c_double), C.byref(st))
    return Layout(rc, coords.reshape(c, n).T.copy(), sources[: st.npasses].copy(),
                  None if S is None else S.reshape(k, n).T.copy(), M.reshape(k, k).T.copy(),
                  E.reshape(k, k).T.copy(), ev, st)


def kcenters(g, P: int, variant: int = 0, parallel: bool = False, nthreads: int = 0):
    """P Kcenters distance passes: (D int32 (n,P), sources).  variant 0 ParHDE, 1 WParHDE, 2 DrawingBase."""
    off, adj, w = _csr_args(g)
    D = np.zeros(g.n * P, dtype=np.int32)
    src = np.zeros(P, dtype=np.int64)
    rc = lib().orc_kcenters(_p(off, C.c_uint32), _p(adj, C.c_uint32), _p(w, C.c_int32), g.n, g.nnz, P, variant,
                            0 if parallel else 1, nthreads, _p(D, C.c_int32), _p(src, C.c_int64))
    if rc != 0:
        raise RuntimeError(f"orc_kcenters failed: {rc}")
    return D.reshape(P, g.n).T.copy(), src


# ----------------------------------------------------------------------------- reference build

def ref_available() -> bool:
    if not os.path.exists(REF_LIB_PATH):
        return False
    try:
        ref()
        return True
    except OSError:  # built for another architecture
        return False


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_LIB_PATH)
        u32p, i32p, f64p, lp = C.POINTER(C.c_uint32), C.POINTER(C.c_int32), C.POINTER(C.c_double), C.POINTER(C.c_long)
        R.ref_dobfs.argtypes = [u32p, u32p, C.c_long, C.c_long, C.c_long, f64p, C.c_int]
        R.ref_deltastep.argtypes = [u32p, u32p, i32p, C.c_long, C.c_long, C.c_long, f64p, C.c_int, C.c_int]
        R.ref_layout.argtypes = [C.c_int, C.c_int, u32p, u32p, i32p, C.c_long, C.c_long, C.c_int, C.c_int, C.c_int,
                                 f64p, lp, C.c_int, C.POINTER(C.c_int)]
        R.ref_layout.restype = C.c_int
        _ref = R
    return _ref


def ref_bfs(g, src: int, nthreads: int = 1) -> np.ndarray:
    off, adj, _ = _csr_args(g)
    d = np.full(g.n, -1.0, dtype=np.float64)
    ref().ref_dobfs(_p(off, C.c_uint32), _p(adj, C.c_uint32), src, g.n, g.nnz, _p(d, C.c_double), nthreads)
    return d


def ref_sssp(g, src: int, nthreads: int = 1, delta: int = 10000) -> np.ndarray:
    off, adj, w = _csr_args(g)
    d = np.full(g.n, -1.0, dtype=np.float64)
    ref().ref_deltastep(_p(off, C.c_uint32), _p(adj, C.c_uint32), _p(w, C.c_int32), src, g.n, g.nnz,
                        _p(d, C.c_double), delta, nthreads)
    return d


def ref_layout(g, algo: str = "ParHDE", strategy: str = "Kcenters", k: int = 10, c: int = 2, nthreads: int = 1):
    """Run the reference pipeline in-process; returns (coords (n, c'), sources)."""
    off, adj, w = _csr_args(g)
    if algo != "wParHDE":
        w = None
    ncap = 3 * k + 8
    coords = np.zeros(g.n * max(c, 2), dtype=np.float64)
    srcs = np.zeros(ncap, dtype=np.int64)
    ns = C.c_int(0)
    nc = ref().ref_layout(ALGOS[algo], STRATEGIES[strategy], _p(off, C.c_uint32), _p(adj, C.c_uint32),
                          _p(w, C.c_int32), g.n, g.nnz, k, c, nthreads, _p(coords, C.c_double),
                          srcs.ctypes.data_as(C.POINTER(C.c_long)), ncap, C.byref(ns))
    if nc < 0:
        raise RuntimeError("ref_layout failed")
    return coords[: g.n * nc].reshape(nc, g.n).T.copy(), srcs[: ns.value].copy()


# ----------------------------------------------------------------------------- the draw tool (draw_oracle.c)

REF_DRAW_PATH = os.path.join(REF_DIR, "draw")


def draw_geometry(x, y):
    """Bounds and image size of draw_graph.c:201-249: (bounds (xmin, xmax, ymin, ymax, aspect),
    (width, height) as computed, (width, height) as corrected); None when the size is not a positive 32-bit number."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    b = np.zeros(5, dtype=np.float64)
    d = np.zeros(4, dtype=np.uint32)
    rc = lib().orc_draw_geometry(_p(x, C.c_double), _p(y, C.c_double), len(x), _p(b, C.c_double),
                                 d.ctypes.data_as(C.POINTER(C.c_uint)))
    if rc != 0:
        return None
    return tuple(b), (int(d[0]), int(d[1])), (int(d[2]), int(d[3]))


def draw(g, x, y):
    """The reference's edge image for graph g at vertex positions (x, y): (rgba (H, W, 4) uint8, max edge length)."""
    geo = draw_geometry(x, y)
    if geo is None:
        raise ValueError("image size is not a positive 32-bit number")
    W, H = geo[2]
    off, adj, _ = _csr_args(g)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    img = np.zeros((H, W, 4), dtype=np.uint8)
    ml = C.c_float(0)
    rc = lib().orc_draw(_p(off, C.c_uint32), _p(adj, C.c_uint32), g.n, g.nnz, _p(x, C.c_double), _p(y, C.c_double),
                        img.ctypes.data_as(C.POINTER(C.c_ubyte)), W, H, C.byref(ml))
    if rc != 0:
        raise RuntimeError("orc_draw failed")
    return img, float(ml.value)


def ref_draw_available() -> bool:
    return os.access(REF_DRAW_PATH, os.X_OK)


def ref_draw(csr_path: str, coords_path: str, png_path: str, ncoords: int, first: int, second: int) -> str:
    """Run the reference's draw binary (one OpenMP thread: its serial order) and return its standard output."""
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([REF_DRAW_PATH, csr_path, coords_path, png_path, str(ncoords), str(first), str(second)],
                       env=env, capture_output=True, text=True, check=True)
    return r.stdout + r.stderr


# ----------------------------------------------------------------------------- dense stages for given pivots

def hde_from_sources(g, sources, k: int, c: int):
    """ParHDE's dense stages (ParHDE.cpp:176-308, DrawingBase.cpp:196-244) in numpy FP64 for a given pivot
    sequence: the BFS column of every source (the C oracle's serial BFS), L2 normalisation, classical
    Gram-Schmidt in the D inner product against the constant column and the accepted columns with the
    reference's 1e-3 discard rule, LS = D S - A S, M = S^T LS, the c eigenvectors of the smallest eigenvalues
    (numpy eigh, the exact eigensolver) and the unit-norm coordinates.  For pivot strategies the C oracle does
    not restate (learned pivots): it checks the dense stages on the GPU's own pivot sequence.
    Returns (coords (n, c), S (n, k), M (k, k), naccepted, ndiscarded)."""
    import scipy.sparse as sp
    n = g.n
    off = g.offsets.astype(np.int64)
    deg = np.diff(off).astype(np.float64)
    A = sp.csr_matrix((np.ones(g.nnz), g.adj.astype(np.int64), off), shape=(n, n))
    u0 = np.full(n, 1.0 / np.sqrt(n))
    Q = []
    nd = 0
    for s in sources:
        if len(Q) >= k:
            break
        x = bfs(g, int(s)).astype(np.float64)
        x = x * (1.0 / np.sqrt(x @ x))
        coef = [(x @ (deg * q)) * (1.0 / (q @ (deg * q))) for q in Q]
        c0 = (x @ (deg * u0)) * (1.0 / (u0 @ (deg * u0)))
        r = x - sum((cq * q for cq, q in zip(coef, Q)), np.zeros(n)) - c0 * u0
        nrm = np.sqrt(r @ r)
        if nrm < 0.001:
            nd += 1
            continue
        Q.append(r * (1.0 / nrm))
    S = np.stack(Q, axis=1)
    LS = deg[:, None] * S - A @ S
    M = S.T @ LS
    w, V = np.linalg.eigh(0.5 * (M + M.T))
    X = S @ V[:, :c]
    X /= np.linalg.norm(X, axis=0)
    return X, S, M, len(Q), nd
