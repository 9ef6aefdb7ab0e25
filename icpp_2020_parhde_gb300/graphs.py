"""Seeded synthetic graphs in the reference's CSR layout.

The reference is run on SuiteSparse matrices converted by ``mtx2csr`` (symmetrised, self-loops and
duplicate edges removed, adjacency lists sorted, largest connected component kept and relabelled in
increasing vertex order: ``mtx2csr.cpp:117-269``).  These generators produce the same kind of CSR
directly, deterministically from a seed (numpy PCG64, identical on x86-64 and aarch64):

* ``mesh``        2-D triangulated grid: 4-neighbour edges plus one diagonal per cell chosen by a coin.
* ``rmat``        R-MAT (Chakrabarti et al.) with Graph500-style label permutation, LCC kept.
* ``grid3d``      3-D 6-neighbour grid, optional symmetric int32 weights uniform in [wmin, wmax].
* ``rgg``         random geometric graph in the unit square/cube, radius chosen for a target mean
                  degree, vertices numbered in spatial-cell order, LCC kept.
"""
from __future__ import annotations

import math

import numpy as np

from .csr_io import CSRGraph


def _csr_from_undirected(n: int, lo: np.ndarray, hi: np.ndarray, w: np.ndarray | None = None) -> CSRGraph:
    """Build a sorted symmetric CSR from unique undirected edges (lo < hi)."""
    src = np.concatenate([lo, hi]).astype(np.int64)
    dst = np.concatenate([hi, lo]).astype(np.int64)
    key = src * n + dst
    order = np.argsort(key, kind="stable")
    src = src[order]
    adj = dst[order].astype(np.uint32)
    ww = None
    if w is not None:
        ww = np.concatenate([w, w]).astype(np.int32)[order]
    counts = np.bincount(src, minlength=n)
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=off[1:])
    return CSRGraph(off.astype(np.uint32) if off[-1] < 2**32 else off, adj, ww)


def _unique_undirected(n: int, u: np.ndarray, v: np.ndarray, w: np.ndarray | None = None):
    u = u.astype(np.int64)
    v = v.astype(np.int64)
    keep = u != v
    u, v = u[keep], v[keep]
    if w is not None:
        w = w[keep]
    lo = np.minimum(u, v)
    hi = np.maximum(u, v)
    key = lo * n + hi
    key_u, first = np.unique(key, return_index=True)
    lo, hi = key_u // n, key_u % n
    return lo, hi, (w[first] if w is not None else None)


def largest_component(g: CSRGraph) -> CSRGraph:
    """Keep the largest connected component, relabelled in increasing vertex order (mtx2csr.cpp:169-269)."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import connected_components

    n = g.n
    a = sp.csr_matrix((np.ones(g.nnz, dtype=np.int8), g.adj.astype(np.int64), g.offsets.astype(np.int64)), shape=(n, n))
    ncomp, lab = connected_components(a, directed=False)
    if ncomp == 1:
        return g
    sizes = np.bincount(lab)
    big = int(np.argmax(sizes))  # lowest label among equal sizes; labels follow first-vertex order
    mask = lab == big
    new_id = np.cumsum(mask) - 1
    deg = np.diff(g.offsets.astype(np.int64))
    src = np.repeat(np.arange(n, dtype=np.int64), deg)
    keep = mask[src]
    adj = new_id[g.adj.astype(np.int64)[keep]].astype(np.uint32)
    counts = deg[mask]
    off = np.zeros(int(mask.sum()) + 1, dtype=np.int64)
    np.cumsum(counts, out=off[1:])
    w = g.weights[keep] if g.weights is not None else None
    return CSRGraph(off.astype(np.uint32) if off[-1] < 2**32 else off, adj, w, g.name)


def mesh(nx: int = 125, ny: int = 125, seed: int = 1) -> CSRGraph:
    """Triangulated 2-D grid: n = nx*ny, |E| = 2*nx*ny - nx - ny + (nx-1)*(ny-1)."""
    rng = np.random.default_rng(seed)
    vid = np.arange(nx * ny, dtype=np.int64).reshape(ny, nx)
    us, vs = [vid[:, :-1].ravel()], [vid[:, 1:].ravel()]  # horizontal
    us.append(vid[:-1, :].ravel())
    vs.append(vid[1:, :].ravel())  # vertical
    coin = rng.integers(0, 2, size=(ny - 1) * (nx - 1)).astype(bool)
    a = vid[:-1, :-1].ravel()
    b = vid[1:, 1:].ravel()
    c = vid[:-1, 1:].ravel()
    d = vid[1:, :-1].ravel()
    us.append(np.where(coin, a, c))
    vs.append(np.where(coin, b, d))
    lo, hi, _ = _unique_undirected(nx * ny, np.concatenate(us), np.concatenate(vs))
    g = _csr_from_undirected(nx * ny, lo, hi)
    g.name = f"mesh{nx}x{ny}_s{seed}"
    return g


def rmat(scale: int, edgefactor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19, seed: int = 1,
         lcc: bool = True) -> CSRGraph:
    """R-MAT graph with 2^scale labels and edgefactor*2^scale generated edges, symmetrised, deduplicated,
    self-loops dropped, labels randomly permuted, largest connected component kept."""
    rng = np.random.default_rng(seed)
    N = 1 << scale
    m = edgefactor * N
    u = np.zeros(m, dtype=np.int64)
    v = np.zeros(m, dtype=np.int64)
    ab, abc = a + b, a + b + c
    for level in range(scale):
        r = rng.random(m)
        ubit = r >= ab
        vbit = ((r >= a) & (r < ab)) | (r >= abc)
        u |= ubit.astype(np.int64) << level
        v |= vbit.astype(np.int64) << level
    perm = rng.permutation(N)
    u = perm[u]
    v = perm[v]
    lo, hi, _ = _unique_undirected(N, u, v)
    del u, v
    g = _csr_from_undirected(N, lo, hi)
    if lcc:
        g = largest_component(g)
    g.name = f"rmat{scale}_ef{edgefactor}_s{seed}"
    return g


def grid3d(L: int, seed: int = 1, weighted: bool = True, wmin: int = 1, wmax: int = 255) -> CSRGraph:
    """L^3 6-neighbour grid; vertex id = x + L*y + L*L*z; neighbours listed in increasing id order.
    Weights (if any) are symmetric and uniform in [wmin, wmax]."""
    rng = np.random.default_rng(seed)
    n = L * L * L
    vid = np.arange(n, dtype=np.int64)
    x = vid % L
    y = (vid // L) % L
    z = vid // (L * L)
    # one weight per undirected edge, indexed by the lower endpoint and the axis
    wx = rng.integers(wmin, wmax + 1, size=n, dtype=np.int32) if weighted else None
    wy = rng.integers(wmin, wmax + 1, size=n, dtype=np.int32) if weighted else None
    wz = rng.integers(wmin, wmax + 1, size=n, dtype=np.int32) if weighted else None
    dirs = [  # (mask, delta, weight array, lower-endpoint offset)
        (z > 0, -L * L, wz, -L * L),
        (y > 0, -L, wy, -L),
        (x > 0, -1, wx, -1),
        (x < L - 1, 1, wx, 0),
        (y < L - 1, L, wy, 0),
        (z < L - 1, L * L, wz, 0),
    ]
    deg = np.zeros(n, dtype=np.int64)
    for msk, _, _, _ in dirs:
        deg += msk
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(deg, out=off[1:])
    nnz = int(off[-1])
    adj = np.empty(nnz, dtype=np.uint32)
    w = np.empty(nnz, dtype=np.int32) if weighted else None
    pos = off[:-1].copy()
    for msk, delta, warr, lo_off in dirs:
        vv = vid[msk]
        p = pos[msk]
        adj[p] = (vv + delta).astype(np.uint32)
        if weighted:
            w[p] = warr[vv + lo_off]
        pos[msk] += 1
    g = CSRGraph(off.astype(np.uint32) if nnz < 2**32 else off, adj, w, f"grid3d_{L}_s{seed}")
    return g


def rgg(n: int, dim: int = 2, avg_degree: float = 8.0, seed: int = 1, lcc: bool = True) -> CSRGraph:
    """Random geometric graph: n uniform points in [0,1)^dim joined when closer than r, with
    r = sqrt(avg_degree/(pi n)) in 2-D and (3 avg_degree/(4 pi n))^(1/3) in 3-D.  Vertices are
    numbered in the row-major order of r-sized cells (a mesh-like numbering), then the LCC is kept."""
    from scipy.spatial import cKDTree

    rng = np.random.default_rng(seed)
    pts = rng.random((n, dim))
    if dim == 2:
        r = math.sqrt(avg_degree / (math.pi * n))
    elif dim == 3:
        r = (3.0 * avg_degree / (4.0 * math.pi * n)) ** (1.0 / 3.0)
    else:
        raise ValueError("dim must be 2 or 3")
    ncell = max(1, int(1.0 / r))
    cell = np.minimum((pts * ncell).astype(np.int64), ncell - 1)
    key = cell[:, 0]
    for d in range(1, dim):
        key = key * ncell + cell[:, d]
    order = np.lexsort((pts[:, 0], key))
    pts = pts[order]
    pairs = cKDTree(pts).query_pairs(r, output_type="ndarray")
    lo, hi, _ = _unique_undirected(n, pairs[:, 0], pairs[:, 1])
    g = _csr_from_undirected(n, lo, hi)
    if lcc:
        g = largest_component(g)
    g.name = f"rgg{dim}d_{n}_s{seed}"
    return g


def path_graph(n: int) -> CSRGraph:
    lo = np.arange(n - 1, dtype=np.int64)
    g = _csr_from_undirected(n, lo, lo + 1)
    g.name = f"path{n}"
    return g


def star_graph(n: int) -> CSRGraph:
    hi = np.arange(1, n, dtype=np.int64)
    g = _csr_from_undirected(n, np.zeros(n - 1, dtype=np.int64), hi)
    g.name = f"star{n}"
    return g


def complete_graph(n: int) -> CSRGraph:
    iu = np.triu_indices(n, 1)
    g = _csr_from_undirected(n, iu[0].astype(np.int64), iu[1].astype(np.int64))
    g.name = f"complete{n}"
    return g


def with_random_weights(g: CSRGraph, seed: int = 1, wmin: int = 1, wmax: int = 255) -> CSRGraph:
    """Attach symmetric int32 weights uniform in [wmin, wmax] to an unweighted CSR."""
    rng = np.random.default_rng(seed)
    n = g.n
    deg = np.diff(g.offsets.astype(np.int64))
    src = np.repeat(np.arange(n, dtype=np.int64), deg)
    dst = g.adj.astype(np.int64)
    lo = np.minimum(src, dst)
    hi = np.maximum(src, dst)
    key = lo * n + hi
    uk, inv = np.unique(key, return_inverse=True)
    wu = rng.integers(wmin, wmax + 1, size=uk.shape[0], dtype=np.int32)
    return CSRGraph(g.offsets, g.adj, wu[inv].astype(np.int32), g.name + f"_w{seed}")


def relabel(g: CSRGraph, perm: np.ndarray) -> CSRGraph:
    """The same graph with vertex v renamed perm[v] (rows and neighbour lists re-sorted).  Kcenters starts
    at vertex 0 and breaks ties by the lowest index, so a relabelled copy shows how a layout depends on that
    choice rather than on the graph."""
    n = g.n
    perm = np.asarray(perm, dtype=np.int64)
    deg = np.diff(g.offsets.astype(np.int64))
    src = perm[np.repeat(np.arange(n, dtype=np.int64), deg)]
    dst = perm[g.adj.astype(np.int64)]
    order = np.argsort(src * n + dst, kind="stable")
    counts = np.bincount(src, minlength=n)
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=off[1:])
    w = g.weights[order] if g.weights is not None else None
    return CSRGraph(off.astype(np.uint32) if off[-1] < 2**32 else off, dst[order].astype(np.uint32), w,
                    g.name + "_relabelled")


def rgg_batch(count: int = 512, nmin: int = 1000, nmax: int = 200_000, avg_degree: float = 8.0, seed: int = 1):
    """`count` random geometric 2-D graphs with vertex counts log-uniform in [nmin, nmax], connection radius
    for mean degree `avg_degree`, largest connected component kept (the batched-layout workload)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(nmin), math.log(nmax), size=count)).astype(np.int64)
    seeds = rng.integers(1, 1 << 31, size=count)
    return [rgg(int(n), dim=2, avg_degree=avg_degree, seed=int(s)) for n, s in zip(sizes, seeds)]
