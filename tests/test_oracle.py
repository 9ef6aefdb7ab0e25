"""The oracle (CPU restatement, oracle/parhde_oracle.c) against the golden fixtures recorded from the
reference itself, and against the live reference build when it is present (this container only)."""
import ctypes
import ctypes.util
import os

import numpy as np
import pytest

from conftest import GOLDEN_NAMES, draw_case_names, golden_runs, load_draw_case, load_golden
from oracle import oracle as orc


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_distances_match_reference_goldens(name):
    g, rec = load_golden(name)
    for i, s in enumerate(rec["bfs_src"]):
        want = rec["bfs_dist"][:, i]
        if g.weights is not None:
            assert np.array_equal(orc.sssp(g, int(s)), want)
            assert np.array_equal(orc.sssp(g, int(s), parallel=True), want)
        else:
            assert np.array_equal(orc.bfs(g, int(s)), want)
            assert np.array_equal(orc.bfs(g, int(s), parallel=True), want)


@pytest.mark.parametrize("case", golden_runs(), ids=lambda c: "%s-%s-k%d-c%d" % c)
def test_layout_matches_reference_goldens(case):
    name, algo, k, c = case
    g, rec = load_golden(name)
    ref_src = rec[f"{algo}_k{k}_c{c}_sources"]
    ref_xy = rec[f"{algo}_k{k}_c{c}_coords"]
    for dist_algo in ("serial", "parallel"):
        L = orc.layout(g, algo, "Kcenters", k, c, nthreads=1, dist_algo=dist_algo)
        if L.status == -5:
            # the reference's pivot-count check is off by one (ParHDE.cpp:192,281): it carries on with
            # k-1 vectors where the oracle reports too few pivots
            assert L.stats.naccepted == k - 1
            continue
        assert L.status == 0
        assert np.array_equal(L.sources, ref_src[: len(L.sources)])
        # one thread, same operation order: the restatement reproduces the reference to the last bit or two
        np.testing.assert_allclose(L.coords, ref_xy, rtol=0, atol=1e-12)


def _one_reduction_mgs(g, sources, k):
    """WParHDE's coupled D-orthogonalisation in the one-reduction form the GPU kernels use (mgs_dots_kernel,
    mgs_solve_kernel, mgs_apply_kernel): per distance column one sweep for r_q = <x0, D y_q> (and the Gram
    row of the newest accepted column), the recurrence c_q G_qq = r_q - sum_{p<q} c_p G_pq, one sweep for
    x = x0 - sum c_q y_q; discard below 1e-3 as WParHDE.cpp:194-204."""
    n = g.n
    off = g.offsets.astype(np.int64)
    d = np.array([float(g.weights[off[i]:off[i + 1]].astype(np.float64).sum()) for i in range(n)])
    Y = [np.full(n, 1.0 / np.sqrt(n))]
    G = np.zeros((k + 1, k + 1))
    gram_cols = 0
    for s in sources:
        if len(Y) > k:
            break
        col = orc.sssp(g, int(s)).astype(np.float64)
        x0 = col * (1.0 / np.sqrt(float(np.sum(col.astype(np.int64) ** 2))))
        j = len(Y)
        if gram_cols < j:
            yg = Y[j - 1] * d
            for p in range(j):
                G[p, j - 1] = Y[p] @ yg
            gram_cols = j
        r = np.array([Y[q] @ (x0 * d) for q in range(j)])
        c = np.zeros(j)
        for q in range(j):
            c[q] = (r[q] - c[:q] @ G[:q, q]) * (1.0 / G[q, q])
        x = x0 - sum(c[q] * Y[q] for q in range(j))
        nrm = np.sqrt(x @ x)
        if nrm >= 0.001:
            Y.append(x * (1.0 / nrm))
    return np.stack(Y[1:k + 1], axis=1)


def test_one_reduction_mgs_matches_reference_mgs():
    """The reorganised MGS equals the reference's sweep-per-column MGS (the oracle follows WParHDE.cpp's
    operation order) to rounding, on the golden weighted grid and on a larger one."""
    from icpp_2020_parhde_gb300 import graphs
    for g, k in ((load_golden("grid12w")[0], 10), (graphs.grid3d(16, seed=3), 16)):
        L = orc.layout(g, "wParHDE", "Kcenters", k, 2, nthreads=1, dist_algo="serial")
        assert L.status == 0
        S = _one_reduction_mgs(g, L.sources, k)
        np.testing.assert_allclose(S, L.S, rtol=0, atol=1e-10)


def test_kcenters_variants_agree_on_connected_graph():
    g, _ = load_golden("rmat13")
    d0, s0 = orc.kcenters(g, 30, 0)
    d1, s1 = orc.kcenters(g, 30, 0, parallel=True, nthreads=4)
    assert np.array_equal(s0, s1) and np.array_equal(d0, d1)


def test_glibc_rand_stream_matches_libc():
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    for seed in (1, 7, 12345):
        libc.srand(seed)
        want = np.array([libc.rand() for _ in range(1000)], dtype=np.int32)
        assert np.array_equal(orc.glibc_rand(seed, 1000), want)


def test_exact_eigensolve_matches_numpy():
    g, _ = load_golden("rmat13")
    L = orc.layout(g, "ParHDE", k=20, c=3, eig="exact", nthreads=2)
    assert L.status == 0
    M = 0.5 * (L.M + L.M.T)
    w, V = np.linalg.eigh(M)
    np.testing.assert_allclose(L.evals, w, rtol=0, atol=1e-12 * np.abs(w).max())
    # eigenvector columns agree up to sign
    for j in range(20):
        assert abs(abs(np.dot(L.evecs[:, j], V[:, j])) - 1) < 1e-8


def test_oracle_errors():
    g, _ = load_golden("mesh125")
    assert orc.layout(g, "ParHDE", k=300, c=2).status == -4  # k out of range
    assert orc.layout(g, "ParHDE", k=10, c=11).status == -4
    gw, _ = load_golden("grid12w")
    from icpp_2020_parhde_gb300.csr_io import CSRGraph
    unweighted = CSRGraph(gw.offsets, gw.adj, None)
    with pytest.raises(ValueError):
        orc.layout(unweighted, "wParHDE", k=5, c=2)
    # two disjoint triangles: disconnected
    off = np.array([0, 2, 4, 6, 8, 10, 12], dtype=np.uint32)
    adj = np.array([1, 2, 0, 2, 0, 1, 4, 5, 3, 5, 3, 4], dtype=np.uint32)
    assert orc.layout(CSRGraph(off, adj), "ParHDE", k=2, c=2).status == -3


@pytest.mark.skipif(not orc.ref_available(), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("algo,k,c", [("ParHDE", 10, 2), ("PivotMDS", 8, 2), ("PHDE", 8, 3)])
def test_oracle_matches_live_reference_rgg(algo, k, c):
    from icpp_2020_parhde_gb300 import graphs
    g = graphs.rgg(5000, dim=2, avg_degree=8, seed=11)
    L = orc.layout(g, algo, "Kcenters", k, c, nthreads=1)
    xy, src = orc.ref_layout(g, algo, "Kcenters", k, c, nthreads=1)
    assert L.status == 0
    assert np.array_equal(L.sources, src)
    np.testing.assert_allclose(L.coords, xy, rtol=0, atol=1e-12)


def test_mtx_oracle_matches_reference_converter():
    """The converter's oracle reproduces the reference mtx2csr's binary CSR byte for byte on every fixture
    (tests/golden/mtx, written by tests/golden/make_mtx_golden.py with the reference build)."""
    import glob
    from oracle import mtx_oracle
    paths = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "mtx", "*.mtx")))
    assert len(paths) >= 5
    for p in paths:
        with open(p[:-4] + ".csr", "rb") as f:
            assert mtx_oracle.mtx2csr_bytes(p) == f.read(), p


# ---------------------------------------------------------------------------------------------- draw
@pytest.mark.parametrize("name", draw_case_names())
def test_draw_oracle_matches_reference_png(name):
    """The draw restatement reproduces the reference draw tool's image (its PNG decoded) pixel for pixel."""
    import pngdecode
    g, x, y, meta, png = load_draw_case(name)
    img, _ = orc.draw(g, x, y)
    ref = pngdecode.read(png)
    assert img.shape == ref.shape
    assert np.array_equal(img, ref)


def test_draw_oracle_geometry_degenerate():
    # equal x: zero range, no image size
    assert orc.draw_geometry(np.full(10, 0.25), np.linspace(-3, 3, 10)) is None
    # equal y = 2: the bounds start at 1 and -1, so the y range is [1, 2] and the image exists
    (xmin, xmax, ymin, ymax, aspect), (w0, h0), (W, H) = orc.draw_geometry(np.linspace(0, 5, 10), np.full(10, 2.0))
    assert (xmin, xmax, ymin, ymax, aspect) == (0.0, 5.0, 1.0, 2.0, 5.0)
    assert (w0, h0, W, H) == (14, 70, 14, 70)


def test_farthest_point_order_restatement():
    """The pivot oracle's farthest-point order against a plain loop over the candidates (first in proposal order
    on ties), on a mesh whose many equal distances make ties common, and with no warm-start columns."""
    from icpp_2020_parhde_gb300 import graphs
    from oracle import pivot_oracle as po
    g = graphs.mesh(40, 30, seed=3)
    Dw, _ = orc.kcenters(g, po.WARM, 0)
    cand = np.arange(0, g.n, 7)[:200]
    dist = np.stack([orc.bfs(g, int(v)) for v in cand], axis=1)[cand]  # (M, M)
    for warm_cols in (Dw[cand], Dw[cand][:, :0]):
        mind = warm_cols.min(axis=1).astype(np.int64) if warm_cols.shape[1] else np.full(len(cand), 2**31 - 1)
        used, want = np.zeros(len(cand), bool), []
        for _ in range(30):
            best = -1
            for i in range(len(cand)):
                if not used[i] and (best < 0 or mind[i] > mind[best]):
                    best = i
            used[best] = True
            want.append(best)
            mind = np.minimum(mind, dist[:, best])
        assert po.farthest_point_order(warm_cols, dist, 30) == want
