"""GPU layout pipeline against the reference's own coordinates (golden fixtures, one-thread reference)
and against the oracle's intermediate matrices.  FP64 path: the tolerance is stated per check."""
import numpy as np
import pytest

from conftest import golden_runs, load_golden, sign_align
from icpp_2020_parhde_gb300 import ParHDE, ParHDEError, PivotMDS, WParHDE, graphs
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

# FP64 end to end; the GPU sums in a different order than the one-thread reference, so results agree
# to rounding amplified by the conditioning of the D-orthogonalisation.
COORD_ATOL = 1e-8


@pytest.mark.parametrize("case", golden_runs(), ids=lambda c: "%s-%s-k%d-c%d" % c)
def test_layout_vs_reference_goldens(gpu_ctx, case):
    name, algo, k, c = case
    g, rec = load_golden(name)
    ref_src = rec[f"{algo}_k{k}_c{c}_sources"]
    ref_xy = rec[f"{algo}_k{k}_c{c}_coords"]
    gpu_ctx.upload(g)
    L = orc.layout(g, algo, "Kcenters", k, c, nthreads=1, dist_algo="serial")
    if L.status != 0:
        with pytest.raises(ParHDEError) as e:
            gpu_ctx.layout(algo, "Kcenters", k, c)
        assert e.value.status == L.status
        return
    r = gpu_ctx.layout(algo, "Kcenters", k, c, extra=True)
    if algo in ("PivotMDS", "PHDE"):
        assert np.array_equal(r.gram, L.M)  # bit-identical C^T C
    assert np.array_equal(r.sources, ref_src[: len(r.sources)])
    assert r.stats["naccepted"] == L.stats.naccepted and r.stats["ndiscarded"] == L.stats.ndiscarded
    # intermediate matrices against the oracle
    np.testing.assert_allclose(r.basis, L.S, rtol=0, atol=1e-9)
    np.testing.assert_allclose(r.gram, L.M, rtol=0, atol=1e-9 * np.abs(L.M).max())
    if _degenerate(L.M, c, largest=algo in ("PivotMDS", "PHDE")):
        # repeated eigenvalues around the picked ones: the power iteration's stopping sweep and the vectors
        # inside the repeated eigenspace depend on rounding, so only the matrices above are comparable
        return
    assert r.stats["eig_iters"] == L.stats.eig_iters
    if algo in ("PivotMDS", "PHDE"):
        # exact centring sums + reference summation order in C^T C, the power iteration and the coordinates
        assert np.array_equal(r.coords, ref_xy), np.abs(r.coords - ref_xy).max()
    else:
        np.testing.assert_allclose(r.coords, ref_xy, rtol=0, atol=COORD_ATOL)


def _degenerate(M, c, largest, rel=1e-6):
    w = np.sort(np.abs(np.linalg.eigvalsh(0.5 * (M + M.T))))
    if largest:
        w = w[::-1]
    scale = max(np.abs(w).max(), 1e-300)
    return bool(np.any(np.abs(np.diff(w[: c + 1])) < rel * scale))


@pytest.mark.parametrize("algo,k,c", [("ParHDE", 10, 2), ("ParHDE", 30, 3), ("PivotMDS", 12, 3), ("PHDE", 12, 2)])
def test_exact_eigensolver_vs_numpy(gpu_ctx, algo, k, c):
    g = graphs.rgg(20000, dim=2, avg_degree=8, seed=21)
    gpu_ctx.upload(g)
    r = gpu_ctx.layout(algo, "Kcenters", k, c, eig="exact", extra=True)
    M = 0.5 * (r.gram + r.gram.T)
    w, V = np.linalg.eigh(M)
    np.testing.assert_allclose(r.evals, w, rtol=0, atol=1e-11 * np.abs(w).max())
    cols = range(c) if algo in ("ParHDE",) else range(k - 1, k - 1 - c, -1)
    Y = V[:, list(cols)]
    X = r.basis @ Y
    X /= np.linalg.norm(X, axis=0)
    np.testing.assert_allclose(sign_align(r.coords, X), X, rtol=0, atol=1e-8)
    L = orc.layout(g, algo, "Kcenters", k, c, eig="exact", nthreads=4)
    np.testing.assert_allclose(sign_align(r.coords, L.coords), L.coords, rtol=0, atol=1e-7)


@pytest.mark.parametrize("algo,k,make", [
    ("ParHDE", 64, lambda: graphs.mesh(150, 80, seed=31)),
    ("ParHDE", 130, lambda: graphs.mesh(150, 80, seed=32)),
    ("wParHDE", 40, lambda: graphs.grid3d(20, seed=33)),
], ids=["parhde-k64", "parhde-k130", "wparhde-k40"])
def test_fp64_large_k_vs_oracle(gpu_ctx, algo, k, make):
    """Large k takes the other FP64 kernel shapes: the Gram with 4 or more outputs per thread or on upper
    tiles, coordinate row tiles of 64 rows, MGS dot sweeps over several column tiles."""
    sp = pytest.importorskip("scipy.sparse")
    g = make()
    gpu_ctx.upload(g)
    r = gpu_ctx.layout(algo, "Kcenters", k, 3, eig="exact", extra=True)
    L = orc.layout(g, algo, "Kcenters", k, 3, eig="exact", nthreads=4)
    assert np.array_equal(r.sources, L.sources)
    np.testing.assert_allclose(r.basis, L.S, rtol=0, atol=1e-9)
    # SpMM + Gram against S^T L S formed in numpy from the GPU's own basis (tight: the kernels alone) ...
    w = np.ones(g.nnz) if g.weights is None else g.weights.astype(np.float64)
    A = sp.csr_matrix((w, g.adj.astype(np.int64), g.offsets.astype(np.int64)), shape=(g.n, g.n))
    Lap = sp.diags(np.asarray(A.sum(axis=1)).ravel()) - A
    Mb = r.basis.T @ (Lap @ r.basis)
    np.testing.assert_allclose(r.gram, Mb, rtol=0, atol=1e-11 * np.abs(Mb).max())
    # ... and against the oracle's, where the late basis columns' conditioning (up to k = 130 nearly
    # collinear distance columns) amplifies the orthogonalisation's rounding differences
    np.testing.assert_allclose(r.gram, L.M, rtol=0, atol=1e-6 * np.abs(L.M).max())
    # the coordinates against the GPU's own basis and Gram (a rectangular mesh: the first four eigenvalues
    # are apart by 2.7e-5 relative or more, so the eigenvectors are well defined)
    w, V = np.linalg.eigh(0.5 * (r.gram + r.gram.T))
    X = r.basis @ V[:, :3]
    X /= np.linalg.norm(X, axis=0)
    np.testing.assert_allclose(sign_align(r.coords, X), X, rtol=0, atol=1e-8)


def test_wparhde_on_larger_grid_vs_oracle(gpu_ctx):
    g = graphs.grid3d(24, seed=8)
    gpu_ctx.upload(g)
    r = gpu_ctx.layout("wParHDE", "Kcenters", 12, 3, extra=True)
    L = orc.layout(g, "wParHDE", "Kcenters", 12, 3, nthreads=4)
    assert np.array_equal(r.sources, L.sources)
    np.testing.assert_allclose(r.coords, L.coords, rtol=0, atol=1e-7)


@pytest.mark.parametrize("strategy", ["RandFine", "RandCoarse"])
def test_random_strategies_vs_oracle(gpu_ctx, strategy):
    g, _ = load_golden("rmat13")
    gpu_ctx.upload(g)
    for algo in ("ParHDE", "PivotMDS"):
        r = gpu_ctx.layout(algo, strategy, 10, 2, seed=5)
        L = orc.layout(g, algo, strategy, 10, 2, seed=5, nthreads=1)
        assert np.array_equal(r.sources, L.sources)
        if algo == "PivotMDS":
            assert np.array_equal(r.coords, L.coords)
        else:
            np.testing.assert_allclose(r.coords, L.coords, rtol=0, atol=1e-8)


def test_layout_errors(gpu_ctx):
    g, _ = load_golden("mesh125")
    gpu_ctx.upload(g)
    for kw, status in [(dict(k=0, c=1), -4), (dict(k=300, c=2), -4), (dict(k=5, c=6), -4)]:
        with pytest.raises(ParHDEError) as e:
            gpu_ctx.layout("ParHDE", **kw)
        assert e.value.status == status
    with pytest.raises(ParHDEError) as e:
        gpu_ctx.layout("wParHDE", k=5, c=2)
    assert e.value.status == -10
    gw, _ = load_golden("grid12w")
    gpu_ctx.upload(gw)
    with pytest.raises(ParHDEError) as e:
        gpu_ctx.layout("ParHDE", k=5, c=2)
    assert e.value.status == -10


def test_reference_class_interface(gpu_ctx):
    g, rec = load_golden("mesh125")
    d = ParHDE(g.offsets, g.adj, None, g.n, g.nnz, 10, 2, 2, verbose=False)
    assert d.run(1) == 0
    xy = d.getCoordinates()
    assert xy.shape == (g.n * 2,)
    np.testing.assert_allclose(xy.reshape(2, g.n).T, rec["ParHDE_k10_c2_coords"], rtol=0, atol=COORD_ATOL)
    p = PivotMDS(g.offsets, g.adj, None, g.n, g.nnz, 10, 2, 2, verbose=False)
    p.run(1)
    np.testing.assert_allclose(p.getCoordinates().reshape(2, g.n).T, rec["PivotMDS_k10_c2_coords"], rtol=0,
                               atol=COORD_ATOL)
    gw, recw = load_golden("grid12w")
    w = WParHDE(gw.offsets, gw.adj, gw.weights, gw.n, gw.nnz, 10, 2, verbose=False)
    w.run(1)
    np.testing.assert_allclose(w.getCoordinates().reshape(2, gw.n).T, recw["wParHDE_k10_c2_coords"], rtol=0,
                               atol=COORD_ATOL)
    with pytest.raises(ParHDEError):
        ParHDE(gw.offsets, gw.adj, gw.weights, gw.n, gw.nnz, 10, 2, 2)


def test_cluster_power_iteration_matches_single_cta_bitwise(gpu_ctx, monkeypatch):
    """The 8-CTA cluster power iteration performs the single-CTA kernel's operations in the same order."""
    g = graphs.rmat(14, seed=8)
    gpu_ctx.upload(g)
    for k in (10, 50):
        a = gpu_ctx.layout("ParHDE", "Kcenters", k, 3, extra=True)
        monkeypatch.setenv("PHDE_POWER_SINGLE_CTA", "1")
        b = gpu_ctx.layout("ParHDE", "Kcenters", k, 3, extra=True)
        monkeypatch.delenv("PHDE_POWER_SINGLE_CTA")
        assert a.stats["eig_iters"] == b.stats["eig_iters"]
        assert np.array_equal(a.evecs, b.evecs) and np.array_equal(a.evals, b.evals)
        assert np.array_equal(a.coords, b.coords)


def test_wparhde_above_2_20_vertices_vs_oracle(gpu_ctx):
    """A weighted 104^3 grid (1,124,864 vertices): graphs of 2^20 vertices or more take the SSSP's narrow band
    (eight times the mean weight) and two CTAs per SM.  Distances, pivots and the layout against the oracle."""
    g = graphs.grid3d(104, seed=9)
    assert g.n >= 1 << 20
    gpu_ctx.upload(g)
    r = gpu_ctx.layout("wParHDE", "Kcenters", 20, 2, extra=True)
    L = orc.layout(g, "wParHDE", "Kcenters", 20, 2, nthreads=16)
    assert L.status == 0
    assert np.array_equal(r.sources, L.sources)
    assert r.stats["naccepted"] == L.stats.naccepted and r.stats["ndiscarded"] == L.stats.ndiscarded
    d = gpu_ctx.distances(r.sources[:3])
    for i in range(3):
        assert np.array_equal(d[:, i], orc.sssp(g, int(r.sources[i]), parallel=True))
    np.testing.assert_allclose(r.gram, L.M, rtol=0, atol=1e-7 * np.abs(L.M).max())
    if not _degenerate(L.M, 2, largest=False, rel=1e-5):
        np.testing.assert_allclose(r.coords, L.coords, rtol=0, atol=1e-6)
