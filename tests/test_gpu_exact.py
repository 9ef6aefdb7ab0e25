"""The exact-Gram FP64 path (PHDE_PREC_EXACT: every n-sized product of the D-orthogonalisation, the Laplacian
product and the coordinates taken from exact integer Gram matrices of the distance columns) against the
reference's own coordinates (golden fixtures) and the FP64 oracle.  The tolerances are the FP64 path's."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import golden_runs, load_golden, sign_align
from icpp_2020_parhde_gb300 import graphs
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

COORD_ATOL = 1e-8


def _degenerate(M, c, rel=1e-6):
    w = np.sort(np.abs(np.linalg.eigvalsh(0.5 * (M + M.T))))
    scale = max(np.abs(w).max(), 1e-300)
    return bool(np.any(np.abs(np.diff(w[: c + 1])) < rel * scale))


def laplacian(g):
    A = sp.csr_matrix((np.ones(g.nnz), g.adj.astype(np.int64), g.offsets.astype(np.int64)), shape=(g.n, g.n))
    return sp.diags(np.asarray(A.sum(axis=1)).ravel()) - A


@pytest.mark.parametrize("case", [c for c in golden_runs() if c[1] == "ParHDE"], ids=lambda c: "%s-%s-k%d-c%d" % c)
def test_exact_vs_reference_goldens(gpu_ctx, case):
    """Same pivots, same accept/discard decisions, the reference's power iteration: the reference's coordinates."""
    name, algo, k, c = case
    g, rec = load_golden(name)
    ref_xy = rec[f"{algo}_k{k}_c{c}_coords"]
    gpu_ctx.upload(g)
    L = orc.layout(g, algo, "Kcenters", k, c, nthreads=1, dist_algo="serial")
    if L.status != 0:
        return  # the off-by-one pivot count of the reference (covered by the FP64 path's test)
    r = gpu_ctx.layout(algo, "Kcenters", k, c, precision="exact", extra=True)
    assert np.array_equal(r.sources, rec[f"{algo}_k{k}_c{c}_sources"][: len(r.sources)])
    assert r.stats["naccepted"] == L.stats.naccepted and r.stats["ndiscarded"] == L.stats.ndiscarded
    np.testing.assert_allclose(r.basis, L.S, rtol=0, atol=1e-9)
    np.testing.assert_allclose(r.gram, L.M, rtol=0, atol=1e-9 * np.abs(L.M).max())
    if _degenerate(L.M, c):
        return
    assert r.stats["eig_iters"] == L.stats.eig_iters
    np.testing.assert_allclose(r.coords, ref_xy, rtol=0, atol=COORD_ATOL)


def hub_mesh():
    """A 300 x 300 mesh plus one vertex joined to every mesh vertex: the hub's row has degree 90,000, so its
    degree times distance needs more than 16 bits and it takes the one-row 32-bit path of the Gram kernel."""
    from icpp_2020_parhde_gb300.csr_io import CSRGraph
    g = graphs.mesh(300, 300, seed=12)
    n = g.n
    A = sp.csr_matrix((np.ones(g.nnz), g.adj.astype(np.int64), g.offsets.astype(np.int64)), shape=(n, n)).tocoo()
    hub = np.full(n, n, dtype=np.int64)
    rows = np.concatenate([A.row, np.arange(n), hub])
    cols = np.concatenate([A.col, hub, np.arange(n)])
    B = sp.csr_matrix((np.ones(len(rows)), (rows, cols)), shape=(n + 1, n + 1))
    B.sort_indices()
    return CSRGraph(B.indptr.astype(np.uint32), B.indices.astype(np.uint32), None)


# Basis tolerance: 1e-9 absolute, except on the hub mesh, where every distance is 0, 1 or 2 and the columns
# are nearly collinear: there the oracle's own FP64 basis is 3.8e-9 away from the same Gram-Schmidt run in
# extended precision (np.longdouble), so the two FP64 computations are compared at 1e-8.
@pytest.mark.parametrize("make,k,c,btol", [
    (lambda: graphs.rmat(16, seed=7), 64, 3, 1e-9),
    (lambda: graphs.rmat(16, seed=7), 50, 3, 1e-9),
    (lambda: graphs.rgg(60000, dim=3, avg_degree=12, seed=2), 64, 3, 1e-9),
    (lambda: graphs.mesh(150, 80, seed=31), 130, 3, 1e-9),
    (lambda: graphs.mesh(900, 12, seed=5), 24, 2, 1e-9),   # diameter above 255: 16-bit packed columns
    (lambda: graphs.rmat(14, seed=3), 20, 7, 1e-9),        # more than four coordinates
    (hub_mesh, 20, 2, 1e-8),                               # a row too heavy for the byte dot products
], ids=["rmat16-k64", "rmat16-k50", "rgg3d-k64", "mesh-k130", "long-mesh-u16", "rmat14-c7", "hub-mesh"])
def test_exact_vs_fp64_oracle(gpu_ctx, make, k, c, btol):
    g = make()
    gpu_ctx.upload(g)
    r = gpu_ctx.layout("ParHDE", "Kcenters", k, c, precision="exact", eig="exact", extra=True)
    L = orc.layout(g, "ParHDE", "Kcenters", k, c, eig="exact", nthreads=8)
    assert L.status == 0
    assert np.array_equal(r.sources, L.sources)
    assert r.stats["naccepted"] == L.stats.naccepted and r.stats["ndiscarded"] == L.stats.ndiscarded
    np.testing.assert_allclose(r.basis, L.S, rtol=0, atol=btol)
    # S^T L S from the GPU's own basis: the exact integer products leave only the k x k rounding
    Mb = r.basis.T @ (laplacian(g) @ r.basis)
    np.testing.assert_allclose(r.gram, Mb, rtol=0, atol=1e-10 * np.abs(Mb).max())
    # against the oracle's vector Gram-Schmidt: both round in FP64 in different orders, amplified by the
    # conditioning of the nearly collinear late columns (the FP64 vector path's tests state 1e-6 at k >= 64)
    tol = 1e-7 if k <= 64 else 1e-6
    np.testing.assert_allclose(r.gram, L.M, rtol=0, atol=tol * np.abs(L.M).max())
    w, V = np.linalg.eigh(0.5 * (r.gram + r.gram.T))
    # the Jacobi eigensolver's own accuracy at k = 64 (FP32 sweeps refined in FP64)
    np.testing.assert_allclose(r.evals, w, rtol=0, atol=1e-9 * np.abs(w).max())
    X = r.basis @ V[:, :c]
    X /= np.linalg.norm(X, axis=0)
    np.testing.assert_allclose(sign_align(r.coords, X), X, rtol=0, atol=1e-9)
    if not _degenerate(L.M, c, rel=1e-5):
        np.testing.assert_allclose(sign_align(r.coords, L.coords), L.coords, rtol=0, atol=1e-7)


def test_exact_learned_pivots_vs_numpy_restatement(gpu_ctx):
    """Learned pivots (no C oracle strategy): the dense stages on the GPU's own pivot sequence against the
    numpy restatement of the reference's normalisation, CGS, Laplacian product, Gram and exact eigensolve."""
    g = graphs.rmat(15, seed=11)
    k, c = 64, 3
    gpu_ctx.upload(g)
    r = gpu_ctx.layout("ParHDE", "Learned", k, c, precision="exact", eig="exact", extra=True)
    X, S, M, na, nd = orc.hde_from_sources(g, r.sources, k, c)
    assert r.stats["naccepted"] == na == k and r.stats["ndiscarded"] == nd
    np.testing.assert_allclose(r.basis, S, rtol=0, atol=1e-9)
    np.testing.assert_allclose(r.gram, M, rtol=0, atol=1e-9 * np.abs(M).max())
    np.testing.assert_allclose(sign_align(r.coords, X), X, rtol=0, atol=1e-7)


def test_exact_discards_like_the_oracle(gpu_ctx):
    """A path graph: the far end's column is a combination of the constant and the near end's columns, so the
    reference discards it; the coefficient-space loop must take the same decision."""
    g = graphs.path_graph(3000)
    k, c = 10, 2
    gpu_ctx.upload(g)
    r = gpu_ctx.layout("ParHDE", "Kcenters", k, c, precision="exact", eig="exact", extra=True)
    L = orc.layout(g, "ParHDE", "Kcenters", k, c, eig="exact", nthreads=4)
    assert L.stats.ndiscarded > 0
    assert r.stats["ndiscarded"] == L.stats.ndiscarded and r.stats["naccepted"] == L.stats.naccepted == k
    np.testing.assert_allclose(r.basis, L.S, rtol=0, atol=1e-9)


def test_exact_out_of_range_takes_fp64_kernels(gpu_ctx):
    """Distances above 65535 (a 70000-vertex path) are outside the exact path's packed range: the layout comes
    from the FP64 vector kernels and still matches the oracle."""
    g = graphs.path_graph(70000)
    gpu_ctx.upload(g)
    r = gpu_ctx.layout("ParHDE", "Kcenters", 6, 2, precision="exact", eig="exact", extra=True)
    L = orc.layout(g, "ParHDE", "Kcenters", 6, 2, eig="exact", nthreads=8)
    assert np.array_equal(r.sources, L.sources)
    np.testing.assert_allclose(r.basis, L.S, rtol=0, atol=1e-9)


def test_exact_rejected_for_other_algorithms(gpu_ctx):
    from icpp_2020_parhde_gb300 import ParHDEError
    g = graphs.mesh(30, 30, seed=1)
    gpu_ctx.upload(g)
    with pytest.raises(ParHDEError) as e:
        gpu_ctx.layout("PivotMDS", "Kcenters", 5, 2, precision="exact")
    assert e.value.status == -1
