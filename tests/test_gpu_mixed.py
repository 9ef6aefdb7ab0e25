"""Mixed precision (PHDE_PREC_MIXED: FP32 basis, CGS2, FP32 SpMM, FP32-product/FP64-sum Gram; FP64 k x k
solve) against the FP64 oracle.  Stated error bounds are the assertions below."""
import numpy as np
import pytest
import scipy.sparse as sp

from icpp_2020_parhde_gb300 import ParHDEError, graphs
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def rayleigh(g, X):
    n = g.n
    A = sp.csr_matrix((np.ones(g.nnz), g.adj.astype(np.int64), g.offsets.astype(np.int64)), shape=(n, n))
    d = np.asarray(A.sum(axis=1)).ravel()
    LX = d[:, None] * X - A @ X
    return np.einsum("ij,ij->j", X, LX) / np.einsum("ij,ij->j", X, X)


def principal_cosines(X, Y):
    qx, _ = np.linalg.qr(X)
    qy, _ = np.linalg.qr(Y)
    return np.linalg.svd(qx.T @ qy, compute_uv=False)


@pytest.mark.parametrize("make,k,c", [
    (lambda: graphs.rmat(15, seed=4), 20, 3),
    (lambda: graphs.rgg(40000, dim=2, avg_degree=8, seed=5), 10, 2),
    (lambda: graphs.mesh(200, 150, seed=6), 16, 2),
], ids=["rmat15", "rgg40k", "mesh200x150"])
def test_mixed_vs_fp64_oracle(gpu_ctx, make, k, c):
    g = make()
    gpu_ctx.upload(g)
    r = gpu_ctx.layout("ParHDE", "Kcenters", k, c, precision="mixed", eig="exact", extra=True)
    L = orc.layout(g, "ParHDE", "Kcenters", k, c, eig="exact", nthreads=4)
    assert np.array_equal(r.sources, L.sources)  # distances and pivots are exact in every precision
    assert r.stats["naccepted"] == L.stats.naccepted == k
    # the k x k matrix S^T L S: FP32 basis and products, FP64 sums -> ~1e-5 relative
    w_m = np.linalg.eigvalsh(0.5 * (r.gram + r.gram.T))
    w_o = np.linalg.eigvalsh(0.5 * (L.M + L.M.T))
    np.testing.assert_allclose(w_m, w_o, rtol=2e-4, atol=2e-4 * np.abs(w_o).max())
    # layout: Rayleigh quotients within 0.1 %, coordinate subspace within 1e-3 (principal cosines)
    rq_m, rq_o = rayleigh(g, r.coords), rayleigh(g, L.coords)
    np.testing.assert_allclose(rq_m, rq_o, rtol=1e-3)
    assert principal_cosines(r.coords, L.coords).min() > 1 - 1e-3


def test_mixed_rejected_for_other_algorithms(gpu_ctx):
    g = graphs.mesh(30, 30, seed=1)
    gpu_ctx.upload(g)
    with pytest.raises(ParHDEError) as e:
        gpu_ctx.layout("PivotMDS", "Kcenters", 5, 2, precision="mixed")
    assert e.value.status == -1


def test_blocked_cgs2_matches_column_cgs2(monkeypatch):
    """The blocked CGS2 (32 candidates per block, coefficient-space accept/discard loop) against the
    column-at-a-time CGS2: same accept/discard decisions, same layout to FP32 accuracy."""
    from icpp_2020_parhde_gb300 import Context
    g = graphs.rmat(15, seed=4)
    k, c = 40, 3
    cb = Context(0)
    cb.upload(g)
    rb = cb.layout("ParHDE", "Kcenters", k, c, precision="mixed", eig="exact")
    monkeypatch.setenv("PHDE_CGS2", "column")
    cc = Context(0)
    cc.upload(g)
    rc = cc.layout("ParHDE", "Kcenters", k, c, precision="mixed", eig="exact")
    for key in ("naccepted", "ndiscarded"):
        assert rb.stats[key] == rc.stats[key]
    np.testing.assert_allclose(rayleigh(g, rb.coords), rayleigh(g, rc.coords), rtol=1e-4)
    assert principal_cosines(rb.coords, rc.coords).min() > 1 - 1e-5


def test_blocked_cgs2_discards_like_the_oracle(gpu_ctx):
    """A path graph: the column of the far end is the near end's reversed (a combination of the constant and
    the first column), so the reference discards it; the blocked loop must take the same decisions."""
    g = graphs.path_graph(3000)
    k, c = 10, 2
    gpu_ctx.upload(g)
    r = gpu_ctx.layout("ParHDE", "Kcenters", k, c, precision="mixed", eig="exact")
    L = orc.layout(g, "ParHDE", "Kcenters", k, c, eig="exact", nthreads=4)
    assert L.stats.ndiscarded > 0
    assert r.stats["ndiscarded"] == L.stats.ndiscarded
    assert r.stats["naccepted"] == L.stats.naccepted == k
    np.testing.assert_allclose(rayleigh(g, r.coords), rayleigh(g, L.coords), rtol=1e-3)


@pytest.mark.parametrize("make,k,c", [
    (lambda: graphs.rmat(16, seed=4), 50, 3),
    (lambda: graphs.rmat(17, seed=5), 64, 3),
    (lambda: graphs.rgg(80000, dim=3, avg_degree=12, seed=6), 50, 3),
    (lambda: graphs.rgg(80000, dim=3, avg_degree=12, seed=7), 64, 3),
], ids=["rmat16-k50", "rmat17-k64", "rgg3d-k50", "rgg3d-k64"])
def test_mixed_vs_fp64_oracle_at_benchmark_k(gpu_ctx, make, k, c):
    """The k the benchmark runs (50 and 64): the blocked CGS2 in FP32 on up to 64 nearly collinear distance
    columns.  Stated error against the FP64 oracle (same pivots, exact eigensolver): the accept/discard count, the
    eigenvalues of S^T L S within 1e-3 relative, every coordinate's Rayleigh quotient within 0.1 %, and the
    coordinate subspace within 1e-3 (principal cosines)."""
    g = make()
    gpu_ctx.upload(g)
    r = gpu_ctx.layout("ParHDE", "Kcenters", k, c, precision="mixed", eig="exact", extra=True)
    L = orc.layout(g, "ParHDE", "Kcenters", k, c, eig="exact", nthreads=8)
    assert L.status == 0
    assert np.array_equal(r.sources, L.sources)
    assert r.stats["naccepted"] == L.stats.naccepted == k and r.stats["ndiscarded"] == L.stats.ndiscarded
    w_m = np.linalg.eigvalsh(0.5 * (r.gram + r.gram.T))
    w_o = np.linalg.eigvalsh(0.5 * (L.M + L.M.T))
    np.testing.assert_allclose(w_m, w_o, rtol=1e-3, atol=1e-3 * np.abs(w_o).max())
    np.testing.assert_allclose(rayleigh(g, r.coords), rayleigh(g, L.coords), rtol=1e-3)
    assert principal_cosines(r.coords, L.coords).min() > 1 - 1e-3
