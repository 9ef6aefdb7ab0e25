"""Batched layouts (phde_batch_upload + phde_layout_batched): many graphs in one call, against the same
graphs laid out one at a time with the same options (Kcenters pivots, mixed precision, Jacobi)."""
import numpy as np
import pytest
import scipy.sparse as sp

from icpp_2020_parhde_gb300 import Context, ParHDEError, graphs
from icpp_2020_parhde_gb300.csr_io import CSRGraph
from conftest import sign_align

pytestmark = pytest.mark.gpu


def rayleigh(g, X):
    A = sp.csr_matrix((np.ones(g.nnz), g.adj.astype(np.int64), g.offsets.astype(np.int64)), shape=(g.n, g.n))
    d = np.asarray(A.sum(axis=1)).ravel()
    return np.einsum("ij,ij->j", X, d[:, None] * X - A @ X) / np.einsum("ij,ij->j", X, X)


def principal_cosines(X, Y):
    qx, _ = np.linalg.qr(X)
    qy, _ = np.linalg.qr(Y)
    return np.linalg.svd(qx.T @ qy, compute_uv=False)


def batch_graphs():
    return [graphs.rgg(3000, dim=2, avg_degree=8, seed=1), graphs.rgg(12000, dim=2, avg_degree=8, seed=2),
            graphs.mesh(60, 50, seed=3), graphs.rgg(1500, dim=2, avg_degree=8, seed=4), graphs.rmat(12, seed=5),
            graphs.rgg(25000, dim=2, avg_degree=8, seed=6), graphs.rgg(8000, dim=3, avg_degree=12, seed=7)]


@pytest.mark.parametrize("k,c", [(10, 2), (20, 3)])
def test_batched_matches_single_layouts(k, c):
    gs = batch_graphs()
    cb = Context(0)
    cb.upload_batch(gs)
    xs, st = cb.layout_batched(k, c)
    assert st["naccepted"] == k and st["npasses"] == 3 * k
    cs = Context(0)
    for g, xb in zip(gs, xs):
        cs.upload(g)
        r = cs.layout("ParHDE", "Kcenters", k, c, precision="mixed", eig="exact")
        np.testing.assert_allclose(np.linalg.norm(xb, axis=0), 1.0, rtol=1e-9)
        np.testing.assert_allclose(rayleigh(g, xb), rayleigh(g, r.coords), rtol=1e-4)
        assert principal_cosines(xb, r.coords).min() > 1 - 1e-5


def test_batched_replay_is_deterministic():
    gs = batch_graphs()[:4]
    cb = Context(0)
    cb.upload_batch(gs)
    x1, s1 = cb.layout_batched(10, 2)
    x2, s2 = cb.layout_batched(10, 2)
    x3, s3 = cb.layout_batched(10, 2)
    assert s1["batch_seg_rows"] == s2["batch_seg_rows"] > 0
    assert s1["ms_batch_tune"] > 0 and s2["ms_batch_tune"] == 0  # tuned once per batch
    for a, b, c in zip(x1, x2, x3):
        assert np.array_equal(a, b) and np.array_equal(b, c)
    # distances stay exact for the batch: a batched upload is an ordinary (disconnected) graph
    d = cb.distances([0, gs[0].n])
    assert (d[: gs[0].n, 0] >= 0).all() and (d[gs[0].n:, 0] == -1).all()


def test_batched_rejects_bad_input():
    good = graphs.rgg(2000, dim=2, avg_degree=8, seed=8)
    cb = Context(0)
    adj = good.adj.copy()
    adj[5] = good.n  # a neighbour outside its own graph
    bad = CSRGraph(good.offsets, adj, None)
    with pytest.raises(ParHDEError) as e:
        cb.upload_batch([good, bad])
    assert e.value.status == -2  # PHDE_ERR_CSR
    tiny = graphs.path_graph(20)
    cb.upload_batch([good, tiny])
    with pytest.raises(ParHDEError) as e:
        cb.layout_batched(10, 2)  # 20 vertices <= 3k pivots
    with pytest.raises(ParHDEError):
        cb.layout_batched(40, 2)  # k above 32 (per-graph pipeline): 20 vertices <= 3k pivots as well


def test_block_per_graph_kcenters_matches_union(monkeypatch):
    """The one-CTA-per-graph Kcenters (large batches) and the whole-grid batched Kcenters give the same
    distance columns and pivots, so the same layouts bit for bit."""
    gs = batch_graphs()
    out = {}
    for mode in ("union", "blocks"):
        monkeypatch.setenv("PHDE_BATCH_BFS", mode)
        cb = Context(0)
        cb.upload_batch(gs)
        xs, st = cb.layout_batched(10, 2)
        out[mode] = [x.copy() for x in xs]
        cb.close()
    for a, b in zip(out["union"], out["blocks"]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("k,c", [(10, 2), (20, 3)])
def test_batched_vs_fp64_oracle(k, c):
    """Every graph of a batch against the FP64 oracle (the reference algorithm with the exact eigensolver) laid
    out on its own: the same pivots, Rayleigh quotients within the mixed path's 0.1 %, and the coordinate
    subspace within 1e-3 (principal cosines)."""
    from oracle import oracle as orc
    gs = batch_graphs()
    cb = Context(0)
    cb.upload_batch(gs)
    xs, st = cb.layout_batched(k, c)
    cs = Context(0)
    for g, xb in zip(gs, xs):
        L = orc.layout(g, "ParHDE", "Kcenters", k, c, eig="exact", nthreads=4)
        assert L.status == 0
        cs.upload(g)
        assert np.array_equal(cs.kcenters(3 * k, 0, want_dist=False)[1], L.sources[: 3 * k])
        np.testing.assert_allclose(rayleigh(g, xb), rayleigh(g, L.coords), rtol=1e-3)
        assert principal_cosines(xb, L.coords).min() > 1 - 1e-3


def learned_batch_graphs():
    return [graphs.rgg(3000, dim=2, avg_degree=8, seed=11), graphs.rgg(12000, dim=2, avg_degree=8, seed=12),
            graphs.mesh(60, 50, seed=13), graphs.rmat(12, seed=14), graphs.rgg(25000, dim=2, avg_degree=8, seed=15),
            graphs.rgg(8000, dim=3, avg_degree=12, seed=16), graphs.rgg(600, dim=2, avg_degree=8, seed=17)]


@pytest.mark.parametrize("k,c", [(10, 2), (20, 3)])
def test_batched_learned_matches_single_learned_layouts(k, c):
    """Learned pivots in a batch (warm start, per-graph feature normalisation and candidates, one multi-source
    sweep for all graphs, per-graph farthest-point order) give every graph the pivots its own learned layout
    takes: the same layout up to the mixed path's rounding, and the per-graph Rayleigh quotients the library
    reports."""
    gs = [g for g in learned_batch_graphs() if g.n > 256]
    cb = Context(0)
    cb.upload_batch(gs)
    xs, st = cb.layout_batched(k, c, strategy="Learned")
    xs = [x.copy() for x in xs]
    rq_lib = cb.batch_rayleigh()
    assert st["naccepted"] == k
    cs = Context(0)
    for i, (g, xb) in enumerate(zip(gs, xs)):
        cs.upload(g)
        r = cs.layout("ParHDE", "Learned", k, c, precision="mixed", eig="exact")
        q = rayleigh(g, xb)
        np.testing.assert_allclose(np.linalg.norm(xb, axis=0), 1.0, rtol=1e-9)
        np.testing.assert_allclose(q, rayleigh(g, r.coords), rtol=1e-4)
        assert principal_cosines(xb, r.coords).min() > 1 - 1e-5
        # the library's quotient is y^T M y / ||S y||^2 over the FP32 basis in FP64; q is taken from the
        # coordinates, which are rounded to FP32 before their normalisation: ~1e-5 apart on these graphs
        np.testing.assert_allclose(rq_lib[i], q, rtol=1e-4)
    # a replay of the captured sequence gives the same layouts bit for bit
    xs2, st2 = cb.layout_batched(k, c, strategy="Learned")
    xs3, st3 = cb.layout_batched(k, c, strategy="Learned")
    assert st3["batch_graph_replay"] == 1
    for a, b in zip(xs, xs3):
        assert np.array_equal(a, b)


def test_batched_learned_rejects_small_graphs():
    gs = learned_batch_graphs()  # the last graph has 256 vertices or fewer after its LCC
    small = [g for g in gs if g.n <= 256]
    if not small:
        gs.append(graphs.path_graph(200))
    cb = Context(0)
    cb.upload_batch(gs)
    with pytest.raises(ParHDEError) as e:
        cb.layout_batched(10, 2, strategy="Learned")
    assert e.value.status == -4


@pytest.mark.parametrize("precision,eig,k,c", [("fp64", "power", 10, 2), ("exact", "exact", 40, 3),
                                               ("mixed", "exact", 40, 2)])
def test_batched_other_options_match_single_layouts(precision, eig, k, c):
    """Options outside the fused batched pipeline (the reference's FP64 arithmetic, exact arithmetic, k above
    32, the power iteration) lay every graph out with the single-graph pipeline on its CSR cut out of the
    union: the coordinates and Rayleigh quotients a single-graph call gives; FP64 with the power iteration
    also against the oracle (the reference algorithm).  The fused pipeline still runs on the batch after."""
    from oracle import oracle as orc
    gs = [graphs.rgg(3000, dim=2, avg_degree=8, seed=41), graphs.mesh(60, 50, seed=42),
          graphs.rmat(12, seed=43), graphs.rgg(5000, dim=3, avg_degree=12, seed=44)]
    cb = Context(0)
    cb.upload_batch(gs)
    xs, st = cb.layout_batched(k, c, precision=precision, eig=eig)
    xs = [x.copy() for x in xs]
    rq = cb.batch_rayleigh()
    assert st["naccepted"] == k
    cs = Context(0)
    for i, (g, xb) in enumerate(zip(gs, xs)):
        cs.upload(g)
        r = cs.layout("ParHDE", "Kcenters", k, c, precision=precision, eig=eig)
        if precision == "exact":  # exact integer sums: the same bits
            assert np.array_equal(xb, r.coords)
        else:  # the same kernels; FP64 (FP32) sums may associate differently between calls
            np.testing.assert_allclose(sign_align(xb, r.coords), r.coords, rtol=0,
                                       atol=1e-10 if precision == "fp64" else 1e-5)
        np.testing.assert_allclose(rq[i], rayleigh(g, xb), rtol=1e-4 if precision == "mixed" else 1e-9)
        if precision == "fp64":
            L = orc.layout(g, "ParHDE", "Kcenters", k, c, nthreads=4)
            assert L.status == 0
            np.testing.assert_allclose(sign_align(xb, L.coords), L.coords, rtol=0, atol=1e-7)
    xf, _ = cb.layout_batched(10, 2)  # the union view is back: the fused pipeline on the same batch
    for g, x in zip(gs, xf):
        assert x.shape == (g.n, 2) and np.all(np.isfinite(x))
