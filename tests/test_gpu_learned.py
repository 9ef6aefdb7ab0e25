"""Learned pivots (PHDE_STRAT_LEARNED): MLP-proposed candidates, one multi-source BFS, farthest-point order.

Acceptance criterion: the layout's Rayleigh quotients (x'Lx / x'x per coordinate, summed over the
coordinates -- the energy the eigensolve minimises) within 2% of the Kcenters layout's, averaged over the
graph and seven relabelled copies of it.  The average matters: Kcenters starts at vertex 0 and breaks ties
by the lowest index, and on an R-MAT graph of 2^16 vertices with k = 20 its own summed quotient moves by up
to 1.48x (single coordinates by up to 2.2x) between relabellings of the same graph, so one pair of runs says
nothing at the 2% level."""
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
    return np.einsum("ij,ij->j", X, d[:, None] * X - A @ X) / np.einsum("ij,ij->j", X, X)


GRAPHS = {
    "rmat16": lambda: graphs.rmat(16, seed=31),
    "rgg2d": lambda: graphs.rgg(60000, dim=2, avg_degree=8, seed=32),
    "rgg3d": lambda: graphs.rgg(60000, dim=3, avg_degree=12, seed=33),
}


@pytest.mark.parametrize("name", sorted(GRAPHS))
def test_learned_pivots_rayleigh_within_2_percent(gpu_ctx, name):
    g = GRAPHS[name]()
    rng = np.random.default_rng(5)
    k, c = 20, 3
    tot_kc, tot_lp = [], []
    for t in range(8):
        gg = g if t == 0 else graphs.relabel(g, rng.permutation(g.n))
        gpu_ctx.upload(gg)
        kc = gpu_ctx.layout("ParHDE", "Kcenters", k, c, eig="exact")
        lp = gpu_ctx.layout("ParHDE", "Learned", k, c, eig="exact")
        assert len(lp.sources) == 3 * k and len(set(lp.sources.tolist())) == 3 * k
        assert lp.stats["naccepted"] == k
        tot_kc.append(rayleigh(gg, kc.coords).sum())
        tot_lp.append(rayleigh(gg, lp.coords).sum())
    assert np.mean(tot_lp) <= 1.02 * np.mean(tot_kc), (tot_lp, tot_kc)


def test_learned_pivot_columns_are_exact(gpu_ctx):
    g = graphs.rmat(15, seed=34)
    gpu_ctx.upload(g)
    lp = gpu_ctx.layout("ParHDE", "Learned", 10, 2, extra=True)
    # the pivots' distance columns came from the multi-source BFS: check a few against the oracle
    d = gpu_ctx.distances(lp.sources[:6])
    for i in range(6):
        assert np.array_equal(d[:, i], orc.bfs(g, int(lp.sources[i])))


def test_learned_only_for_parhde(gpu_ctx):
    g = graphs.mesh(30, 30, seed=2)
    gpu_ctx.upload(g)
    with pytest.raises(ParHDEError):
        gpu_ctx.layout("PivotMDS", "Learned", 5, 2)


# ---- acceptance in the library: PHDE_STRAT_LEARNED_CHECKED and the structural fallback ----

def _model_size():
    return 64 * 4 + 64 + 64 * 64 + 64 + 64 + 1


def _clustering_model():
    """A pivot model that prefers the vertices closest to the warm-start pivots (score = sigmoid(-10 f2), f2 the
    warm start's normalised minimum distance): every proposed candidate sits next to a pivot already taken."""
    w = np.zeros(_model_size(), np.float32)
    w[0 * 4 + 2] = 1.0                       # W1[0][2]: hidden unit 0 = f2
    w[64 * 4 + 64 + 0] = 1.0                 # W2[0][0]: second layer passes it on
    w[64 * 4 + 64 + 64 * 64 + 64 + 0] = -10  # w3[0]: the farther, the lower the score
    return w


@pytest.mark.parametrize("precision", ["exact", "mixed", "fp64"])
def test_rayleigh_quotients_in_stats(gpu_ctx, precision):
    g = graphs.rmat(14, seed=41)
    gpu_ctx.upload(g)
    r = gpu_ctx.layout("ParHDE", "Learned", 12, 3, precision=precision, eig="exact")
    assert r.stats["pivot_outcome"] == 1
    # y^T (S^T L S) y / ||S y||^2 from the pipeline's own k x k matrix: FP64-exact for the exact-Gram and FP64
    # paths; the mixed path's S^T L S carries its FP32 products
    tol = 1e-5 if precision == "mixed" else 1e-9
    np.testing.assert_allclose(r.stats["rayleigh"][:3], rayleigh(g, r.coords), rtol=tol)
    assert r.stats["rayleigh"][3:] == [0.0] * 5


def test_learned_checked_rejects_a_clustering_model():
    """A model whose candidates all crowd around the warm-start pivots gives a much worse layout: the checked
    strategy must reject it and return the Kcenters layout itself (same coordinates, same pivots)."""
    from icpp_2020_parhde_gb300 import Context
    g = graphs.rgg(40000, dim=2, avg_degree=8, seed=42)
    k, c = 20, 2
    with Context(0) as ctx:
        ctx.upload(g)
        kc = ctx.layout("ParHDE", "Kcenters", k, c, precision="exact", eig="exact")
        ctx.set_pivot_model(_clustering_model())
        bad = ctx.layout("ParHDE", "Learned", k, c, precision="exact", eig="exact")
        r = ctx.layout("ParHDE", "LearnedChecked", k, c, precision="exact", eig="exact")
    assert sum(rayleigh(g, bad.coords)) > 1.02 * sum(rayleigh(g, kc.coords))
    assert r.stats["pivot_outcome"] == 2
    assert np.array_equal(r.coords, kc.coords) and np.array_equal(r.sources, kc.sources)
    np.testing.assert_allclose(r.stats["rayleigh_kcenters"][:c], rayleigh(g, kc.coords), rtol=1e-9)
    np.testing.assert_allclose(r.stats["rayleigh"][:c], rayleigh(g, bad.coords), rtol=1e-9)
    assert r.stats["ms_check"] > 0 and r.stats["ms_total"] > r.stats["ms_check"]


def test_learned_checked_with_a_zero_model():
    """All-zero weights score every vertex alike.  Whatever the rule decides, the checked strategy returns either
    the learned layout (the same as PHDE_STRAT_LEARNED's) or the Kcenters layout, and says which."""
    from icpp_2020_parhde_gb300 import Context
    g = graphs.rmat(15, seed=43)
    k, c = 16, 3
    with Context(0) as ctx:
        ctx.upload(g)
        ctx.set_pivot_model(np.zeros(_model_size(), np.float32))
        kc = ctx.layout("ParHDE", "Kcenters", k, c, precision="exact", eig="exact")
        lp = ctx.layout("ParHDE", "Learned", k, c, precision="exact", eig="exact")
        for rule in ("sum", "each"):
            ctx.set_pivot_check(rule, 0.02)
            r = ctx.layout("ParHDE", "LearnedChecked", k, c, precision="exact", eig="exact")
            ql, qk = rayleigh(g, lp.coords), rayleigh(g, kc.coords)
            ok = ql.sum() <= 1.02 * qk.sum() if rule == "sum" else bool(np.all(ql <= 1.02 * qk))
            assert r.stats["pivot_outcome"] == (1 if ok else 2), (rule, ql, qk)
            want = lp if ok else kc
            assert np.array_equal(r.coords, want.coords) and np.array_equal(r.sources, want.sources)


def test_learned_falls_back_when_the_search_is_too_deep(gpu_ctx):
    """A 70000-vertex path: the multi-source BFS's 16-bit level record overflows, so the learned proposal gives
    no layout; PHDE_STRAT_LEARNED returns the Kcenters layout and says so."""
    g = graphs.path_graph(70000)
    gpu_ctx.upload(g)
    r = gpu_ctx.layout("ParHDE", "Learned", 6, 2, precision="exact", eig="exact")
    kc = gpu_ctx.layout("ParHDE", "Kcenters", 6, 2, precision="exact", eig="exact")
    assert r.stats["pivot_outcome"] == 3
    assert np.array_equal(r.coords, kc.coords) and np.array_equal(r.sources, kc.sources)


def test_pivot_check_arguments(gpu_ctx):
    with pytest.raises(ParHDEError):
        gpu_ctx._check(gpu_ctx._L.phde_set_pivot_check(gpu_ctx._h, 7, 0.02))
    with pytest.raises(ParHDEError):
        gpu_ctx.set_pivot_check("sum", -1.0)
    gpu_ctx.set_pivot_check("sum", 0.02)


@pytest.mark.parametrize("make", [lambda: graphs.rmat(15, seed=44), lambda: graphs.rgg(30000, dim=3, avg_degree=12, seed=45)],
                         ids=["rmat15", "rgg3d"])
def test_feature_and_mlp_kernels_vs_numpy(gpu_ctx, make):
    """feature_raw_kernel + mlp_score_kernel against the numpy restatement (oracle/pivot_oracle.py) on the warm
    start of the oracle's own Kcenters: the warm distances bit-exact, every score within 1e-5 relative (FP32
    log / exp and summation order differ), and the same 256 candidates except where scores tie within that
    tolerance at the cut."""
    from oracle import pivot_oracle as po
    g = make()
    gpu_ctx.upload(g)
    sc, d0, cand = gpu_ctx.pivot_scores(256)
    D, _ = orc.kcenters(g, po.WARM, 0)
    d0_ref = D.min(axis=1)
    assert np.array_equal(d0, d0_ref)
    ref = po.scores(po.features(g, d0_ref), po.load_weights())
    np.testing.assert_allclose(sc, ref, rtol=1e-5, atol=1e-7)
    order = np.lexsort((np.arange(g.n), -ref.astype(np.float64)))  # score descending, index ascending
    want = order[:256]
    cut = ref[want[-1]]
    differ = set(cand.tolist()) ^ set(want.tolist())
    assert all(abs(float(ref[v]) - float(cut)) <= 1e-5 * abs(float(cut)) + 1e-7 for v in differ), sorted(differ)[:8]
    # candidates come best first: their GPU scores are non-increasing
    assert np.all(np.diff(sc[cand].astype(np.float64)) <= 0)


@pytest.mark.parametrize("make,k", [(lambda: graphs.rmat(14, seed=51), 20), (lambda: graphs.rgg(20000, dim=3, avg_degree=12, seed=52), 16),
                                    (lambda: graphs.mesh(120, 90, seed=53), 24)], ids=["rmat14", "rgg3d", "mesh"])
def test_learned_pivot_order_vs_oracle(gpu_ctx, make, k):
    """The learned strategy's whole pivot sequence against a CPU restatement, given the proposal's candidates:
    the warm start is the oracle's Kcenters (the first 8 pivots), the candidates' distances come from the
    oracle's one-source BFS (the GPU reads them from its multi-source sweep), and the rest is the
    farthest-point order of oracle/pivot_oracle.py -- the same 3k sources in the same order."""
    from oracle import pivot_oracle as po
    g = make()
    gpu_ctx.upload(g)
    _, _, cand = gpu_ctx.pivot_scores(256)
    lp = gpu_ctx.layout("ParHDE", "Learned", k, 2, precision="exact", eig="exact")
    P = 3 * k
    Dw, warm = orc.kcenters(g, po.WARM, 0)
    assert np.array_equal(lp.sources[: po.WARM], warm)
    dist = np.stack([orc.bfs(g, int(v)) for v in cand], axis=1)  # (n, M): column j from candidate j
    order = po.farthest_point_order(Dw[cand], dist[cand], P - po.WARM)
    assert np.array_equal(lp.sources[po.WARM:], cand[order])
