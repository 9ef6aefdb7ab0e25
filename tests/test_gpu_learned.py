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
