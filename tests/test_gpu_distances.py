"""GPU distance kernels against the reference's own distance columns (golden fixtures) and the oracle:
bit-exact hop counts and weighted distances, identical Kcenters pivot order."""
import numpy as np
import pytest

from conftest import GOLDEN_NAMES, golden_runs, load_golden
from icpp_2020_parhde_gb300 import DOBFS, DeltaStep, ParHDEError, graphs
from icpp_2020_parhde_gb300.csr_io import CSRGraph
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_distances_bit_exact_vs_reference(gpu_ctx, name):
    g, rec = load_golden(name)
    gpu_ctx.upload(g)
    d = gpu_ctx.distances(rec["bfs_src"])
    assert d.dtype == np.int32
    assert np.array_equal(d, rec["bfs_dist"])


@pytest.mark.parametrize("case", [c for c in golden_runs()], ids=lambda c: "%s-%s-k%d-c%d" % c)
def test_kcenters_pivot_order_vs_reference(gpu_ctx, case):
    name, algo, k, c = case
    g, rec = load_golden(name)
    ref = rec[f"{algo}_k{k}_c{c}_sources"]
    gpu_ctx.upload(g)
    if algo == "wParHDE":
        pytest.skip("WParHDE interleaves selection with orthogonalisation; covered by the layout tests")
    passes = 3 * k if algo == "ParHDE" else k
    D, src = gpu_ctx.kcenters(passes, 0 if algo == "ParHDE" else 2)
    assert np.array_equal(src, ref[:passes])
    Do, so = orc.kcenters(g, passes, 0 if algo == "ParHDE" else 2)
    assert np.array_equal(D, Do)


@pytest.mark.parametrize("make", [
    lambda: graphs.rmat(16, seed=1),
    lambda: graphs.rgg(60000, dim=2, avg_degree=8, seed=2),
    lambda: graphs.rgg(40000, dim=3, avg_degree=12, seed=3),
    lambda: graphs.mesh(300, 200, seed=4),
], ids=["rmat16", "rgg2d", "rgg3d", "mesh300x200"])
def test_bfs_and_kcenters_exact_vs_oracle(gpu_ctx, make):
    g = make()
    gpu_ctx.upload(g)
    rng = np.random.default_rng(5)
    src = rng.integers(0, g.n, size=4)
    d = gpu_ctx.distances(src)
    for i, s in enumerate(src):
        assert np.array_equal(d[:, i], orc.bfs(g, int(s)))
    D, s = gpu_ctx.kcenters(24, 0)
    Do, so = orc.kcenters(g, 24, 0, parallel=True)
    assert np.array_equal(s, so) and np.array_equal(D, Do)


@pytest.mark.parametrize("L,seed", [(20, 1), (32, 2)])
def test_sssp_exact_vs_oracle(gpu_ctx, L, seed):
    g = graphs.grid3d(L, seed=seed)
    gpu_ctx.upload(g)
    src = [0, g.n - 1, g.n // 2]
    d = gpu_ctx.distances(src)
    for i, s in enumerate(src):
        assert np.array_equal(d[:, i], orc.sssp(g, s))


@pytest.mark.parametrize("local,ctas,delta", [("0", "2", None), ("1", "1", None), ("4", "2", "40"), ("16", "1", "7")])
def test_sssp_round_shapes_exact(gpu_ctx, monkeypatch, local, ctas, delta):
    """The block-local round count, resident CTAs per SM and band width change the work, never the
    distances: a weighted grid and a weighted R-MAT (hubs: several chunks per block) under each shape."""
    monkeypatch.setenv("PHDE_SSSP_LOCAL", local)
    monkeypatch.setenv("PHDE_SSSP_CTAS", ctas)
    if delta is None:
        monkeypatch.delenv("PHDE_SSSP_DELTA", raising=False)
    else:
        monkeypatch.setenv("PHDE_SSSP_DELTA", delta)
    for g in (graphs.grid3d(24, seed=4), graphs.with_random_weights(graphs.rmat(13, seed=5), seed=6, wmin=1, wmax=300)):
        gpu_ctx.upload(g)
        src = [0, g.n - 1, g.n // 3]
        d = gpu_ctx.distances(src)
        for i, s in enumerate(src):
            assert np.array_equal(d[:, i], orc.sssp(g, s))


def test_sssp_exact_on_weighted_rmat(gpu_ctx):
    g = graphs.with_random_weights(graphs.rmat(14, seed=9), seed=3, wmin=1, wmax=1000)
    gpu_ctx.upload(g)
    d = gpu_ctx.distances([0, 17, 999])
    for i, s in enumerate([0, 17, 999]):
        assert np.array_equal(d[:, i], orc.sssp(g, s))


def _two_triangles(weighted=False):
    off = np.array([0, 2, 4, 6, 8, 10, 12], dtype=np.uint32)
    adj = np.array([1, 2, 0, 2, 0, 1, 4, 5, 3, 5, 3, 4], dtype=np.uint32)
    w = np.full(12, 3, dtype=np.int32) if weighted else None
    return CSRGraph(off, adj, w)


def test_disconnected_distances_and_layout_error(gpu_ctx):
    g = _two_triangles()
    gpu_ctx.upload(g)
    d = gpu_ctx.distances([0])
    assert list(d[:, 0]) == [0, 1, 1, -1, -1, -1]
    with pytest.raises(ParHDEError) as e:
        gpu_ctx.layout("ParHDE", k=2, c=2)
    assert e.value.status == -3
    gw = _two_triangles(weighted=True)
    gpu_ctx.upload(gw)
    d = gpu_ctx.distances([4])
    assert list(d[:, 0]) == [orc.SSSP_INF] * 3 + [3, 0, 3]


def test_reference_shaped_dobfs_and_deltastep():
    g = _two_triangles()
    dists = np.full(6, -7.0)
    DOBFS(g.offsets, g.adj, 1, 6, 12, dists)
    assert list(dists) == [1, 0, 1, -7, -7, -7]  # unreached entries untouched (bfs.cc:144-185)
    gw, rec = load_golden("grid12w")
    dist = np.zeros(gw.n)
    DeltaStep(gw.offsets, gw.adj, gw.weights, 1000, gw.n, gw.nnz, dist, 10000)
    assert np.array_equal(dist.astype(np.int32), rec["bfs_dist"][:, 1])


def test_csr_validation_rejects_bad_input(gpu_ctx):
    off = np.array([0, 2, 1, 3], dtype=np.uint32)  # decreasing offsets
    adj = np.array([1, 2, 0], dtype=np.uint32)
    with pytest.raises(ParHDEError) as e:
        gpu_ctx.upload(CSRGraph(off, adj))
    assert e.value.status == -2
    off = np.array([0, 1, 2], dtype=np.uint32)
    adj = np.array([1, 5], dtype=np.uint32)  # neighbour out of range
    with pytest.raises(ParHDEError) as e:
        gpu_ctx.upload(CSRGraph(off, adj))
    assert e.value.status == -2


def test_bounded_wait_times_out_and_context_survives(gpu_ctx):
    assert gpu_ctx.selftest_barrier_timeout(50) == -8  # PHDE_ERR_TIMEOUT
    g, rec = load_golden("mesh125")
    gpu_ctx.upload(g)
    assert np.array_equal(gpu_ctx.distances(rec["bfs_src"]), rec["bfs_dist"])


@pytest.mark.parametrize("nsrc", [5, 64, 100, 300])
def test_multi_source_bfs_bit_exact(gpu_ctx, nsrc):
    """phde_distances with several sources runs the bitset multi-source BFS (up to 256 sources per sweep)."""
    g = graphs.rmat(15, seed=12)
    gpu_ctx.upload(g)
    rng = np.random.default_rng(nsrc)
    src = rng.integers(0, g.n, size=nsrc)
    src[1] = src[0]  # a repeated source is allowed
    d = gpu_ctx.distances(src)
    for i in range(0, nsrc, max(1, nsrc // 7)):
        assert np.array_equal(d[:, i], orc.bfs(g, int(src[i]))), i
    assert np.array_equal(d[:, 0], d[:, 1])


@pytest.mark.parametrize("window", ["0", "1"])
@pytest.mark.parametrize("make,nsrc", [
    (lambda: graphs.rgg(40000, dim=3, avg_degree=12, seed=3), 256),
    (lambda: graphs.rgg(30000, dim=2, avg_degree=8, seed=5), 100),
    (lambda: graphs.rmat(14, seed=2), 256),
], ids=["rgg3d-256", "rgg2d-100", "rmat14-256"])
def test_multi_source_bfs_window_modes(gpu_ctx, monkeypatch, make, nsrc, window):
    """Dense levels with and without the shared-memory frontier window (chosen by index locality; forced here
    both ways, also on the R-MAT graph whose numbering is not local) give the one-source BFS columns."""
    monkeypatch.setenv("PHDE_MSBFS_WINDOW", window)
    g = make()
    gpu_ctx.upload(g)
    rng = np.random.default_rng(nsrc + 7)
    src = rng.integers(0, g.n, size=nsrc)
    d = gpu_ctx.distances(src)
    for i in range(0, nsrc, max(1, nsrc // 9)):
        assert np.array_equal(d[:, i], orc.bfs(g, int(src[i]))), i


def test_multi_source_bfs_on_mesh_and_disconnected(gpu_ctx):
    g, rec = load_golden("mesh125")
    gpu_ctx.upload(g)
    src = np.concatenate([rec["bfs_src"], np.arange(0, 15625, 1000)])
    d = gpu_ctx.distances(src)
    assert np.array_equal(d[:, :3], rec["bfs_dist"])
    for i in range(3, len(src)):
        assert np.array_equal(d[:, i], orc.bfs(g, int(src[i])))
    g2 = _two_triangles()
    gpu_ctx.upload(g2)
    d = gpu_ctx.distances([0, 1, 3, 5])
    assert list(d[:, 0]) == [0, 1, 1, -1, -1, -1] and list(d[:, 2]) == [-1, -1, -1, 0, 1, 1]
