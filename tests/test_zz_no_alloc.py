"""phde_bfs_noalloc: the BFS entry point for callers that may not allocate device memory.

Such callers -- code whose device memory belongs to its own pool allocator, code on a latency-critical
path where cudaMalloc would synchronise the device, plugins handed only pre-allocated buffers -- pass the
graph and the output column as device pointers; the library's scratch is a fixed array inside the
library.  This file is collected last so that a run stopping at the first failure has already run
every other test.  The device buffers here are the CALLER's (allocated by the test through torch);
the entry point itself must not change the device's free memory.
"""
import ctypes as C

import numpy as np
import pytest

from icpp_2020_parhde_gb300 import graphs

pytestmark = pytest.mark.gpu


def _setup(g):
    torch = pytest.importorskip("torch")
    off = torch.tensor(g.offsets.astype(np.int64), device="cuda")
    adj = torch.tensor(g.adj.astype(np.int32), device="cuda")  # same bits as uint32 (all ids < 2^31)
    dist = torch.empty(g.n, dtype=torch.int32, device="cuda")
    return torch, off, adj, dist


def test_noalloc_bfs_matches_existing_entry_point_twice():
    from icpp_2020_parhde_gb300 import Context, _lib, graphs
    from oracle import oracle as orc

    L = _lib.load()
    g = graphs.rmat(16, seed=2)
    torch, off, adj, dist = _setup(g)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    sources = [0, g.n // 3]
    with Context(0) as ctx:
        ctx.upload(g)
        want = ctx.distances(sources)
    # first call: one-time lookup of the scratch address
    assert L.phde_bfs_noalloc(off.data_ptr(), adj.data_ptr(), g.n, g.nnz, sources[0], dist.data_ptr(), stream) == 0
    free0 = torch.cuda.mem_get_info()[0]
    for i, s in enumerate(sources):  # two calls in a row; integer distances must agree exactly
        rc = L.phde_bfs_noalloc(off.data_ptr(), adj.data_ptr(), g.n, g.nnz, s, dist.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()
        got = dist.cpu().numpy()
        assert np.array_equal(got, want[:, i])
        assert np.array_equal(got, orc.bfs(g, s))  # and the oracle's BFS, not only the library's own
    assert torch.cuda.mem_get_info()[0] == free0  # the calls allocated no device memory


@pytest.mark.parametrize("make", [lambda: graphs.mesh(900, 40, seed=4), lambda: graphs.path_graph(5000)],
                         ids=["long-mesh", "path"])
def test_noalloc_bfs_matches_oracle_on_long_searches(make):
    """Graphs with hundreds to thousands of levels, so the search switches between top-down and bottom-up
    steps many times, against the oracle's BFS, on two calls in a row from different sources."""
    from icpp_2020_parhde_gb300 import _lib
    from oracle import oracle as orc

    L = _lib.load()
    g = make()
    torch, off, adj, dist = _setup(g)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for s in (0, g.n - 1):
        assert L.phde_bfs_noalloc(off.data_ptr(), adj.data_ptr(), g.n, g.nnz, s, dist.data_ptr(), stream) == 0
        torch.cuda.synchronize()
        assert np.array_equal(dist.cpu().numpy(), orc.bfs(g, s))


def test_noalloc_bfs_rejects_graphs_beyond_capacity():
    from icpp_2020_parhde_gb300 import _lib, graphs

    L = _lib.load()
    g = graphs.path_graph(8)
    torch, off, adj, dist = _setup(g)
    n_too_big = _lib.NOALLOC_MAX_VERTICES + 1
    rc = L.phde_bfs_noalloc(off.data_ptr(), adj.data_ptr(), n_too_big, g.nnz, 0, dist.data_ptr(), None)
    assert rc == -12  # PHDE_ERR_TOO_LARGE, nothing launched
