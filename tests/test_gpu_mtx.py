"""The GPU Matrix Market converter (phde_graph_from_entries, lib/mtx2csr) against the reference converter's
golden output (tests/golden/mtx) and the oracle restatement (oracle/mtx_oracle.py) on larger random inputs."""
import glob
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN_DIR, ROOT
from icpp_2020_parhde_gb300 import Context, graphs
from oracle import mtx_oracle

pytestmark = pytest.mark.gpu
FIXTURES = sorted(glob.glob(os.path.join(GOLDEN_DIR, "mtx", "*.mtx")))


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_mtx2csr_driver_matches_reference(path, tmp_path):
    out = tmp_path / "g.csr"
    exe = os.path.join(ROOT, "icpp_2020_parhde_gb300", "lib", "mtx2csr")
    r = subprocess.run([exe, path, str(out)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    with open(path[:-4] + ".csr", "rb") as f:
        assert out.read_bytes() == f.read()


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_graph_from_entries_matches_reference(gpu_ctx, path):
    u, v, w, n1, n2, sym, pattern = mtx_oracle.parse_mtx(path)
    info = gpu_ctx.graph_from_entries(u, v, w, n1, n2 if not sym else n1, sym)
    g = gpu_ctx.download()
    got = mtx_oracle.csr_bytes(g.offsets, g.adj, g.weights if pattern == 2 else None)
    with open(path[:-4] + ".csr", "rb") as f:
        assert got == f.read()
    _, _, _, oinfo = mtx_oracle.convert(u, v, w, n1, n2 if not sym else n1, sym)
    assert info == oinfo


@pytest.mark.parametrize("case", ["sym", "sym_weighted", "bipartite"])
def test_graph_from_entries_random_vs_oracle(gpu_ctx, case):
    rng = np.random.default_rng({"sym": 1, "sym_weighted": 2, "bipartite": 3}[case])
    n1 = 6000
    n2 = n1 if case != "bipartite" else 4500
    m = 30000
    u = rng.integers(1, n1 + 1, m)
    v = rng.integers(1, n2 + 1, m)
    u[:500] = v[:500] if case != "bipartite" else u[:500]  # self loops
    u = np.concatenate([u, u[:3000]])  # repeated entries
    v = np.concatenate([v, v[:3000]])
    w = rng.integers(-100, 100, u.shape[0]) if case == "sym_weighted" else None
    sym = case != "bipartite"
    info = gpu_ctx.graph_from_entries(u, v, w, n1, n2, sym)
    g = gpu_ctx.download()
    off, adj, ws, oinfo = mtx_oracle.convert(u, v, w, n1, n2, sym)
    assert info == oinfo
    assert np.array_equal(g.offsets, off) and np.array_equal(g.adj, adj)
    if w is not None:
        assert np.array_equal(g.weights, ws)


def test_converted_graph_lays_out(gpu_ctx):
    """The converter leaves the graph uploaded: a layout runs on it directly."""
    g = graphs.mesh(40, 30, seed=7)
    src = np.repeat(np.arange(g.n), np.diff(g.offsets.astype(np.int64)))
    keep = src < g.adj
    gpu_ctx.graph_from_entries(src[keep] + 1, g.adj[keep].astype(np.int64) + 1, None, g.n, g.n, True)
    r = gpu_ctx.layout("ParHDE", "Kcenters", 10, 2)
    gpu_ctx.upload(g)
    r2 = gpu_ctx.layout("ParHDE", "Kcenters", 10, 2)
    assert np.array_equal(r.coords, r2.coords)
