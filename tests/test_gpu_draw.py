"""The GPU rasteriser (phde_draw, phde_draw_write_png, lib/draw) against the reference draw tool's images
(tests/golden/draw) and the draw oracle (oracle/draw_oracle.c) on larger graphs, bit-exact per pixel."""
import os
import subprocess

import numpy as np
import pytest

import pngdecode
from conftest import ROOT, draw_case_names, load_draw_case
from icpp_2020_parhde_gb300 import ParHDEError, graphs
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
DRAW_EXE = os.path.join(ROOT, "icpp_2020_parhde_gb300", "lib", "draw")


def gpu_image(ctx, g, x, y):
    ctx.upload(g)
    info = ctx.draw(x, y)
    return ctx.draw_image(), info


@pytest.mark.parametrize("name", draw_case_names())
def test_draw_matches_reference_png(gpu_ctx, name):
    g, x, y, meta, png = load_draw_case(name)
    img, info = gpu_image(gpu_ctx, g, x, y)
    ref = pngdecode.read(png)
    assert img.shape == ref.shape
    assert np.array_equal(img, ref)
    _, ml = orc.draw(g, x, y)
    assert info["max_edge_length"] == np.float32(ml)


@pytest.mark.parametrize("name", draw_case_names())
def test_draw_driver_matches_reference_png(name, tmp_path):
    """lib/draw, the drop-in for the reference's command line, writes a PNG of the reference's pixels."""
    _, _, _, meta, png = load_draw_case(name)
    base = png[:-4]
    out = str(tmp_path / "out.png")
    r = subprocess.run([DRAW_EXE, base + ".csr", base + ".nxyz", out, str(meta["ncoords"]), str(meta["first"]),
                        str(meta["second"])], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Max edge length:" in r.stdout and "Corrected width" in r.stderr
    assert np.array_equal(pngdecode.read(out), pngdecode.read(png))


def _random_positions(n, seed, spread=(10.0, 6.0)):
    rng = np.random.default_rng(seed)
    return rng.uniform(-spread[0], spread[0], n), rng.uniform(-spread[1], spread[1], n)


@pytest.mark.parametrize("case", ["mesh_layout", "rmat_layout", "rgg_positions", "random_dense", "star_hub"])
def test_draw_matches_oracle(gpu_ctx, case, tmp_path):
    """Larger graphs: layouts from the GPU pipeline, geometric positions (bin 0 past its counter) and random
    positions (every counter exhausted); the PNG path decodes to the same pixels."""
    if case == "mesh_layout":
        g = graphs.mesh(90, 70, seed=4)
        gpu_ctx.upload(g)
        xy = gpu_ctx.layout("ParHDE", "Kcenters", k=10, c=2).coords
        x, y = xy[:, 0].copy(), xy[:, 1].copy()
    elif case == "rmat_layout":
        g = graphs.rmat(13, 8, seed=3)
        gpu_ctx.upload(g)
        xy = gpu_ctx.layout("ParHDE", "Kcenters", k=10, c=2).coords
        x, y = xy[:, 0].copy(), xy[:, 1].copy()
    elif case == "rgg_positions":
        rng = np.random.default_rng(5)
        n = 6000
        pts = rng.random((n, 2))
        order = np.lexsort((pts[:, 1], pts[:, 0]))
        pts = pts[order]
        pairs = []
        cell = np.floor(pts * 40).astype(np.int64)
        key = cell[:, 0] * 41 + cell[:, 1]
        buckets = {}
        for i, kk in enumerate(key):
            buckets.setdefault(int(kk), []).append(i)
        r2 = 0.02 ** 2
        for i in range(n):
            cx, cy = cell[i]
            for ax in (cx - 1, cx, cx + 1):
                for ay in (cy - 1, cy, cy + 1):
                    for j in buckets.get(int(ax * 41 + ay), ()):
                        if j > i:
                            d2 = ((pts[i] - pts[j]) ** 2).sum()
                            if d2 < r2:
                                pairs.append((i, j))
        pairs.append((0, n - 1))  # one long edge: nearly every other edge lands in bin 0
        g = _csr(n, pairs)
        x, y = pts[:, 0].copy(), pts[:, 1].copy()
    elif case == "random_dense":
        rng = np.random.default_rng(9)
        n = 3000
        g = _csr(n, rng.integers(0, n, (40000, 2)))
        x, y = _random_positions(n, 11)
    else:
        n = 5000
        g = _csr(n, [(0, i) for i in range(1, n)] + [(i, i + 1) for i in range(1, n - 1)])
        x, y = _random_positions(n, 12, (3.0, 0.5))
    img, info = gpu_image(gpu_ctx, g, x, y)
    ref, ml = orc.draw(g, x, y)
    assert img.shape == ref.shape
    bad = np.argwhere((img != ref).any(axis=2))
    assert bad.shape[0] == 0, "%d pixels differ, first at %s: %s vs %s" % (
        bad.shape[0], bad[0], img[tuple(bad[0])], ref[tuple(bad[0])])
    assert info["max_edge_length"] == np.float32(ml)
    assert info["pixels"] > 0 and info["gpu_launches"] >= 5
    path = str(tmp_path / "img.png")
    gpu_ctx.draw_png(path, nthreads=4)
    assert np.array_equal(pngdecode.read(path), ref)


def test_draw_rejects_bad_coordinates(gpu_ctx):
    g = graphs.path_graph(10)
    gpu_ctx.upload(g)
    x = np.linspace(0, 3, 10)
    y = np.linspace(-2, 2, 10)
    x[4] = np.nan
    with pytest.raises(ParHDEError):
        gpu_ctx.draw(x, y)
    with pytest.raises(ParHDEError):  # a zero x range: no image width
        gpu_ctx.draw(np.full(10, 0.5), y)
    x[4] = 1.0
    gpu_ctx.draw(x, y)  # the context stays usable


def test_draw_property_large(gpu_ctx):
    """A layout of a 1M-entry graph: the image agrees with the oracle, and the reported pixel writes equal the
    sum of the Bresenham line lengths."""
    g = graphs.rmat(16, 8, seed=2)
    gpu_ctx.upload(g)
    xy = gpu_ctx.layout("ParHDE", "Kcenters", k=10, c=2, precision="mixed", eig="exact").coords
    x, y = xy[:, 0].copy(), xy[:, 1].copy()
    img, info = gpu_image(gpu_ctx, g, x, y)
    ref, _ = orc.draw(g, x, y)
    assert np.array_equal(img, ref)
    # the pixel count is the sum of Bresenham line lengths, computed here from the oracle's pixel positions
    (xmin, xmax, ymin, ymax, _), _, (W, H) = orc.draw_geometry(x, y)
    px = np.clip((-xmin + x) * (1.0 / (xmax - xmin)) * W, 0, W - 1).astype(np.int64)
    py = np.clip((-ymin + y) * (1.0 / (ymax - ymin)) * H, 0, H - 1).astype(np.int64)
    src = np.repeat(np.arange(g.n), np.diff(g.offsets.astype(np.int64)))
    L = np.maximum(np.abs(px[g.adj] - px[src]), np.abs(py[g.adj] - py[src])) + 1
    assert info["pixels"] == int(L.sum())


def _csr(n, pairs):
    p = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    p = p[p[:, 0] != p[:, 1]]
    d = np.unique(np.concatenate([p, p[:, ::-1]]), axis=0)
    off = np.zeros(n + 1, dtype=np.int64)
    np.add.at(off, d[:, 0] + 1, 1)
    from icpp_2020_parhde_gb300.csr_io import CSRGraph
    return CSRGraph(np.cumsum(off).astype(np.uint32), d[:, 1].astype(np.uint32), None, "draw")


def test_draw_plain_raster_variant_matches(monkeypatch):
    """PHDE_DRAW_RASTER=plain (an atomic for every pixel write, tiles in order) draws the same image."""
    from icpp_2020_parhde_gb300 import Context
    g, x, y, meta, png = load_draw_case("random_spread")
    monkeypatch.setenv("PHDE_DRAW_RASTER", "plain")
    with Context(0) as ctx:
        img, _ = gpu_image(ctx, g, x, y)
    assert np.array_equal(img, pngdecode.read(png))
