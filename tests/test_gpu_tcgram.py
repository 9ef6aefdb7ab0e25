"""The tensor-core Gram kernel (tcgen05, three-way BF16 split, FP32 accumulation in TMEM) behind the mixed
path's Gram products, through phde_gram_f32, against FP64 products of the same FP32 inputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ref(A, B, w=None):
    A64 = A.astype(np.float64)
    B64 = B.astype(np.float64)
    if w is not None:  # the kernel scales B's rows by (float) w in FP32, as the CGS2 projections do
        B64 = (B * w.astype(np.float32)[:, None]).astype(np.float64)
    return A64.T @ B64, np.abs(A64).T @ np.abs(B64)


def test_gram_small_integers_exact(gpu_ctx):
    """Small integers are exact in every part: any layout or descriptor error shows as a wrong entry."""
    rng = np.random.default_rng(1)
    for n, p, q in [(64, 32, 32), (200, 50, 50), (1000, 64, 64), (129, 7, 3), (3000, 130, 70)]:
        A = rng.integers(-8, 9, (n, p)).astype(np.float32)
        B = rng.integers(-8, 9, (n, q)).astype(np.float32)
        G = gpu_ctx.gram_f32(A, B)
        ref, _ = _ref(A, B)
        assert np.array_equal(G, ref), (n, p, q, np.argwhere(G != ref)[:5])


@pytest.mark.parametrize("n,p,q,weighted,nsplit", [
    (100_003, 50, 50, False, 0), (65_536, 64, 64, True, 7), (4_097, 33, 17, True, 1), (250_000, 100, 51, False, 0),
    (7, 3, 5, False, 0), (0, 4, 4, False, 0)])
def test_gram_random_fp32_faithful(gpu_ctx, n, p, q, weighted, nsplit):
    rng = np.random.default_rng(n + p)
    A = (rng.standard_normal((n, p)) / np.sqrt(max(n, 1))).astype(np.float32)
    B = (rng.standard_normal((n, q)) * rng.uniform(0.1, 10, q) / np.sqrt(max(n, 1))).astype(np.float32)
    w = rng.uniform(1, 300, n) if weighted else None
    G = gpu_ctx.gram_f32(A, B, w, nsplit=nsplit)
    ref, mag = _ref(A, B, w)
    err = np.abs(G - ref) / np.maximum(mag, 1e-300)
    # FP32 accumulation over each CTA's rows: a few units of 2^-24 times sqrt(rows), far below 1e-5
    assert err.max() < 2e-6, err.max()


@pytest.mark.parametrize("mode", ["0", "all"])
def test_mixed_layout_gram_engines_agree(mode, monkeypatch):
    """The mixed layout with its Gram products on the CUDA cores (PHDE_TC_GRAM=0) or with the CGS2 Grams on the
    tensor cores too (PHDE_TC_GRAM=all) takes the same pivots and accept/discard decisions as the default, with
    coordinates equal up to FP32 rounding."""
    from icpp_2020_parhde_gb300 import Context, graphs
    g = graphs.rmat(14, 8, seed=5)
    with Context(0) as ctx:
        ctx.upload(g)
        ref = ctx.layout("ParHDE", "Kcenters", k=40, c=3, precision="mixed", eig="exact")
    monkeypatch.setenv("PHDE_TC_GRAM", mode)
    with Context(0) as ctx:
        ctx.upload(g)
        r = ctx.layout("ParHDE", "Kcenters", k=40, c=3, precision="mixed", eig="exact")
    assert np.array_equal(r.sources, ref.sources)
    assert r.stats["naccepted"] == ref.stats["naccepted"] and r.stats["ndiscarded"] == ref.stats["ndiscarded"]
    for j in range(3):
        a, b = r.coords[:, j], ref.coords[:, j]
        if np.dot(a, b) < 0:
            b = -b
        assert np.abs(a - b).max() < 1e-3, (j, np.abs(a - b).max())
