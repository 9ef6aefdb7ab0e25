"""The layouts' exact eigensolver (phde_symeig: FP32 Jacobi sweeps, FP64 orthonormalisation and similarity, FP64
rotations of unseparated pairs, perturbation refinement, FP64 sweeps when a wanted eigenvalue is not separated)
on symmetric matrices built from known spectra: separated, clustered away from the wanted eigenvalues,
degenerate among the wanted ones, exactly diagonal with repeats; against numpy's eigh and the spectrum."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def built(spec, seed):
    rng = np.random.default_rng(seed)
    k = len(spec)
    Q, _ = np.linalg.qr(rng.standard_normal((k, k)))
    M = Q @ np.diag(spec) @ Q.T
    return 0.5 * (M + M.T)


def signed(Y):
    """Each column signed so that its entry of largest magnitude is positive (the solver's convention)."""
    Y = Y.copy()
    for j in range(Y.shape[1]):
        i = np.argmax(np.abs(Y[:, j]))
        if Y[i, j] < 0:
            Y[:, j] = -Y[:, j]
    return Y


def wanted(w, V, c, largest):
    cols = list(range(len(w) - 1, len(w) - 1 - c, -1)) if largest else list(range(c))
    return w[cols], V[:, cols]


def check_solve(gpu_ctx, M, c, largest):
    """Eigenvalues to 1e-11 of the spectral radius (FP32 sweeps, then FP64 work on a basis orthonormalised to
    second order), residuals and orthonormality of the returned eigenvectors."""
    ev, Y, _ = gpu_ctx.symeig(M, c, largest)
    w, V = np.linalg.eigh(M)
    scale = np.abs(w).max()
    np.testing.assert_allclose(ev, w, rtol=0, atol=1e-11 * scale)
    lw, Vw = wanted(w, V, c, largest)
    np.testing.assert_allclose(M @ Y - Y * lw, 0, atol=1e-10 * scale)
    np.testing.assert_allclose(Y.T @ Y, np.eye(c), atol=1e-11)
    return ev, Y, w, Vw


@pytest.mark.parametrize("k,c,largest", [(64, 3, False), (96, 4, False), (40, 3, True), (1, 1, False)])
def test_separated_spectrum(gpu_ctx, k, c, largest):
    rng = np.random.default_rng(k)
    spec = np.arange(1, k + 1, dtype=np.float64) + 0.3 * rng.random(k)
    M = built(spec, seed=k + 1)
    ev, Y, w, Vw = check_solve(gpu_ctx, M, c, largest)
    np.testing.assert_allclose(Y, signed(Vw), rtol=0, atol=1e-9)


@pytest.mark.parametrize("k,c,largest", [(64, 3, False), (96, 3, False), (64, 2, True)])
def test_clusters_away_from_the_wanted_eigenvalues(gpu_ctx, k, c, largest):
    """Exactly repeated and nearly repeated eigenvalues (gaps 1e-12 .. 1e-5 relative) among the unwanted ones:
    the targeted FP64 rotations settle them, the wanted eigenpairs stay exact."""
    rest = [10.0] * 5 + [10 + 1e-10, 10 + 1e-7, 10 + 1e-4, 30.0, 30.0, 30 + 1e-9]
    head = [1.0, 2.0, 3.5]
    tail = list(np.linspace(40.0, 90.0, k - len(rest) - len(head)))
    spec = np.array(head + rest + tail)
    if largest:
        spec = spec.max() + 1.0 - spec  # the clusters sit below the wanted largest eigenvalues
    M = built(spec, seed=7 * k)
    ev, Y, w, Vw = check_solve(gpu_ctx, M, c, largest)
    np.testing.assert_allclose(Y, signed(Vw), rtol=0, atol=1e-9)
    np.testing.assert_allclose(np.sort(ev), np.sort(spec), rtol=0, atol=1e-11 * np.abs(spec).max())


def test_degenerate_wanted_eigenvalues(gpu_ctx):
    """A repeated wanted eigenvalue: any orthonormal basis of its eigenspace is an answer; the solver's spans it."""
    k = 48
    spec = np.array([1.0, 1.0, 2.0] + list(np.linspace(5.0, 60.0, k - 3)))
    M = built(spec, seed=5)
    ev, Y, w, Vw = check_solve(gpu_ctx, M, 3, False)
    P = Vw[:, :2] @ Vw[:, :2].T
    np.testing.assert_allclose(Y[:, :2] - P @ Y[:, :2], 0, atol=1e-9)
    np.testing.assert_allclose(Y[:, 2], signed(Vw[:, 2:3])[:, 0], rtol=0, atol=1e-9)


def test_exactly_diagonal_with_repeats(gpu_ctx):
    """Zero couplings between equal diagonal entries (no rotation applies) give finite, exact results."""
    spec = np.array([3.0, 1.0, 2.0, 7.0, 7.0, 7.0, 9.0, 9.0, 11.0, 4.0])
    ev, Y, _ = gpu_ctx.symeig(np.diag(spec), 3, False)
    np.testing.assert_array_equal(ev, np.sort(spec))
    E = np.zeros((len(spec), 3))
    E[[1, 2, 0], [0, 1, 2]] = 1.0
    np.testing.assert_array_equal(Y, E)


def test_bad_arguments(gpu_ctx):
    from icpp_2020_parhde_gb300 import ParHDEError
    with pytest.raises(ParHDEError):
        gpu_ctx.symeig(np.eye(4), 5)
