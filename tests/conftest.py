"""Shared fixtures.  `-m gpu` tests need a GB300 and call the CUDA library through the C ABI;
everything else runs on the CPU (oracle vs golden fixtures, host logic, library symbols)."""
import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from icpp_2020_parhde_gb300.csr_io import CSRGraph  # noqa: E402

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libparhde_gb300.so")


def load_golden(name: str):
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    rec = {k: z[k] for k in z.files}
    g = CSRGraph(rec["csr_offsets"], rec["csr_adj"], rec.get("csr_weights"), name)
    return g, rec


GOLDEN_NAMES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def golden_runs():
    """(case, algo, k, c) for every reference layout recorded in the fixtures."""
    out = []
    for name in GOLDEN_NAMES:
        z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
        for key in z.files:
            if key.endswith("_coords"):
                algo, k, c, _ = key.split("_")
                out.append((name, algo, int(k[1:]), int(c[1:])))
    return out


def sign_align(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Flip the columns of a to best match b (eigenvector signs are arbitrary up to the sign rule)."""
    a = a.copy()
    for j in range(a.shape[1]):
        if np.dot(a[:, j], b[:, j]) < 0:
            a[:, j] = -a[:, j]
    return a


@pytest.fixture(scope="session")
def gpu_ctx():
    from icpp_2020_parhde_gb300 import Context
    ctx = Context(0)
    yield ctx
    ctx.close()
