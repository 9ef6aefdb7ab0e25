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


# ---- draw fixtures (tests/golden/draw, made by tests/golden/make_draw_golden.py) ----
DRAW_DIR = os.path.join(GOLDEN_DIR, "draw")


def draw_case_names():
    import json
    path = os.path.join(DRAW_DIR, "cases.json")
    return sorted(json.load(open(path))) if os.path.exists(path) else []


def load_draw_case(name: str):
    """(graph, x, y, meta, reference png path): the coordinate columns the case's command line selects,
    parsed from the .nxyz text as the reference's fscanf("%lf") reads them."""
    import json
    from icpp_2020_parhde_gb300.csr_io import read_csr
    meta = json.load(open(os.path.join(DRAW_DIR, "cases.json")))[name]
    base = os.path.join(DRAW_DIR, name)
    g = read_csr(base + ".csr")
    with open(base + ".nxyz") as f:
        rows = np.array([[float(t) for t in line.split(",")] for line in f if line.strip()], dtype=np.float64)
    return g, rows[:, meta["first"] - 1].copy(), rows[:, meta["second"] - 1].copy(), meta, base + ".png"
