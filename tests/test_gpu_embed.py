"""The drop-in `embed` driver (csrc/embed.cpp over the C++ class interface): same flags, same CSR input,
same .nxyz output as the reference driver (spectralDrawing.cpp:67-203)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import load_golden
from icpp_2020_parhde_gb300 import build as pbuild
from icpp_2020_parhde_gb300 import csr_io

pytestmark = pytest.mark.gpu


def _embed(args, cwd):
    pbuild.build()
    return subprocess.run([pbuild.EMBED_PATH] + args, cwd=cwd, capture_output=True, text=True, timeout=300)


def test_embed_pivotmds_output_is_byte_identical(tmp_path):
    g, rec = load_golden("mesh125")
    p = str(tmp_path / "mesh.csr")
    csr_io.write_csr(p, g)
    r = _embed([p, "-a", "PivotMDS", "-r", "10", "-c", "2"], str(tmp_path))
    assert r.returncode == 0, r.stderr
    assert "Total mean time" in r.stdout and "Writing coordinates to file" in r.stdout
    assert open(p + "_hde.nxyz").read() == csr_io.format_nxyz(rec["PivotMDS_k10_c2_coords"])


def test_embed_parhde_and_weighted(tmp_path):
    g, rec = load_golden("rmat13")
    p = str(tmp_path / "r.csr")
    csr_io.write_csr(p, g)
    r = _embed([p, "-r", "10", "-c", "3"], str(tmp_path))
    assert r.returncode == 0, r.stderr
    assert "HDE mean time" in r.stdout
    xy = csr_io.read_nxyz(p + "_hde.nxyz")
    np.testing.assert_allclose(xy, rec["ParHDE_k10_c3_coords"], rtol=1e-5, atol=1e-7)  # 6 significant digits
    gw, recw = load_golden("grid12w")
    pw = str(tmp_path / "w.csr")
    csr_io.write_csr(pw, gw)
    r = _embed([pw, "-w", "1", "-a", "wParHDE", "-r", "10"], str(tmp_path))
    assert r.returncode == 0, r.stderr
    np.testing.assert_allclose(csr_io.read_nxyz(pw + "_hde.nxyz"), recw["wParHDE_k10_c2_coords"], rtol=1e-5,
                               atol=1e-7)


def test_embed_errors(tmp_path):
    r = _embed([str(tmp_path / "missing.csr")], str(tmp_path))
    assert r.returncode == 1 and "Could not open input file" in r.stdout
    g, _ = load_golden("path20")
    p = str(tmp_path / "p.csr")
    csr_io.write_csr(p, g)
    r = _embed([p, "-a", "Nope"], str(tmp_path))
    assert r.returncode != 0 and "Unrecognized algorithm" in r.stderr
    r = _embed([p, "-p", "Nope"], str(tmp_path))
    assert r.returncode != 0 and "Unrecognized Strategy" in r.stderr
