"""Host-side logic that needs no GPU: file formats, generators, and the C ABI library's exports."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden
from icpp_2020_parhde_gb300 import csr_io, graphs
from icpp_2020_parhde_gb300 import build as pbuild


def test_csr_roundtrip(tmp_path):
    g, _ = load_golden("grid12w")
    p = str(tmp_path / "g.csr")
    csr_io.write_csr(p, g)
    h = csr_io.read_csr(p, weighted=True)
    assert np.array_equal(h.offsets, g.offsets) and np.array_equal(h.adj, g.adj)
    assert np.array_equal(h.weights, g.weights)
    hdr = np.fromfile(p, dtype="<i8", count=6)
    assert list(hdr) == [g.n, g.nnz, 1, 0, 1, 0]  # mtx2csr.cpp:281-291
    with open(p, "r+b") as f:
        f.truncate(100)
    with pytest.raises(ValueError):
        csr_io.read_csr(p)


def test_nxyz_format_matches_ostream_default():
    # std::ostream default float format: %g, 6 significant digits (spectralDrawing.cpp:59-61)
    xy = np.array([[0.1234567, -1e-7], [12345678.0, 0.0], [-0.5, 1.0 / 3.0]])
    assert csr_io.format_nxyz(xy) == "0.123457,-1e-07\n1.23457e+07,0\n-0.5,0.333333\n"


def test_generators_sizes():
    g = graphs.mesh(125, 125, seed=1)
    assert g.n == 15625 and g.nnz == 2 * 46376
    g = graphs.grid3d(8, weighted=True, seed=2)
    assert g.n == 512 and g.nnz == 2 * 3 * 7 * 64
    assert g.weights.min() >= 1 and g.weights.max() <= 255
    # weights are symmetric
    deg = np.diff(g.offsets.astype(np.int64))
    src = np.repeat(np.arange(g.n), deg)
    w = {(int(a), int(b)): int(c) for a, b, c in zip(src, g.adj, g.weights)}
    assert all(w[(b, a)] == c for (a, b), c in w.items())
    g = graphs.rmat(10, seed=4)
    assert np.all(np.diff(g.offsets.astype(np.int64)) > 0)  # LCC: no isolated vertices
    for i in range(0, g.n, 97):
        row = g.adj[g.offsets[i]:g.offsets[i + 1]]
        assert np.all(np.diff(row.astype(np.int64)) > 0) and i not in row  # sorted, no dups, no self loops


def _declared_functions():
    decl = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            decl |= set(re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(phde_\w+)\s*\(", txt, re.M))
    return decl


def test_library_exports_every_declared_symbol():
    path = pbuild.build()
    lib = ctypes.CDLL(path)
    decl = _declared_functions()
    assert len(decl) >= 15
    missing = [f for f in sorted(decl) if not hasattr(lib, f)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    for f in decl:
        assert re.search(r"\bT %s$" % f, out, re.M), f


def test_ctypes_mirrors_match_the_c_abi(tmp_path):
    """Every ctypes structure of the Python binding has the size and field offsets of its C declaration in
    include/parhde.h (compiled here with the host compiler)."""
    from icpp_2020_parhde_gb300 import _lib
    structs = {"phde_layout_opts": _lib.LayoutOpts, "phde_layout_stats": _lib.LayoutStats,
               "phde_layout_extra": _lib.LayoutExtra, "phde_graph_desc": _lib.GraphDesc,
               "phde_csr_info": _lib.CsrInfo, "phde_draw_info": _lib.DrawInfo}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "parhde.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ["  return 0;", "}"]
    src = tmp_path / "abi.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "abi"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n"):
        if ln:
            a, b, v = ln.split()
            got[(a, b)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


@pytest.mark.parametrize("extra,algo", [(["--rmat-scale", "12"], "ParHDE"),
                                        (["--graph", "grid3d", "--grid-l", "20"], "wParHDE")])
def test_bench_reference_arm_contract(extra, algo):
    """`bench.py --impl reference` (the reference algorithm on the host cores) prints one JSON line with the
    contract's keys; the weighted configuration runs WParHDE."""
    import json
    r = subprocess.run(["python", os.path.join(ROOT, "bench.py"), "--impl", "reference", "--k", "8", "--c", "2",
                        "--steps", "1", "--warmup", "0"] + extra, capture_output=True, text=True, timeout=300,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["config"]["workload"].startswith(algo + " ")
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("port", "reference")


def test_status_strings_without_gpu():
    lib = ctypes.CDLL(pbuild.build())
    lib.phde_status_string.restype = ctypes.c_char_p
    assert lib.phde_status_string(0) == b"ok"
    assert b"connected" in lib.phde_status_string(-3)
    assert lib.phde_version() >= 10000


def test_status_codes_agree_with_oracle():
    txt = open(os.path.join(ROOT, "include", "parhde.h")).read()
    codes = dict(re.findall(r"#define PHDE_(ERR_\w+|OK)\s+\(?(-?\d+)\)?", txt))
    src = open(os.path.join(ROOT, "oracle", "parhde_oracle.c")).read()
    for name, val in re.findall(r"#define ORC_(ERR_\w+|OK)\s+\(?(-?\d+)\)?", src):
        key = {"ERR_K_RANGE": "ERR_K_RANGE"}.get(name, name)
        assert codes[key] == val, name


@pytest.mark.skipif(not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "embed")), reason="reference build absent")
def test_nxyz_writer_matches_reference_embed(tmp_path):
    """The reference's own embed binary writes the .nxyz; our formatter reproduces it byte for byte."""
    from oracle import oracle as orc
    g, rec = load_golden("mesh125")
    p = str(tmp_path / "mesh.csr")
    csr_io.write_csr(p, g)
    env = dict(os.environ, OMP_NUM_THREADS="1")
    subprocess.run([orc.REF_EMBED_PATH, p, "-a", "PivotMDS", "-r", "10", "-c", "2"], check=True, env=env,
                   stdout=subprocess.DEVNULL)
    ref_text = open(p + "_hde.nxyz").read()
    assert csr_io.format_nxyz(rec["PivotMDS_k10_c2_coords"]) == ref_text


def test_relabel_is_isomorphic():
    g = graphs.rmat(10, seed=3)
    perm = np.random.default_rng(1).permutation(g.n)
    h = graphs.relabel(g, perm)
    assert h.n == g.n and h.nnz == g.nnz
    deg_g = np.diff(g.offsets.astype(np.int64))
    deg_h = np.diff(h.offsets.astype(np.int64))
    assert np.array_equal(deg_h[perm], deg_g)
    for v in (0, 5, g.n - 1):
        nb = np.sort(perm[g.adj[g.offsets[v]:g.offsets[v + 1]].astype(np.int64)])
        assert np.array_equal(h.adj[h.offsets[perm[v]]:h.offsets[perm[v] + 1]].astype(np.int64), nb)


def test_fast_nxyz_writer_is_byte_identical(tmp_path):
    """phde_write_nxyz (parallel host formatter in the library) against the %g formatting of the
    reference's writeCoords, on values that exercise every %g branch."""
    from icpp_2020_parhde_gb300 import write_nxyz_fast
    rng = np.random.default_rng(3)
    n = 20000
    X = rng.standard_normal((n, 3)) * np.logspace(-12, 12, n)[:, None]
    X[:8, 0] = [0.0, -0.0, 1e-5, 1e-4, 123456.5, 1234567.0, 0.1 + 0.2, -9.999995e-7]
    X[:4, 1] = [np.inf, -np.inf, 1e300, -1e-300]
    for c, nth in ((2, 1), (3, 0), (3, 7)):
        p1, p2 = tmp_path / "a.nxyz", tmp_path / "b.nxyz"
        csr_io.write_nxyz(str(p1), X[:, :c])
        write_nxyz_fast(str(p2), X[:, :c], nthreads=nth)
        assert p1.read_bytes() == p2.read_bytes()


def test_png_writer_round_trip(tmp_path):
    """phde_write_png (host code of the library): palette images of 1, 2, 4 and 8 bits, and RGBA, decode to the
    same pixels."""
    import pngdecode
    from icpp_2020_parhde_gb300 import write_png
    rng = np.random.default_rng(7)
    for (H, W, ncol) in [(7, 5, 2), (40, 33, 4), (33, 257, 9), (64, 64, 200), (50, 70, 300), (1, 1, 1), (3, 1000, 17)]:
        cols = rng.integers(0, 256, (ncol, 4), dtype=np.uint8)
        idx = rng.integers(0, ncol, (H, W))
        idx[:, : W // 2] = 0  # long runs
        img = cols[idx]
        path = str(tmp_path / ("t%d_%d_%d.png" % (H, W, ncol)))
        write_png(path, img, nthreads=3)
        assert np.array_equal(pngdecode.read(path), img)
    # a larger image spread over many deflate ranges
    img = np.zeros((1500, 1200, 4), np.uint8)
    img[..., 3] = 255
    img[::7, :, 0] = 200
    img[:, ::13, 1] = 100
    path = str(tmp_path / "big.png")
    write_png(path, img, nthreads=8)
    assert np.array_equal(pngdecode.read(path), img)


def test_embed_driver_command_line_without_gpu(tmp_path):
    """lib/embed keeps the reference's command line (spectralDrawing.cpp:67-115): no argument prints the
    usage line, -h the option list, an unknown algorithm or strategy aborts with the reference's message,
    and a missing input file is reported before any device work."""
    pbuild.build()
    r = subprocess.run([pbuild.EMBED_PATH], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Usage:" in r.stderr
    r = subprocess.run([pbuild.EMBED_PATH, "x.csr", "-h"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "-r <value> : Number of pivots (default=10)" in r.stdout
    r = subprocess.run([pbuild.EMBED_PATH, "x.csr", "-a", "Spring"], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "Unrecognized algorithm" in r.stderr
    r = subprocess.run([pbuild.EMBED_PATH, "x.csr", "-p", "Median"], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "Unrecognized Strategy" in r.stderr
    r = subprocess.run([pbuild.EMBED_PATH, str(tmp_path / "missing.csr")], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 1 and "Could not open input file" in r.stdout


def test_mtx2csr_driver_command_line_without_gpu(tmp_path):
    """lib/mtx2csr keeps the reference converter's command line: a wrong argument count prints the usage line,
    an unreadable input is reported before any device work."""
    pbuild.build()
    exe = os.path.join(os.path.dirname(pbuild.EMBED_PATH), "mtx2csr")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Usage:" in r.stdout and "<MM filename> <binary CSR filename>" in r.stdout
    r = subprocess.run([exe, str(tmp_path / "missing.mtx"), str(tmp_path / "out.csr")], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1 and "could not open input file" in r.stdout
    assert not (tmp_path / "out.csr").exists()


def test_draw_driver_usage_without_gpu():
    """lib/draw keeps the reference's command line: a wrong argument count prints the usage line and fails."""
    pbuild.build()
    r = subprocess.run([pbuild.DRAW_PATH], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert "Usage:" in r.stderr and "<first coord> <second coord>" in r.stderr
