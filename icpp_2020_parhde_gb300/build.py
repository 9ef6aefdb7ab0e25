"""Build the GB300 layout library in-tree.

``libparhde_gb300.so``  every ``csrc/*.cu`` compiled for sm_103a (``-gencode arch=compute_103a,code=sm_103a``)
                        plus the library's host C++ (the reference-interface classes ``csrc/drawing.cpp``,
                        the parallel ``.nxyz`` writer ``csrc/nxyz.cpp``, the PNG writer ``csrc/png.cpp``),
                        C ABI in ``include/parhde.h``.
``embed``, ``mtx2csr``, ``draw``  the drop-in drivers (``csrc/embed.cpp``, ``csrc/mtx2csr.cpp``,
                        ``csrc/draw.cpp``), linked against the library.

Translation units are compiled in parallel and only when a source or header is newer than its object.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ_DIR = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libparhde_gb300.so")
EMBED_PATH = os.path.join(LIB_DIR, "embed")
MTX2CSR_PATH = os.path.join(LIB_DIR, "mtx2csr")
DRAW_PATH = os.path.join(LIB_DIR, "draw")
DRIVERS = ("embed.cpp", "mtx2csr.cpp", "draw.cpp")  # sources with a main(): built as executables, not into the library

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libparhde_gb300.so")


def _headers() -> list[str]:
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(
        os.path.join(INCLUDE, "*.h"))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    if r.stdout.strip() and os.environ.get("PHDE_BUILD_VERBOSE"):
        print(r.stdout)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    nv = nvcc()
    hdrs = _headers()
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    common = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]
    jobs = []
    objs = []
    for src in cu:
        obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            cmd = [nv] + ARCH + common + ["-c", src, "-o", obj]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    # host C++ of the library (the reference-interface classes, the .nxyz writer); embed.cpp is the driver
    for cpp in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        if os.path.basename(cpp) in DRIVERS:
            continue
        obj = os.path.join(OBJ_DIR, os.path.basename(cpp) + ".o")
        objs.append(obj)
        if force or _stale(obj, [cpp] + hdrs):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-pthread", "-I" + INCLUDE, "-c", cpp, "-o", obj])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB_PATH, objs):
        tmp = LIB_PATH + ".tmp"
        _run([nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"])
        os.replace(tmp, LIB_PATH)
    for drv in DRIVERS:  # command-line drop-ins, linked against the library
        src = os.path.join(CSRC, drv)
        exe = os.path.join(LIB_DIR, os.path.splitext(drv)[0])
        if os.path.exists(src) and (force or _stale(exe, [src, LIB_PATH] + hdrs)):
            _run(["g++", "-std=c++17", "-O2", "-pthread", "-I" + INCLUDE, src, "-o", exe, "-L" + LIB_DIR,
                  "-lparhde_gb300", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print("built", LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas-info" in sys.argv)
