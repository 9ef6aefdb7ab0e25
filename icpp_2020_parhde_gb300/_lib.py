"""ctypes binding of ``libparhde_gb300.so`` (C ABI declared in ``include/parhde.h``).

There is no fallback: if the shared library is missing or CUDA is unavailable, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

PHDE_OK = 0
STATUS = {
    0: "PHDE_OK", -1: "PHDE_ERR_INVALID", -2: "PHDE_ERR_CSR", -3: "PHDE_ERR_DISCONNECTED", -4: "PHDE_ERR_K_RANGE",
    -5: "PHDE_ERR_TOO_FEW_PIVOTS", -6: "PHDE_ERR_OOM", -7: "PHDE_ERR_NOCONVERGE", -8: "PHDE_ERR_TIMEOUT",
    -9: "PHDE_ERR_CUDA", -10: "PHDE_ERR_WEIGHTS", -11: "PHDE_ERR_NO_GRAPH", -12: "PHDE_ERR_TOO_LARGE",
}
NOALLOC_MAX_VERTICES = 1048576
ALGOS = {"PivotMDS": 0, "PHDE": 1, "wParHDE": 2, "WParHDE": 2, "ParHDE": 3}
STRATEGIES = {"RandCoarse": 0, "RandFine": 1, "Kcenters": 2, "Learned": 3, "LearnedChecked": 4}
OUTCOMES = {0: "reference strategy", 1: "learned", 2: "rejected: Kcenters", 3: "failed: Kcenters"}
PRECISIONS = {"fp64": 0, "mixed": 1, "exact": 2}
EIGS = {"power": 0, "exact": 1}

# every symbol include/parhde.h declares
EXPORTS = [
    "phde_create", "phde_destroy", "phde_last_error", "phde_status_string", "phde_version", "phde_graph_upload",
    "phde_graph_n", "phde_graph_nnz", "phde_layout", "phde_distances", "phde_kcenters", "phde_DOBFS",
    "phde_DeltaStep", "phde_selftest_barrier_timeout", "phde_launch_count", "phde_bfs_noalloc",
    "phde_set_pivot_model", "phde_batch_upload", "phde_layout_batched", "phde_write_nxyz",
    "phde_graph_from_entries", "phde_graph_download", "phde_draw", "phde_draw_download", "phde_draw_write_png",
    "phde_write_png", "phde_gram_f32", "phde_set_pivot_check", "phde_pivot_scores", "phde_batch_rayleigh",
    "phde_symeig",
]


class LayoutOpts(C.Structure):
    _fields_ = [("algo", C.c_int), ("strategy", C.c_int), ("k", C.c_int), ("c", C.c_int), ("precision", C.c_int),
                ("eig", C.c_int), ("seed", C.c_uint64), ("verbose", C.c_int)]


class CsrInfo(C.Structure):
    _fields_ = [("n_in", C.c_int64), ("nnz_dedup", C.c_int64), ("ncomponents", C.c_int64), ("n", C.c_int64),
                ("nnz", C.c_int64)]


class GraphDesc(C.Structure):
    _fields_ = [("offsets", C.c_void_p), ("offset_bytes", C.c_int), ("adj", C.c_void_p), ("n", C.c_int64),
                ("nnz", C.c_int64)]


class LayoutStats(C.Structure):
    _fields_ = [("status", C.c_int), ("npasses", C.c_int), ("naccepted", C.c_int), ("ndiscarded", C.c_int),
                ("eig_iters", C.c_int), ("gpu_launches", C.c_int), ("ms_dist", C.c_double), ("ms_orth", C.c_double),
                ("ms_mmult", C.c_double), ("ms_eig", C.c_double), ("ms_coords", C.c_double),
                ("ms_total", C.c_double), ("edges_examined", C.c_int64), ("ms_dist_kernel", C.c_double),
                ("dist_kernel_launches", C.c_int), ("ms_msbfs_kernel", C.c_double), ("msbfs_levels", C.c_int),
                ("batch_graph_replay", C.c_int), ("batch_seg_rows", C.c_int), ("ms_batch_tune", C.c_double),
                ("sssp_rounds", C.c_int64), ("pivot_outcome", C.c_int), ("rayleigh", C.c_double * 8),
                ("rayleigh_kcenters", C.c_double * 8), ("ms_check", C.c_double), ("ms_lap_kernel", C.c_double)]

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_}
        for f in ("rayleigh", "rayleigh_kcenters"):
            d[f] = list(d[f])
        return d


class DrawInfo(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("width_computed", C.c_uint32),
                ("height_computed", C.c_uint32), ("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double),
                ("ymax", C.c_double), ("aspect", C.c_double), ("max_edge_length", C.c_float),
                ("gpu_launches", C.c_int), ("pixels", C.c_int64), ("ms_device", C.c_double),
                ("ms_raster", C.c_double), ("ms_total", C.c_double)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class LayoutExtra(C.Structure):
    _fields_ = [("basis", C.POINTER(C.c_double)), ("gram", C.POINTER(C.c_double)), ("evecs", C.POINTER(C.c_double)),
                ("evals", C.POINTER(C.c_double))]


_lib = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(path: str | None = None):
    """Load the library (building it first if it is missing and nvcc is present)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or lib_path()
    if not os.path.exists(path):
        _build.build()
    L = C.CDLL(path)
    vp, i64, u32p, i32p, f64p, i64p = C.c_void_p, C.c_int64, C.POINTER(C.c_uint32), C.POINTER(C.c_int32), \
        C.POINTER(C.c_double), C.POINTER(C.c_int64)
    L.phde_create.argtypes = [C.POINTER(vp), C.c_int]
    L.phde_destroy.argtypes = [vp]
    L.phde_destroy.restype = None
    L.phde_last_error.argtypes = [vp]
    L.phde_last_error.restype = C.c_char_p
    L.phde_status_string.argtypes = [C.c_int]
    L.phde_status_string.restype = C.c_char_p
    L.phde_graph_upload.argtypes = [vp, vp, C.c_int, u32p, i32p, i64, i64]
    L.phde_graph_n.argtypes = [vp]
    L.phde_graph_n.restype = i64
    L.phde_graph_nnz.argtypes = [vp]
    L.phde_graph_nnz.restype = i64
    L.phde_layout.argtypes = [vp, C.POINTER(LayoutOpts), f64p, i64p, C.POINTER(LayoutExtra), C.POINTER(LayoutStats)]
    L.phde_distances.argtypes = [vp, i64p, C.c_int, i32p]
    L.phde_kcenters.argtypes = [vp, C.c_int, C.c_int, i32p, i64p]
    L.phde_DOBFS.argtypes = [u32p, u32p, C.c_long, C.c_long, C.c_long, f64p, C.c_int, C.c_int]
    L.phde_DeltaStep.argtypes = [u32p, u32p, i32p, C.c_long, C.c_long, C.c_long, f64p, C.c_int32]
    L.phde_selftest_barrier_timeout.argtypes = [vp, C.c_int]
    L.phde_launch_count.argtypes = [vp]
    L.phde_launch_count.restype = i64
    L.phde_bfs_noalloc.argtypes = [vp, vp, i64, i64, i64, vp, vp]
    L.phde_set_pivot_model.argtypes = [vp, C.POINTER(C.c_float), C.c_int]
    L.phde_set_pivot_check.argtypes = [vp, C.c_int, C.c_double]
    L.phde_pivot_scores.argtypes = [vp, C.POINTER(C.c_float), i32p, i64p, C.c_int]
    L.phde_batch_upload.argtypes = [vp, C.POINTER(GraphDesc), C.c_int]
    L.phde_layout_batched.argtypes = [vp, C.POINTER(LayoutOpts), f64p, C.POINTER(LayoutStats)]
    L.phde_batch_rayleigh.argtypes = [vp, f64p]
    L.phde_write_nxyz.argtypes = [C.c_char_p, f64p, i64, C.c_int, C.c_int]
    L.phde_graph_from_entries.argtypes = [vp, u32p, u32p, i32p, i64, i64, i64, C.c_int, C.POINTER(CsrInfo)]
    L.phde_graph_download.argtypes = [vp, u32p, u32p, i32p]
    f32p = C.POINTER(C.c_float)
    L.phde_gram_f32.argtypes = [vp, f32p, C.c_int, C.c_int, f32p, C.c_int, C.c_int, f64p, i64, C.c_int, f64p]
    L.phde_symeig.argtypes = [vp, f64p, C.c_int, C.c_int, C.c_int, f64p, f64p, C.POINTER(C.c_int)]
    L.phde_draw.argtypes = [vp, f64p, f64p, C.POINTER(DrawInfo)]
    L.phde_draw_download.argtypes = [vp, C.POINTER(C.c_uint8), C.c_size_t]
    L.phde_draw_write_png.argtypes = [vp, C.c_char_p, C.c_int]
    L.phde_write_png.argtypes = [C.c_char_p, C.POINTER(C.c_uint8), C.c_uint32, C.c_uint32, C.c_int]
    _lib = L
    return L
