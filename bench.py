"""Benchmark: ParHDE layout throughput on one GB300 (layout TEPS = k * nnz / time per graph).

Workload (one step = one full layout of one graph):
  ParHDE, Kcenters pivots, k = 50, c = 3, on a seeded synthetic R-MAT graph of scale 20, edgefactor 16,
  (a, b, c) = (0.57, 0.19, 0.19), symmetrised, self-loops and duplicates removed, largest connected
  component kept.  Distances exact (int32), dense stages FP64.

Reported:
  value      layout TEPS with the CSR resident in device memory, from the library's CUDA events on its
             stream (degrees, 3k Kcenters BFS passes, D-orthogonalisation, SpMM, Gram, eigensolve,
             coordinates, and the copy of the n x c coordinates to host memory); L2 flushed between steps.
  e2e        the same metric through the C ABI with pinned HOST buffers: phde_graph_upload (H2D) +
             phde_layout (coordinates D2H), host wall clock.
  roofline   the dominant kernel (the persistent Kcenters BFS): algorithmic bytes per launch / its
             event-timed duration, against the measured HBM copy bandwidth.
  cpu_baseline  the oracle port (OpenMP, all host threads) on the same graph.

N > 1 GPUs: replicas only -- every rank lays out its own copy of the graph; value = all ranks' graphs /
max-over-ranks time (weak scaling).  --impl reference times the reference algorithm on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "layout edges/sec (TEPS) and ms per graph, learned+batched vs plain, at stated error"
UNIT = "edges/s"
HBM_FALLBACK_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--rmat-scale", type=int, default=20)
    ap.add_argument("--k", type=int, default=50)
    ap.add_argument("--c", type=int, default=3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-reps", type=int, default=3)
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    return ap.parse_args()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_graph(args):
    from icpp_2020_parhde_gb300 import graphs
    t = time.time()
    g = graphs.rmat(args.rmat_scale, 16, 0.57, 0.19, 0.19, seed=args.seed)
    return g, time.time() - t


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, x: float) -> float:
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rayleigh_quotients(g, X):
    """x^T L x / x^T x per coordinate column (L = D - A)."""
    import scipy.sparse as sp
    n = g.n
    A = sp.csr_matrix((np.ones(g.nnz, dtype=np.float64), g.adj.astype(np.int64), g.offsets.astype(np.int64)),
                      shape=(n, n))
    d = np.asarray(A.sum(axis=1)).ravel()
    LX = d[:, None] * X - A @ X
    return np.einsum("ij,ij->j", X, LX) / np.einsum("ij,ij->j", X, X)


def cpu_baseline(g, args, reps):
    from oracle import oracle as orc
    ncores = os.cpu_count() or 1
    ts = []
    for _ in range(reps):
        L = orc.layout(g, "ParHDE", "Kcenters", args.k, args.c, nthreads=ncores, dist_algo="parallel", want_S=False)
        if L.status != 0:
            raise RuntimeError("oracle layout failed: %d" % L.status)
        ts.append(L.stats.t_total)
    t = float(np.median(ts))
    return {"value": args.k * g.nnz / t, "unit": UNIT, "cores": ncores, "kind": "port",
            "sample": "%d full ParHDE layouts (k=%d, c=%d) of the same graph, median %.3f s, OpenMP oracle port "
                      "(reference algorithm: DO-BFS Kcenters, CGS, SpMM, Gram, power iteration)" % (reps, args.k, args.c, t),
            "ms_per_graph": t * 1e3}


def run_reference(args):
    ws, rank, local = dist_init()
    if rank != 0:
        return
    g, _ = make_graph(args)
    from oracle import oracle as orc
    ncores = os.cpu_count() or 1
    for _ in range(args.warmup):
        orc.layout(g, "ParHDE", "Kcenters", args.k, args.c, nthreads=ncores, want_S=False)
    t0 = time.perf_counter()
    ts = []
    for _ in range(args.steps):
        L = orc.layout(g, "ParHDE", "Kcenters", args.k, args.c, nthreads=ncores, want_S=False)
        ts.append(L.stats.t_total)
    wall = time.perf_counter() - t0
    t = float(np.mean(ts))
    v = args.k * g.nnz / t
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "ParHDE Kcenters layout, R-MAT scale %d ef16 LCC (n=%d, nnz=%d), k=%d, c=%d"
                                   % (args.rmat_scale, g.n, g.nnz, args.k, args.c),
                       "n": g.n, "nnz": g.nnz, "k": args.k, "c": args.c},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": ncores, "kind": "port",
                             "sample": "%d full layouts after %d warm-up, OpenMP oracle port of the reference algorithm"
                                       % (args.steps, args.warmup)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line), flush=True)


def run_gb300(args):
    ws, rank, local = dist_init()
    import torch
    torch.cuda.set_device(local)
    from icpp_2020_parhde_gb300 import Context, _lib
    g, gen_s = make_graph(args)
    ctx = Context(local)
    n, nnz, k, c = g.n, g.nnz, args.k, args.c
    # pinned host copies of the inputs (e2e path) and of the output
    off_h = torch.from_numpy(g.offsets.astype(np.uint32)).pin_memory()
    adj_h = torch.from_numpy(g.adj.astype(np.uint32)).pin_memory()
    xy_h = torch.empty(n * c, dtype=torch.float64).pin_memory()
    from icpp_2020_parhde_gb300.csr_io import CSRGraph
    gp = CSRGraph(off_h.numpy(), adj_h.numpy(), None)
    ctx.upload(gp)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2

    def flush_l2():
        flush.fill_(1.0)
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        ctx.layout("ParHDE", "Kcenters", k, c, coords_out=xy_h.numpy())
    # ---- device-resident timed region ----
    flush_l2()
    barrier(ws)
    torch.cuda.synchronize()
    stats = []
    launches0 = ctx.launch_count
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush_l2()
            r = ctx.layout("ParHDE", "Kcenters", k, c, coords_out=xy_h.numpy())
            stats.append(r.stats)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    barrier(ws)
    launches = ctx.launch_count - launches0
    ms_steps = [s["ms_total"] for s in stats]
    ms_mean = float(np.mean(ms_steps))
    ms_max = allmax(ws, ms_mean)
    value = ws * k * nnz / (ms_max * 1e-3)
    # ---- end to end through the C ABI with host buffers ----
    e2e_t = []
    for i in range(args.steps):
        flush_l2()
        barrier(ws)
        t1 = time.perf_counter()
        ctx.upload(gp)
        r = ctx.layout("ParHDE", "Kcenters", k, c, coords_out=xy_h.numpy())
        e2e_t.append(time.perf_counter() - t1)
    e2e_s = allmax(ws, float(np.mean(e2e_t)))
    h2d = 4 * (n + 1) + 4 * nnz
    d2h = 8 * n * c + 8 * 3 * k
    # ---- roofline of the dominant kernel: the persistent Kcenters BFS (3k passes per launch) ----
    P = 3 * k
    bytes_per_pass = 8 * (n + 1) + 4 * nnz + 4 * n + 12 * n  # CSR read once, column write, Kcenters fold
    kern_ms = float(np.mean([s["ms_dist_kernel"] for s in stats]))
    achieved = P * bytes_per_pass / (kern_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    traffic = None
    tp = os.path.join(ROOT, "profiles", "kcenters_bfs_rmat20_traffic.json")
    if os.path.exists(tp):
        try:
            traffic = json.load(open(tp)).get("bytes_per_launch")
        except Exception:
            traffic = None
    mixed = None
    if not args.no_mixed:
        # mixed precision (FP32 basis / CGS2 / SpMM, FP64 k x k solve): same workload, stated error vs FP64
        xy64 = xy_h.numpy().reshape(c, n).T.copy()
        ms_mixed = []
        for _ in range(args.warmup):
            ctx.layout("ParHDE", "Kcenters", k, c, precision="mixed", coords_out=xy_h.numpy())
        for _ in range(args.steps):
            flush_l2()
            rm = ctx.layout("ParHDE", "Kcenters", k, c, precision="mixed", coords_out=xy_h.numpy())
            ms_mixed.append(rm.stats["ms_total"])
        xym = xy_h.numpy().reshape(c, n).T.copy()
        rq64, rqm = rayleigh_quotients(g, xy64), rayleigh_quotients(g, xym)
        msm = allmax(ws, float(np.mean(ms_mixed)))
        mixed = {"value": ws * k * nnz / (msm * 1e-3), "unit": UNIT, "ms_per_graph": msm, "dtype": "f32+f64",
                 "phases_ms": {kk: rm.stats[kk] for kk in ("ms_dist", "ms_orth", "ms_mmult", "ms_eig", "ms_coords")},
                 "rayleigh_fp64": rq64.tolist(), "rayleigh_mixed": rqm.tolist(),
                 "rayleigh_rel_err_max": float(np.max(np.abs(rqm - rq64) / np.abs(rq64))),
                 "eig_iters": rm.stats["eig_iters"], "naccepted": rm.stats["naccepted"]}
    learned = None
    if not args.no_learned:
        # learned pivots (one multi-source BFS instead of 3k serial passes), same workload and precision;
        # accepted when the layout's Rayleigh quotient (sum over coordinates of x'Lx / x'x) is within 2% of
        # the plain Kcenters layout's
        xy64 = None
        r64 = ctx.layout("ParHDE", "Kcenters", k, c, coords_out=xy_h.numpy())
        xy64 = xy_h.numpy().reshape(c, n).T.copy()
        for _ in range(args.warmup):
            ctx.layout("ParHDE", "Learned", k, c, coords_out=xy_h.numpy())
        ms_l = []
        for _ in range(args.steps):
            flush_l2()
            rl = ctx.layout("ParHDE", "Learned", k, c, coords_out=xy_h.numpy())
            ms_l.append(rl.stats["ms_total"])
        xyl = xy_h.numpy().reshape(c, n).T.copy()
        ms_lm = []
        for _ in range(args.steps):
            flush_l2()
            rlm = ctx.layout("ParHDE", "Learned", k, c, precision="mixed", coords_out=xy_h.numpy())
            ms_lm.append(rlm.stats["ms_total"])
        xylm = xy_h.numpy().reshape(c, n).T.copy()
        rq_p, rq_l, rq_lm = rayleigh_quotients(g, xy64), rayleigh_quotients(g, xyl), rayleigh_quotients(g, xylm)
        msl, mslm = allmax(ws, float(np.mean(ms_l))), allmax(ws, float(np.mean(ms_lm)))
        learned = {"value": ws * k * nnz / (msl * 1e-3), "unit": UNIT, "ms_per_graph": msl, "dtype": "f64",
                   "speedup_vs_plain": ms_max / msl,
                   "phases_ms": {kk: rl.stats[kk] for kk in ("ms_dist", "ms_orth", "ms_mmult", "ms_eig", "ms_coords")},
                   "rayleigh_plain": rq_p.tolist(), "rayleigh_learned": rq_l.tolist(),
                   "rayleigh_total_ratio": float(rq_l.sum() / rq_p.sum()),
                   "accepted_within_2pct": bool(rq_l.sum() <= 1.02 * rq_p.sum()),
                   "mixed": {"value": ws * k * nnz / (mslm * 1e-3), "ms_per_graph": mslm, "dtype": "f32+f64",
                             "speedup_vs_plain": ms_max / mslm, "rayleigh": rq_lm.tolist(),
                             "rayleigh_total_ratio": float(rq_lm.sum() / rq_p.sum()),
                             "accepted_within_2pct": bool(rq_lm.sum() <= 1.02 * rq_p.sum())}}
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "ParHDE Kcenters layout, R-MAT scale %d ef16 (a=.57,b=.19,c=.19) LCC, k=%d, c=%d, FP64"
                               % (args.rmat_scale, k, c),
                   "n": n, "nnz": nnz, "k": k, "c": c, "parallelism": "replicas%d" % ws if ws > 1 else "single",
                   "l2": "flushed between timed steps (256 MB write)", "graph_gen_s": round(gen_s, 1)},
        "ms_per_graph": ms_max,
        "phases_ms": {kk: float(np.mean([s[kk] for s in stats])) for kk in
                      ("ms_dist", "ms_orth", "ms_mmult", "ms_eig", "ms_coords", "ms_dist_kernel")},
        "wall_s_timed_region": wall,
        "e2e": {"value": ws * k * nnz / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_graph": e2e_s * 1e3},
        "gpu_launches": launches,
        "roofline": {"kernel": "kcenters_bfs_kernel", "bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
                     "algorithmic_bytes_per_launch": P * bytes_per_pass, "kernel_ms": kern_ms},
        "clocks": clk.summary(),
        "stats_last": stats[-1],
        "mixed_precision": mixed,
        "learned_pivots": learned,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(g, args, args.cpu_reps)
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
