"""Benchmark: ParHDE layout throughput on one GB300 (layout TEPS = k * nnz / time per graph).

Workload (one step = one full layout of one graph): ParHDE, k = 50, c = 3, on a seeded synthetic R-MAT graph
of scale 20, edgefactor 16, (a, b, c) = (0.57, 0.19, 0.19), symmetrised, self-loops and duplicates removed,
largest connected component kept (n = 646,362, nnz = 31,403,988 for seed 1).  --rmat-scale/--k/--c select
other sizes (scale 22 with k = 64 is the learned-pivot target size); --graph grid3d --k 20 --c 2 times the
weighted configuration (WParHDE with delta-stepping SSSP, FP64) on a 256^3 grid with weights in [1, 255].

Pipelines timed (each from the CSR resident in device memory to the n x c coordinates in host memory, by the
library's CUDA events on its stream; L2 flushed between steps):
  learned_mixed        the headline: learned pivots (Kcenters warm start, MLP-scored candidates, one
                       multi-source BFS, farthest-point order), FP32 n-sized stages with FP64 sums, blocked
                       CGS2, FP64 Jacobi for the k x k eigenproblem
  plain                the reference pipeline on the GPU: Kcenters (3k serial BFS passes), FP64, power iteration
  kcenters_mixed       control: Kcenters pivots, otherwise the headline's precision and eigensolver
  kcenters_fp64_exact  control: Kcenters pivots, FP64, Jacobi (the precision error is stated against it)

Reported:
  value       headline TEPS; if the learned pivots fail the acceptance test (mean summed Rayleigh quotient
              over the graph and relabelled copies more than 2% above Kcenters'), plain Kcenters is the
              fallback and its TEPS is the value
  e2e         the same metric through the C ABI with pinned HOST buffers: phde_graph_upload (H2D) +
              phde_layout (coordinates D2H), host wall clock
  roofline    the headline's dominant kernel (the 256-source bitset BFS sweep): algorithmic bytes per
              launch / its event-timed duration, against the measured HBM copy bandwidth; traffic from the
              committed ncu capture; roofline_plain does the same for the plain pipeline's Kcenters BFS
  cpu_baseline  the oracle port of the reference algorithm (OpenMP, all host threads) on the same graph
  batched     512 random geometric graphs laid out in one phde_layout_batched call, against one call each
  draw        the draw tool on the headline layout: Bresenham pixel writes per second of device time, the
              end-to-end path to a PNG file, and the one-thread oracle's rate on an R-MAT-16 sample

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
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--graph", default="rmat", choices=["rmat", "rgg3d", "grid3d"],
                    help="grid3d: the weighted configuration (WParHDE, delta-stepping SSSP, FP64) on an L^3 grid")
    ap.add_argument("--grid-l", type=int, default=256, help="side of the weighted 3-D grid")
    ap.add_argument("--rmat-scale", type=int, default=20)
    ap.add_argument("--rgg-n", type=int, default=8_000_000, help="vertices of the 3-D random geometric graph")
    ap.add_argument("--k", type=int, default=50)
    ap.add_argument("--c", type=int, default=3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-reps", type=int, default=3)
    ap.add_argument("--no-extra", action="store_true", help="skip the two Kcenters control pipelines")
    ap.add_argument("--no-accept", action="store_true", help="skip the learned-pivot acceptance check")
    ap.add_argument("--relabellings", type=int, default=4)
    ap.add_argument("--no-batched", action="store_true", help="skip the 512-graph batched layout measurement")
    ap.add_argument("--no-draw", action="store_true", help="skip the draw-tool measurement")
    ap.add_argument("--batch-count", type=int, default=512)
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


def profiled_traffic(name):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) recorded in profiles/<name>."""
    try:
        with open(os.path.join(ROOT, "profiles", name)) as f:
            for line in f:
                if line.startswith("dram_bytes_per_launch:"):
                    return int(line.split(":")[1])
    except OSError:
        pass
    return None


def make_graph(args):
    from icpp_2020_parhde_gb300 import graphs
    t = time.time()
    if args.graph == "rgg3d":
        g = graphs.rgg(args.rgg_n, dim=3, avg_degree=12, seed=args.seed)
    elif args.graph == "grid3d":
        g = graphs.grid3d(args.grid_l, seed=args.seed, weighted=True)
    else:
        g = graphs.rmat(args.rmat_scale, 16, 0.57, 0.19, 0.19, seed=args.seed)
    return g, time.time() - t


def graph_desc(args):
    if args.graph == "grid3d":
        return "a %d^3 6-neighbour grid with int32 weights uniform in [1, 255]" % args.grid_l
    if args.graph == "rgg3d":
        return "a 3-D random geometric graph (%d points in the unit cube, radius for mean degree 12, LCC)" % args.rgg_n
    return ("an R-MAT scale-%d graph (edgefactor 16, a=.57 b=.19 c=.19, symmetrised, LCC)" % args.rmat_scale)


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
    algo = "wParHDE" if args.graph == "grid3d" else "ParHDE"  # the weighted configuration runs WParHDE
    for _ in range(args.warmup):
        orc.layout(g, algo, "Kcenters", args.k, args.c, nthreads=ncores, want_S=False)
    t0 = time.perf_counter()
    ts = []
    for _ in range(args.steps):
        L = orc.layout(g, algo, "Kcenters", args.k, args.c, nthreads=ncores, want_S=False)
        ts.append(L.stats.t_total)
    wall = time.perf_counter() - t0
    t = float(np.mean(ts))
    v = args.k * g.nnz / t
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "%s Kcenters layout of %s (n=%d, nnz=%d), k=%d, c=%d"
                                   % (algo, graph_desc(args), g.n, g.nnz, args.k, args.c),
                       "n": g.n, "nnz": g.nnz, "k": args.k, "c": args.c},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": ncores, "kind": "port",
                             "sample": "%d full layouts after %d warm-up, OpenMP oracle port of the reference algorithm"
                                       % (args.steps, args.warmup)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line), flush=True)


PIPELINES = {
    # the GB300 pipeline: learned pivots (one multi-source BFS), FP32 n-sized stages with FP64 sums, blocked
    # CGS2, FP64 k x k Jacobi eigensolve
    "learned_mixed": dict(strategy="Learned", precision="mixed", eig="exact"),
    # the reference pipeline on the GPU: Kcenters (3k serial BFS passes), FP64 throughout, power iteration
    "plain": dict(strategy="Kcenters", precision="fp64", eig="power"),
    # isolates the pivot choice (same precision and eigensolver as the headline)
    "kcenters_mixed": dict(strategy="Kcenters", precision="mixed", eig="exact"),
    # isolates the precision (same pivots and eigensolver as kcenters_mixed)
    "kcenters_fp64_exact": dict(strategy="Kcenters", precision="fp64", eig="exact"),
}
PHASES = ("ms_dist", "ms_orth", "ms_mmult", "ms_eig", "ms_coords", "ms_total")


def run_gb300(args):
    ws, rank, local = dist_init()
    import torch
    torch.cuda.set_device(local)
    from icpp_2020_parhde_gb300 import Context, graphs
    from icpp_2020_parhde_gb300.csr_io import CSRGraph
    g, gen_s = make_graph(args)
    ctx = Context(local)
    n, nnz, k, c = g.n, g.nnz, args.k, args.c
    # pinned host copies of the inputs (e2e path) and of the output
    off_h = torch.from_numpy(g.offsets.astype(np.uint32)).pin_memory()
    adj_h = torch.from_numpy(g.adj.astype(np.uint32)).pin_memory()
    xy_h = torch.empty(n * c, dtype=torch.float64).pin_memory()
    gp = CSRGraph(off_h.numpy(), adj_h.numpy(), None)
    ctx.upload(gp)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2

    def flush_l2():
        flush.fill_(1.0)
        torch.cuda.synchronize()

    def run(name):
        return ctx.layout("ParHDE", k=k, c=c, coords_out=xy_h.numpy(), **PIPELINES[name])

    def coords():
        return xy_h.numpy().reshape(c, n).T.copy()

    def timed(name, steps, sampler=None):
        for _ in range(args.warmup):
            run(name)
        flush_l2()
        barrier(ws)
        torch.cuda.synchronize()
        stats = []
        l0 = ctx.launch_count
        t0 = time.perf_counter()
        for _ in range(steps):
            flush_l2()
            stats.append(run(name).stats)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        barrier(ws)
        ms = allmax(ws, float(np.mean([s["ms_total"] for s in stats])))
        return {"ms": ms, "stats": stats, "launches": ctx.launch_count - l0, "wall": wall,
                "phases_ms": {p: float(np.mean([s[p] for s in stats])) for p in PHASES}}

    # ---- headline: device-resident timed region; clocks sampled over every timed region below ----
    clk = ClockSampler(local).__enter__()
    head = timed("learned_mixed", args.steps)
    xy_head = coords()
    # ---- end to end through the C ABI: pinned host CSR -> phde_graph_upload -> phde_layout -> host coords ----
    e2e_t = []
    for _ in range(args.steps):
        flush_l2()
        barrier(ws)
        t1 = time.perf_counter()
        ctx.upload(gp)
        run("learned_mixed")
        e2e_t.append(time.perf_counter() - t1)
    e2e_s = allmax(ws, float(np.mean(e2e_t)))
    h2d = 4 * (n + 1) + 4 * nnz
    d2h = 8 * n * c + 8 * 3 * k
    # ---- the reference pipeline on the GPU, and the two controls ----
    plain = timed("plain", args.steps)
    rq_plain = rayleigh_quotients(g, coords())
    ctl = {}
    if not args.no_extra:
        for name in ("kcenters_mixed", "kcenters_fp64_exact"):
            ctl[name] = timed(name, max(1, args.steps // 2))
            ctl[name]["rq"] = rayleigh_quotients(g, coords())
    clk.__exit__(None, None, None)
    rq_head = rayleigh_quotients(g, xy_head)
    # ---- acceptance of the learned pivots: summed Rayleigh quotient vs Kcenters (same precision and
    #      eigensolver), averaged over the graph and relabelled copies (Kcenters starts at vertex 0 and breaks
    #      ties by the lowest index; its own quotient moves by tens of percent between relabellings) ----
    acc = {"relabellings": [], "criterion": "mean summed RQ(learned) <= 1.02 * mean summed RQ(Kcenters)"}
    if not args.no_accept:
        rng = np.random.default_rng(11)
        tot_l, tot_k = [], []
        for t in range(args.relabellings):
            gg = g if t == 0 else graphs.relabel(g, rng.permutation(n))
            ctx.upload(gg)
            ctx.layout("ParHDE", k=k, c=c, coords_out=xy_h.numpy(), **PIPELINES["learned_mixed"])
            ql = rayleigh_quotients(gg, coords())
            ctx.layout("ParHDE", k=k, c=c, coords_out=xy_h.numpy(), **PIPELINES["kcenters_mixed"])
            qk = rayleigh_quotients(gg, coords())
            tot_l.append(float(ql.sum()))
            tot_k.append(float(qk.sum()))
            acc["relabellings"].append({"learned": ql.tolist(), "kcenters": qk.tolist()})
        acc["ratio_of_means"] = float(np.mean(tot_l) / np.mean(tot_k))
        acc["accepted"] = bool(acc["ratio_of_means"] <= 1.02)
        ctx.upload(gp)
    else:
        acc["accepted"] = None
    # learned pivots rejected -> plain Kcenters is the fallback, and the headline is its number
    fallback = acc["accepted"] is False
    hl = plain if fallback else head
    value = ws * k * nnz / (hl["ms"] * 1e-3)
    # ---- roofline of the headline's dominant kernel: the multi-source BFS sweep ----
    peak, peak_kind = peaks()
    roof = None
    last = head["stats"][-1]
    if not fallback and last.get("ms_msbfs_kernel", 0) > 0:
        lv = last["msbfs_levels"]
        per_level = 8 * (n + 1) + 4 * nnz + 2 * n * 32  # offsets + adjacency + frontier words in and out
        bytes_launch = lv * per_level
        kern_ms = float(np.mean([s["ms_msbfs_kernel"] for s in head["stats"]]))
        achieved = bytes_launch / (kern_ms * 1e-3) / 1e9
        traffic = profiled_traffic("msbfs_kernel_rmat20.md") if (args.graph, args.rmat_scale, k) == ("rmat", 20, 50) else None
        roof = {"kernel": "msbfs_kernel<4>", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "peak_source": ("measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback"),
                "algorithmic_bytes_per_launch": bytes_launch, "levels": lv, "kernel_ms": kern_ms}
    # the plain pipeline's dominant kernel: the persistent Kcenters BFS (3k passes in one launch)
    lp = plain["stats"][-1]
    P = 3 * k
    kc_bytes = P * (8 * (n + 1) + 4 * nnz + 4 * n + 12 * n)  # per pass: CSR once, column write, selection fold
    kc_ms = float(np.mean([s["ms_dist_kernel"] for s in plain["stats"]]))
    kc_ach = kc_bytes / (kc_ms * 1e-3) / 1e9
    roof_plain = {"kernel": "kcenters_bfs_kernel", "bound": "hbm", "achieved": kc_ach, "peak": peak, "unit": "GB/s",
                  "frac": kc_ach / peak, "traffic": None, "algorithmic_bytes_per_launch": kc_bytes,
                  "kernel_ms": kc_ms, "passes": lp["npasses"],
                  "note": "direction-optimising passes read far less than the whole CSR; bytes counted as if each "
                          "pass read it once"}
    if rank != 0:
        return

    def summary(t, rq=None, ref_ms=None):
        d = {"value": ws * k * nnz / (t["ms"] * 1e-3), "unit": UNIT, "ms_per_graph": t["ms"],
             "phases_ms": t["phases_ms"], "gpu_launches_per_step": t["launches"] / max(1, len(t["stats"]))}
        if rq is not None:
            d["rayleigh"] = [float(x) for x in rq]
        if ref_ms is not None:
            d["speedup_vs_plain"] = ref_ms / t["ms"]
        return d

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": hl["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32 distances, f32 n-sized stages with f64 sums, f64 k x k" if not fallback else "f64",
        "data": "synthetic",
        "config": {"workload": "ParHDE layout of %s, k=%d pivots, %d coordinates" % (graph_desc(args), k, c),
                   "pipeline": "plain Kcenters fallback" if fallback else "learned pivots + mixed precision + exact eigensolve",
                   "n": n, "nnz": nnz, "k": k, "c": c, "parallelism": "replicas%d" % ws if ws > 1 else "single",
                   "l2": "flushed between timed steps (256 MB write)", "graph_gen_s": round(gen_s, 1)},
        "ms_per_graph": hl["ms"],
        "phases_ms": hl["phases_ms"],
        "speedup_vs_plain": plain["ms"] / hl["ms"],
        "e2e": {"value": ws * k * nnz / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_graph": e2e_s * 1e3, "path": "phde_graph_upload + phde_layout, pinned host buffers"},
        "gpu_launches": hl["launches"],
        "roofline": roof,
        "roofline_plain": roof_plain,
        "clocks": clk.summary(),
        "headline_stats_last": hl["stats"][-1],
        "learned_acceptance": acc,
        "pipelines": {
            "learned_mixed": summary(head, rq_head, plain["ms"]),
            "plain": summary(plain, rq_plain),
            **{kk: summary(v, v["rq"], plain["ms"]) for kk, v in ctl.items()},
        },
    }
    if "kcenters_mixed" in ctl and "kcenters_fp64_exact" in ctl:
        a, b = ctl["kcenters_mixed"]["rq"], ctl["kcenters_fp64_exact"]["rq"]
        line["mixed_precision_error"] = {"rayleigh_rel_err_max": float(np.max(np.abs(a - b) / np.abs(b))),
                                         "vs": "Kcenters FP64 with the same pivots and eigensolver"}
    if not args.no_batched:
        line["batched"] = run_batched(args, local, flush_l2)
    if not args.no_draw:
        line["draw"] = run_draw(args, ctx, gp, xy_head, flush_l2)
        ctx.upload(gp)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(g, args, args.cpu_reps)
    print(json.dumps(line), flush=True)
    ctx.close()


def run_draw(args, ctx, g, xy, flush_l2):
    """The draw tool on the headline layout: its first two coordinates rasterised (phde_draw: bounds, scaling,
    Bresenham lines of every CSR entry, colour counters, palette scanlines).  value = Bresenham pixel writes per
    second of device time; e2e = host coordinates -> PNG file through the C ABI (phde_draw + phde_draw_write_png,
    deflate on the host threads).  The CPU baseline is the one-thread oracle (the reference's serial order) on a
    bounded sample: an R-MAT scale-16 layout from the same pipeline."""
    import tempfile
    from icpp_2020_parhde_gb300 import graphs
    x, y = np.ascontiguousarray(xy[:, 0]), np.ascontiguousarray(xy[:, 1])
    ctx.upload(g)
    for _ in range(args.warmup):
        info = ctx.draw(x, y)
    dev, ras = [], []
    steps = max(3, args.steps // 6)
    for _ in range(steps):
        flush_l2()
        info = ctx.draw(x, y)
        dev.append(info["ms_device"])
        ras.append(info["ms_raster"])
    path = os.path.join(tempfile.mkdtemp(), "draw.png")
    e2e = []
    for _ in range(steps):
        flush_l2()
        t1 = time.perf_counter()
        ctx.draw(x, y)
        ctx.draw_png(path, 0)
        e2e.append(time.perf_counter() - t1)
    png_bytes = os.path.getsize(path)
    px = info["pixels"]
    out = {"workload": "draw of the headline layout (coordinates 1 and 2) of %s: %d x %d image, %d CSR entries"
                       % (graph_desc(args), info["width"], info["height"], g.nnz),
           "value": px / (np.mean(dev) * 1e-3), "unit": "pixel writes/s", "pixels_per_step": px,
           "ms_device": float(np.mean(dev)), "ms_raster": float(np.mean(ras)),
           "e2e": {"value": px / float(np.mean(e2e)), "unit": "pixel writes/s", "ms": float(np.mean(e2e)) * 1e3,
                   "path": "phde_draw + phde_draw_write_png (host coordinates to PNG file)",
                   "h2d_bytes_per_step": 16 * g.n, "png_bytes": png_bytes},
           "gpu_launches": info["gpu_launches"]}
    if not args.no_cpu_baseline:
        from oracle import oracle as orc
        gs = graphs.rmat(16, 16, seed=args.seed)
        ctx.upload(gs)
        xs = ctx.layout("ParHDE", k=args.k, c=2, **PIPELINES["learned_mixed"]).coords
        sx, sy = np.ascontiguousarray(xs[:, 0]), np.ascontiguousarray(xs[:, 1])
        info_s = ctx.draw(sx, sy)
        t1 = time.perf_counter()
        ref, _ = orc.draw(gs, sx, sy)
        t_cpu = time.perf_counter() - t1
        same = bool(np.array_equal(ref, ctx.draw_image()))
        out["cpu_baseline"] = {"value": info_s["pixels"] / t_cpu, "unit": "pixel writes/s", "cores": 1, "kind": "port",
                               "sample": "R-MAT scale 16 layout (n = %d, %d entries, %d pixel writes) drawn by the "
                                         "one-thread oracle in %.2f s; identical image on the GPU: %s"
                                         % (gs.n, gs.nnz, info_s["pixels"], t_cpu, same)}
    return out


def run_batched(args, local, flush_l2):
    """Many graphs in one call: --batch-count random geometric 2-D graphs (n log-uniform in 1k..200k, mean
    degree 8, LCC), k = 10, c = 2, laid out by phde_layout_batched, against the same graphs laid out one call
    each (Kcenters + mixed + Jacobi, and the plain FP64 pipeline).  All device-event times, CSR resident."""
    import torch
    from icpp_2020_parhde_gb300 import Context, graphs
    k, c = 10, 2
    t = time.time()
    gs = graphs.rgg_batch(args.batch_count, seed=args.seed)
    gen_s = time.time() - t
    ntot, nnz_tot = sum(g.n for g in gs), sum(g.nnz for g in gs)
    cb = Context(local)
    cb.upload_batch(gs)
    out = torch.empty(ntot * c, dtype=torch.float64).pin_memory()
    _, st0 = cb.layout_batched(k, c, coords_out=out.numpy())  # first call: autotune + capture
    for _ in range(args.warmup):
        cb.layout_batched(k, c, coords_out=out.numpy())
    ms = []
    steps = max(3, args.steps // 10)
    for _ in range(steps):
        flush_l2()
        _, st = cb.layout_batched(k, c, coords_out=out.numpy())
        ms.append(st["ms_total"])
    xs = [x.copy() for x in cb.layout_batched(k, c, coords_out=out.numpy())[0]]
    t_b = float(np.mean(ms))
    # end to end: the batch's host CSR arrays uploaded and laid out
    e2e = []
    for _ in range(steps):
        t1 = time.perf_counter()
        cb.upload_batch(gs)
        cb.layout_batched(k, c, coords_out=out.numpy())
        e2e.append(time.perf_counter() - t1)
    cb.close()
    # one call per graph
    cs = Context(local)
    loop = {"kcenters_mixed": 0.0, "plain": 0.0}
    rq_err = []
    for i, g in enumerate(gs):
        cs.upload(g)
        for name in loop:
            r = cs.layout("ParHDE", k=k, c=c, **PIPELINES[name])
            loop[name] += r.stats["ms_total"]
            if name == "kcenters_mixed" and i % 64 == 0:
                a, b = rayleigh_quotients(g, xs[i]), rayleigh_quotients(g, r.coords)
                rq_err.append(float(np.max(np.abs(a - b) / np.abs(b))))
    cs.close()
    return {"workload": "%d random geometric 2-D graphs, n log-uniform in [1000, 200000], mean degree 8, LCC "
                        "(sum n = %d, sum nnz = %d), ParHDE k=%d, c=%d, Kcenters, mixed precision, Jacobi"
                        % (len(gs), ntot, nnz_tot, k, c),
            "value": k * nnz_tot / (t_b * 1e-3), "unit": UNIT, "ms_per_batch": t_b, "ms_per_graph": t_b / len(gs),
            "e2e_ms_per_batch": float(np.mean(e2e)) * 1e3,
            "loop_ms_per_batch": {kk: v for kk, v in loop.items()},
            "speedup_vs_loop": {kk: v / t_b for kk, v in loop.items()},
            "cuda_graph_replay": bool(st["batch_graph_replay"]), "autotuned_segment_rows": st["batch_seg_rows"],
            "autotune_first_call_ms": st0["ms_batch_tune"], "gpu_launches_per_batch": st["gpu_launches"],
            "rayleigh_rel_err_vs_single_max": max(rq_err) if rq_err else None, "graph_gen_s": round(gen_s, 1)}


def run_weighted(args):
    """The weighted configuration: WParHDE (Kcenters pivots by delta-stepping SSSP, coupled MGS, FP64 as the
    reference) with k pivots and c coordinates on a weighted 3-D grid; same timing rules as the headline."""
    ws, rank, local = dist_init()
    import torch
    torch.cuda.set_device(local)
    from icpp_2020_parhde_gb300 import Context, graphs
    from icpp_2020_parhde_gb300.csr_io import CSRGraph
    g, gen_s = make_graph(args)
    ctx = Context(local)
    n, nnz, k, c = g.n, g.nnz, args.k, args.c
    # pinned host copies of the inputs (end-to-end path) and of the output
    off_h = torch.from_numpy(g.offsets.astype(np.uint32)).pin_memory()
    adj_h = torch.from_numpy(g.adj.astype(np.uint32)).pin_memory()
    w_h = torch.from_numpy(g.weights.astype(np.int32)).pin_memory()
    gp = CSRGraph(off_h.numpy(), adj_h.numpy(), w_h.numpy())
    ctx.upload(gp)
    xy_h = torch.empty(n * c, dtype=torch.float64).pin_memory()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def run():
        return ctx.layout("wParHDE", "Kcenters", k=k, c=c, precision="fp64", eig="power", coords_out=xy_h.numpy())

    for _ in range(args.warmup):
        run()
    clk = ClockSampler(local).__enter__()
    barrier(ws)
    torch.cuda.synchronize()
    stats = []
    l0 = ctx.launch_count
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        stats.append(run().stats)
    torch.cuda.synchronize()
    barrier(ws)
    ms = allmax(ws, float(np.mean([st["ms_total"] for st in stats])))
    launches = ctx.launch_count - l0
    e2e_t = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        ctx.upload(gp)
        run()
        e2e_t.append(time.perf_counter() - t1)
    clk.__exit__(None, None, None)
    e2e_s = allmax(ws, float(np.mean(e2e_t)))
    if rank != 0:
        return
    line = {"metric": METRIC, "value": ws * k * nnz / (ms * 1e-3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32 distances, f64", "data": "synthetic",
            "config": {"workload": "WParHDE layout of %s, k=%d pivots, %d coordinates" % (graph_desc(args), k, c),
                       "n": n, "nnz": nnz, "k": k, "c": c, "l2": "flushed between timed steps (256 MB write)",
                       "graph_gen_s": round(gen_s, 1)},
            "phases_ms": {p: float(np.mean([st[p] for st in stats])) for p in PHASES},
            "e2e": {"value": ws * k * nnz / e2e_s, "unit": UNIT, "ms_per_graph": e2e_s * 1e3,
                    "h2d_bytes_per_step": 4 * (n + 1) + 8 * nnz, "d2h_bytes_per_step": 8 * n * c,
                    "timing": "mean of %d host-timed calls: upload from pinned host CSR + layout + coordinates to "
                              "pinned host memory" % len(e2e_t), "ms_each": [round(x * 1e3, 1) for x in e2e_t]},
            "gpu_launches": launches, "clocks": clk.summary(),
            "sssp": {"grid_rounds_per_layout": float(np.mean([st["sssp_rounds"] for st in stats])),
                     "edges_relaxed_per_layout": float(np.mean([st["edges_examined"] for st in stats])),
                     "passes_per_layout": float(np.mean([st["npasses"] for st in stats]))}}
    if not args.no_cpu_baseline:
        from oracle import oracle as orc
        gs = graphs.grid3d(64, seed=args.seed, weighted=True)
        t1 = time.perf_counter()
        orc.layout(gs, "wParHDE", "Kcenters", k, c, nthreads=os.cpu_count() or 1, want_S=False)
        t_cpu = time.perf_counter() - t1
        line["cpu_baseline"] = {"value": k * gs.nnz / t_cpu, "unit": UNIT, "cores": os.cpu_count() or 1,
                                "kind": "port", "sample": "one layout of a 64^3 weighted grid (nnz = %d) in %.2f s"
                                                          % (gs.nnz, t_cpu)}
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.graph == "grid3d":
        run_weighted(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
