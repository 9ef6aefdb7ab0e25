"""Benchmark: ParHDE layout throughput on one GB300 (layout TEPS = k * nnz / time per graph).

Headline workload (one step = one full layout of one graph): ParHDE with k = 64 pivots and c = 3 coordinates
on a seeded synthetic R-MAT graph of scale 22, edgefactor 16, (a, b, c) = (0.57, 0.19, 0.19), symmetrised,
self-loops and duplicates removed, largest connected component kept (n = 2,394,430, nnz = 128,305,124 for
seed 1) -- the learned-pivot configuration's R-MAT graph.  The reference publishes no numbers and no dataset
for it; the graph is generated, as its shape and sizes prescribe.

Pipelines (each timed from the CSR resident in device memory to the n x c coordinates in pinned host memory, by
the library's CUDA events on its stream; the 513 MB CSR is larger than L2 and L2 is flushed between steps too):
  learned_exact    the headline: learned pivots (Kcenters warm start, MLP-scored candidates, one multi-source
                   BFS, farthest-point order), then the reference's FP64 dense stages computed from exact
                   integer Gram matrices of the distance columns (no rounding in any n-sized sum; FP64
                   coefficient-space Gram-Schmidt and k x k products), Jacobi eigensolve
  plain            the reference pipeline on the GPU: Kcenters (3k serial BFS passes), FP64 vector kernels,
                   the reference's power iteration
  kcenters_exact   control: Kcenters pivots, otherwise the headline's stages (isolates the pivot proposal)
  learned_checked  the headline with its acceptance test in the same call (PHDE_STRAT_LEARNED_CHECKED: the
                   Kcenters layout too, the learned one returned only when its Rayleigh quotients pass)
  learned_mixed    the headline's pivots with FP32 n-sized stages (error stated against learned_exact)
Every pipeline has an end-to-end time: phde_graph_upload from pinned host CSR + phde_layout (coordinates to
pinned host memory), host wall clock.

Other configurations, as sub-keys (each with its own end-to-end time and a CPU baseline on the same graph):
  rmat20     R-MAT scale 20, k = 50, c = 3 (plain vs the exact and mixed-precision paths)
  rgg3d      3-D random geometric graph, 8M points, mean degree 12, k = 64, c = 3
  weighted   WParHDE (delta-stepping SSSP, coupled MGS, FP64) on a 256^3 grid, weights uniform in [1, 255],
             k = 20, c = 2
  batched    512 random geometric 2-D graphs laid out by one phde_layout_batched call, k = 10, c = 2
  draw       the draw tool on the headline layout (Bresenham pixel writes per second)

cpu_baseline: the oracle (a C/OpenMP restatement of the reference algorithm, pinned bit for bit to the
reference built from its own sources) on the host cores, on the same graph.  --impl reference times the same on
the headline's graph, k and c (the reference's own build needs its sources, which exist only where the
reference tree does).

N > 1 GPUs: replicas only -- every rank lays out its own copy of the graph; value = all ranks' graphs /
max-over-ranks time (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
import traceback

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "layout edges/sec (TEPS) and ms per graph, learned+batched vs plain, at stated error"
UNIT = "edges/s"
HBM_FALLBACK_GBS = 6800.0
SUBS = ("rmat20", "rgg3d", "weighted", "batched", "draw")


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--graph", default="rmat", choices=["rmat", "rgg3d", "grid3d"],
                    help="headline graph (default: the R-MAT graph of the learned-pivot configuration)")
    ap.add_argument("--rmat-scale", type=int, default=22)
    ap.add_argument("--rgg-n", type=int, default=8_000_000)
    ap.add_argument("--grid-l", type=int, default=256)
    ap.add_argument("--k", type=int, default=64)
    ap.add_argument("--c", type=int, default=3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-reps", type=int, default=1)
    ap.add_argument("--relabellings", type=int, default=2, help="graph copies for the averaged acceptance rule")
    ap.add_argument("--subs", default=",".join(SUBS), help="comma-separated sub-keys to measure ('' for none)")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--controls", default="plain,kcenters_exact,learned_checked,learned_mixed",
                    help="pipelines timed beside the headline ('' for none)")
    return ap.parse_args(argv)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed regions run."""

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
            self.t = threading.Thread(target=self._read, args=(self.proc,), daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self, proc):
        for line in proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=5)
            self.proc = None


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


# ---------------------------------------------------------------------------------------------- workloads

def rmat_desc(scale):
    return "an R-MAT scale-%d graph (edgefactor 16, a=.57 b=.19 c=.19, symmetrised, LCC)" % scale


def rgg3d_desc(n):
    return "a 3-D random geometric graph (%d points in the unit cube, radius for mean degree 12, LCC)" % n


def grid_desc(L):
    return "a %d^3 6-neighbour grid with int32 weights uniform in [1, 255]" % L


def make_graph(kind, args):
    from icpp_2020_parhde_gb300 import graphs
    t = time.time()
    if kind == "rgg3d":
        g = graphs.rgg(args.rgg_n, dim=3, avg_degree=12, seed=args.seed)
        desc = rgg3d_desc(args.rgg_n)
    elif kind == "grid3d":
        g = graphs.grid3d(args.grid_l, seed=args.seed, weighted=True)
        desc = grid_desc(args.grid_l)
    elif kind == "rmat20":
        g = graphs.rmat(20, 16, 0.57, 0.19, 0.19, seed=args.seed)
        desc = rmat_desc(20)
    else:
        g = graphs.rmat(args.rmat_scale, 16, 0.57, 0.19, 0.19, seed=args.seed)
        desc = rmat_desc(args.rmat_scale)
    return g, desc, time.time() - t


def workload_config(algo, desc, g, k, c):
    """The config dict both arms print for the same workload (the pipeline is named outside it)."""
    return {"workload": "%s layout of %s (n=%d, nnz=%d), k=%d pivots, %d coordinates" % (algo, desc, g.n, g.nnz, k, c),
            "algorithm": algo, "n": int(g.n), "nnz": int(g.nnz), "k": k, "c": c}


# ---------------------------------------------------------------------------------------------- multi-rank

def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
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


# ---------------------------------------------------------------------------------------------- helpers

def rayleigh_quotients(g, X):
    """x^T L x / x^T x per coordinate column (L = D - A, weighted when the graph is)."""
    import scipy.sparse as sp
    n = g.n
    w = np.ones(g.nnz) if g.weights is None else g.weights.astype(np.float64)
    A = sp.csr_matrix((w, g.adj.astype(np.int64), g.offsets.astype(np.int64)), shape=(n, n))
    d = np.asarray(A.sum(axis=1)).ravel()
    LX = d[:, None] * X - A @ X
    return np.einsum("ij,ij->j", X, LX) / np.einsum("ij,ij->j", X, X)


def cpu_layout(g, algo, k, c, reps, desc):
    """The oracle's reference algorithm (Kcenters, CGS / coupled MGS, SpMM, Gram, power iteration) on all host
    cores, `reps` full layouts of the graph: median time."""
    from oracle import oracle as orc
    ncores = os.cpu_count() or 1
    ts = []
    for _ in range(max(1, reps)):
        t0 = time.perf_counter()
        L = orc.layout(g, algo, "Kcenters", k, c, nthreads=ncores, want_S=False)
        ts.append(time.perf_counter() - t0)
        if L.status != 0:
            raise RuntimeError("oracle layout failed: %d" % L.status)
    t = float(np.median(ts))
    return {"value": k * g.nnz / t, "unit": UNIT, "cores": ncores, "kind": "port", "ms_per_graph": t * 1e3,
            "sample": "%d full %s layout(s) of %s (k=%d, c=%d), median %.2f s: the OpenMP oracle port of the "
                      "reference algorithm" % (len(ts), algo, desc, k, c, t)}


class Runner:
    """Timed layouts of one uploaded graph: device time (library events) and end to end (upload + layout)."""

    def __init__(self, ctx, g, gp, algo, k, c, xy, flush_l2, ws):
        self.ctx, self.g, self.gp, self.algo, self.k, self.c = ctx, g, gp, algo, k, c
        self.xy, self.flush_l2, self.ws = xy, flush_l2, ws

    def run(self, p):
        return self.ctx.layout(self.algo, k=self.k, c=self.c, coords_out=self.xy.numpy(), **p)

    def coords(self):
        return self.xy.numpy().reshape(self.c, self.g.n).T.copy()

    def timed(self, p, steps, warmup):
        import torch
        for _ in range(warmup):
            self.run(p)
        self.flush_l2()
        barrier(self.ws)
        torch.cuda.synchronize()
        stats = []
        l0 = self.ctx.launch_count
        for _ in range(steps):
            self.flush_l2()
            stats.append(self.run(p).stats)
        torch.cuda.synchronize()
        barrier(self.ws)
        ms = allmax(self.ws, float(np.mean([s["ms_total"] for s in stats])))
        ph = {q: float(np.mean([s[q] for s in stats]))
              for q in ("ms_dist", "ms_orth", "ms_mmult", "ms_eig", "ms_coords", "ms_total")}
        return {"ms": ms, "stats": stats, "launches": (self.ctx.launch_count - l0) / max(1, steps), "phases": ph}

    def e2e(self, p, steps):
        ts, tu = [], []
        for _ in range(steps):
            self.flush_l2()
            barrier(self.ws)
            t1 = time.perf_counter()
            self.ctx.upload(self.gp)
            t2 = time.perf_counter()
            self.run(p)
            ts.append(time.perf_counter() - t1)
            tu.append(t2 - t1)
        self.upload_ms = float(np.mean(tu)) * 1e3
        return allmax(self.ws, float(np.mean(ts))) * 1e3

    def h2d_probe(self):
        """Host-to-device bandwidth of the pinned adjacency array alone (one plain copy, no kernels)."""
        import torch
        src = self.gp._pinned[1]
        dst = torch.empty_like(src, device="cuda")
        for _ in range(2):
            dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(3):
            dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        t = (time.perf_counter() - t1) / 3
        return {"bytes": int(src.numel() * 4), "ms": t * 1e3, "gbs": src.numel() * 4 / t / 1e9}

    def h2d(self):
        g = self.g
        return 4 * (g.n + 1) + 4 * g.nnz + (4 * g.nnz if g.weights is not None else 0)

    def d2h(self):
        return 8 * self.g.n * self.c


def pinned_graph(g):
    import torch
    from icpp_2020_parhde_gb300.csr_io import CSRGraph
    off = torch.from_numpy(np.ascontiguousarray(g.offsets, dtype=np.uint32)).pin_memory()
    adj = torch.from_numpy(np.ascontiguousarray(g.adj, dtype=np.uint32)).pin_memory()
    w = None if g.weights is None else torch.from_numpy(np.ascontiguousarray(g.weights, dtype=np.int32)).pin_memory()
    keep = (off, adj, w)
    gp = CSRGraph(off.numpy(), adj.numpy(), None if w is None else w.numpy())
    gp._pinned = keep
    return gp


def summary(r, k, nnz, ws, e2e_ms=None, h2d=0, d2h=0, rq=None, extra=None):
    d = {"value": ws * k * nnz / (r["ms"] * 1e-3), "unit": UNIT, "ms_per_graph": r["ms"], "phases_ms": r["phases"],
         "gpu_launches_per_step": r["launches"]}
    if e2e_ms is not None:
        d["e2e"] = {"value": ws * k * nnz / (e2e_ms * 1e-3), "unit": UNIT, "ms_per_graph": e2e_ms,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
    if rq is not None:
        d["rayleigh"] = [float(x) for x in rq]
    if extra:
        d.update(extra)
    return d


P_LEARNED = dict(strategy="Learned", precision="exact", eig="exact")
P_PLAIN = dict(strategy="Kcenters", precision="fp64", eig="power")
P_KC = dict(strategy="Kcenters", precision="exact", eig="exact")
P_CHECKED = dict(strategy="LearnedChecked", precision="exact", eig="exact")
P_MIXED = dict(strategy="Learned", precision="mixed", eig="exact")
P_KC_MIXED = dict(strategy="Kcenters", precision="mixed", eig="exact")


# ---------------------------------------------------------------------------------------------- the reference arm

def run_reference(args):
    ws, rank, local = dist_init()
    if rank != 0:
        return
    kind = {"rmat": "rmat", "rgg3d": "rgg3d", "grid3d": "grid3d"}[args.graph]
    g, desc, _ = make_graph(kind, args)
    from oracle import oracle as orc
    ncores = os.cpu_count() or 1
    algo = "wParHDE" if args.graph == "grid3d" else "ParHDE"
    for _ in range(args.warmup):
        orc.layout(g, algo, "Kcenters", args.k, args.c, nthreads=ncores, want_S=False)
    t0 = time.perf_counter()
    ts = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        L = orc.layout(g, algo, "Kcenters", args.k, args.c, nthreads=ncores, want_S=False)
        ts.append(time.perf_counter() - t1)
        if L.status != 0:
            raise RuntimeError("oracle layout failed: %d" % L.status)
    wall = time.perf_counter() - t0
    t = float(np.mean(ts))
    v = args.k * g.nnz / t
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(algo, desc, g, args.k, args.c),
            "pipeline": "the reference algorithm (Kcenters, CGS, SpMM, Gram, power iteration) as the OpenMP oracle "
                        "port, FP64",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": ncores, "kind": "port",
                             "sample": "%d full layouts after %d warm-up on %d threads (the port is pinned bit for "
                                       "bit to the reference built from its sources at one thread)"
                                       % (args.steps, args.warmup, ncores)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------- our arm

def run_gb300(args):
    ws, rank, local = dist_init()
    import torch
    torch.cuda.set_device(local)
    from icpp_2020_parhde_gb300 import Context, graphs
    if args.graph == "grid3d":
        return run_weighted_headline(args, ws, rank, local)
    kind = "rgg3d" if args.graph == "rgg3d" else "rmat"
    g, desc, gen_s = make_graph(kind, args)
    n, nnz, k, c = g.n, g.nnz, args.k, args.c
    ctx = Context(local)
    gp = pinned_graph(g)
    xy = torch.empty(n * c, dtype=torch.float64).pin_memory()
    ctx.upload(gp)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2

    def flush_l2():
        flush.fill_(1.0)
        torch.cuda.synchronize()

    R = Runner(ctx, g, gp, "ParHDE", k, c, xy, flush_l2, ws)
    sub_steps = max(3, args.steps // 4)
    controls = [x for x in args.controls.split(",") if x]
    pipes = [(name, p) for name, p in (("plain", P_PLAIN), ("kcenters_exact", P_KC), ("learned_checked", P_CHECKED),
                                       ("learned_mixed", P_MIXED)) if name in controls]
    # ---- end to end through the C ABI first, before the clock sampler ever runs: a polling nvidia-smi slows
    #      host <-> device copies several-fold on these machines, also for seconds after it exits (the R-MAT 22
    #      adjacency upload: 2.6 ms without it, 9.5-15 ms with it running or recently stopped) ----
    R.run(P_LEARNED)
    e2e_head = R.e2e(P_LEARNED, args.steps)
    upload_head = R.upload_ms
    e2e_ctl = {}
    for name, p in pipes:
        R.run(p)
        e2e_ctl[name] = R.e2e(p, sub_steps)
    # ---- device-resident timed regions, clocks sampled: the headline, then the reference pipeline on the GPU,
    #      the pivot control, the checked strategy, mixed precision ----
    clk = ClockSampler(local).__enter__()
    head = R.timed(P_LEARNED, args.steps, args.warmup)
    xy_head = R.coords()
    st_head = head["stats"][-1]
    ctl = {}
    for name, p in pipes:
        r = R.timed(p, sub_steps, 1 if name == "learned_checked" else 2)
        r["rq"] = rayleigh_quotients(g, R.coords())
        r["e2e"] = e2e_ctl[name]
        ctl[name] = r
    clk.__exit__(None, None, None)
    rq_head = rayleigh_quotients(g, xy_head)
    # ---- acceptance of the learned pivots against Kcenters (same precision and eigensolver): the per-coordinate
    #      rule and the summed rule on this graph, and the summed rule averaged over relabelled copies ----
    acc = {}
    if "kcenters_exact" in ctl:
        rq_kc = ctl["kcenters_exact"]["rq"]
        acc = {"per_coordinate_ratio": [float(a / b) for a, b in zip(rq_head, rq_kc)],
               "sum_ratio": float(rq_head.sum() / rq_kc.sum())}
        acc["accepted_each_2pct"] = bool(max(acc["per_coordinate_ratio"]) <= 1.02)
        acc["accepted_sum_2pct"] = bool(acc["sum_ratio"] <= 1.02)
        if "learned_checked" in ctl:
            acc["checked_strategy_outcome"] = ctl["learned_checked"]["stats"][-1]["pivot_outcome"]
        rel = []
        rng = np.random.default_rng(11)
        for t in range(1, max(1, args.relabellings)):
            gg = graphs.relabel(g, rng.permutation(n))
            ctx.upload(gg)
            ql = rayleigh_quotients(gg, ctx.layout("ParHDE", k=k, c=c, **P_LEARNED).coords)
            qk = rayleigh_quotients(gg, ctx.layout("ParHDE", k=k, c=c, **P_KC).coords)
            rel.append({"learned": ql.tolist(), "kcenters": qk.tolist()})
        ctx.upload(gp)
        if rel:
            tl = [rq_head.sum()] + [sum(r["learned"]) for r in rel]
            tk = [rq_kc.sum()] + [sum(r["kcenters"]) for r in rel]
            acc["relabelled_copies"] = rel
            acc["mean_sum_ratio_over_copies"] = float(np.mean(tl) / np.mean(tk))
    # ---- rooflines: the headline's two largest kernels, measured live by the library's events ----
    peak, peak_kind = peaks()
    pk_src = ("measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback")
    roof = None
    if st_head.get("ms_msbfs_kernel", 0) > 0:
        lv = st_head["msbfs_levels"]
        per_level = 8 * (n + 1) + 4 * nnz + 2 * n * 32  # offsets + adjacency + frontier words in and out
        b = lv * per_level
        kern_ms = float(np.mean([s["ms_msbfs_kernel"] for s in head["stats"]]))
        ach = b / (kern_ms * 1e-3) / 1e9
        roof = {"kernel": "msbfs_kernel<4>", "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": ach / peak, "traffic": profiled_traffic("msbfs_kernel_rmat22.md" if args.rmat_scale == 22 and
                                                                 kind == "rmat" else "none"),
                "peak_source": pk_src, "algorithmic_bytes_per_launch": b, "levels": lv, "kernel_ms": kern_ms}
    roof_lap = None
    if st_head.get("ms_lap_kernel", 0) > 0:
        kp = 64 if k <= 64 else (128 if k <= 128 else 256)
        zb = 1  # R-MAT distances stay below 256: one byte per packed distance
        b = 8 * (n + 1) + 4 * nnz + n * kp * zb  # CSR once, the packed distance rows once
        kern_ms = float(np.mean([s["ms_lap_kernel"] for s in head["stats"]]))
        ach = b / (kern_ms * 1e-3) / 1e9
        roof_lap = {"kernel": "lgram_kernel<uint8_t,64,4>", "bound": "hbm", "achieved": ach, "peak": peak,
                    "unit": "GB/s", "frac": ach / peak,
                    "traffic": profiled_traffic("lgram_kernel_rmat22.md" if args.rmat_scale == 22 and kind == "rmat"
                                                else "none"),
                    "peak_source": pk_src, "algorithmic_bytes_per_launch": b, "kernel_ms": kern_ms,
                    "gathered_bytes_per_launch": nnz // 2 * kp * zb}  # each undirected edge's upper end
    if rank != 0:
        return
    h2d, d2h = R.h2d(), R.d2h()
    line = {
        "metric": METRIC, "value": ws * k * nnz / (head["ms"] * 1e-3), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config("ParHDE", desc, g, k, c),
        "pipeline": "learned pivots + exact-Gram FP64 dense stages + exact eigensolve",
        "arithmetic": "int32 distances (bit-exact); every n-sized product as an exact int64 sum of integer products; "
                      "FP64 coefficient-space Gram-Schmidt, k x k Gram and eigensolve; coordinates as exact 62-bit "
                      "fixed-point row sums rounded once to FP64",
        "timing": {"l2": "inputs larger than L2 (513 MB CSR) and L2 flushed between timed steps (256 MB write)",
                   "device": "library CUDA events on its stream, mean over the timed steps, max over ranks",
                   "graph_gen_s": round(gen_s, 1)},
        "ms_per_graph": head["ms"],
        "phases_ms": head["phases"],
        "e2e": {"value": ws * k * nnz / (e2e_head * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_graph": e2e_head, "upload_ms": upload_head,
                "h2d_copy_probe": R.h2d_probe(),
                "path": "phde_graph_upload from pinned host CSR + phde_layout (coordinates to pinned host memory)"},
        "gpu_launches": int(round(head["launches"] * args.steps)),
        "roofline": roof,
        "roofline_lap_gram": roof_lap,
        "clocks": clk.summary(),
        "headline_stats_last": st_head,
        "learned_acceptance": acc,
        "pipelines": {"learned_exact": summary(head, k, nnz, ws, e2e_head, h2d, d2h, rq_head)},
    }
    for name, r in ctl.items():
        extra = {}
        if name == "learned_checked":
            extra = {"outcome": r["stats"][-1]["pivot_outcome"],
                     "ms_check": float(np.mean([s["ms_check"] for s in r["stats"]]))}
        if name == "learned_mixed":
            extra = {"rayleigh_rel_err_vs_learned_exact": float(np.max(np.abs(r["rq"] - rq_head) / np.abs(rq_head)))}
        line["pipelines"][name] = summary(r, k, nnz, ws, r["e2e"], h2d, d2h, r["rq"], extra)
    for name, key in (("plain", "speedup_vs_plain"), ("kcenters_exact", "speedup_vs_kcenters_same_stages")):
        if name in ctl:
            line[key] = {"device": ctl[name]["ms"] / head["ms"], "e2e": ctl[name]["e2e"] / e2e_head}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_layout(g, "ParHDE", k, c, args.cpu_reps, desc)
    subs = [s for s in args.subs.split(",") if s]
    line["configs"] = {}
    for s in subs:
        t0 = time.time()
        try:
            if s == "draw":
                line["configs"][s] = run_draw(args, ctx, gp, g, desc, xy_head, flush_l2)
            elif s == "rmat20":
                line["configs"][s] = run_single(args, local, "rmat20", 50, 3, flush_l2)
            elif s == "rgg3d":
                line["configs"][s] = run_single(args, local, "rgg3d", 64, 3, flush_l2)
            elif s == "weighted":
                line["configs"][s] = run_weighted(args, local, flush_l2)
            elif s == "batched":
                line["configs"][s] = run_batched(args, local, flush_l2)
        except Exception as e:  # a sub-measurement must not cost the headline line
            line["configs"][s] = {"error": "%s: %s" % (type(e).__name__, e), "trace": traceback.format_exc()[-800:]}
        line["configs"].setdefault(s, {})["bench_wall_s"] = round(time.time() - t0, 1)
    print(json.dumps(line), flush=True)
    ctx.close()


def run_single(args, local, kind, k, c, flush_l2):
    """Another single-graph configuration: learned + exact (headline pipeline), plain, the Kcenters control and
    the mixed-precision path, each with its end-to-end time; the CPU baseline on the same graph."""
    import torch
    from icpp_2020_parhde_gb300 import Context
    g, desc, gen_s = make_graph(kind, args)
    ctx = Context(local)
    gp = pinned_graph(g)
    xy = torch.empty(g.n * c, dtype=torch.float64).pin_memory()
    ctx.upload(gp)
    R = Runner(ctx, g, gp, "ParHDE", k, c, xy, flush_l2, 1)
    steps = max(3, args.steps // 5)
    out = {"config": workload_config("ParHDE", desc, g, k, c), "graph_gen_s": round(gen_s, 1), "pipelines": {}}
    rq = {}
    for name, p in (("learned_exact", P_LEARNED), ("plain", P_PLAIN), ("kcenters_exact", P_KC),
                    ("learned_mixed", P_MIXED), ("kcenters_mixed", P_KC_MIXED)):
        r = R.timed(p, steps, 2)
        rq[name] = rayleigh_quotients(g, R.coords())
        e = R.e2e(p, steps)
        out["pipelines"][name] = summary(r, k, g.nnz, 1, e, R.h2d(), R.d2h(), rq[name])
    out["value"] = out["pipelines"]["learned_exact"]["value"]
    out["speedup_vs_plain"] = {"device": out["pipelines"]["plain"]["ms_per_graph"] /
                               out["pipelines"]["learned_exact"]["ms_per_graph"],
                               "e2e": out["pipelines"]["plain"]["e2e"]["ms_per_graph"] /
                               out["pipelines"]["learned_exact"]["e2e"]["ms_per_graph"]}
    out["learned_vs_kcenters_rayleigh"] = {"per_coordinate_ratio": (rq["learned_exact"] / rq["kcenters_exact"]).tolist(),
                                           "sum_ratio": float(rq["learned_exact"].sum() / rq["kcenters_exact"].sum())}
    out["mixed_rayleigh_rel_err_vs_exact_same_pivots"] = float(
        np.max(np.abs(rq["kcenters_mixed"] - rq["kcenters_exact"]) / np.abs(rq["kcenters_exact"])))
    ctx.close()
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_layout(g, "ParHDE", k, c, 3 if g.nnz < 50_000_000 else 1, desc)
    return out


def run_weighted(args, local, flush_l2, clk=None):
    # clk: a ClockSampler (not yet started) to run around the device-timed region only, after the end-to-end
    # loop (see the headline's note on nvidia-smi)
    """The weighted configuration: WParHDE (Kcenters pivots by delta-stepping SSSP, coupled MGS, FP64 as the
    reference) on the weighted 3-D grid; CPU baseline: one oracle layout of the same graph."""
    import torch
    from icpp_2020_parhde_gb300 import Context
    k, c = 20, 2
    g, desc, gen_s = make_graph("grid3d", args)
    ctx = Context(local)
    gp = pinned_graph(g)
    xy = torch.empty(g.n * c, dtype=torch.float64).pin_memory()
    ctx.upload(gp)
    R = Runner(ctx, g, gp, "wParHDE", k, c, xy, flush_l2, 1)
    p = dict(strategy="Kcenters", precision="fp64", eig="power")
    steps = max(3, args.steps // 5)
    R.run(p)
    e = R.e2e(p, steps)
    if clk:
        clk.__enter__()
    r = R.timed(p, steps, 2)
    if clk:
        clk.__exit__(None, None, None)
    st = r["stats"]
    out = summary(r, k, g.nnz, 1, e, R.h2d(), R.d2h(), rayleigh_quotients(g, R.coords()))
    out.update({"config": workload_config("wParHDE", desc, g, k, c), "graph_gen_s": round(gen_s, 1),
                "pipeline": "WParHDE: Kcenters by delta-stepping SSSP, coupled MGS, FP64, power iteration",
                "sssp": {"grid_rounds_per_layout": float(np.mean([s["sssp_rounds"] for s in st])),
                         "edges_relaxed_per_layout": float(np.mean([s["edges_examined"] for s in st])),
                         "passes_per_layout": float(np.mean([s["npasses"] for s in st]))}})
    ctx.close()
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_layout(g, "wParHDE", k, c, 1, desc)
    return out


def run_weighted_headline(args, ws, rank, local):
    """--graph grid3d: the weighted configuration as the headline line."""
    import torch
    torch.cuda.set_device(local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def flush_l2():
        flush.fill_(1.0)
        torch.cuda.synchronize()

    clk = ClockSampler(local)
    out = run_weighted(args, local, flush_l2, clk)
    if rank != 0:
        return
    line = {"metric": METRIC, "value": out["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": out["ms_per_graph"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": out.pop("config"),
            "e2e": out.pop("e2e"), "clocks": clk.summary(), **out}
    print(json.dumps(line), flush=True)


def run_batched(args, local, flush_l2):
    """Many graphs in one call: --batch-count random geometric 2-D graphs (n log-uniform in 1k..200k, mean
    degree 8, LCC), k = 10, c = 2, laid out by phde_layout_batched, against the same graphs laid out one call
    each; CPU baseline: the oracle looping over the same graphs."""
    import torch
    from icpp_2020_parhde_gb300 import Context, graphs
    from oracle import oracle as orc
    k, c = 10, 2
    t = time.time()
    gs = graphs.rgg_batch(args.batch_count, seed=args.seed)
    gen_s = time.time() - t
    ntot, nnz_tot = sum(g.n for g in gs), sum(g.nnz for g in gs)
    cb = Context(local)
    cb.upload_batch(gs)
    out = torch.empty(ntot * c, dtype=torch.float64).pin_memory()
    steps = max(3, args.steps // 5)
    timing, rqs = {}, {}
    for strat in ("Kcenters", "Learned"):
        _, st0 = cb.layout_batched(k, c, coords_out=out.numpy(), strategy=strat)  # tunes (first) / runs uncaptured
        for _ in range(3):
            cb.layout_batched(k, c, coords_out=out.numpy(), strategy=strat)   # captures, then replays
        ms = []
        for _ in range(steps):
            flush_l2()
            _, st = cb.layout_batched(k, c, coords_out=out.numpy(), strategy=strat)
            ms.append(st["ms_total"])
        rqs[strat] = cb.batch_rayleigh()
        if strat == "Kcenters":
            xs = [x.copy() for x in cb.layout_batched(k, c, coords_out=out.numpy())[0]]
            st_kc, st0_kc = st, st0
        e2e = []
        for _ in range(steps):
            flush_l2()
            t1 = time.perf_counter()
            cb.upload_batch(gs)
            cb.layout_batched(k, c, coords_out=out.numpy(), strategy=strat)
            e2e.append(time.perf_counter() - t1)
        timing[strat] = {"ms_per_batch": float(np.mean(ms)), "e2e_ms_per_batch": float(np.mean(e2e)) * 1e3,
                         "gpu_launches_per_batch": st["gpu_launches"], "cuda_graph_replay": bool(st["batch_graph_replay"])}
    cb.close()
    st, st0 = st_kc, st0_kc
    t_b = timing["Kcenters"]["ms_per_batch"]
    e2e = [timing["Kcenters"]["e2e_ms_per_batch"] * 1e-3]
    # the learned pivots' acceptance per graph, against the batch's Kcenters layouts (same precision and solver)
    ql, qk = rqs["Learned"], rqs["Kcenters"]
    sum_ratio = ql.sum(axis=1) / qk.sum(axis=1)
    learned_check = {"graphs": len(gs), "sum_ratio_mean": float(np.mean(sum_ratio)),
                     "sum_ratio_max": float(np.max(sum_ratio)),
                     "graphs_within_2pct_sum": int(np.sum(sum_ratio <= 1.02)),
                     "graphs_within_2pct_each": int(np.sum(np.all(ql <= 1.02 * qk, axis=1))),
                     "mean_sum_ratio_over_graphs_weighted": float(ql.sum() / qk.sum())}
    cs = Context(local)
    loop = {"kcenters_mixed": 0.0, "plain": 0.0}
    rq_err = []
    for i, g in enumerate(gs):
        cs.upload(g)
        for name, p in (("kcenters_mixed", P_KC_MIXED), ("plain", P_PLAIN)):
            r = cs.layout("ParHDE", k=k, c=c, **p)
            loop[name] += r.stats["ms_total"]
            if name == "kcenters_mixed" and i % 64 == 0:
                a, b = rayleigh_quotients(g, xs[i]), rayleigh_quotients(g, r.coords)
                rq_err.append(float(np.max(np.abs(a - b) / np.abs(b))))
    cs.close()
    e2e_ms = float(np.mean(e2e)) * 1e3
    res = {"config": {"workload": "%d random geometric 2-D graphs, n log-uniform in [1000, 200000], mean degree 8, LCC "
                                  "(sum n = %d, sum nnz = %d), ParHDE k=%d, c=%d" % (len(gs), ntot, nnz_tot, k, c),
                      "graphs": len(gs), "n": ntot, "nnz": nnz_tot, "k": k, "c": c},
           "pipeline": "Kcenters, mixed precision, Jacobi; one persistent Kcenters launch + one CUDA graph replay",
           "value": k * nnz_tot / (t_b * 1e-3), "unit": UNIT, "ms_per_batch": t_b, "ms_per_graph": t_b / len(gs),
           "learned": {"value": k * nnz_tot / (timing["Learned"]["ms_per_batch"] * 1e-3), "unit": UNIT,
                       **timing["Learned"],
                       "speedup_vs_kcenters_batched": {
                           "device": t_b / timing["Learned"]["ms_per_batch"],
                           "e2e": timing["Kcenters"]["e2e_ms_per_batch"] / timing["Learned"]["e2e_ms_per_batch"]},
                       "rayleigh_check_vs_kcenters": learned_check},
           "e2e": {"value": k * nnz_tot / (e2e_ms * 1e-3), "unit": UNIT, "ms_per_batch": e2e_ms,
                   "h2d_bytes_per_step": 4 * (ntot + len(gs)) + 4 * nnz_tot, "d2h_bytes_per_step": 8 * ntot * c},
           "loop_ms_per_batch": loop, "speedup_vs_loop": {kk: v / t_b for kk, v in loop.items()},
           "cuda_graph_replay": bool(st["batch_graph_replay"]), "autotuned_segment_rows": st["batch_seg_rows"],
           "autotune_first_call_ms": st0["ms_batch_tune"], "gpu_launches_per_batch": st["gpu_launches"],
           "rayleigh_rel_err_vs_single_max": max(rq_err) if rq_err else None, "graph_gen_s": round(gen_s, 1)}
    if not args.no_cpu_baseline:
        ncores = os.cpu_count() or 1
        t1 = time.perf_counter()
        for g in gs:
            L = orc.layout(g, "ParHDE", "Kcenters", k, c, nthreads=ncores, want_S=False)
            if L.status != 0:
                raise RuntimeError("oracle layout failed: %d" % L.status)
        t_cpu = time.perf_counter() - t1
        res["cpu_baseline"] = {"value": k * nnz_tot / t_cpu, "unit": UNIT, "cores": ncores, "kind": "port",
                               "ms_per_batch": t_cpu * 1e3,
                               "sample": "the oracle port of the reference algorithm looping over the same %d graphs "
                                         "(one layout each) in %.1f s" % (len(gs), t_cpu)}
    return res


def run_draw(args, ctx, gp, g, desc, xy, flush_l2):
    """The draw tool on the headline layout: its first two coordinates rasterised (phde_draw).  value = Bresenham
    pixel writes per second of device time; e2e = host coordinates -> PNG file through the C ABI.  CPU baseline:
    the one-thread oracle (the reference's serial order) on an R-MAT-16 layout."""
    import tempfile
    from icpp_2020_parhde_gb300 import graphs
    from oracle import oracle as orc
    x, y = np.ascontiguousarray(xy[:, 0]), np.ascontiguousarray(xy[:, 1])
    ctx.upload(gp)
    for _ in range(3):
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
    px = info["pixels"]
    out = {"config": {"workload": "draw of the headline layout (coordinates 1 and 2) of %s: %d x %d image, %d CSR "
                                  "entries" % (desc, info["width"], info["height"], g.nnz)},
           "value": px / (np.mean(dev) * 1e-3), "unit": "pixel writes/s", "pixels_per_step": px,
           "ms_device": float(np.mean(dev)), "ms_raster": float(np.mean(ras)),
           "e2e": {"value": px / float(np.mean(e2e)), "unit": "pixel writes/s", "ms": float(np.mean(e2e)) * 1e3,
                   "path": "phde_draw + phde_draw_write_png (host coordinates to PNG file)",
                   "h2d_bytes_per_step": 16 * g.n, "d2h_bytes_per_step": 0, "png_bytes": os.path.getsize(path)},
           "gpu_launches": info["gpu_launches"]}
    if not args.no_cpu_baseline:
        gs = graphs.rmat(16, 16, seed=args.seed)
        ctx.upload(gs)
        xs = ctx.layout("ParHDE", k=20, c=2, **P_LEARNED).coords
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
        ctx.upload(gp)
    return out


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
