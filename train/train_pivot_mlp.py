"""Train the pivot-scoring MLP of the learned pivot strategy (PHDE_STRAT_LEARNED).

Training data: seeded R-MAT and random geometric (2-D and 3-D) graphs.  On each, Kcenters (k = 64, the
reference's farthest-first rule, ParHDE.cpp:118-157, computed with the CPU oracle) runs 3k passes; the
first WARM passes are the warm start the layout runs exactly, and the pivots Kcenters picks after them are
the positive vertices.  Features are the four the GPU kernel computes (csrc/learned.cu): log-degree, log of
the neighbour-degree sum, the warm start's minimum distance to its pivots, and the share of neighbours
with a larger minimum distance, each normalised per graph.  The 4 -> 64 -> 64 -> 1 ReLU network is trained with a
class-weighted logistic loss under BF16 autocast; the FP32 weights are written to
icpp_2020_parhde_gb300/csrc/pivot_mlp_weights.h (compiled into the library) and a summary to
train/pivot_mlp_train.json.  An offline tool: the library never imports it.

    python train/train_pivot_mlp.py [--graphs 200] [--max-n 100000]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "icpp_2020_parhde_gb300")
sys.path.insert(0, ROOT)

from oracle.pivot_oracle import WARM, features  # noqa: E402  (the numpy restatement of the GPU features)


def training_graphs(count: int, max_n: int, seed: int):
    from icpp_2020_parhde_gb300 import graphs
    rng = np.random.default_rng(seed)
    for i in range(count):
        kind = i % 3
        n = int(math.exp(rng.uniform(math.log(10_000), math.log(max_n))))
        s = int(rng.integers(1, 1 << 30))
        if kind == 0:
            scale = max(12, min(20, int(round(math.log2(n / 0.8)))))
            yield graphs.rmat(scale, 16, seed=s)
        elif kind == 1:
            yield graphs.rgg(n, dim=2, avg_degree=8, seed=s)
        else:
            yield graphs.rgg(n, dim=3, avg_degree=12, seed=s)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--graphs", type=int, default=200)
    ap.add_argument("--max-n", type=int, default=100_000)
    ap.add_argument("--k", type=int, default=64)
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--seed", type=int, default=2020)
    args = ap.parse_args(argv)
    import torch
    from oracle import oracle as orc  # the CPU oracle computes the Kcenters labels

    torch.manual_seed(args.seed)
    P = 3 * args.k
    X, Y, sizes = [], [], []
    t0 = time.time()
    for gi, g in enumerate(training_graphs(args.graphs, args.max_n, args.seed)):
        D, piv = orc.kcenters(g, min(P, g.n - 1), 0, parallel=True)
        d0 = D[:, :WARM].min(axis=1).astype(np.int64)
        y = np.zeros(g.n, dtype=np.float32)
        y[piv[WARM:]] = 1.0
        X.append(features(g, d0))
        Y.append(y)
        sizes.append((g.name, g.n, g.nnz))
        if gi % 20 == 0:
            print(f"[{time.time() - t0:6.1f}s] graph {gi}: {g.name} n={g.n} nnz={g.nnz}", flush=True)
    X = torch.from_numpy(np.concatenate(X))
    Y = torch.from_numpy(np.concatenate(Y))
    pos = float(Y.sum())
    pos_weight = torch.tensor([(len(Y) - pos) / max(pos, 1.0)])
    model = torch.nn.Sequential(torch.nn.Linear(4, 64), torch.nn.ReLU(), torch.nn.Linear(64, 64), torch.nn.ReLU(),
                                torch.nn.Linear(64, 1))
    opt = torch.optim.Adam(model.parameters(), lr=3e-3)
    lossf = torch.nn.BCEWithLogitsLoss(pos_weight=pos_weight)
    bs = 65536
    history = []
    for ep in range(args.epochs):
        perm = torch.randperm(len(Y))
        tot = 0.0
        for b in range(0, len(Y), bs):
            idx = perm[b:b + bs]
            with torch.autocast("cpu", dtype=torch.bfloat16):
                logits = model(X[idx]).squeeze(1)
            loss = lossf(logits.float(), Y[idx])
            opt.zero_grad()
            loss.backward()
            opt.step()
            tot += float(loss) * len(idx)
        history.append(tot / len(Y))
        print(f"epoch {ep}: loss {history[-1]:.4f}", flush=True)
    # ranking quality: share of Kcenters pivots among each graph's 256 best-scored vertices
    with torch.no_grad():
        s = model(X).squeeze(1).numpy()
    hits, off = [], 0
    for (_, n, _), y in zip(sizes, np.split(Y.numpy(), np.cumsum([z[1] for z in sizes])[:-1])):
        top = np.argsort(-s[off:off + n], kind="stable")[:256]
        hits.append(float(y[top].sum() / max(y.sum(), 1)))
        off += n
    W1 = model[0].weight.detach().float().numpy()  # (64, 4)
    b1 = model[0].bias.detach().float().numpy()
    W2 = model[2].weight.detach().float().numpy()  # (64, 64)
    b2 = model[2].bias.detach().float().numpy()
    w3 = model[4].weight.detach().float().numpy().ravel()
    b3 = model[4].bias.detach().float().numpy()
    flat = np.concatenate([W1.ravel(), b1, W2.ravel(), b2, w3, b3]).astype(np.float32)
    hdr = os.path.join(PKG, "csrc", "pivot_mlp_weights.h")
    with open(hdr, "w") as f:
        f.write("// Generated by train/train_pivot_mlp.py -- do not edit.\n")
        f.write("// Pivot-scoring MLP 4 -> 64 -> 64 -> 1 (ReLU): W1[64][4], b1[64], W2[64][64], b2[64], w3[64], b3.\n")
        f.write("#pragma once\nstatic const float kPivotMlpWeights[%d] = {\n" % flat.size)
        for i in range(0, flat.size, 8):
            f.write("    " + ", ".join("%.9ef" % v for v in flat[i:i + 8]) + ",\n")
        f.write("};\n")
    summary = {"graphs": len(sizes), "vertices": int(len(Y)), "positives": int(pos), "k": args.k, "P": P,
               "warm": WARM,
               "epochs": args.epochs, "loss": history, "mean_kcenters_pivots_in_top256": float(np.mean(hits)),
               "max_n": args.max_n, "seed": args.seed, "train_seconds": time.time() - t0,
               "training_graphs": [f"{a} n={b} nnz={c}" for a, b, c in sizes]}
    with open(os.path.join(HERE, "pivot_mlp_train.json"), "w") as f:
        json.dump(summary, f, indent=1)
    print(json.dumps({k: v for k, v in summary.items() if k != "training_graphs"}, indent=1))


if __name__ == "__main__":
    main()
