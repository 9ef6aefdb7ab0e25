"""Numpy restatement of the learned pivot proposal's scoring (csrc/learned.cu): the four per-vertex features
and the 4 -> 64 -> 64 -> 1 ReLU network's FP32 forward pass with the sigmoid output.

TEST INFRASTRUCTURE: the checker of the GPU feature and scoring kernels (tests/), and the feature definition
the offline trainer (train/train_pivot_mlp.py) labels with.  The library never imports it.
"""
from __future__ import annotations

import os

import numpy as np

WARM = 8  # PHDE_LEARNED_WARM in include/parhde.h: exact Kcenters passes before the candidates are scored
HIDDEN = 64
WEIGHTS_H = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "icpp_2020_parhde_gb300",
                         "csrc", "pivot_mlp_weights.h")


def features(g, d0: np.ndarray) -> np.ndarray:
    """(n, 4) float32: log(1+deg)/log(1+max deg), log(1+sum of neighbour degrees)/log(1+its max),
    d0/max d0 (d0 = the warm start's minimum distance to its pivots), and the share of neighbours with a
    larger d0 -- the features of feature_raw_kernel / mlp_score_kernel, in FP64 then rounded."""
    off = g.offsets.astype(np.int64)
    adj = g.adj.astype(np.int64)
    n = g.n
    deg = np.diff(off).astype(np.float64)
    src = np.repeat(np.arange(n), np.diff(off))
    hop2 = np.bincount(src, weights=deg[adj], minlength=n)
    outw = np.bincount(src, weights=(d0[adj] > d0[src]).astype(np.float64), minlength=n)
    f = np.zeros((n, 4), dtype=np.float64)
    f[:, 0] = np.log1p(deg) / max(np.log1p(deg.max()), 1e-30)
    f[:, 1] = np.log1p(hop2) / max(np.log1p(hop2.max()), 1e-30)
    f[:, 2] = np.maximum(d0, 0) / max(d0.max(), 1)
    f[:, 3] = np.where(deg > 0, outw / np.maximum(deg, 1), 0.0)
    return f.astype(np.float32)


def load_weights(path: str = WEIGHTS_H) -> np.ndarray:
    """The compiled-in weights (W1[64][4], b1[64], W2[64][64], b2[64], w3[64], b3) from the generated header."""
    txt = open(path).read()
    body = txt[txt.index("{") + 1: txt.rindex("}")]
    return np.array([float(t.rstrip("f")) for t in body.replace("\n", " ").split(",") if t.strip()], dtype=np.float32)


def scores(f: np.ndarray, w: np.ndarray) -> np.ndarray:
    """sigmoid(w3 . relu(W2 relu(W1 f + b1) + b2) + b3) per vertex, in FP32."""
    H = HIDDEN
    W1 = w[: H * 4].reshape(H, 4)
    b1 = w[H * 4: H * 5]
    W2 = w[H * 5: H * 5 + H * H].reshape(H, H)
    b2 = w[H * 5 + H * H: H * 6 + H * H]
    w3 = w[H * 6 + H * H: H * 7 + H * H]
    b3 = w[H * 7 + H * H]
    h1 = np.maximum(f.astype(np.float32) @ W1.T + b1, 0).astype(np.float32)
    h2 = np.maximum(h1 @ W2.T + b2, 0).astype(np.float32)
    z = (h2 @ w3 + b3).astype(np.float32)
    return (1.0 / (1.0 + np.exp(-z.astype(np.float64)))).astype(np.float32)


def farthest_point_order(D_warm: np.ndarray, C: np.ndarray, npick: int) -> list[int]:
    """The learned strategy's pivot order after the warm start (the host loop of csrc/api.cu's learned path):
    D_warm (M, P0) = the candidates' distances to the warm-start pivots, C (M, M) = the candidates' pairwise
    distances (C[i, j] from candidate j to candidate i); candidates in proposal order (best score first).
    Each step takes the unused candidate farthest from every pivot taken so far -- the first in proposal order
    on ties -- and folds its distances into the minima.  Returns candidate indices."""
    M = C.shape[0]
    mind = D_warm.min(axis=1).astype(np.int64) if D_warm.shape[1] else np.full(M, np.iinfo(np.int32).max, np.int64)
    used = np.zeros(M, dtype=bool)
    order = []
    for _ in range(min(npick, M)):
        cand = np.where(~used, mind, -1)
        best = int(np.argmax(cand))  # first maximum: proposal order on ties
        if used[best]:
            break
        used[best] = True
        order.append(best)
        mind = np.minimum(mind, C[:, best])
    return order
