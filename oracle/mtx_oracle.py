"""CPU restatement of the reference's Matrix Market converter (test infrastructure: the oracle of
phde_graph_from_entries and lib/mtx2csr; nothing in the product imports it).

Follows mtx2csr.cpp step by step:
  header words (mtx2csr.cpp:44-80): "coordinate" required, "general" -> not symmetric, "real" weights read and
    dropped, "integer" weights kept;
  size line and reading mode (:84-105): a general square matrix is read as an undirected graph, a general
    non-square one as a bipartite graph with rows numbered after the columns;
  entries (:106-131): symmetric -> both directions, self loops dropped; bipartite -> rows shifted by n2;
  per-vertex sort of (neighbour, weight) pairs and removal of parallel entries keeping the first (:134-160);
  components by BFS in vertex order, the largest kept (the first found on ties) (:168-207);
  renumbering in increasing order and the binary CSR (:209-296): six int64 header words
  {n, nnz, 1, 0, 1, 0}, uint32 offsets, uint32 adjacency, int32 weights for integer matrices.
"""
from __future__ import annotations

import numpy as np


def parse_mtx(path: str):
    """-> (u, v, w or None, n1, n2, symmetric, pattern) with 1-indexed u, v as the file holds them."""
    symmetric, pattern = 1, 1
    n1 = n2 = m = 0
    rows = []
    first = True
    with open(path) as f:
        for line in f:
            if line.startswith("%"):
                if line.startswith("%%"):
                    if "coordinate" not in line:
                        raise ValueError("not in coordinate format")
                    if "general" in line:
                        symmetric = 0
                    if "pattern" not in line:
                        if "real" in line:
                            pattern = 0
                        if "integer" in line:
                            pattern = 2
                continue
            if not line.strip():
                continue
            if first:
                n1, n2, m = (int(x) for x in line.split()[:3])
                first = False
                if not symmetric and n1 == n2:
                    symmetric = 1
                continue
            rows.append(line.split())
    u = np.array([int(r[0]) for r in rows], dtype=np.int64)
    v = np.array([int(r[1]) for r in rows], dtype=np.int64)
    w = np.array([int(r[2]) for r in rows], dtype=np.int64) if pattern == 2 else None
    return u, v, w, n1, n2, symmetric, pattern


def convert(u, v, w, n1, n2, symmetric):
    """-> (offsets uint32, adj uint32, weights int32 or None, info dict)."""
    u = np.asarray(u, dtype=np.int64)
    v = np.asarray(v, dtype=np.int64)
    wt = np.ones(u.shape[0], dtype=np.int64) if w is None else np.asarray(w, dtype=np.int64)
    N = n1 if symmetric else n1 + n2
    if symmetric:
        keep = u != v
        s = np.concatenate([u[keep] - 1, v[keep] - 1])
        d = np.concatenate([v[keep] - 1, u[keep] - 1])
        ww = np.concatenate([wt[keep], wt[keep]])
    else:
        r = u - 1 + n2
        s = np.concatenate([r, v - 1])
        d = np.concatenate([v - 1, r])
        ww = np.concatenate([wt, wt])
    order = np.lexsort((ww, d, s))  # per vertex, (neighbour, weight) ascending
    s, d, ww = s[order], d[order], ww[order]
    first = np.ones(s.shape[0], dtype=bool)
    first[1:] = (s[1:] != s[:-1]) | (d[1:] != d[:-1])
    s, d, ww = s[first], d[first], ww[first]
    deg = np.bincount(s, minlength=N)
    off = np.zeros(N + 1, dtype=np.int64)
    np.cumsum(deg, out=off[1:])
    # components by BFS in vertex order; the largest (first found on ties)
    comp = np.zeros(N, dtype=np.int64)
    ncomp, best, best_size = 0, 0, 0
    for i in range(N):
        if comp[i]:
            continue
        ncomp += 1
        comp[i] = ncomp
        stack, size = [i], 1
        while stack:
            x = stack.pop()
            for y in d[off[x]:off[x + 1]]:
                if not comp[y]:
                    comp[y] = ncomp
                    stack.append(int(y))
                    size += 1
        if size > best_size:
            best, best_size = ncomp, size
    keepv = comp == best
    newid = np.cumsum(keepv) - 1
    ke = keepv[s]
    s2, d2, w2 = newid[s[ke]], newid[d[ke]], ww[ke]
    n = int(keepv.sum())
    off2 = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(s2, minlength=n), out=off2[1:])
    info = {"n_in": N, "nnz_dedup": int(s.shape[0]), "ncomponents": ncomp, "n": n, "nnz": int(s2.shape[0])}
    return (off2.astype(np.uint32), d2.astype(np.uint32), None if w is None else w2.astype(np.int32), info)


def csr_bytes(off, adj, weights) -> bytes:
    n, m = off.shape[0] - 1, adj.shape[0]
    hdr = np.array([n, m, 1, 0, 1, 0], dtype=np.int64).tobytes()
    body = off.astype(np.uint32).tobytes() + adj.astype(np.uint32).tobytes()
    if weights is not None:
        body += weights.astype(np.int32).tobytes()
    return hdr + body


def mtx2csr_bytes(path: str) -> bytes:
    u, v, w, n1, n2, sym, pattern = parse_mtx(path)
    off, adj, ws, _ = convert(u, v, w, n1, n2, sym)
    return csr_bytes(off, adj, ws if pattern == 2 else None)
