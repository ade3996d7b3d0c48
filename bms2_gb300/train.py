"""Training data and training of the learned query-vertex cost model.

Samples are query vertices.  Features come from bms_query_features (label
frequency, degree, ring membership, candidate-set size, ...).  The target is
a vertex's root-level search-tree size: log2(1 + mean number of DFS
assignments it receives per mapped pair when the search starts at it), logged
by the library's own join (count-all, EXACT).  One logged run per root rank r
searches every query from its vertex r (the rest in a breadth-first order from
it) with explicit orders (BMS_ORDER_GIVEN), so every vertex is logged as a
root once.  The order built from the predictions (lowest cost first, then the
cheapest frontier vertex, placed neighbours counting in its favour) starts at
the vertices whose first search level is smallest.  (Assignments logged in the
plain query-index order measure a vertex's position in that order more than
the vertex: ordering by them, even exactly, cuts expansions far less.)
Training runs on the GPU with the library's own forward, backward and Adam
kernels (bfloat16 weights, fp32 accumulation).
"""
from __future__ import annotations

from collections import deque

import numpy as np

from .native import COUNT_ALL, ORDER_GIVEN, ORDER_GMCR, SEM_EXACT, Context


def _neighbours(queries: dict, g: int) -> list[list[int]]:
    go, ro, ci = queries["graph_offsets"], queries["row_offsets"], queries["column_indices"]
    s, e = int(go[g]), int(go[g + 1])
    return [sorted(int(x) - s for x in ci[int(ro[v]):int(ro[v + 1])]) for v in range(s, e)]


def rooted_orders(queries: dict, r: int) -> np.ndarray:
    """Per query with more than r vertices: vertex r first, then breadth-first
    from it (lowest local id first; any unreached vertex after); smaller
    queries keep the query-index order."""
    go = np.asarray(queries["graph_offsets"], dtype=np.int64)
    out = np.zeros(int(go[-1]), dtype=np.uint8)
    for g in range(len(go) - 1):
        s, e = int(go[g]), int(go[g + 1])
        n = e - s
        if n <= r:
            out[s:e] = np.arange(n)
            continue
        nb = _neighbours(queries, g)
        seen = [False] * n
        order, todo = [], deque([r])
        seen[r] = True
        while len(order) < n:
            if not todo:
                u0 = seen.index(False)
                seen[u0] = True
                todo.append(u0)
            u = todo.popleft()
            order.append(u)
            for w in nb[u]:
                if not seen[w]:
                    seen[w] = True
                    todo.append(w)
        out[s:e] = order
    return out


def greedy_orders(queries: dict, cost: np.ndarray) -> np.ndarray:
    """Per query, a connected order: the vertex of lowest cost first, then the
    frontier vertex (adjacent to the placed ones; any vertex when none is)
    minimising cost - (placed neighbours).  order[qoff + t] = local vertex."""
    go = np.asarray(queries["graph_offsets"], dtype=np.int64)
    out = np.zeros(int(go[-1]), dtype=np.uint8)
    for g in range(len(go) - 1):
        s, e = int(go[g]), int(go[g + 1])
        n = e - s
        if n == 0:
            continue
        nb = _neighbours(queries, g)
        c = np.asarray(cost[s:e], dtype=np.float64)
        placed = np.zeros(n, bool)
        pn = np.zeros(n)
        order = [int(np.argmin(c))]
        placed[order[0]] = True
        for w in nb[order[0]]:
            pn[w] += 1
        while len(order) < n:
            front = np.nonzero(~placed & (pn > 0))[0]
            if len(front) == 0:
                front = np.nonzero(~placed)[0]
            u = int(front[np.argmin(c[front] - pn[front])])
            order.append(u)
            placed[u] = True
            for w in nb[u]:
                pn[w] += 1
        out[s:e] = order
    return out


def collect(ctx: Context, refine_steps: int, queries: dict) -> tuple[np.ndarray, np.ndarray]:
    """(features [n, 12], targets [n]) of every vertex of every query of the
    loaded batch (`queries`: its CSR arrays) that has at least one mapped pair;
    the target is the vertex's logged root-level search-tree size."""
    ctx.run(refine_steps, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
    x = ctx.query_features()
    _, qidx = ctx.gmcr()
    st = ctx.stats()
    pairs = np.bincount(qidx, minlength=st["n_query_graphs"]).astype(np.float64)
    go = np.asarray(queries["graph_offsets"], dtype=np.int64)
    sizes = np.diff(go)
    q_of = np.repeat(np.arange(len(sizes)), sizes)
    rank = np.arange(int(go[-1])) - go[q_of]  # local id of every vertex
    root = np.zeros(int(go[-1]), dtype=np.float64)
    ctx.set_logging(True)
    try:
        for r in range(int(sizes.max()) if len(sizes) else 0):
            ctx.set_query_order(rooted_orders(queries, r))
            ctx.run(refine_steps, COUNT_ALL, ORDER_GIVEN, SEM_EXACT)
            v = ctx.vertex_expansions().astype(np.float64)
            mine = rank == r
            root[mine] = v[mine]  # the root's assignments: its candidates, pair by pair
    finally:
        ctx.set_logging(False)
    p = pairs[q_of]
    keep = p > 0
    y = np.log2(1.0 + root[keep] / p[keep]).astype(np.float32)
    return x[keep].astype(np.float32), y


def train(ctx: Context, x: np.ndarray, y: np.ndarray, seed: int = 1, epochs: int = 200, batch: int = 256,
          lr: float = 3e-3) -> float:
    return ctx.model_train(x, y, epochs=epochs, batch=batch, lr=lr, seed=seed)
