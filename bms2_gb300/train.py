"""Training data and training of the learned query-vertex cost model.

Samples are query vertices.  Features come from bms_query_features (label
frequency, degree, ring membership, candidate-set size, ...); the target is
log2(1 + mean number of DFS assignments the vertex receives per mapped pair)
logged by the library in a plain (query-index) order, count-all, EXACT run.
Training runs on the GPU with the library's own forward, backward and Adam
kernels (bfloat16 weights, fp32 accumulation).
"""
from __future__ import annotations

import numpy as np

from .native import COUNT_ALL, ORDER_GMCR, SEM_EXACT, Context


def collect(ctx: Context, refine_steps: int) -> tuple[np.ndarray, np.ndarray]:
    """(features [n, 12], targets [n]) of every vertex of every query that has
    at least one mapped pair, from one logged plain-order run."""
    ctx.set_logging(True)
    try:
        ctx.run(refine_steps, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
    finally:
        ctx.set_logging(False)
    x = ctx.query_features()
    e = ctx.vertex_expansions().astype(np.float64)
    off, qidx = ctx.gmcr()
    st = ctx.stats()
    pairs = np.bincount(qidx, minlength=st["n_query_graphs"]).astype(np.float64)
    goff = ctx.query_graph_offsets().astype(np.int64)
    q_of = np.repeat(np.arange(len(goff) - 1), np.diff(goff))
    p = pairs[q_of]
    keep = p > 0
    y = np.log2(1.0 + e[keep] / p[keep]).astype(np.float32)
    return x[keep].astype(np.float32), y


def train(ctx: Context, x: np.ndarray, y: np.ndarray, seed: int = 1, epochs: int = 200, batch: int = 256,
          lr: float = 3e-3) -> float:
    return ctx.model_train(x, y, epochs=epochs, batch=batch, lr=lr, seed=seed)
