"""Data-graph shards across ranks (one process per GPU).

Pairs are independent, so a batch of data graphs is split across ranks with
the queries replicated on every rank; each rank runs the whole pipeline on its
shard and the only exchange is the final reduction of totals (and the maximum
of the timed region over ranks).  No collective touches the data path.

`lpt_owners` restates the reference MPI driver's load balancing
(BMS2_mpi.cpp:78-157): cost of a data graph = nodes^2 + edges, graphs sorted by
decreasing cost, each given to the currently least-loaded rank (the lowest
rank on ties).  The sort here is stable, so equal costs keep their input
order and the assignment is deterministic.
"""
from __future__ import annotations

import numpy as np


def graph_costs(arrays: dict) -> np.ndarray:
    """nodes^2 + edges per data graph (edges = CSR entries / 2 for the
    symmetric batches the format describes); at least 1."""
    go = np.asarray(arrays["graph_offsets"], dtype=np.int64)
    ro = np.asarray(arrays["row_offsets"], dtype=np.int64)
    nodes = go[1:] - go[:-1]
    entries = ro[go[1:]] - ro[go[:-1]]
    cost = nodes.astype(np.float64) ** 2 + (entries // 2).astype(np.float64)
    return np.maximum(cost, 1.0)


def lpt_owners(costs: np.ndarray, world: int) -> np.ndarray:
    """Rank owning each graph: largest cost first, to the least-loaded rank."""
    if world < 1:
        raise ValueError("world must be >= 1")
    owners = np.zeros(len(costs), dtype=np.int32)
    load = np.zeros(world, dtype=np.float64)
    for i in np.argsort(-np.asarray(costs, dtype=np.float64), kind="stable"):
        r = int(np.argmin(load))  # first minimum: lowest rank on ties
        owners[i] = r
        load[r] += costs[i]
    return owners


def take_graphs(arrays: dict, idx: np.ndarray) -> dict:
    """The CSR batch of graphs `idx` (in that order), ids rebased."""
    go = np.asarray(arrays["graph_offsets"], dtype=np.int64)
    ro = np.asarray(arrays["row_offsets"], dtype=np.int64)
    ci = np.asarray(arrays["column_indices"], dtype=np.int64)
    nl, el = arrays["node_labels"], arrays["edge_labels"]
    out_go, out_ro, out_ci, out_nl, out_el = [0], [], [], [], []
    n_nodes = n_entries = 0
    for g in np.asarray(idx, dtype=np.int64):
        s, e = int(go[g]), int(go[g + 1])
        rs, re = int(ro[s]), int(ro[e])
        out_ci.append(ci[rs:re] - s + n_nodes)
        out_ro.append(ro[s + 1:e + 1] - rs + n_entries)
        out_nl.append(nl[s:e])
        out_el.append(el[rs:re])
        n_nodes += e - s
        n_entries += re - rs
        out_go.append(n_nodes)
    cat = lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt)  # noqa: E731
    return {"graph_offsets": np.asarray(out_go, dtype=np.uint32),
            "row_offsets": np.concatenate([np.zeros(1, np.int64)] + out_ro).astype(np.uint32),
            "column_indices": cat(out_ci, np.uint32), "node_labels": cat(out_nl, np.uint8),
            "edge_labels": cat(out_el, np.uint8)}


def reduce_totals(total_matches: int, valid_pairs: int, seconds: float, device=None) -> tuple[int, int, float]:
    """Sum of matches and valid pairs, maximum of the timed seconds, over all
    ranks of the default process group (gloo on CPU, NCCL with `device`)."""
    import torch
    import torch.distributed as dist

    s = torch.tensor([total_matches, valid_pairs], dtype=torch.int64, device=device)
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(s, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return int(s[0].item()), int(s[1].item()), float(t[0].item())
