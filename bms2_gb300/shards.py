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


def lpt_owners_native(arrays: dict, world: int) -> np.ndarray:
    """lpt_owners(graph_costs(arrays), world) computed by libbms
    (bms_shard_lpt), for batches of millions of graphs."""
    import ctypes as C

    from .native import _check, _ptr, lib

    go = np.ascontiguousarray(arrays["graph_offsets"], dtype=np.uint32)
    ro = np.ascontiguousarray(arrays["row_offsets"], dtype=np.uint32)
    owners = np.zeros(max(len(go) - 1, 1), dtype=np.uint32)
    _check(lib().bms_shard_lpt(len(go) - 1, _ptr(go, C.c_uint32), _ptr(ro, C.c_uint32), world,
                               _ptr(owners, C.c_uint32), None))
    return owners[: len(go) - 1].astype(np.int32)


def take_graphs(arrays: dict, idx: np.ndarray) -> dict:
    """The CSR batch of graphs `idx` (in that order), ids rebased."""
    go = np.asarray(arrays["graph_offsets"], dtype=np.int64)
    ro = np.asarray(arrays["row_offsets"], dtype=np.int64)
    ci = np.asarray(arrays["column_indices"], dtype=np.int64)
    nl, el = np.asarray(arrays["node_labels"]), np.asarray(arrays["edge_labels"])
    idx = np.asarray(idx, dtype=np.int64)
    sizes = go[idx + 1] - go[idx]
    new_go = np.zeros(len(idx) + 1, np.int64)
    np.cumsum(sizes, out=new_go[1:])
    # the nodes taken, in order, and the graph each belongs to
    node_src = np.repeat(go[idx] - new_go[:-1], sizes) + np.arange(new_go[-1])
    ent = ro[node_src + 1] - ro[node_src]
    new_ro = np.zeros(len(node_src) + 1, np.int64)
    np.cumsum(ent, out=new_ro[1:])
    ent_src = np.repeat(ro[node_src] - new_ro[:-1], ent) + np.arange(new_ro[-1])
    # a column id moves with its graph: old id - old graph start + new graph start
    shift = np.repeat(np.repeat(new_go[:-1] - go[idx], sizes), ent)
    return {"graph_offsets": new_go.astype(np.uint32), "row_offsets": new_ro.astype(np.uint32),
            "column_indices": (ci[ent_src] + shift).astype(np.uint32), "node_labels": nl[node_src].astype(np.uint8),
            "edge_labels": el[ent_src].astype(np.uint8)}


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
