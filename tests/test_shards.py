"""Data-graph shards across ranks, on CPU: LPT assignment, shard extraction,
and two gloo ranks whose reduced totals and reassembled per-pair counts equal
one process over the whole batch (the oracle computes every rank's pairs)."""
import os
import socket

import numpy as np
import pytest

import oracle
from bms2_gb300 import shards, workloads


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_lpt_owners_follow_the_reference_rule():
    # costs 9, 7, 6, 5, 4 on 2 ranks: 9->0, 7->1, 6->1 (7 < 9), 5->0 (9 < 13), 4->1 (13 < 14)
    owners = shards.lpt_owners(np.array([4.0, 9.0, 6.0, 5.0, 7.0]), 2)
    assert owners.tolist() == [1, 0, 1, 0, 1]
    # ties keep the input order and go to the lowest rank
    assert shards.lpt_owners(np.array([1.0, 1.0, 1.0]), 2).tolist() == [0, 1, 0]
    with pytest.raises(ValueError):
        shards.lpt_owners(np.array([1.0]), 0)


def test_graph_costs_are_nodes_squared_plus_edges():
    q, d = workloads.make("mol1k", 3, n_data=20, n_queries=2)
    a = d.arrays()
    go, ro = a["graph_offsets"].astype(np.int64), a["row_offsets"].astype(np.int64)
    n = go[1:] - go[:-1]
    e = (ro[go[1:]] - ro[go[:-1]]) // 2
    assert np.array_equal(shards.graph_costs(a), np.maximum(n * n + e, 1).astype(np.float64))


def test_take_graphs_round_trip():
    _, d = workloads.make("mol1k", 4, n_data=30, n_queries=2)
    a = d.arrays()
    idx = np.array([5, 0, 29, 7])
    sub = shards.take_graphs(a, idx)
    go = a["graph_offsets"]
    for j, g in enumerate(idx):
        s, e = int(go[g]), int(go[g + 1])
        ss, se = int(sub["graph_offsets"][j]), int(sub["graph_offsets"][j + 1])
        assert np.array_equal(sub["node_labels"][ss:se], a["node_labels"][s:e])
        rows = a["row_offsets"][s:e + 1] - a["row_offsets"][s]
        assert np.array_equal(sub["row_offsets"][ss:se + 1] - sub["row_offsets"][ss], rows)
        cols = a["column_indices"][a["row_offsets"][s]:a["row_offsets"][e]] - s
        assert np.array_equal(sub["column_indices"][sub["row_offsets"][ss]:sub["row_offsets"][se]] - ss, cols)
    assert len(shards.take_graphs(a, np.array([], dtype=np.int64))["graph_offsets"]) == 1


def _rank(rank: int, world: int, port: int, out_dir: str) -> None:
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        q, d = workloads.make("mol1k", 11, n_data=60, n_queries=8)
        a = d.arrays()
        owners = shards.lpt_owners(shards.graph_costs(a), world)
        mine = np.nonzero(owners == rank)[0]
        res = oracle.run_pipeline(q, shards.take_graphs(a, mine), 2)
        dense = res.pair_counts_dense(q.n_graphs)
        total, valid, t = shards.reduce_totals(int(res.counts.sum()), int(len(res.qidx)), 0.5 + rank)
        np.save(os.path.join(out_dir, f"rank{rank}.npy"), dense)
        np.save(os.path.join(out_dir, f"idx{rank}.npy"), mine)
        if rank == 0:
            np.save(os.path.join(out_dir, "reduced.npy"), np.array([total, valid, t]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_equal_one_process(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    q, d = workloads.make("mol1k", 11, n_data=60, n_queries=8)
    whole = oracle.run_pipeline(q, d, 2)
    total, valid, t = np.load(tmp_path / "reduced.npy")
    assert int(total) == int(whole.counts.sum())
    assert int(valid) == len(whole.qidx)
    assert t == 1.5  # the slower rank's time
    dense = np.zeros((q.n_graphs, d.n_graphs), np.uint64)
    seen = np.zeros(d.n_graphs, bool)
    for r in range(world):
        idx = np.load(tmp_path / f"idx{r}.npy")
        dense[:, idx] = np.load(tmp_path / f"rank{r}.npy")
        seen[idx] = True
    assert seen.all()
    assert np.array_equal(dense, whole.pair_counts_dense(q.n_graphs))


def test_native_lpt_equals_the_restatement():
    # bms_shard_lpt (libbms, host code) and lpt_owners give the same owners,
    # ties included (many equal costs among small molecules)
    for n, world in ((1, 3), (500, 2), (3000, 8)):
        _, d = workloads.make("mol1k", 7, n_data=n, n_queries=2)
        a = d.arrays()
        assert np.array_equal(shards.lpt_owners_native(a, world), shards.lpt_owners(shards.graph_costs(a), world))
