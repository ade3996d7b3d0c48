"""Two ranks running the engine over LPT shards of one batch (gloo on CPU for
the final reduction, both ranks on cuda:0: their kernels never wait on each
other).  The reduced totals and the per-pair counts reassembled from the
ranks must equal one engine run over the whole batch and the oracle.  This is
the host side of the multi-GPU path (BMS2_mpi.cpp:78-157, 245, 551) exercised
with the real engine; every call of this run has one GPU, so the ranks share
it."""
import os
import socket

import numpy as np
import pytest

import oracle
from bms2_gb300 import COUNT_ALL, DATA, ORDER_GMCR, QUERY, SEM_EXACT, Context, Graphs, shards, workloads

pytestmark = pytest.mark.gpu

R = 6


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _batch():
    return workloads.make("mol1k", 31, n_data=400, n_queries=20)


def _rank(rank: int, world: int, port: int, out_dir: str) -> None:
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        q, d = _batch()
        a = d.arrays()
        owners = shards.lpt_owners_native(a, world)
        mine = np.nonzero(owners == rank)[0]
        with Context(0) as ctx:
            ctx.load(QUERY, q)
            ctx.load(DATA, Graphs.from_csr(**shards.take_graphs(a, mine)))
            total = ctx.run(R, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
            off, qidx = ctx.gmcr()
            counts = ctx.pair_counts()
            valid = int(ctx.stats()["n_valid_pairs"])
        dense = np.zeros((q.n_graphs, len(mine)), np.uint64)
        for g in range(len(mine)):
            dense[qidx[off[g]:off[g + 1]], g] = counts[off[g]:off[g + 1]]
        tot, val, t = shards.reduce_totals(int(total), valid, 1.0 + rank)
        np.save(os.path.join(out_dir, f"rank{rank}.npy"), dense)
        np.save(os.path.join(out_dir, f"idx{rank}.npy"), mine)
        if rank == 0:
            np.save(os.path.join(out_dir, "reduced.npy"), np.array([tot, val, t]))
    finally:
        dist.destroy_process_group()


def test_two_ranks_of_the_engine_equal_one_run(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    q, d = _batch()
    want = oracle.run_pipeline(q, d, R, keep_steps=False)
    with Context(0) as ctx:
        ctx.load(QUERY, q)
        ctx.load(DATA, d)
        whole = ctx.run(R, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
    assert whole == want.total
    total, valid, t = np.load(tmp_path / "reduced.npy")
    assert int(total) == want.total
    assert int(valid) == len(want.qidx)
    assert t == 2.0  # the slower rank's time
    dense = np.zeros((q.n_graphs, d.n_graphs), np.uint64)
    seen = np.zeros(d.n_graphs, bool)
    for r in range(world):
        idx = np.load(tmp_path / f"idx{r}.npy")
        dense[:, idx] = np.load(tmp_path / f"rank{r}.npy")
        seen[idx] = True
    assert seen.all()
    assert np.array_equal(dense, want.pair_counts_dense(q.n_graphs))
