"""The engine against the oracle on a sample with the shape of the 1M-graph
batched workload: log-normal data graphs of 5-120 atoms (all three size
classes of the join: <= 32, 33-64 and 65-128 nodes) and queries of 3-40 nodes,
R = 6, with CUDA-graph capture and replay and with subtree splitting forced
on, in EXACT and REFERENCE_DFS semantics, count-all and find-first.  Every
per-pair count and every GMCR row is compared, not only totals."""
import numpy as np
import pytest

import oracle
from bms2_gb300 import (COUNT_ALL, DATA, FIND_FIRST, ORDER_GMCR, QUERY, SEM_EXACT, SEM_REFERENCE_DFS, workloads)
from bms2_gb300.native import OPT_CUDA_GRAPH, OPT_SPLIT_BUDGET

pytestmark = pytest.mark.gpu

R = 6


@pytest.fixture(scope="module")
def sample():
    q, d = workloads.make("mol1m", 4242, n_data=20000, n_queries=200)
    da, qa = d.arrays(), q.arrays()
    dsz = np.diff(da["graph_offsets"].astype(np.int64))
    qsz = np.diff(qa["graph_offsets"].astype(np.int64))
    # the shape this file is about: every size class and long queries present
    assert (dsz <= 32).sum() > 0 and ((dsz > 32) & (dsz <= 64)).sum() > 0 and (dsz > 64).sum() > 0
    assert qsz.max() > 30 and qsz.min() <= 5
    exact = oracle.run_pipeline(qa, da, R, keep_steps=False)
    first = oracle.run_pipeline(qa, da, R, find_first=True, keep_steps=False)
    literal = oracle.run_pipeline(qa, da, R, dfs_literal=True, keep_steps=False)
    return q, d, exact, first, literal


def _check(ctx, want, total):
    off, qidx = ctx.gmcr()
    assert np.array_equal(off, want.offsets)
    assert np.array_equal(qidx, want.qidx)
    assert np.array_equal(ctx.pair_counts(), want.counts)
    assert total == want.total


def test_exact_count_all_eager_capture_replay(ctx, sample):
    q, d, exact, _, _ = sample
    ctx.load(QUERY, q)
    ctx.load(DATA, d)
    assert exact.total > 0
    exps = None
    for _ in range(3):  # eager, capture + launch, replay
        total = ctx.run(R, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
        _check(ctx, exact, total)
        if exps is None:
            exps = ctx.pair_expansions()
            assert np.array_equal(exps, exact.expansions)
        else:
            assert np.array_equal(ctx.pair_expansions(), exps)


def test_exact_find_first(ctx, sample):
    q, d, exact, first, _ = sample
    ctx.load(QUERY, q)
    ctx.load(DATA, d)
    for _ in range(2):
        total = ctx.run(R, FIND_FIRST, ORDER_GMCR, SEM_EXACT)
        _check(ctx, first, total)
    assert np.array_equal(first.counts, (exact.counts > 0).astype(np.uint64))


@pytest.mark.parametrize("budget", [8, 200])
def test_subtree_splitting_forced(ctx, sample, budget):
    q, d, exact, _, _ = sample
    ctx.load(QUERY, q)
    ctx.load(DATA, d)
    try:
        ctx.set_option(OPT_SPLIT_BUDGET, budget)
        for _ in range(2):
            total = ctx.run(R, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
            _check(ctx, exact, total)
            assert np.array_equal(ctx.pair_expansions(), exact.expansions)
    finally:
        ctx.set_option(OPT_SPLIT_BUDGET, 1024)


def test_reference_dfs_equals_the_literal_oracle(ctx, sample):
    q, d, _, _, literal = sample
    ctx.load(QUERY, q)
    ctx.load(DATA, d)
    for graph in (0, 1, 1):
        ctx.set_option(OPT_CUDA_GRAPH, graph)
        total = ctx.run(R, COUNT_ALL, ORDER_GMCR, SEM_REFERENCE_DFS)
        _check(ctx, literal, total)
    ctx.set_option(OPT_CUDA_GRAPH, 1)
