"""Clustered join (BMS_OPT_USE_CS, the reference driver's --use-cs) on the GPU
against the oracle's restatement, bit for bit: per-pair counts, totals,
prototype matches and (count-all) expansions, through the C ABI."""
import numpy as np
import pytest

import oracle
from bms2_gb300 import (COUNT_ALL, DATA, FIND_FIRST, OPT_CUDA_GRAPH, OPT_USE_CS, ORDER_GMCR, ORDER_LEARNED, QUERY,
                        SEM_EXACT, SEM_REFERENCE_DFS, BmsError, Graphs, workloads)
from tests.kat_graphs import C, chain, line, star

pytestmark = pytest.mark.gpu

MODES = [(COUNT_ALL, SEM_EXACT), (FIND_FIRST, SEM_EXACT), (COUNT_ALL, SEM_REFERENCE_DFS),
         (FIND_FIRST, SEM_REFERENCE_DFS)]


def graphs(*gs) -> Graphs:
    return Graphs.parse_text("\n".join(line(*g) for g in gs) + "\n")


@pytest.fixture
def cs(ctx):
    ctx.set_option(OPT_USE_CS, 1)
    yield ctx
    ctx.set_option(OPT_USE_CS, 0)


@pytest.fixture(scope="module")
def cluster():
    # data graphs of 6..100 atoms (all three size classes); a prototype of 3..5
    # nodes common enough to match in many graphs
    d = Graphs.synth_molecules(600, 21, 0, 0, 0, 6, 100, 1, 4)
    return workloads.make_cluster(d, 40, 21, proto_nodes=(3, 5)), d


def check(ctx, q, d, R, mode, sem, staged=False):
    want = oracle.run_pipeline(q, d, R, find_first=mode == FIND_FIRST, dfs_literal=sem == SEM_REFERENCE_DFS,
                               cs=True)
    ctx.load(QUERY, q)
    ctx.load(DATA, d)
    if staged:
        ctx.signatures(R)
        ctx.filter()
        for k in range(1, R + 1):
            ctx.refine(k)
        ctx.map()
        total = ctx.join(mode, ORDER_GMCR, sem)
    else:
        total = ctx.run(R, mode, ORDER_GMCR, sem)
    off, qidx = ctx.gmcr()
    assert np.array_equal(off, want.offsets) and np.array_equal(qidx, want.qidx)
    assert np.array_equal(ctx.pair_counts(), want.counts)
    assert total == want.total
    st = ctx.stats()
    assert st["n_partial_matches"] == want.n_partial
    if mode == COUNT_ALL:
        assert np.array_equal(ctx.pair_expansions(), want.expansions)
        assert st["expansions"] == int(want.expansions.sum()) + want.partial_exps
    return want


@pytest.mark.parametrize("R", [0, 2, 6])
@pytest.mark.parametrize("mode,sem", MODES)
def test_fused_clustered_join_bit_exact(cs, cluster, R, mode, sem):
    q, d = cluster
    want = check(cs, q, d, R, mode, sem)
    assert want.n_partial > 0 and want.total > 0


@pytest.mark.parametrize("R", [2, 6])
@pytest.mark.parametrize("mode,sem", MODES)
def test_ring_prototype_cluster_bit_exact(cs, R, mode, sem):
    d = Graphs.synth_molecules(800, 23, 0, 0, 0, 6, 110, 1, 4)
    c = workloads.make_cluster(d, 30, 23, proto="ring")
    want = check(cs, c, d, R, mode, sem)
    assert want.n_partial > 0 and want.total > 0


@pytest.mark.parametrize("mode,sem", MODES)
def test_staged_clustered_join_bit_exact(cs, cluster, mode, sem):
    q, d = cluster
    check(cs, q, d, 2, mode, sem, staged=True)


def with_one_node_prototype(c: Graphs) -> Graphs:
    """The cluster behind a new prototype: one node labelled like every
    member's first node (the old prototype becomes a member)."""
    a = c.arrays()
    lab = int(a["node_labels"][0])
    return Graphs.from_csr(np.concatenate([[0], a["graph_offsets"] + 1]),
                           np.concatenate([[0], a["row_offsets"]]), a["column_indices"] + 1,
                           np.concatenate([[lab], a["node_labels"]]), a["edge_labels"])


@pytest.mark.parametrize("staged", [False, True])
def test_single_node_prototype(cs, cluster, staged):
    # the prototype's own pair is never valid (gmcr.hpp:64): its matches come
    # from the one-node candidate test (fused) or the dense matrix (staged)
    c, d = cluster
    q = with_one_node_prototype(c)
    for mode, sem in MODES:
        for R in (0, 2, 6):
            want = check(cs, q, d, R, mode, sem, staged=staged)
            assert want.n_partial > 0


def test_members_smaller_than_or_equal_to_the_prototype(cs):
    q = graphs(chain(3), chain(2), chain(3))
    d = graphs(star(3), chain(4), star(4))
    for mode, sem in MODES:
        check(cs, q, d, 0, mode, sem)


def test_hand_derived_counts(cs):
    q, d = graphs(([C], []), star(3)), graphs(star(4))
    cs.load(QUERY, q)
    cs.load(DATA, d)
    assert cs.run(0, COUNT_ALL, ORDER_GMCR, SEM_EXACT) == 24
    assert cs.stats()["n_partial_matches"] == 5
    assert cs.run(0, COUNT_ALL, ORDER_GMCR, SEM_REFERENCE_DFS) == 8


def test_exact_clustered_equals_plain_join_at_two_refine_steps(ctx, cluster):
    q, d = cluster
    ctx.load(QUERY, q)
    ctx.load(DATA, d)
    plain = ctx.run(2, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
    pc = ctx.pair_counts()
    ctx.set_option(OPT_USE_CS, 1)
    try:
        assert ctx.run(2, COUNT_ALL, ORDER_GMCR, SEM_EXACT) == plain
        assert np.array_equal(ctx.pair_counts(), pc)
    finally:
        ctx.set_option(OPT_USE_CS, 0)


def test_cuda_graph_replay_and_batches(cs, cluster):
    q, d = cluster
    want = oracle.run_pipeline(q, d, 6, cs=True)
    cs.load(QUERY, q)
    cs.load(DATA, d)
    cs.set_option(OPT_CUDA_GRAPH, 1)
    for _ in range(3):  # eager, capture, replay
        assert cs.run(6, COUNT_ALL, ORDER_GMCR, SEM_EXACT) == want.total
        assert np.array_equal(cs.pair_counts(), want.counts)
        assert cs.stats()["n_partial_matches"] == want.n_partial
    total, per_query = cs.run_batches(d, 97, 6, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
    assert total == want.total
    assert np.array_equal(per_query, want.pair_counts_dense(q.n_graphs).sum(axis=1).astype(np.uint64))


def test_learned_order_is_refused(cs, cluster):
    q, d = cluster
    cs.load(QUERY, q)
    cs.load(DATA, d)
    with pytest.raises(BmsError):
        cs.run(2, COUNT_ALL, ORDER_LEARNED, SEM_EXACT)
