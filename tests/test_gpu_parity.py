"""CUDA path against the oracle, through the C ABI (libbms.so), bit for bit.

Every stage of the staged pipeline (signatures, filter, each refine step, GMCR,
join) and the fused pipeline are compared with the CPU oracle on the same seeded
inputs; EXACT counts are also compared with the networkx answer key.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from bms2_gb300 import (COUNT_ALL, DATA, FIND_FIRST, ORDER_GMCR, QUERY, SEM_EXACT, SEM_REFERENCE_DFS, BmsError,
                        Graphs, shards, workloads)
from tests.kat_graphs import C, N, O, WILD, chain, line, ring, star

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).with_name("golden") / "nx_small.json"


def graphs(*gs) -> Graphs:
    return Graphs.parse_text("\n".join(line(*g) for g in gs) + "\n")


def mixed_workload(seed=3, n_data=300, n_queries=24):
    """Seeded molecules plus hand-built edge cases appended to both sides."""
    q, d = workloads.make("mol1k", seed, n_data=n_data, n_queries=n_queries)
    extra_q = [ring(6), star(2), ([WILD, C], [(0, 1)]), ([20, C], [(0, 1)]), ([C], []), chain(4)]
    extra_d = [ring(6), star(3), ([O, C], [(0, 1)]), ([20, C, C], [(0, 1), (1, 2)]), ring(5),
               (ring(5)[0], ring(5)[1] + [(0, 1)]),  # repeated CSR entries
               ([C] * 0, [])]  # an empty data graph
    tmp = []
    for g, extra in ((q, extra_q), (d, extra_d)):
        a = g.arrays()
        txt = _text(a) + "".join(line(*x) + "\n" for x in extra)
        tmp.append(Graphs.parse_text(txt))
    return tmp[0], tmp[1]


def _text(a) -> str:
    go, ro, ci, nl, el = (a["graph_offsets"], a["row_offsets"], a["column_indices"], a["node_labels"],
                          a["edge_labels"])
    out = []
    for g in range(len(go) - 1):
        s, e = int(go[g]), int(go[g + 1])
        labels = [int(x) for x in nl[s:e]]
        edges = [(v - s, int(ci[i]) - s) for v in range(s, e) for i in range(int(ro[v]), int(ro[v + 1]))
                 if int(ci[i]) >= v]
        out.append(line(labels, edges) + "\n")
    return "".join(out)


@pytest.fixture(scope="module")
def wl():
    return mixed_workload()


def load(ctx, q, d):
    ctx.load(QUERY, q)
    ctx.load(DATA, d)


@pytest.mark.parametrize("R", [0, 6])
def test_signatures_bit_exact(ctx, wl, R):
    q, d = wl
    load(ctx, q, d)
    ctx.signatures(R)
    for kind, g in ((QUERY, q), (DATA, d)):
        want = oracle.signatures(g.arrays(), R)
        got = ctx.signatures_of(kind, R)
        assert np.array_equal(got["label_gen"], want.label_gen)
        assert np.array_equal(got["path"], want.path)
        assert np.array_equal(got["cycle"], want.cycle)
        assert np.array_equal(got["shells"], want.shells)


@pytest.mark.parametrize("R", [0, 3, 6])
def test_staged_filter_refine_map_bit_exact(ctx, wl, R):
    q, d = wl
    want = oracle.run_pipeline(q, d, R, join=False)
    load(ctx, q, d)
    ctx.signatures(R)
    ctx.filter()
    assert np.array_equal(ctx.candidates(), want.cand_filter)
    for k in range(1, R + 1):
        ctx.refine(k)
        assert np.array_equal(ctx.candidates(), want.cand_steps[k - 1]), f"refine step {k}"
    T = ctx.map()
    off, qidx = ctx.gmcr()
    assert T == len(want.qidx)
    assert np.array_equal(off, want.offsets)
    assert np.array_equal(qidx, want.qidx)


MODES = [(COUNT_ALL, SEM_EXACT), (FIND_FIRST, SEM_EXACT), (COUNT_ALL, SEM_REFERENCE_DFS),
         (FIND_FIRST, SEM_REFERENCE_DFS)]


@pytest.mark.parametrize("mode,sem", MODES)
def test_staged_join_counts_bit_exact(ctx, wl, mode, sem):
    q, d = wl
    R = 2
    want = oracle.run_pipeline(q, d, R, find_first=mode == FIND_FIRST, dfs_literal=sem == SEM_REFERENCE_DFS)
    load(ctx, q, d)
    ctx.signatures(R)
    ctx.filter()
    for k in range(1, R + 1):
        ctx.refine(k)
    ctx.map()
    total = ctx.join(mode, ORDER_GMCR, sem)
    assert np.array_equal(ctx.pair_counts(), want.counts)
    assert total == want.total


@pytest.mark.parametrize("R", [0, 2, 6])
@pytest.mark.parametrize("mode,sem", MODES)
def test_fused_run_bit_exact(ctx, wl, R, mode, sem):
    q, d = wl
    want = oracle.run_pipeline(q, d, R, find_first=mode == FIND_FIRST, dfs_literal=sem == SEM_REFERENCE_DFS)
    load(ctx, q, d)
    total = ctx.run(R, mode, ORDER_GMCR, sem)
    off, qidx = ctx.gmcr()
    assert np.array_equal(off, want.offsets)
    assert np.array_equal(qidx, want.qidx)
    assert np.array_equal(ctx.pair_counts(), want.counts)
    assert total == want.total
    st = ctx.stats()
    assert st["n_valid_pairs"] == len(want.qidx)
    assert st["n_pairs"] == q.n_graphs * d.n_graphs


@pytest.mark.parametrize("seed", [17, 32])
def test_literal_dfs_paths_that_repeat_a_node(ctx, seed):
    # in these seeded workloads the reference DFS's stale clear unmarks a node
    # on the path and the search maps that node a second time (pairs found by a
    # search over seeds); the induced test then has to compare position by
    # position, as isValidMapping_fast_bitwise does (isomorphism.hpp:266-285)
    q, d = workloads.make("mol1k", seed, n_data=60, n_queries=12)
    for mode in (COUNT_ALL, FIND_FIRST):
        want = oracle.run_pipeline(q, d, 0, find_first=mode == FIND_FIRST, dfs_literal=True)
        load(ctx, q, d)
        assert ctx.run(0, mode, ORDER_GMCR, SEM_REFERENCE_DFS) == want.total
        assert np.array_equal(ctx.pair_counts(), want.counts)
        if mode == COUNT_ALL:
            assert np.array_equal(ctx.pair_expansions(), want.expansions)


def test_fused_expansions_match_oracle_exact_plain_order(ctx, wl):
    # oracle expansions count the reference DFS's successful pushes per pair;
    # the engine's bitset DFS makes the same assignments in EXACT mode
    q, d = wl
    want = oracle.run_pipeline(q, d, 2)
    load(ctx, q, d)
    ctx.run(2, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
    got = ctx.pair_expansions()
    counted = want.counts > 0
    assert np.array_equal(got[counted], want.expansions[counted])


@pytest.mark.parametrize("R", [0, 2])
def test_fused_matches_networkx_answer_key(ctx, R):
    g = json.loads(GOLDEN.read_text())
    q = Graphs.parse_text(g["query_text"])
    d = Graphs.parse_text(g["data_text"])
    load(ctx, q, d)
    ctx.run(R, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
    off, qidx = ctx.gmcr()
    counts = ctx.pair_counts()
    dense = np.zeros((g["n_queries"], g["n_data"]), np.uint64)
    for di in range(g["n_data"]):
        for t in range(off[di], off[di + 1]):
            dense[qidx[t], di] = counts[t]
    want = np.zeros_like(dense)
    for qi, di, c in g["counts"]:
        want[qi, di] = c
    assert np.array_equal(dense, want)


def test_large_graphs_two_word_bitsets(ctx):
    # data graphs of 65-128 nodes and queries of 31-64 nodes (beyond the
    # reference's 64/30 domain: generalized semantics, same in the oracle)
    d = Graphs.synth_molecules(60, 5, 0, 0, 0, 65, 128, 1, 4)
    q = Graphs.synth_queries(d, 10, 6, 31, 40)
    q2 = Graphs.synth_queries(d, 10, 7, 3, 10)
    for qq in (q, q2):
        for R in (0, 4):
            want = oracle.run_pipeline(qq, d, R)
            load(ctx, qq, d)
            ctx.run(R, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
            assert np.array_equal(ctx.pair_counts(), want.counts)
            ctx.signatures(R)
            got = ctx.signatures_of(DATA, R)
            assert np.array_equal(got["cycle"], want.d_sigs.cycle)
            assert np.array_equal(got["shells"], want.d_sigs.shells)


def test_join_counted_and_in_row_tests_agree(ctx):
    # Data graphs of 8-120 nodes cover all three record classes (32-bit, one
    # and two 64-bit words).  Molecules have in-degrees <= 4, so the join uses
    # its counted induced test; appending a star with 9 leaves (in-degree 9)
    # switches the whole batch to the in-row test.  Counts and expansions of
    # the shared pairs must not change, and both equal the oracle.
    d = Graphs.synth_molecules(150, 11, 0, 0, 0, 8, 120, 1, 4)
    q = Graphs.synth_queries(d, 16, 12, 3, 12)
    d_hub = Graphs.parse_text(_text(d.arrays()) + line(*star(9)) + "\n")
    results = []
    for dd in (d, d_hub):
        want = oracle.run_pipeline(q, dd, 2)
        load(ctx, q, dd)
        ctx.run(2, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
        counts, exps = ctx.pair_counts(), ctx.pair_expansions()
        assert np.array_equal(counts, want.counts)
        results.append((counts, exps))
    n = len(results[0][0])
    assert n > 0 and results[0][0].sum() > 0
    assert np.array_equal(results[1][0][:n], results[0][0])
    assert np.array_equal(results[1][1][:n], results[0][1])


@pytest.mark.parametrize("budget,cap", [(1, 0), (3, 0), (64, 0), (2, 16), (1, 1)])
def test_join_subtree_splitting_is_exact(ctx, budget, cap):
    # A search passing `budget` expansions hands its unexplored subtrees to the
    # next round (cap: subtree buffer entries; tiny caps force the buffer-full
    # path, where a search keeps its work).  Counts and per-pair expansions must
    # equal the unsplit join and the oracle, in both induced-test variants and
    # in find-first mode.
    from bms2_gb300.native import OPT_SPLIT_BUDGET, OPT_SUBTREE_CAP
    d = Graphs.synth_molecules(120, 21, 0, 0, 0, 8, 120, 1, 4)
    q = Graphs.synth_queries(d, 12, 22, 3, 12)
    d_hub = Graphs.parse_text(_text(d.arrays()) + line(*star(9)) + "\n")
    try:
        for dd in (d, d_hub):
            load(ctx, q, dd)
            for mode in (COUNT_ALL, FIND_FIRST):
                want = oracle.run_pipeline(q, dd, 2, find_first=mode == FIND_FIRST)
                ctx.set_option(OPT_SPLIT_BUDGET, 0)
                ctx.run(2, mode, ORDER_GMCR, SEM_EXACT)
                base_counts, base_exps = ctx.pair_counts(), ctx.pair_expansions()
                ctx.set_option(OPT_SPLIT_BUDGET, budget)
                ctx.set_option(OPT_SUBTREE_CAP, cap)
                total = ctx.run(2, mode, ORDER_GMCR, SEM_EXACT)
                assert np.array_equal(ctx.pair_counts(), want.counts)
                assert total == want.total
                if mode == COUNT_ALL:
                    assert np.array_equal(base_counts, want.counts)
                    assert np.array_equal(ctx.pair_expansions(), base_exps)
    finally:
        ctx.set_option(OPT_SPLIT_BUDGET, 1024)
        ctx.set_option(OPT_SUBTREE_CAP, 0)


def test_cuda_graph_replay_equals_eager(ctx):
    # bms_run captures its device work as a CUDA graph on the second run with
    # unchanged inputs and settings and replays it afterwards; every replay must
    # give the eager results, and any change (option, reload) must be honoured.
    from bms2_gb300.native import OPT_CUDA_GRAPH, OPT_SPLIT_BUDGET
    q, d = workloads.make("mol1k", 5, n_data=400, n_queries=20)
    q2, d2 = workloads.make("mol1k", 6, n_data=250, n_queries=15)
    want = oracle.run_pipeline(q, d, 3)
    want2 = oracle.run_pipeline(q2, d2, 3)

    def run_all(sem=SEM_EXACT):
        total = ctx.run(3, COUNT_ALL, ORDER_GMCR, sem)
        return total, ctx.pair_counts(), ctx.pair_expansions(), ctx.stats()["kernel_launches"]

    try:
        ctx.set_option(OPT_CUDA_GRAPH, 0)
        load(ctx, q, d)
        eager = run_all()
        assert eager[0] == want.total and np.array_equal(eager[1], want.counts)
        ctx.set_option(OPT_CUDA_GRAPH, 1)
        for _ in range(4):  # eager, capture + launch, replay, replay
            got = run_all()
            assert got[0] == eager[0]
            assert np.array_equal(got[1], eager[1]) and np.array_equal(got[2], eager[2])
            assert got[3] == eager[3]
        ctx.set_option(OPT_SPLIT_BUDGET, 2)  # a changed option is a new plan
        for _ in range(3):
            got = run_all()
            assert np.array_equal(got[1], eager[1]) and np.array_equal(got[2], eager[2])
        ctx.set_option(OPT_SPLIT_BUDGET, 1024)
        load(ctx, q2, d2)  # new inputs of other sizes
        for _ in range(3):
            got = run_all()
            assert got[0] == want2.total and np.array_equal(got[1], want2.counts)
        want_lit = oracle.run_pipeline(q2, d2, 3, dfs_literal=True)
        for _ in range(3):
            got = run_all(SEM_REFERENCE_DFS)
            assert np.array_equal(got[1], want_lit.counts)
    finally:
        ctx.set_option(OPT_CUDA_GRAPH, 1)
        ctx.set_option(OPT_SPLIT_BUDGET, 1024)


@pytest.mark.parametrize("batch", [1, 37, 500, 0])
def test_batched_run_equals_one_run(ctx, batch):
    # the data side in slices of `batch` graphs (0: the reference's 100,000,
    # i.e. one slice): the total and every query's matches equal the oracle
    # over the whole batch, in count-all and find-first modes
    d = Graphs.synth_molecules(240, 51, 0, 0, 0, 6, 100, 1, 4)
    q = Graphs.synth_queries(d, 12, 52, 3, 10)
    for mode in (COUNT_ALL, FIND_FIRST):
        want = oracle.run_pipeline(q, d, 2, find_first=mode == FIND_FIRST)
        dense = want.pair_counts_dense(q.n_graphs)
        ctx.load(QUERY, q)
        total, per_query = ctx.run_batches(d, batch, 2, mode, ORDER_GMCR, SEM_EXACT)
        assert total == want.total
        assert np.array_equal(per_query, dense.sum(axis=1).astype(np.uint64))
    # the context keeps the last slice: its pairs equal a run over that slice
    last = d.n_graphs - (d.n_graphs % batch or batch) if batch else 0
    tail = Graphs.from_csr(**shards.take_graphs(d.arrays(), np.arange(last, d.n_graphs)))
    assert ctx.stats()["n_data_graphs"] == tail.n_graphs
    assert np.array_equal(ctx.pair_counts(), oracle.run_pipeline(q, tail, 2, find_first=True).counts)


@pytest.mark.parametrize("window", [1, 53, 0])
def test_resident_windows_equal_one_run(ctx, window):
    # the data batch stays in HBM and windows of it are views: totals and
    # per-query matches equal the oracle, in count-all and find-first modes;
    # loading an ordinary data side afterwards replaces the views
    d = Graphs.synth_molecules(230, 71, 0, 0, 0, 6, 110, 1, 4)
    q = Graphs.synth_queries(d, 11, 72, 3, 10)
    ctx.load(QUERY, q)
    ctx.load_resident(d)
    for mode in (COUNT_ALL, FIND_FIRST):
        want = oracle.run_pipeline(q, d, 2, find_first=mode == FIND_FIRST)
        total, per_query = ctx.run_resident(window, 2, mode, ORDER_GMCR, SEM_EXACT)
        assert total == want.total
        assert np.array_equal(per_query, want.pair_counts_dense(q.n_graphs).sum(axis=1).astype(np.uint64))
    res, bat = ctx.run_resident(window, 2), ctx.run_batches(d, window, 2)
    assert res[0] == bat[0] and np.array_equal(res[1], bat[1])
    small = Graphs.from_csr(**shards.take_graphs(d.arrays(), np.arange(40)))
    ctx.load(DATA, small)
    assert ctx.run(2, COUNT_ALL, ORDER_GMCR, SEM_EXACT) == oracle.run_pipeline(q, small, 2).total
    total, _ = ctx.run_resident(window, 2)  # the resident batch is still there
    assert total == oracle.run_pipeline(q, d, 2).total


@pytest.mark.parametrize("window", [37, 0])
def test_resident_signatures_computed_once(ctx, window):
    # BMS_OPT_RESIDENT_SIGNATURES: the data side's signatures are computed once
    # for the whole resident batch; later windows and calls reuse them (no
    # signature time), with the same results; R and a new batch recompute
    from bms2_gb300 import OPT_RESIDENT_SIGNATURES

    d = Graphs.synth_molecules(260, 81, 0, 0, 0, 6, 110, 1, 4)
    q = Graphs.synth_queries(d, 12, 82, 3, 10)
    ctx.load(QUERY, q)
    ctx.load_resident(d)
    ctx.set_option(OPT_RESIDENT_SIGNATURES, 1)
    try:
        for R in (2, 6, 2):
            want = oracle.run_pipeline(q, d, R)
            dense = want.pair_counts_dense(q.n_graphs).sum(axis=1).astype(np.uint64)
            for call in range(2):
                total, per_query = ctx.run_resident(window, R)
                assert total == want.total and np.array_equal(per_query, dense)
            # the second call reused every window's signatures
            assert ctx.stats()["ms_signatures"] < 1.0
        d2 = Graphs.synth_molecules(150, 83, 0, 0, 0, 6, 110, 1, 4)
        ctx.load_resident(d2)
        total, _ = ctx.run_resident(window, 2)
        assert total == oracle.run_pipeline(q, d2, 2).total
    finally:
        ctx.set_option(OPT_RESIDENT_SIGNATURES, 0)
    total, _ = ctx.run_resident(window, 2)
    assert total == oracle.run_pipeline(q, d2, 2).total


def test_embeddings_equal_the_oracle(ctx):
    # every embedding of a pair (not only the count), sorted, against the
    # oracle's enumeration (itself pinned against networkx); graphs of up to
    # 110 nodes, queries of up to 10
    d = Graphs.synth_molecules(90, 81, 0, 0, 0, 6, 110, 1, 4)
    q = Graphs.synth_queries(d, 10, 82, 3, 10)
    want = oracle.run_pipeline(q, d, 2)
    load(ctx, q, d)
    ctx.run(2, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
    assert np.array_equal(ctx.pair_counts(), want.counts)
    picked = [t for t in range(len(want.counts)) if 0 < want.counts[t] <= 3000][:120]
    assert len(picked) >= 40
    for t in picked:
        got = ctx.embeddings(t)
        assert np.array_equal(got, oracle.pair_embeddings(q, d, want, t)), t
    first = ctx.embeddings(picked[0], max_embeddings=1)
    assert np.array_equal(first, ctx.embeddings(picked[0])[:1])
    zero = [t for t in range(len(want.counts)) if want.counts[t] == 0]
    if zero:
        assert ctx.embeddings(zero[0]).shape[0] == 0
    ctx.run(2, FIND_FIRST, ORDER_GMCR, SEM_EXACT)
    with pytest.raises(BmsError):
        ctx.embeddings(picked[0])


def test_pinned_batch_gives_the_same_results(ctx):
    d = Graphs.synth_molecules(300, 61, 0, 0, 0, 6, 80, 1, 4)
    q = Graphs.synth_queries(d, 10, 62, 3, 9)
    ctx.load(QUERY, q)
    plain = ctx.run_batches(d, 64, 2)
    d.pin()
    d.pin()  # pinning twice is a no-op
    pinned = ctx.run_batches(d, 64, 2)
    d.unpin()
    assert plain[0] == pinned[0] and np.array_equal(plain[1], pinned[1])
    d.pin()  # freed while pinned: the ranges are released with the batch
    del d


def test_many_entries_graph_reads_rows_from_global_memory(ctx):
    # a 127-leaf star with every edge listed 5 times: 1270 CSR entries (more
    # than the 1024 staged in shared memory), repeated entries, 128 nodes
    labels = [C] + [C if i % 4 else N for i in range(127)]
    edges = [(0, i + 1) for i in range(127) for _ in range(5)]
    d = graphs((labels, edges), ring(6))
    q = graphs(star(2), chain(3), ([N, C], [(0, 1)]), ([C, N, C], [(0, 1), (0, 2)]))
    for R in (0, 2):
        want = oracle.run_pipeline(q, d, R)
        load(ctx, q, d)
        ctx.run(R, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
        assert np.array_equal(ctx.pair_counts(), want.counts)
        ctx.signatures(R)
        got = ctx.signatures_of(DATA, R)
        for k in ("label_gen", "path", "cycle", "shells"):
            assert np.array_equal(got[k], getattr(want.d_sigs, k)), k
    assert want.counts.max() == 95 * 94  # ordered pairs of the 95 carbon leaves


def test_mol100k_sample_fused_equals_staged_equals_oracle(ctx):
    q, d = workloads.make("mol100k", 1, n_data=3000, n_queries=60)
    R = 6
    want = oracle.run_pipeline(q, d, R, keep_steps=False)
    load(ctx, q, d)
    total = ctx.run(R, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
    assert np.array_equal(ctx.pair_counts(), want.counts)
    assert total == want.total
    ctx.signatures(R)
    ctx.filter()
    for k in range(1, R + 1):
        ctx.refine(k)
    ctx.map()
    assert ctx.join(COUNT_ALL, ORDER_GMCR, SEM_EXACT) == total


def test_runs_are_deterministic(ctx, wl):
    q, d = wl
    load(ctx, q, d)
    a = ctx.run(6, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
    ca = ctx.pair_counts().copy()
    b = ctx.run(6, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
    assert a == b and np.array_equal(ca, ctx.pair_counts())


def test_invalid_column_is_reported(ctx):
    q = graphs(chain(2))
    ctx.load(QUERY, q)
    ctx.load_csr(DATA, [0, 2], [0, 1, 2], [1, 5], [8, 8])
    with pytest.raises(BmsError) as e:
        ctx.run(1)
    assert e.value.status == -1


def test_oversized_graph_is_rejected_at_load(ctx):
    big = graphs(chain(129))
    with pytest.raises(BmsError) as e:
        ctx.load(DATA, big)
    assert e.value.status == -6
    with pytest.raises(BmsError):
        ctx.load(QUERY, graphs(chain(65)))


def test_stage_order_is_enforced(ctx, wl):
    q, d = wl
    load(ctx, q, d)
    with pytest.raises(BmsError) as e:
        ctx.filter()
    assert e.value.status == -5
    with pytest.raises(BmsError):
        ctx.map()


def test_expansion_budget_marks_pairs_incomplete(ctx):
    q = graphs(chain(8))
    d = graphs(*[chain(40) for _ in range(4)])
    load(ctx, q, d)
    ctx.set_expansion_budget(5)
    try:
        with pytest.raises(BmsError) as e:
            ctx.run(0, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
        assert e.value.status == -8
        assert ctx.stats()["n_incomplete"] > 0
        assert ctx.pair_status().max() == 1
    finally:
        ctx.set_expansion_budget(0)
    full = ctx.run(0, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
    assert full == oracle.run_pipeline(q, d, 0).total


@pytest.mark.parametrize("split", [(0, 0, 0), (1, 1, 1), (1, 0, 1), (0, 1, 0)])
def test_task_granularity_does_not_change_counts(ctx, split):
    # per size bucket: one task per pair (0) or per (pair, root) (1); data
    # graphs of 8-120 nodes fill all three buckets
    d = Graphs.synth_molecules(150, 31, 0, 0, 0, 8, 120, 1, 4)
    q = Graphs.synth_queries(d, 14, 32, 3, 12)
    want = oracle.run_pipeline(q, d, 3)
    load(ctx, q, d)
    sched = ctx.schedule()
    try:
        ctx.set_schedule({**sched, "split_depth": list(split) + [0]})
        assert ctx.run(3, COUNT_ALL, ORDER_GMCR, SEM_EXACT) == want.total
        assert np.array_equal(ctx.pair_counts(), want.counts)
        assert ctx.run(3, FIND_FIRST, ORDER_GMCR, SEM_EXACT) == int((want.counts > 0).sum())
    finally:
        ctx.set_schedule(sched)


@pytest.mark.parametrize("lanes,words", [(1, 32), (2, 64), (4, 32), (8, 64), (32, 64), (32, 32)])
def test_lanes_per_pair_and_word_width_keep_counts(ctx, lanes, words):
    # lanes per pair (lane g of a group takes the roots of rank g mod lanes)
    # and the search sets' machine word change the schedule, never a count or
    # an expansion; all three size classes, count-all and find-first
    # (expansions are compared with the default schedule's: pairs that the
    # fused filter's label screen proves empty are never searched, so their
    # expansions are 0 where the oracle's search spends a few)
    d = Graphs.synth_molecules(300, 43, 0, 0, 0, 5, 120, 1, 4)
    q = Graphs.synth_queries(d, 14, 44, 3, 16)
    load(ctx, q, d)
    before = ctx.schedule()
    try:
        base = dict(before)
        base["split_depth"] = [0, 0, 0, 0]
        ctx.set_schedule(base)
        ctx.run(2, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
        base_exps = ctx.pair_expansions().copy()
        s = dict(base)
        s["lanes_per_pair"] = [lanes] * 3 + [1]
        s["word_bits"] = [32, words, words, 64]
        ctx.set_schedule(s)
        for mode in (COUNT_ALL, FIND_FIRST):
            want = oracle.run_pipeline(q, d, 2, find_first=mode == FIND_FIRST)
            total = ctx.run(2, mode, ORDER_GMCR, SEM_EXACT)
            assert total == want.total
            assert np.array_equal(ctx.pair_counts(), want.counts)
            if mode == COUNT_ALL:
                assert np.array_equal(ctx.pair_expansions(), base_exps)
    finally:
        ctx.set_schedule(before)


def test_autotune_picks_a_valid_schedule_and_keeps_counts(ctx):
    d = Graphs.synth_molecules(400, 41, 0, 0, 0, 8, 120, 1, 4)
    q = Graphs.synth_queries(d, 16, 42, 3, 14)
    want = oracle.run_pipeline(q, d, 2)
    load(ctx, q, d)
    before = ctx.schedule()
    try:
        s = ctx.autotune(2)
        assert s["max_data_nodes"][:3] == [32, 64, 128] and s["word_bits"][0] == 32
        for k in range(3):
            assert s["word_bits"][k] in (32, 64)
            assert s["lanes_per_pair"][k] in (1, 2, 4, 8, 32)
            assert s["blocks_per_sm"][k] in (2, 3, 4, 6, 8, 12)
            assert s["warps_per_block"][k] in (2, 4, 8)
            assert s["steps"][k] in (16, 32, 64)
            assert s["refill"][k] in (1, 2, 4, 8)
            assert s["split_budget"][k] in (0, 256, 1024, 4096)
            assert s["split_depth"][k] in (0, 1)
            assert s["ms"][k] >= 0.0
        assert ctx.schedule() == s
        assert ctx.run(2, COUNT_ALL, ORDER_GMCR, SEM_EXACT) == want.total
        assert np.array_equal(ctx.pair_counts(), want.counts)
    finally:
        ctx.set_schedule(before)


@pytest.mark.parametrize("kernel", [0, 1])
@pytest.mark.parametrize("R", [0, 6])
def test_both_fused_filter_kernels_bit_exact(ctx, wl, kernel, R):
    from bms2_gb300.native import OPT_FILTER_KERNEL

    q, d = wl
    want = oracle.run_pipeline(q, d, R)
    load(ctx, q, d)
    try:
        ctx.set_option(OPT_FILTER_KERNEL, kernel)
        total = ctx.run(R, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
        off, qidx = ctx.gmcr()
        assert np.array_equal(off, want.offsets) and np.array_equal(qidx, want.qidx)
        assert np.array_equal(ctx.pair_counts(), want.counts) and total == want.total
    finally:
        ctx.set_option(OPT_FILTER_KERNEL, 0)


def test_sliced_filter_slow_clauses(ctx):
    # labels >= 16, degree > 16 and cycle counts > 8 fall outside the mask table
    big = ([C] + [30] * 20, [(0, i + 1) for i in range(20)])  # degree-20 centre, label-30 leaves
    kq = ([C] + list(range(16, 33)), [(0, i + 1) for i in range(17)])  # degree 17, leaves labelled 16..32
    kd = ([C] + list(range(16, 34)), [(0, i + 1) for i in range(18)])  # one embedding of kq
    k8 = ([C] * 8, [(i, j) for i in range(8) for j in range(i + 1, 8)])  # 420 5-cycles through each node
    q = graphs(([C, 30], [(0, 1)]), kq, k8, ([30, C, 30], [(0, 1), (1, 2)]))
    d = graphs(big, k8, kd, ring(6))
    for R in (0, 2):
        want = oracle.run_pipeline(q, d, R)
        load(ctx, q, d)
        assert ctx.run(R, COUNT_ALL, ORDER_GMCR, SEM_EXACT) == want.total
        assert np.array_equal(ctx.pair_counts(), want.counts)
    assert want.total == 20 + 20 * 19 + 40320 + 1 + 1  # the [C,30] edge also sits once in kd


def test_results_into_page_locked_memory(ctx, wl):
    # results read into page-locked memory (aligned and at an 8-byte offset)
    # equal those read into ordinary memory
    import ctypes

    torch = pytest.importorskip("torch")
    from bms2_gb300 import native

    q, d = wl
    load(ctx, q, d)
    ctx.run(2, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
    want = ctx.pair_counts()
    T = len(want)
    buf = torch.zeros(8 * T + 24, dtype=torch.uint8).pin_memory()
    for off in (0, 8):
        buf.zero_()
        ptr = ctypes.cast(buf.data_ptr() + off, native._u64p)
        native._check(native.lib().bms_get_pair_counts(ctx.handle, ptr, T), ctx.handle)
        got = buf.numpy()[off:off + 8 * T].view(np.uint64)
        assert np.array_equal(got, want)
