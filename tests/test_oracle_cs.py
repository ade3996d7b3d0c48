"""The clustered join of the oracle (the reference driver's --use-cs,
BMS2.cpp:218-296; isomorphism.hpp:756-977, 1021-1178): hand-derived known
answers, and the properties that pin it against the plain join."""
import numpy as np
import pytest

import oracle
from bms2_gb300 import Graphs, workloads
from tests.kat_graphs import C, chain, line, star


def graphs(*gs) -> Graphs:
    return Graphs.parse_text("\n".join(line(*g) for g in gs) + "\n")


def run(q, d, R=0, **kw):
    return oracle.run_pipeline(graphs(*q), graphs(*d), R, cs=True, **kw)


def test_single_node_prototype_star():
    # P = one carbon: every carbon of the data graph is a match (5 in a 4-leaf
    # star).  The member (centre + 3 leaves, centre first) extends only the
    # centre's match: 4*3*2 = 24 ordered leaf triples.
    r = run([([C], []), star(3)], [star(4)])
    assert r.n_partial == 5
    assert r.total == 24
    # literal DFS, per branch root a: frame 2 takes b, the leaf frame counts c
    # and d and clears only d (the last one); c then stays visited, d finds no
    # leaf left: 2 per branch root, 4 branch roots -> 8
    assert run([([C], []), star(3)], [star(4)], dfs_literal=True).total == 8


def test_literal_branch_roots_restart_visited():
    # joinWithPartialMatches gives each branch root a fresh visited set
    # (isomorphism.hpp:881-887): centre + 2 leaves in a 3-leaf star counts all
    # 6, where the plain literal join stops at 2
    assert run([([C], []), star(2)], [star(3)], dfs_literal=True).total == 6
    assert oracle.run_pipeline(graphs(star(2)), graphs(star(3)), 0, dfs_literal=True).total == 2


def test_members_smaller_than_or_equal_to_the_prototype():
    # P = 3-chain; in a 3-leaf star its matches put the centre in the middle: 6.
    # A 2-chain member adds nothing (end > |V(q)|), a 3-chain member adds one
    # per match (end == |V(q)|), isomorphism.hpp:854-864
    r = run([chain(3), chain(2), chain(3)], [star(3)])
    assert r.n_partial == 6
    dense = r.pair_counts_dense(3)[:, 0]
    assert dense.tolist() == [6, 0, 6]
    ff = run([chain(3), chain(2), chain(3)], [star(3)], find_first=True)
    assert ff.pair_counts_dense(3)[:, 0].tolist() == [1, 0, 1]


def test_empty_prototype_runs_the_plain_join():
    # BMS2.cpp:220-233: a depth of 0 keeps the plain join
    q = Graphs.from_csr([0, 0, 3], [0, 1, 2, 2], [1, 0], [C, C, C])
    d = graphs(chain(3))
    a = oracle.run_pipeline(q, d, 0, cs=True)
    b = oracle.run_pipeline(q, d, 0)
    assert a.n_partial == 0 and np.array_equal(a.counts, b.counts)


@pytest.mark.parametrize("seed", [7, 11])
def test_exact_clustered_equals_plain_join_at_two_refine_steps(seed):
    # members contain the prototype as an induced subgraph, and at R <= 2 every
    # filter is sound for induced embeddings, so both joins count all of them
    _, d = workloads.make("mol1k", seed, n_data=500, n_queries=2)
    c = workloads.make_cluster(d, 40, seed, proto_nodes=(3, 5))
    for R in (0, 2):
        a = oracle.run_pipeline(c, d, R)
        b = oracle.run_pipeline(c, d, R, cs=True)
        assert np.array_equal(a.counts, b.counts)
        assert b.n_partial > 0 and b.total > 0
        # the shared prefix is searched once per data graph: less work
        assert int(b.expansions.sum()) + b.partial_exps < int(a.expansions.sum())


def test_ring_prototype_cluster():
    # a pure carbon ring prototype (the reference's ring clusters): its members
    # keep the ring first, and the shared ring search halves the work
    _, d = workloads.make("mol1k", 3, n_data=600, n_queries=2)
    c = workloads.make_cluster(d, 30, 5, proto="ring")
    a = c.arrays()
    p = int(a["graph_offsets"][1])
    assert p in (5, 6) and (a["node_labels"][:p] == 8).all()
    x = oracle.run_pipeline(c, d, 2)
    y = oracle.run_pipeline(c, d, 2, cs=True)
    assert np.array_equal(x.counts, y.counts) and y.total > 0
    assert int(y.expansions.sum()) + y.partial_exps < int(x.expansions.sum())


def test_find_first_is_existence_of_a_clustered_match():
    _, d = workloads.make("mol1k", 5, n_data=300, n_queries=2)
    c = workloads.make_cluster(d, 25, 5, proto_nodes=(3, 5))
    for lit in (False, True):
        a = oracle.run_pipeline(c, d, 6, cs=True, dfs_literal=lit)
        f = oracle.run_pipeline(c, d, 6, cs=True, dfs_literal=lit, find_first=True)
        assert np.array_equal(f.counts, (a.counts > 0).astype(np.uint64))


def test_cluster_layout_lists_the_prototype_first():
    # generate_cs.py:338-362: a member's first |V(P)| nodes induce P, labels equal
    _, d = workloads.make("mol1k", 9, n_data=300, n_queries=2)
    c = workloads.make_cluster(d, 20, 9)
    a = c.arrays()
    go, ro, ci, nl = a["graph_offsets"], a["row_offsets"], a["column_indices"], a["node_labels"]

    def adj(g):
        s, e = int(go[g]), int(go[g + 1])
        return {(u - s, int(w) - s) for u in range(s, e) for w in ci[ro[u]:ro[u + 1]]}

    p = int(go[1] - go[0])
    pa = adj(0)
    for g in range(1, c.n_graphs):
        s = int(go[g])
        assert int(go[g + 1]) - s > p
        assert np.array_equal(nl[s:s + p], nl[0:p])
        assert {(u, w) for (u, w) in adj(g) if u < p and w < p} == pa
