"""Known-answer tests of the CPU oracle (hand-derived values).

The reference ships no tests or golden vectors, so these values are derived by
hand from its code (file:line in each test) and pin the oracle.
"""
import numpy as np
import pytest

import oracle
from bms2_gb300 import Graphs
from tests.kat_graphs import C, N, O, WILD, chain, line, ring, star


def graphs(*gs) -> Graphs:
    return Graphs.parse_text("\n".join(line(*g) for g in gs) + "\n")


def total(q, d, R=0, **kw):
    return oracle.run_pipeline(graphs(*q), graphs(*d), R, **kw).total


def test_ring_in_ring_exact_counts_every_automorphism():
    # a 6-ring has 12 automorphisms; every one is an induced embedding
    assert total([ring(6)], [ring(6)]) == 12
    assert total([ring(5)], [ring(5)]) == 10


def test_ring_in_ring_reference_dfs_counts_half():
    # isomorphism.hpp:414-448: frame 1 takes a1, later a5; a1 keeps its visited
    # bit, so the second orientation can never close the ring: 1 per root
    assert total([ring(6)], [ring(6)], dfs_literal=True) == 6


def test_star_reference_dfs_stale_visited_bits():
    # centre + 3 leaves, query centre + 2 leaves: 3*2 = 6 embeddings; the
    # literal DFS finds (b,c), (b,d), then c and d stay visited: 2
    assert total([star(2)], [star(3)]) == 6
    assert total([star(2)], [star(3)], dfs_literal=True) == 2


def test_find_first_is_one_per_matching_pair():
    assert total([ring(6)], [ring(6), ring(6), ring(5)], find_first=True) == 2


def test_single_node_query_never_mapped():
    # gmcr.hpp:64 requires more than one query node
    r = oracle.run_pipeline(graphs(([C], [])), graphs(ring(6)), 0)
    assert len(r.qidx) == 0 and r.total == 0


def test_induced_semantics():
    # a 3-chain is not an induced subgraph of a triangle
    assert total([chain(3)], [ring(3)]) == 0
    assert total([chain(3)], [chain(3)]) == 2


def test_exact_distance_shells_prune_at_step_3():
    # 4-chain in a 5-ring: 10 induced embeddings; the chain end sees a carbon at
    # distance 3, a 5-ring node has no node at distance 3 (signature.hpp:358-382)
    assert total([chain(4)], [ring(5)], R=2) == 10
    assert total([chain(4)], [ring(5)], R=3) == 0


def test_wildcard_query_label():
    # isomorphism.hpp:78: a query label 255 matches any data label
    assert total([([WILD, C], [(0, 1)])], [([O, C], [(0, 1)])]) == 1
    assert total([([WILD, C], [(0, 1)])], [([C, C], [(0, 1)])]) == 2
    assert total([([N, C], [(0, 1)])], [([O, C], [(0, 1)])]) == 0


def test_labels_above_15_match_by_equality_and_are_ignored_by_shells():
    q = ([20, C], [(0, 1)])
    d = ([20, C, C], [(0, 1), (1, 2)])
    assert total([q], [d], R=2) == 1
    s = oracle.signatures(graphs(d).arrays(), 1)
    assert s.shells[0][1] == (1 << (4 * 8))  # only the carbon neighbour is counted


def test_cycle_signatures():
    # signature.hpp:658-714: closures counted per direction and halved
    s = oracle.signatures(graphs(ring(6)).arrays(), 0)
    assert (s.cycle == np.array([0, 0, 1, 0])).all()
    s = oracle.signatures(graphs(ring(5)).arrays(), 0)
    assert (s.cycle == np.array([1, 0, 0, 0])).all()
    s = oracle.signatures(graphs(ring(6, [N, C, C, C, C, C])).arrays(), 0)
    assert (s.cycle == np.array([0, 0, 0, 1])).all()


def test_cycle_signature_follows_repeated_csr_entries():
    # a repeated edge 0-1 doubles every 5-ring path through it: 4 closures / 2
    labels, edges = ring(5)
    edges = edges + [(0, 1)]
    s = oracle.signatures(graphs((labels, edges)).arrays(), 0)
    assert (s.cycle[:, 0] == 2).all()


def test_label_signature_saturates_at_15():
    # signature.hpp:43-50
    s = oracle.signatures(graphs(star(17)).arrays(), 0)
    assert (s.label_gen[0] >> (4 * C)) & 15 == 15
    assert (s.label_gen[1] >> (4 * C)) & 15 == 1


def test_shells_are_exact_distance_histograms():
    s = oracle.signatures(graphs(chain(5)).arrays(), 6)
    end = s.shells[:, 0]
    one_c = 1 << (4 * C)
    assert list(end) == [one_c, one_c, one_c, one_c, 0, 0]


def _fmix32(h):
    h ^= h >> 16
    h = (h * 0x85EBCA6B) & 0xFFFFFFFF
    h ^= h >> 13
    h = (h * 0xC2B2AE35) & 0xFFFFFFFF
    h ^= h >> 16
    return h


def _combine(a, b):
    return (a ^ ((b + 0x9E3779B9 + ((a << 6) & 0xFFFFFFFF) + (a >> 2)) & 0xFFFFFFFF)) & 0xFFFFFFFF


def _insert(bits, v):
    h = v
    for _ in range(3):
        bits[(h & 255) >> 6] |= 1 << (h & 63)
        h = _fmix32(h)


def test_path_signature_matches_python_restatement():
    # signature.hpp:393-437, 472-519 restated independently in Python
    labels, edges = [N, C, O, C], [(0, 1), (1, 2), (2, 3), (3, 1)]
    g = graphs((labels, edges)).arrays()
    s = oracle.signatures(g, 0)
    adj = {i: [] for i in range(4)}
    rp, ci = g["row_offsets"], g["column_indices"]
    for u in range(4):
        adj[u] = [int(x) for x in ci[rp[u]:rp[u + 1]]]
    for u in range(4):
        bits = [0, 0, 0, 0]
        for v in adj[u]:
            for w in adj[v]:
                if w == u:
                    continue
                h2 = _combine(labels[u], _combine(labels[v], labels[w]))
                _insert(bits, _fmix32(h2))
                for x in adj[w]:
                    if x in (v, u):
                        continue
                    _insert(bits, _fmix32(_combine(h2, labels[x])))
        assert list(s.path[u]) == bits


def test_x86_reading_equals_generalized_inside_64_nodes():
    from bms2_gb300 import workloads

    q, d = workloads.make("mol1k", 3, n_data=300, n_queries=12)
    for R in (0, 6):
        a = oracle.run_pipeline(q, d, R)
        b = oracle.run_pipeline(q, d, R, x86=True)
        assert np.array_equal(a.d_sigs.shells, b.d_sigs.shells)
        assert np.array_equal(a.d_sigs.cycle, b.d_sigs.cycle)
        assert np.array_equal(a.counts, b.counts)


def test_x86_reading_aliases_above_64_nodes():
    # a 70-node carbon chain: on x86 the 64-bit visited/shell bitsets alias
    # local ids modulo 64 (utils.hpp:95-97) and cycle signatures are zero
    # (signature.hpp:614); the generalized reading does neither
    g = graphs(chain(70)).arrays()
    gen = oracle.signatures(g, 3)
    x86 = oracle.signatures(g, 3, x86=True)
    assert not np.array_equal(gen.shells, x86.shells)
    g2 = graphs(ring(70)).arrays()
    assert oracle.signatures(g2, 0, x86=True).cycle.sum() == 0


@pytest.mark.parametrize("R", [0, 2, 6])
def test_find_first_equals_min_count_one(R):
    from bms2_gb300 import workloads

    q, d = workloads.make("mol1k", 5, n_data=200, n_queries=10)
    a = oracle.run_pipeline(q, d, R)
    b = oracle.run_pipeline(q, d, R, find_first=True)
    assert np.array_equal(np.minimum(a.counts, 1), b.counts)
