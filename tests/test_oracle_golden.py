"""The oracle's EXACT counts against the networkx answer key (tests/golden)."""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from bms2_gb300 import Graphs, workloads

GOLDEN = Path(__file__).with_name("golden") / "nx_small.json"


def golden():
    g = json.loads(GOLDEN.read_text())
    q = Graphs.parse_text(g["query_text"])
    d = Graphs.parse_text(g["data_text"])
    dense = np.zeros((g["n_queries"], g["n_data"]), np.uint64)
    for qi, di, c in g["counts"]:
        dense[qi, di] = c
    return q, d, dense


@pytest.mark.parametrize("R", [0, 1, 2])
def test_oracle_exact_counts_match_networkx(R):
    q, d, want = golden()
    r = oracle.run_pipeline(q, d, R)
    assert np.array_equal(r.pair_counts_dense(q.n_graphs), want)


def test_oracle_find_first_matches_networkx_existence():
    q, d, want = golden()
    r = oracle.run_pipeline(q, d, 2, find_first=True)
    assert np.array_equal(r.pair_counts_dense(q.n_graphs), np.minimum(want, 1))


def test_refinement_beyond_two_steps_only_removes_matches():
    # exact-distance shells at k >= 3 are unsound (embeddings can shorten
    # distances), so counts may only drop, never grow
    q, d, want = golden()
    r = oracle.run_pipeline(q, d, 6)
    got = r.pair_counts_dense(q.n_graphs)
    assert (got <= want).all()


def test_live_networkx_cross_check():
    nx = pytest.importorskip("networkx")
    from networkx.algorithms import isomorphism as iso

    q, d = workloads.make("mol1k", 23, n_data=40, n_queries=8)
    r = oracle.run_pipeline(q, d, 2)
    got = r.pair_counts_dense(q.n_graphs)

    def to_nx(a):
        out = []
        go, ro, ci, nl = a["graph_offsets"], a["row_offsets"], a["column_indices"], a["node_labels"]
        for g in range(len(go) - 1):
            s, e = int(go[g]), int(go[g + 1])
            G = nx.Graph()
            G.add_nodes_from((v - s, {"l": int(nl[v])}) for v in range(s, e))
            G.add_edges_from((v - s, int(ci[i]) - s) for v in range(s, e) for i in range(int(ro[v]), int(ro[v + 1])))
            out.append(G)
        return out

    Q, D = to_nx(q.arrays()), to_nx(d.arrays())
    for qi, qq in enumerate(Q):
        for di, dd in enumerate(D):
            gm = iso.GraphMatcher(dd, qq, node_match=lambda a, b: b["l"] == 255 or a["l"] == b["l"])
            want = sum(1 for _ in gm.subgraph_isomorphisms_iter()) if qq.number_of_nodes() > 1 else 0
            assert got[qi, di] == want, (qi, di)


def test_oracle_embeddings_match_networkx():
    # every embedding (not only the count) of every GMCR pair at R = 2, against
    # networkx's induced label-preserving subgraph isomorphisms
    nx = pytest.importorskip("networkx")
    from networkx.algorithms import isomorphism as iso

    q, d = workloads.make("mol1k", 29, n_data=25, n_queries=6)
    r = oracle.run_pipeline(q, d, 2)
    qa, da = q.arrays(), d.arrays()

    def graph(a, g):
        go, ro, ci, nl = a["graph_offsets"], a["row_offsets"], a["column_indices"], a["node_labels"]
        s, e = int(go[g]), int(go[g + 1])
        G = nx.Graph()
        G.add_nodes_from((v - s, {"l": int(nl[v])}) for v in range(s, e))
        G.add_edges_from((v - s, int(ci[i]) - s) for v in range(s, e) for i in range(int(ro[v]), int(ro[v + 1])))
        return G

    checked = 0
    for di in range(d.n_graphs):
        for t in range(int(r.offsets[di]), int(r.offsets[di + 1])):
            qi = int(r.qidx[t])
            got = oracle.pair_embeddings(q, d, r, t)
            assert len(got) == int(r.counts[t])
            qq, dd = graph(qa, qi), graph(da, di)
            gm = iso.GraphMatcher(dd, qq, node_match=lambda a, b: b["l"] == 255 or a["l"] == b["l"])
            want = sorted(tuple(inv[u] for u in range(qq.number_of_nodes()))
                          for inv in ({v: k for k, v in m.items()} for m in gm.subgraph_isomorphisms_iter()))
            assert [tuple(int(x) for x in row) for row in got] == want, (qi, di)
            checked += 1
    assert checked > 20


GOLDEN_LARGE = Path(__file__).with_name("golden") / "nx_large.json"


def golden_large():
    g = json.loads(GOLDEN_LARGE.read_text())
    q = Graphs.parse_text(g["query_text"])
    d = Graphs.parse_text(g["data_text"])
    dense = np.zeros((g["n_queries"], g["n_data"]), np.uint64)
    for qi, di, c in g["counts"]:
        dense[qi, di] = c
    return q, d, dense


@pytest.mark.parametrize("R", [0, 2])
def test_oracle_counts_match_networkx_beyond_64_nodes(R):
    # data graphs of 65-128 nodes and queries of up to 40: the generalized
    # reading (bitsets as wide as the graph, cycle signatures for every size,
    # no 30-node join arrays) keeps every filter sound, so EXACT counts equal
    # the independent answer key
    q, d, want = golden_large()
    assert int(np.diff(d.arrays()["graph_offsets"]).min()) > 64
    assert int(np.diff(q.arrays()["graph_offsets"]).max()) > 30
    r = oracle.run_pipeline(q, d, R)
    assert np.array_equal(r.pair_counts_dense(q.n_graphs), want)


def test_x86_reading_loses_matches_beyond_64_nodes():
    # the reference's own reading zeroes the data side's cycle signatures above
    # 64 nodes (signature.hpp:614), so queries with cycles lose their matches
    q, d, want = golden_large()
    r = oracle.run_pipeline(q, d, 0, x86=True)
    got = r.pair_counts_dense(q.n_graphs)
    assert (got <= want).all() and got.sum() < want.sum()
