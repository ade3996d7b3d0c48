"""Generate tests/golden/nx_small.json: an independent answer key.

Embedding counts are computed with networkx's VF2 GraphMatcher, which
enumerates node-induced, label-preserving subgraph isomorphisms — the exact
semantics of the engine.  With at most 2 refinement steps every filter of the
reference is sound (embeddings preserve labels, degrees, walks, cycles and
distances 1 and 2), so the oracle's and the engine's EXACT counts must equal
these.  Inputs are a seeded synthetic molecular workload plus hand-built
graphs, stored as text in the reference format (graph.hpp:150-202).

Run from the repository root:  python tests/golden/make_golden.py
`python tests/golden/make_golden.py large` writes tests/golden/nx_large.json
instead: the same answer key for data graphs of 65-128 nodes and queries of up
to 40 nodes, beyond the reference's 64-node bitsets and 30-node join arrays,
where the engine's generalized reading applies.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import networkx as nx
from networkx.algorithms import isomorphism as iso

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from bms2_gb300 import Graphs, workloads  # noqa: E402
from bms2_gb300.build import build  # noqa: E402
from tests.kat_graphs import C, N, O, WILD, chain, line, ring, star  # noqa: E402

WILDCARD = 255


def to_nx(arrays: dict) -> list[nx.Graph]:
    out = []
    go, ro, ci, nl = arrays["graph_offsets"], arrays["row_offsets"], arrays["column_indices"], arrays["node_labels"]
    for g in range(len(go) - 1):
        s, e = int(go[g]), int(go[g + 1])
        G = nx.Graph()
        for v in range(s, e):
            G.add_node(v - s, label=int(nl[v]))
        for v in range(s, e):
            for i in range(int(ro[v]), int(ro[v + 1])):
                w = int(ci[i])
                if w != v:
                    G.add_edge(v - s, w - s)
        out.append(G)
    return out


def count(data: nx.Graph, query: nx.Graph) -> int:
    if query.number_of_nodes() < 2:
        return 0  # gmcr.hpp:64: single-node queries are never mapped
    nm = lambda a, b: b["label"] == WILDCARD or a["label"] == b["label"]  # noqa: E731
    gm = iso.GraphMatcher(data, query, node_match=nm)
    return sum(1 for _ in gm.subgraph_isomorphisms_iter())


def text_of(g: Graphs, tmp: Path) -> str:
    g.write_file(tmp)
    return tmp.read_text()


def main() -> None:
    build()
    q, d = workloads.make("mol1k", 11, n_data=150, n_queries=16)
    tmp = ROOT / "_work" / "golden_tmp.txt"
    tmp.parent.mkdir(exist_ok=True)
    q_text, d_text = text_of(q, tmp), text_of(d, tmp)
    # hand-built cases appended to both sides
    kat_q = [ring(6), ring(5), chain(4), star(2), ([WILD, C], [(0, 1)]), ([N, C, O], [(0, 1), (1, 2)]), chain(3)]
    kat_d = [ring(6), ring(5), star(3), ([O, C], [(0, 1)]), ring(3), ([N, C, O, C], [(0, 1), (1, 2), (2, 3)])]
    q_text += "".join(line(*g) + "\n" for g in kat_q)
    d_text += "".join(line(*g) + "\n" for g in kat_d)
    qg = Graphs.parse_text(q_text)
    dg = Graphs.parse_text(d_text)
    Q, D = to_nx(qg.arrays()), to_nx(dg.arrays())
    counts = []
    for qi, qq in enumerate(Q):
        for di, dd in enumerate(D):
            c = count(dd, qq)
            if c:
                counts.append([qi, di, c])
    out = {
        "about": "networkx VF2 induced, label-preserving embedding counts (answer key for EXACT semantics, R <= 2)",
        "generator": "tests/golden/make_golden.py",
        "networkx": nx.__version__,
        "query_text": q_text,
        "data_text": d_text,
        "n_queries": len(Q),
        "n_data": len(D),
        "counts": counts,
    }
    path = Path(__file__).with_name("nx_small.json")
    path.write_text(json.dumps(out, separators=(",", ":")))
    print(f"{path}: {len(counts)} non-zero pairs, total {sum(c[2] for c in counts)}")


def main_large() -> None:
    build()
    d = Graphs.synth_molecules(30, 29, 0, 0, 0, 65, 128, 1, 4)
    q = Graphs.synth_queries(d, 12, 31, 3, 8, 0.25, 0.0)
    q_big = Graphs.synth_queries(d, 8, 37, 31, 40, 0.0, 0.0)  # beyond the reference's 30-node join arrays
    tmp = ROOT / "_work" / "golden_tmp.txt"
    tmp.parent.mkdir(exist_ok=True)
    q_text, d_text = text_of(q, tmp) + text_of(q_big, tmp), text_of(d, tmp)
    q_text += "".join(line(*g) + "\n" for g in [ring(6), chain(5), star(3)])
    qg = Graphs.parse_text(q_text)
    dg = Graphs.parse_text(d_text)
    Q, D = to_nx(qg.arrays()), to_nx(dg.arrays())
    counts = [[qi, di, c] for qi, qq in enumerate(Q) for di, dd in enumerate(D) if (c := count(dd, qq))]
    out = {
        "about": "networkx VF2 induced, label-preserving embedding counts for data graphs of 65-128 nodes "
                 "and queries of up to 40 nodes (answer key for EXACT semantics, R <= 2)",
        "generator": "tests/golden/make_golden.py large",
        "networkx": nx.__version__,
        "query_text": q_text,
        "data_text": d_text,
        "n_queries": len(Q),
        "n_data": len(D),
        "counts": counts,
    }
    path = Path(__file__).with_name("nx_large.json")
    path.write_text(json.dumps(out, separators=(",", ":")))
    print(f"{path}: {len(counts)} non-zero pairs, total {sum(c[2] for c in counts)}")


if __name__ == "__main__":
    if sys.argv[1:] == ["large"]:
        main_large()
    else:
        main()
