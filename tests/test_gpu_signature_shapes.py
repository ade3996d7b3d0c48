"""Node signatures of graph shapes that molecules seldom have, against the
oracle bit for bit: dense graphs with many crossing 5- and 6-cycles (complete
graphs, random graphs up to 128 nodes, one label or two), graphs whose rows
are not symmetric (the in-sets differ from the rows), and asymmetric rows with
repeated entries.  The cycle signature counts closures through every node
(signature.hpp:591-719); symmetric graphs without repeated entries take the
kernel's canonical enumeration, the others its per-node walks."""
import numpy as np
import pytest

import oracle
from bms2_gb300 import DATA, QUERY, Graphs

pytestmark = pytest.mark.gpu

KEYS = ("label_gen", "path", "cycle", "shells")


def csr(rows_of_graphs, labels_of_graphs):
    """Batched CSR from per-graph lists of rows (local ids) and labels."""
    go, ro, ci, nl = [0], [0], [], []
    for rows, labels in zip(rows_of_graphs, labels_of_graphs):
        base = go[-1]
        for r in rows:
            ci.extend(base + int(c) for c in r)
            ro.append(len(ci))
        nl.extend(labels)
        go.append(base + len(rows))
    return Graphs.from_csr(np.array(go), np.array(ro), np.array(ci), np.array(nl, np.uint8))


def random_graph(rng, n, p, directed=False, repeats=0.0):
    a = rng.random((n, n)) < p
    np.fill_diagonal(a, False)
    if not directed:
        a = np.triu(a, 1)
        a = a | a.T
    rows = []
    for v in range(n):
        r = list(np.flatnonzero(a[v]))
        r += [c for c in r if rng.random() < repeats]
        rows.append(sorted(r))
    return rows


def check(ctx, g, steps=(0, 2, 6)):
    arrays = g.arrays()
    q = csr([[[1], [0]]], [[6, 6]])
    for R in steps:
        want = oracle.signatures(arrays, R)
        ctx.load(DATA, g)
        ctx.load(QUERY, q)
        ctx.signatures(R)
        got = ctx.signatures_of(DATA, R)
        for k in KEYS:
            assert np.array_equal(got[k], getattr(want, k)), (k, R)


def test_complete_and_dense_symmetric_graphs(ctx):
    rng = np.random.default_rng(7)
    rows, labels = [], []
    for n in (5, 6, 7, 8, 9, 12):  # complete graphs: every node on many 5- and 6-cycles
        rows.append([[c for c in range(n) if c != v] for v in range(n)])
        labels.append([6] * n)
    for n, p in ((16, 0.5), (24, 0.3), (31, 0.25), (40, 0.15), (64, 0.08), (65, 0.08), (100, 0.05), (128, 0.04)):
        rows.append(random_graph(rng, n, p))
        labels.append(list(rng.choice([6, 7], n, p=[0.8, 0.2])))
    check(ctx, csr(rows, labels))


def test_fused_rings_one_label(ctx):
    # ladders and prisms: each rung closes 4-, 6- and larger cycles sharing edges
    rows, labels = [], []
    for k in (3, 4, 5, 8, 20):
        n = 2 * k
        adj = [set() for _ in range(n)]
        for i in range(k):
            for u, v in ((i, (i + 1) % k), (k + i, k + (i + 1) % k), (i, k + i)):
                adj[u].add(v)
                adj[v].add(u)
        rows.append([sorted(r) for r in adj])
        labels.append([6] * n if k != 5 else [6, 7] * k)
    check(ctx, csr(rows, labels))


def test_asymmetric_rows(ctx):
    rng = np.random.default_rng(11)
    rows, labels = [], []
    for n, p in ((6, 0.4), (12, 0.3), (30, 0.15), (33, 0.12), (70, 0.05), (128, 0.03)):
        rows.append(random_graph(rng, n, p, directed=True))
        labels.append(list(rng.choice([6, 7, 8], n)))
    g = csr(rows, labels)
    a = g.arrays()
    ro, ci = a["row_offsets"].astype(np.int64), a["column_indices"]
    pairs = {(v, int(ci[i])) for v in range(len(ro) - 1) for i in range(ro[v], ro[v + 1])}
    assert any((w, v) not in pairs for v, w in pairs)  # really asymmetric
    check(ctx, g)


def test_asymmetric_rows_with_repeated_entries(ctx):
    rng = np.random.default_rng(13)
    rows, labels = [], []
    for n, p in ((8, 0.4), (20, 0.2), (50, 0.08)):
        rows.append(random_graph(rng, n, p, directed=True, repeats=0.3))
        labels.append(list(rng.choice([6, 7], n)))
    for n, p in ((10, 0.4), (40, 0.1)):  # symmetric rows, some entries twice
        rows.append(random_graph(rng, n, p, repeats=0.3))
        labels.append([6] * n)
    check(ctx, csr(rows, labels))
