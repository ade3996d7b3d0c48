"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference measures on converted public SMARTS sets; those cannot be
converted here (no rdkit), so seeded synthetic molecular graphs with the stated
distributions stand in for them.  Every workload is a pure function of its seed.

  mol1k     1,000 data graphs of 10-40 atoms (uniform), 20 queries of 3-12 nodes
  mol100k   100,000 data graphs, N(28, 9) atoms clipped to 10-60, 600 queries of
            5-30 nodes of which 30% are pure-carbon chains or rings
  mol1m     1,000,000 data graphs, log-normal atoms (median 25, sigma 0.55)
            clipped to 5-120, 1,000 queries of 3-40 nodes
  mol10m    10,000,000 data graphs as mol1m (about 290M atoms, drawn in ten
            seeded blocks of 1,000,000), 3,000 queries of 3-40 nodes of which
            20% are adversarial symmetric patterns
Element mix C 72%, N 12%, O 11%, S 2%, F 1.5%, Cl 1%, Br 0.5%; degree <= 4;
1-4 rings per molecule; bonds single/double/triple/aromatic 60/20/2/18%.
"""
from __future__ import annotations

from dataclasses import dataclass

from .native import SIZE_LOGNORMAL, SIZE_NORMAL, SIZE_UNIFORM, Graphs


@dataclass(frozen=True)
class Workload:
    name: str
    n_data: int
    size_dist: int
    p0: float
    p1: float
    min_atoms: int
    max_atoms: int
    n_queries: int
    q_min: int
    q_max: int
    frac_carbon: float
    frac_adversarial: float


WORKLOADS = {
    "mol1k": Workload("mol1k", 1_000, SIZE_UNIFORM, 0, 0, 10, 40, 20, 3, 12, 0.0, 0.0),
    "mol100k": Workload("mol100k", 100_000, SIZE_NORMAL, 28.0, 9.0, 10, 60, 600, 5, 30, 0.3, 0.0),
    "mol1m": Workload("mol1m", 1_000_000, SIZE_LOGNORMAL, 25.0, 0.55, 5, 120, 1_000, 3, 40, 0.0, 0.0),
    "mol10m": Workload("mol10m", 10_000_000, SIZE_LOGNORMAL, 25.0, 0.55, 5, 120, 3_000, 3, 40, 0.0, 0.2),
}


BLOCK_GRAPHS = 1_000_000


def block_seed(seed: int, b: int) -> int:
    """Seed of block b of a data batch: block 0 keeps the batch's seed, so any
    batch of at most BLOCK_GRAPHS graphs is one sequential draw."""
    return seed if b == 0 else (seed * 0x9E3779B1 + 0x7F4A7C15 * b) & 0xFFFFFFFFFFFFFFFF


def _molecules(w: Workload, n: int, seed: int) -> Graphs:
    """n data graphs of workload w: blocks of BLOCK_GRAPHS graphs, each a
    sequential draw with its own seed, generated on parallel threads and
    concatenated in block order."""
    if n <= BLOCK_GRAPHS:
        return Graphs.synth_molecules(n, seed, w.size_dist, w.p0, w.p1, w.min_atoms, w.max_atoms, 1, 4)
    import concurrent.futures as cf
    import os

    import numpy as np

    sizes = [min(BLOCK_GRAPHS, n - b) for b in range(0, n, BLOCK_GRAPHS)]

    def one(b: int) -> dict:
        g = Graphs.synth_molecules(sizes[b], block_seed(seed, b), w.size_dist, w.p0, w.p1, w.min_atoms, w.max_atoms,
                                   1, 4)
        return g.arrays()

    with cf.ThreadPoolExecutor(max_workers=min(len(sizes), os.cpu_count() or 1)) as ex:
        parts = list(ex.map(one, range(len(sizes))))
    node_base = np.cumsum([0] + [len(p["node_labels"]) for p in parts])
    entry_base = np.cumsum([0] + [len(p["column_indices"]) for p in parts])
    go = np.concatenate([parts[0]["graph_offsets"][:1]] +
                        [p["graph_offsets"][1:].astype(np.uint64) + node_base[i] for i, p in enumerate(parts)])
    ro = np.concatenate([parts[0]["row_offsets"][:1]] +
                        [p["row_offsets"][1:].astype(np.uint64) + entry_base[i] for i, p in enumerate(parts)])
    ci = np.concatenate([p["column_indices"].astype(np.uint64) + node_base[i] for i, p in enumerate(parts)])
    if go[-1] >= 1 << 32 or ro[-1] >= 1 << 32:
        raise ValueError("batch exceeds 32-bit node or entry ids")
    return Graphs.from_csr(go.astype(np.uint32), ro.astype(np.uint32), ci.astype(np.uint32),
                           np.concatenate([p["node_labels"] for p in parts]),
                           np.concatenate([p["edge_labels"] for p in parts]))


def make_data(name: str, seed: int = 1, n_data: int | None = None) -> Graphs:
    """The data graphs of a named workload alone (as make draws them)."""
    w = WORKLOADS[name]
    return _molecules(w, n_data or w.n_data, seed)


def make(name: str, seed: int = 1, n_data: int | None = None, n_queries: int | None = None) -> tuple[Graphs, Graphs]:
    """(queries, data) of a named workload; n_data / n_queries shrink it.
    Batches of more than BLOCK_GRAPHS data graphs are drawn in seeded blocks
    (block_seed) on parallel threads."""
    w = WORKLOADS[name]
    data = _molecules(w, n_data or w.n_data, seed)
    queries = Graphs.synth_queries(data, n_queries or w.n_queries, seed + 1000003, w.q_min, w.q_max, w.frac_carbon,
                                   w.frac_adversarial)
    return queries, data


# ------------------------------------------------------------------ clusters
def _graph_at(a: dict, g: int):
    """(labels, rows, edge labels) of graph g of a CSR batch (dict of arrays),
    local ids; rows[u] lists u's neighbours in CSR order."""
    go, ro, ci, el, nl = (a["graph_offsets"], a["row_offsets"], a["column_indices"], a["edge_labels"],
                          a["node_labels"])
    s, e = int(go[g]), int(go[g + 1])
    rows, elab = [], []
    for u in range(s, e):
        a, b = int(ro[u]), int(ro[u + 1])
        rows.append([int(x) - s for x in ci[a:b]])
        elab.append([int(x) for x in el[a:b]])
    return [int(x) for x in nl[s:e]], rows, elab


def _grow(rng, rows, nodes: list, k: int) -> list:
    """Add up to k nodes to `nodes`, each a random neighbour of the set so far."""
    out = list(nodes)
    inside = set(out)
    for _ in range(k):
        frontier = sorted({w for u in out for w in rows[u] if w not in inside})
        if not frontier:
            break
        w = frontier[int(rng.integers(len(frontier)))]
        out.append(w)
        inside.add(w)
    return out


def _find_induced(p_lab, p_adj, lab, rows, cap: int = 20000):
    """One label-preserving induced embedding of the prototype (its nodes in
    order, each after a neighbour) in a graph, or None; gives up after `cap` tries."""
    adj = [set(r) for r in rows]
    n, m = len(p_lab), len(lab)
    assign: list[int] = []
    tries = [0]

    def rec(i: int) -> bool:
        if i == n:
            return True
        prev = [j for j in p_adj[i] if j < i]
        pool = sorted(adj[assign[prev[0]]]) if prev else range(m)
        for v in pool:
            tries[0] += 1
            if tries[0] > cap:
                return False
            if lab[v] != p_lab[i] or v in assign:
                continue
            if all((j in p_adj[i]) == (assign[j] in adj[v]) for j in range(i)):
                assign.append(v)
                if rec(i + 1):
                    return True
                assign.pop()
        return False

    return list(assign) if rec(0) else None


def _find_ring(lab, rows, label: int = 8, sizes=(6, 5)):
    """A chordless ring of `label` atoms (6 atoms, else 5) in ring order, or None."""
    adj = [set(r) for r in rows]
    for size in sizes:
        for s in range(len(lab)):
            if lab[s] != label:
                continue
            stack = [[s]]
            while stack:
                path = stack.pop()
                u = path[-1]
                if len(path) == size:
                    if s in adj[u] and all(path[j] not in adj[path[i]] for i in range(size)
                                           for j in range(i + 2, size) if not (i == 0 and j == size - 1)):
                        return path
                    continue
                stack.extend(path + [w] for w in sorted(adj[u]) if w > s and w not in path and lab[w] == label)
    return None


def make_cluster(data: Graphs, n_members: int, seed: int, proto_nodes: tuple[int, int] = (5, 8),
                 extra_nodes: tuple[int, int] = (1, 12), n_sources: int = 24, proto: str = "grow",
                 source_graphs: int = 100_000) -> Graphs:
    """make_cluster_arrays on a Graphs batch, as a Graphs batch."""
    return Graphs.from_csr(**make_cluster_arrays(data.arrays(), n_members, seed, proto_nodes, extra_nodes, n_sources,
                                                 proto, source_graphs))


def make_cluster_arrays(data: dict, n_members: int, seed: int, proto_nodes: tuple[int, int] = (5, 8),
                        extra_nodes: tuple[int, int] = (1, 12), n_sources: int = 24, proto: str = "grow",
                        source_graphs: int = 100_000) -> dict:
    """A query cluster in the layout of the reference's cluster files
    (generate_cs.py:338-362, 555-577): graph 0 is the prototype P; each member
    is P plus 1..12 further atoms grown around an induced occurrence of P in one
    of up to n_sources data graphs, with P's nodes first, in P's order.
    proto="grow": P is a connected induced subgraph of proto_nodes atoms of a
    random data graph, numbered in discovery order; proto="ring": P is a
    chordless carbon ring of 6 (else 5) atoms in ring order, the reference's
    pure-ring clusters (generate_cs.py:259, 323: listed first).  (The reference
    clusters real molecules by maximum common substructure with rdkit, which is
    absent here; this keeps its file convention.)  The prototype and its
    occurrences come from the first `source_graphs` data graphs, so any prefix of
    the same data set at least that long yields the same cluster."""
    import numpy as np

    rng = np.random.default_rng(seed)
    v = data
    go = v["graph_offsets"]
    G = min(len(go) - 1, source_graphs)
    sizes = go[1:G + 1].astype(np.int64) - go[:G]
    want = proto_nodes[1] + extra_nodes[1]
    big = np.nonzero(sizes >= want)[0]
    pool = big if len(big) else np.array([int(np.argmax(sizes))])
    if proto == "ring":
        ring = None
        for g in rng.permutation(pool)[:2000]:
            g0 = int(g)
            lab0, rows0, el0 = _graph_at(v, g0)
            ring = _find_ring(lab0, rows0)
            if ring is not None:
                break
        if ring is None:
            raise ValueError("no carbon ring of 5 or 6 atoms in the sampled data graphs")
        proto_list = ring
    else:
        g0 = int(pool[int(rng.integers(len(pool)))])
        lab0, rows0, el0 = _graph_at(v, g0)
        p = int(rng.integers(proto_nodes[0], proto_nodes[1] + 1))
        proto_list = _grow(rng, rows0, [int(rng.integers(len(lab0)))], p - 1)
    proto = proto_list
    p = len(proto)
    p_lab = [lab0[u] for u in proto]
    pos = {u: i for i, u in enumerate(proto)}
    p_adj = [{pos[w] for w in rows0[u] if w in pos} for u in proto]
    occ = [(g0, proto)]
    for g in rng.permutation(G)[: 50 * n_sources]:
        if len(occ) >= n_sources:
            break
        g = int(g)
        if g == g0 or sizes[g] < p:
            continue
        lab, rows, _ = _graph_at(v, g)
        emb = _find_induced(p_lab, p_adj, lab, rows)
        if emb is not None:
            occ.append((g, emb))
    cache = {g0: (lab0, rows0, el0)}
    graphs = [(g0, proto)]
    for _ in range(n_members):
        g, emb = occ[int(rng.integers(len(occ)))]
        if g not in cache:
            cache[g] = _graph_at(v, g)
        k = int(rng.integers(extra_nodes[0], extra_nodes[1] + 1))
        graphs.append((g, _grow(rng, cache[g][1], emb, k)))
    # induced subgraphs, CSR entries in each source row's order
    goff, roff, cols, labs, elabs = [0], [0], [], [], []
    for g, nodes in graphs:
        lab, rows, el = cache[g]
        local = {u: i for i, u in enumerate(nodes)}
        base = goff[-1]
        for u in nodes:
            for w, l in zip(rows[u], el[u]):
                if w in local:
                    cols.append(base + local[w])
                    elabs.append(l)
            roff.append(len(cols))
            labs.append(lab[u])
        goff.append(base + len(nodes))
    return {"graph_offsets": np.array(goff, np.uint32), "row_offsets": np.array(roff, np.uint32),
            "column_indices": np.array(cols, np.uint32), "node_labels": np.array(labs, np.uint8),
            "edge_labels": np.array(elabs, np.uint8)}
