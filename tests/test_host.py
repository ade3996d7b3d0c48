"""Host-side logic of libbms without a GPU: parser, writer, generator, the
C ABI surface.  No compute call is made."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from bms2_gb300 import BmsError, Graphs, native, workloads

ROOT = Path(__file__).resolve().parent.parent


def test_library_exports_every_declared_symbol():
    header = (ROOT / "include" / "bms.h").read_text()
    declared = set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(bms_[a-z_0-9]+)\s*\(", header, re.M))
    assert len(declared) >= 40
    lib = ctypes.CDLL(str(native.LIB_PATH))
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, missing
    bound = {name for name, _, _ in native.SIGNATURES}
    assert declared == bound, declared ^ bound
    assert native.lib().bms_abi_version() == 2


def test_parse_csr_follows_toCSRGraph():
    # graph.hpp:212-243: rows in edge order, v appended to u's row and u to v's
    g = Graphs.parse_text("n#3 l#11 0 8 1 7 2 8 e#2 0 1 2 1 2 1\n")
    a = g.arrays()
    assert a["graph_offsets"].tolist() == [0, 3]
    assert a["row_offsets"].tolist() == [0, 1, 3, 4]
    assert a["column_indices"].tolist() == [1, 0, 2, 1]
    assert a["node_labels"].tolist() == [8, 7, 8]
    assert a["edge_labels"].tolist() == [2, 2, 1, 1]


def test_parse_edges_without_labels_default_to_zero():
    a = Graphs.parse_text("n#2 l#11 0 8 1 8 e#1 0 1").arrays()
    assert a["edge_labels"].tolist() == [0, 0]


def test_parse_labels_truncate_to_uint8():
    # label_t is uint8 (types.hpp:12); -1 becomes the wildcard 255
    a = Graphs.parse_text("n#2 l#11 0 -1 1 264 e#1 0 1").arrays()
    assert a["node_labels"].tolist() == [255, 8]


def test_parse_self_loop_leaves_second_slot_at_zero():
    # toCSRGraph writes the same slot twice for (a, a) and skips the next one
    a = Graphs.parse_text("n#3 l#11 0 8 1 8 2 8 e#2 1 1 1 2").arrays()
    assert a["row_offsets"].tolist() == [0, 0, 3, 4]
    assert a["column_indices"].tolist() == [1, 0, 2, 1]


def test_parse_rejects_malformed_lines_and_can_skip_them():
    with pytest.raises(BmsError) as e:
        Graphs.parse_text("n#2 l#11 0 8 1 8 e#2 0 1\n")
    assert e.value.status == -1 and "Invalid graph format" in str(e.value)
    with pytest.raises(BmsError):
        Graphs.parse_text("n#2 l#11 0 8 5 8 e#0\n")
    g = Graphs.parse_text("n#2 l#11 0 8 1 8 e#1 0 1\nbroken\n\nn#1 l#11 0 7 e#0\n", skip_invalid=True)
    assert g.n_graphs == 2


def test_parse_max_graphs():
    txt = "n#1 l#11 0 8 e#0\n" * 5
    assert Graphs.parse_text(txt, max_graphs=3).n_graphs == 3


def test_write_then_parse_round_trip(tmp_path):
    q, d = workloads.make("mol1k", 2, n_data=50, n_queries=5)
    p = tmp_path / "d.txt"
    d.write_file(p)
    back = Graphs.parse_file(p)
    a, b = d.arrays(), back.arrays()
    for k in ("graph_offsets", "row_offsets", "node_labels"):
        assert np.array_equal(a[k], b[k]), k
    # same adjacency sets per node (entry order may differ)
    for v in range(len(a["node_labels"])):
        ra = sorted(a["column_indices"][a["row_offsets"][v]:a["row_offsets"][v + 1]])
        rb = sorted(b["column_indices"][b["row_offsets"][v]:b["row_offsets"][v + 1]])
        assert ra == rb


def test_parallel_parse_equals_serial_parse(tmp_path):
    # buffers above 16 MiB are split at line boundaries across threads; the
    # pieces must concatenate to exactly the serial parse (max_graphs forces
    # the serial path), and the first malformed line keeps its number
    d = Graphs.synth_molecules(70_000, 17, 0, 0, 0, 10, 40, 1, 4)
    path = tmp_path / "big.txt"
    d.write_file(path)
    text = path.read_bytes()
    assert len(text) > (17 << 20)
    par = Graphs.parse_file(path).arrays()
    ser = Graphs.parse_file(path, max_graphs=d.n_graphs).arrays()
    ref = d.arrays()
    for k in ref:
        assert np.array_equal(par[k], ser[k]), k
        assert np.array_equal(par[k], ref[k]), k
    lines = text.split(b"\n")
    bad = len(lines) - 100
    lines[bad] = b"n#2 l#1 garbage"
    path.write_bytes(b"\n".join(lines))
    msgs = []
    for mg in (0, d.n_graphs + 1):
        with pytest.raises(BmsError) as e:
            Graphs.parse_file(path, max_graphs=mg)
        msgs.append(str(e.value))
    assert msgs[0] == msgs[1] and f"line {bad + 1}:" in msgs[0]
    skipped = Graphs.parse_file(path, skip_invalid=True)
    assert skipped.n_graphs == d.n_graphs - 1
    # a malformed line in the first and in a middle piece keeps its number too
    for bad2 in (4, len(lines) // 2):
        lines2 = list(lines)
        lines2[bad2] = b"n#3 l#3 0 8 1 8"
        path.write_bytes(b"\n".join(lines2))
        with pytest.raises(BmsError) as e:
            Graphs.parse_file(path)
        assert f"line {bad2 + 1}:" in str(e.value)


def test_parse_file_missing_is_eio(tmp_path):
    with pytest.raises(BmsError) as e:
        Graphs.parse_file(tmp_path / "nope.txt")
    assert e.value.status == -4


def test_synthetic_workloads_are_seeded_and_shaped():
    q1, d1 = workloads.make("mol1k", 7)
    q2, d2 = workloads.make("mol1k", 7)
    for a, b in ((q1.arrays(), q2.arrays()), (d1.arrays(), d2.arrays())):
        for k in a:
            assert np.array_equal(a[k], b[k])
    a = d1.arrays()
    sizes = np.diff(a["graph_offsets"])
    assert d1.n_graphs == 1000 and sizes.min() >= 10 and sizes.max() <= 40
    deg = np.diff(a["row_offsets"])
    assert deg.max() <= 4
    frac = np.bincount(a["node_labels"], minlength=11) / len(a["node_labels"])
    assert abs(frac[8] - 0.72) < 0.02 and abs(frac[0] - 0.12) < 0.02 and abs(frac[7] - 0.11) < 0.02
    qs = np.diff(q1.arrays()["graph_offsets"])
    assert q1.n_graphs == 20 and qs.min() >= 3 and qs.max() <= 12
    # connected, symmetric, no self-loops
    ro, ci = a["row_offsets"], a["column_indices"]
    for v in range(0, len(a["node_labels"]), 97):
        for i in range(ro[v], ro[v + 1]):
            w = ci[i]
            assert w != v and v in ci[ro[w]:ro[w + 1]]


def test_queries_are_connected_induced_subgraphs():
    q, d = workloads.make("mol1k", 9, n_data=200, n_queries=30)
    a = q.arrays()
    go, ro, ci = a["graph_offsets"], a["row_offsets"], a["column_indices"]
    for g in range(len(go) - 1):
        s, e = go[g], go[g + 1]
        seen, stack = {s}, [s]
        while stack:
            v = stack.pop()
            for w in ci[ro[v]:ro[v + 1]]:
                if w not in seen:
                    seen.add(int(w))
                    stack.append(int(w))
        assert len(seen) == e - s


def test_from_csr_validates():
    with pytest.raises(BmsError):
        Graphs.from_csr([1, 2], [0, 0], [], [8])
    g = Graphs.from_csr([0, 2], [0, 1, 2], [1, 0], [8, 8])
    assert g.n_graphs == 1 and g.n_nodes == 2


def test_filter_size():
    q, _ = workloads.make("mol1k", 4)
    f = q.filter_size(5, 8)
    sizes = np.diff(f.arrays()["graph_offsets"])
    assert len(sizes) and sizes.min() >= 5 and sizes.max() <= 8


def test_status_names():
    L = native.lib()
    assert L.bms_status_name(-5) == b"BMS_ESTATE"
    assert L.bms_feature_name(0) == b"log2_mean_candidates"
    assert len(native.feature_names()) == 12


def test_outside_reference_domain_shares():
    import bench

    q = [0, 3, 33, 40]  # query sizes 3, 30, 7: none above 30
    d = [0, 64, 129, 139, 139]  # data sizes 64, 65, 10, 0: one of four above 64
    got = bench.outside_reference_domain(q, d)
    assert got == {"data_graphs_over_64_nodes": 0.25, "queries_over_30_nodes": 0.0, "pairs": 0.25}
    got = bench.outside_reference_domain([0, 31, 32], d)  # one of two queries above 30
    assert got["queries_over_30_nodes"] == 0.5 and got["pairs"] == 1.0 - 0.75 * 0.5
    g = Graphs.synth_molecules(50, 3, 0, 0, 0, 60, 70, 1, 4)
    off = bench.graph_offsets(g)
    assert np.array_equal(off, g.arrays()["graph_offsets"])
    assert bench.outside_reference_domain([0, 5], off)["data_graphs_over_64_nodes"] > 0


def test_parallel_parse_with_empty_pieces():
    # 40 MiB of blank lines between two halves: the middle pieces of the
    # parallel parse hold no graph and must merge to the serial result
    d = Graphs.synth_molecules(2000, 19, 0, 0, 0, 10, 40, 1, 4)
    import tempfile, os
    with tempfile.TemporaryDirectory() as t:
        p = os.path.join(t, "g.txt")
        d.write_file(p)
        text = open(p, "rb").read()
    lines = text.split(b"\n")
    half = len(lines) // 2
    buf = b"\n".join(lines[:half]) + b"\n" + b"\n" * (40 << 20) + b"\n".join(lines[half:])
    par = Graphs.parse_text(buf).arrays()
    ref = d.arrays()
    for k in ref:
        assert np.array_equal(par[k], ref[k]), k


def test_bench_algorithmic_bytes_follow_their_definitions():
    import bench

    # filter + refine: Qn*Dn/8 candidate bits once, (45 + 8R) bytes per node on both sides
    assert bench.algorithmic_filter_bytes(16, 1000, 6) == 16 * 1000 / 8 + (1000 + 16) * (45 + 48)
    assert bench.algorithmic_filter_bytes(0, 0, 6) == 0
    # signatures: CSR read once (5 per node + 4 per entry), 48 + 8R bytes written per node
    assert bench.algorithmic_signature_bytes(10, 22, 6) == 10 * 5 + 22 * 4 + 10 * (48 + 48)
    empty = bench.graph_offsets(Graphs.parse_text(""))
    assert empty.tolist() == [0]
