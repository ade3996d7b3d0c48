"""Generate tests/golden/ref_*.npz: outputs of the reference's own code.

The reference's headers (AnySparse/BMS2, library/include) are compiled on the
CPU against a host-only SYCL stand-in by oracle/ref/build_ref.py (patches
disclosed there) and run by oracle/ref/ref_driver.cpp on seeded inputs in the
reference text format (graph.hpp:150-202).  Each fixture holds the input texts
and every intermediate the reference produces: the batched CSR of both sides
(its parser and createDeviceCSRGraph), label signatures as generated, path and
cycle signatures, the distance-shell signatures of every refinement step, the
dense candidate matrix after the filter and after every refinement step, the
GMCR offsets and query indices, and the join's totals in find-first and
find-all mode.

Inputs stay inside the reference's domain (data graphs of at most 64 nodes,
queries of at most 30, no empty data graph: its range mask shifts a 32-bit
word by 32 there, candidates.hpp:90).

Run from the repository root, where the reference tree is readable:
    python tests/golden/make_ref_golden.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from bms2_gb300 import workloads  # noqa: E402
from bms2_gb300.build import build  # noqa: E402
from oracle.ref import build_ref  # noqa: E402
from tests.kat_graphs import C, N, O, WILD, chain, line, ring, star  # noqa: E402

OUT = Path(__file__).resolve().parent
R = 6
DTYPES = {"u8": np.uint8, "u16": np.uint16, "u32": np.uint32, "u64": np.uint64}


def text_of(a: dict) -> str:
    """The reference text format of a CSR batch: one edge per symmetric pair of
    entries (u < v, in u's row order), with its edge label."""
    go, ro, ci, nl, el = (a["graph_offsets"], a["row_offsets"], a["column_indices"], a["node_labels"],
                          a["edge_labels"])
    lines = []
    for g in range(len(go) - 1):
        s, e = int(go[g]), int(go[g + 1])
        parts = [f"n#{e - s}", "l#11"]
        for v in range(s, e):
            parts += [str(v - s), str(int(nl[v]))]
        edges = [(v - s, int(ci[i]) - s, int(el[i])) for v in range(s, e) for i in range(int(ro[v]), int(ro[v + 1]))
                 if int(ci[i]) > v]
        parts.append(f"e#{len(edges)}")
        for u, v, l in edges:
            parts += [str(u), str(v), str(l)]
        lines.append(" ".join(parts))
    return "\n".join(lines) + "\n"


# hand-built graphs at the edges of the reference's rules
EXTRA_QUERIES = [
    line(*ring(6)), line(*star(2)), line([WILD, C], [(0, 1)]), line([20, C], [(0, 1)]), line([C], []),
    line(*chain(4)), line([C, C, O], [(0, 1), (1, 2), (2, 0)]), line(*ring(5, [C, C, N, C, C])),
]
EXTRA_DATA = [
    line(*ring(6)), line(*star(3)), line([O, C], [(0, 1)]), line([20, C, C], [(0, 1), (1, 2)]), line(*ring(5)),
    line(ring(5)[0], ring(5)[1] + [(0, 1)]),            # a repeated edge: repeated CSR entries
    line([C, C, C], [(0, 1), (1, 1), (1, 2)]),          # a self-loop (graph.hpp:229-240)
    line([C] * 16 + [N] * 2, [(i, i + 1) for i in range(17)] + [(0, 5), (5, 10)]),
]


def cases():
    q, d = workloads.make("mol1k", 11, n_data=250, n_queries=20)
    yield "mol1k", text_of(q.arrays()) + "\n".join(EXTRA_QUERIES) + "\n", text_of(d.arrays()) + "\n".join(
        EXTRA_DATA) + "\n"
    q, d = workloads.make("mol100k", 12, n_data=120, n_queries=24)
    d = d.filter_size(1, 64)
    yield "mol100k", text_of(q.arrays()), text_of(d.arrays())


def run_case(driver: Path, name: str, qtext: str, dtext: str) -> Path:
    with tempfile.TemporaryDirectory() as tmp:
        t = Path(tmp)
        (t / "q.txt").write_text(qtext)
        (t / "d.txt").write_text(dtext)
        out = t / "out"
        out.mkdir()
        subprocess.run([str(driver), str(t / "q.txt"), str(t / "d.txt"), str(R), str(out), "join"], check=True)
        arrays = {"query_text": np.frombuffer(qtext.encode(), np.uint8), "data_text": np.frombuffer(dtext.encode(), np.uint8),
                  "refine_steps": np.array([R], np.int32)}
        for row in (out / "manifest.txt").read_text().split("\n"):
            if not row.strip():
                continue
            key, dt, n = row.split()
            arrays[key] = np.fromfile(out / f"{key}.bin", dtype=DTYPES[dt], count=int(n))
        path = OUT / f"ref_{name}.npz"
        np.savez_compressed(path, **arrays)
        return path


def main(ref_root: str | None = None) -> None:
    build()
    driver = build_ref.build(Path(ref_root) if ref_root else build_ref.DEFAULT_REF)
    for name, qtext, dtext in cases():
        p = run_case(driver, name, qtext, dtext)
        print(p, p.stat().st_size)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
