"""Fixtures made by the reference's own code (tests/golden/ref_*.npz).

tests/golden/make_ref_golden.py compiles the reference's headers on the CPU
against a host-only SYCL stand-in (oracle/ref/, patches disclosed in
oracle/ref/build_ref.py) and records every intermediate of its pipeline on
seeded inputs.  This module loads them for the oracle and engine tests.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).with_name("golden")
CASES = ["mol1k", "mol100k"]


def load(name: str) -> dict:
    with np.load(GOLDEN / f"ref_{name}.npz") as z:
        return {k: z[k] for k in z.files}


def texts(f: dict) -> tuple[bytes, bytes]:
    return bytes(f["query_text"]), bytes(f["data_text"])


def n_nodes(f: dict, side: str) -> int:
    return len(f[f"{side}_node_labels"])


def candidates(f: dict, key: str) -> np.ndarray:
    """A dense candidate matrix of the fixture as [query nodes, words]."""
    qn = n_nodes(f, "q")
    return f[key].reshape(qn, -1)
