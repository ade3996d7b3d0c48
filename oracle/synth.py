"""Seeded synthetic workloads for the CPU side, without the engine library.

Test infrastructure only.  The CPU-baseline arm of the benchmark must run the
restated reference pipeline with nothing of the GPU engine mapped into its
process, yet on exactly the inputs the engine sees.  The generator source
(bms2_gb300/csrc/synth.cpp and the host graph container graphs.cpp) is
therefore compiled a second time, on its own, into oracle/_build/libsynth.so;
the same seed gives byte-identical CSR arrays in both libraries.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libsynth.so"

_lib = None


class _View(C.Structure):
    _fields_ = [("n_graphs", C.c_uint32), ("max_nodes", C.c_uint32), ("n_nodes", C.c_uint64),
                ("n_entries", C.c_uint64), ("graph_offsets", C.POINTER(C.c_uint32)),
                ("row_offsets", C.POINTER(C.c_uint32)), ("column_indices", C.POINTER(C.c_uint32)),
                ("node_labels", C.POINTER(C.c_uint8)), ("edge_labels", C.POINTER(C.c_uint8))]


class _MolParams(C.Structure):
    _fields_ = [("n_graphs", C.c_uint32), ("size_dist", C.c_uint32), ("p0", C.c_double), ("p1", C.c_double),
                ("min_nodes", C.c_uint32), ("max_nodes", C.c_uint32), ("min_rings", C.c_uint32),
                ("max_rings", C.c_uint32)]


class _QueryParams(C.Structure):
    _fields_ = [("n_queries", C.c_uint32), ("min_nodes", C.c_uint32), ("max_nodes", C.c_uint32),
                ("frac_carbon", C.c_double), ("frac_adversarial", C.c_double)]


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from bms2_gb300 import build as _b

            _b.build_synth()
        L = C.CDLL(str(LIB_PATH))
        L.bms_synth_molecules.restype = C.c_int
        L.bms_synth_molecules.argtypes = [C.POINTER(_MolParams), C.c_uint64, C.POINTER(C.c_void_p)]
        L.bms_synth_queries.restype = C.c_int
        L.bms_synth_queries.argtypes = [C.POINTER(_QueryParams), C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]
        L.bms_graphs_view_of.restype = C.c_int
        L.bms_graphs_view_of.argtypes = [C.c_void_p, C.POINTER(_View)]
        L.bms_graphs_free.restype = None
        L.bms_graphs_free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _arrays(h) -> dict:
    v = _View()
    if load().bms_graphs_view_of(h, C.byref(v)) != 0:
        raise RuntimeError("bms_graphs_view_of failed")

    def arr(p, n, dt):
        return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True) if n else np.zeros(0, dt)

    return {"graph_offsets": arr(v.graph_offsets, v.n_graphs + 1, np.uint32),
            "row_offsets": arr(v.row_offsets, v.n_nodes + 1, np.uint32),
            "column_indices": arr(v.column_indices, v.n_entries, np.uint32),
            "node_labels": arr(v.node_labels, v.n_nodes, np.uint8),
            "edge_labels": arr(v.edge_labels, v.n_entries, np.uint8)}


def make(name: str, seed: int = 1, n_data: int | None = None, n_queries: int | None = None) -> tuple[dict, dict]:
    """(queries, data) CSR dicts of a named workload, identical to
    bms2_gb300.workloads.make(name, seed, n_data, n_queries).arrays()."""
    from bms2_gb300.workloads import WORKLOADS

    w = WORKLOADS[name]
    L = load()
    hd, hq = C.c_void_p(), C.c_void_p()
    mp = _MolParams(n_data or w.n_data, w.size_dist, w.p0, w.p1, w.min_atoms, w.max_atoms, 1, 4)
    if L.bms_synth_molecules(C.byref(mp), seed, C.byref(hd)) != 0:
        raise RuntimeError("bms_synth_molecules failed")
    try:
        qp = _QueryParams(n_queries or w.n_queries, w.q_min, w.q_max, w.frac_carbon, w.frac_adversarial)
        if L.bms_synth_queries(C.byref(qp), hd, seed + 1000003, C.byref(hq)) != 0:
            raise RuntimeError("bms_synth_queries failed")
        try:
            return _arrays(hq), _arrays(hd)
        finally:
            L.bms_graphs_free(hq)
    finally:
        L.bms_graphs_free(hd)
