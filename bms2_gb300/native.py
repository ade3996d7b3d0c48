"""ctypes binding of libbms.so (the C ABI in include/bms.h).

Used by the test-suite and bench.py.  Loading fails loudly when the library has
not been built: there is no Python or CPU fallback for any stage.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import build as _build

LIB_PATH = Path(os.environ.get("BMS_LIB", str(_build.LIB)))

BMS_OK = 0
STATUS = {0: "BMS_OK", -1: "BMS_EINVAL", -2: "BMS_ENOMEM", -3: "BMS_ECUDA", -4: "BMS_EIO", -5: "BMS_ESTATE",
          -6: "BMS_EUNSUPPORTED", -7: "BMS_ETIMEDOUT", -8: "BMS_EINCOMPLETE", -9: "BMS_ENODEV"}
QUERY, DATA = 0, 1
FIND_FIRST, COUNT_ALL = 0, 1
ORDER_GMCR, ORDER_LEARNED, ORDER_GIVEN = 0, 1, 2
SEM_EXACT, SEM_REFERENCE_DFS = 0, 1
SIZE_UNIFORM, SIZE_NORMAL, SIZE_LOGNORMAL = 0, 1, 2
NUM_FEATURES = 12
MLP_PARAMS = 64 * 12 + 64 + 64 * 64 + 64 + 64 + 1
SCHED_BUCKETS = 4
(OPT_FILTER_KERNEL, OPT_JOIN_STEPS, OPT_SPLIT_BUDGET, OPT_SUBTREE_CAP, OPT_CUDA_GRAPH, OPT_USE_CS,
 OPT_RESIDENT_SIGNATURES) = 1, 2, 3, 4, 5, 6, 7
FILTER_SLICED, FILTER_BALLOT = 0, 1


class BmsError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class GraphsView(C.Structure):
    _fields_ = [("n_graphs", C.c_uint32), ("max_nodes", C.c_uint32), ("n_nodes", C.c_uint64),
                ("n_entries", C.c_uint64), ("graph_offsets", C.POINTER(C.c_uint32)),
                ("row_offsets", C.POINTER(C.c_uint32)), ("column_indices", C.POINTER(C.c_uint32)),
                ("node_labels", C.POINTER(C.c_uint8)), ("edge_labels", C.POINTER(C.c_uint8))]


class MolParams(C.Structure):
    _fields_ = [("n_graphs", C.c_uint32), ("size_dist", C.c_uint32), ("p0", C.c_double), ("p1", C.c_double),
                ("min_nodes", C.c_uint32), ("max_nodes", C.c_uint32), ("min_rings", C.c_uint32),
                ("max_rings", C.c_uint32)]


class QueryParams(C.Structure):
    _fields_ = [("n_queries", C.c_uint32), ("min_nodes", C.c_uint32), ("max_nodes", C.c_uint32),
                ("frac_carbon", C.c_double), ("frac_adversarial", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("n_query_graphs", C.c_uint32), ("n_data_graphs", C.c_uint32), ("n_query_nodes", C.c_uint64),
                ("n_data_nodes", C.c_uint64), ("n_pairs", C.c_uint64), ("n_valid_pairs", C.c_uint64),
                ("n_incomplete", C.c_uint64), ("total_matches", C.c_uint64), ("expansions", C.c_uint64),
                ("refine_steps", C.c_uint32), ("last_mode", C.c_uint32), ("last_order", C.c_uint32),
                ("last_semantics", C.c_uint32), ("ms_signatures", C.c_float), ("ms_filter", C.c_float),
                ("ms_refine", C.c_float), ("ms_map", C.c_float), ("ms_order", C.c_float), ("ms_join", C.c_float),
                ("ms_total", C.c_float), ("kernel_launches", C.c_uint64), ("n_partial_matches", C.c_uint64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Schedule(C.Structure):
    _fields_ = [("max_data_nodes", C.c_uint32 * SCHED_BUCKETS), ("word_bits", C.c_uint32 * SCHED_BUCKETS),
                ("split_depth", C.c_uint32 * SCHED_BUCKETS), ("blocks_per_sm", C.c_uint32 * SCHED_BUCKETS),
                ("warps_per_block", C.c_uint32 * SCHED_BUCKETS), ("steps", C.c_uint32 * SCHED_BUCKETS),
                ("refill", C.c_uint32 * SCHED_BUCKETS), ("split_budget", C.c_uint32 * SCHED_BUCKETS),
                ("lanes_per_pair", C.c_uint32 * SCHED_BUCKETS), ("ms", C.c_float * SCHED_BUCKETS)]

    def as_dict(self) -> dict:
        return {k: list(getattr(self, k)) for k, _ in self._fields_}


_u32p = C.POINTER(C.c_uint32)
_u64p = C.POINTER(C.c_uint64)
_u16p = C.POINTER(C.c_uint16)
_u8p = C.POINTER(C.c_uint8)
_f32p = C.POINTER(C.c_float)
_vp = C.c_void_p

# (name, restype, argtypes) for every function of include/bms.h
SIGNATURES = [
    ("bms_last_error", C.c_char_p, [_vp]),
    ("bms_status_name", C.c_char_p, [C.c_int]),
    ("bms_abi_version", C.c_int, []),
    ("bms_graphs_parse_file", C.c_int, [C.c_char_p, C.c_uint32, C.c_int, C.POINTER(_vp)]),
    ("bms_graphs_parse_text", C.c_int, [C.c_char_p, C.c_size_t, C.c_uint32, C.c_int, C.POINTER(_vp)]),
    ("bms_graphs_from_csr", C.c_int, [C.c_uint32, _u32p, _u32p, _u32p, _u8p, _u8p, C.POINTER(_vp)]),
    ("bms_graphs_view_of", C.c_int, [_vp, C.POINTER(GraphsView)]),
    ("bms_graphs_write_file", C.c_int, [_vp, C.c_char_p]),
    ("bms_graphs_filter_size", C.c_int, [_vp, C.c_uint32, C.c_uint32, C.POINTER(_vp)]),
    ("bms_graphs_free", None, [_vp]),
    ("bms_graphs_pin", C.c_int, [_vp]),
    ("bms_graphs_unpin", C.c_int, [_vp]),
    ("bms_synth_molecules", C.c_int, [C.POINTER(MolParams), C.c_uint64, C.POINTER(_vp)]),
    ("bms_synth_queries", C.c_int, [C.POINTER(QueryParams), _vp, C.c_uint64, C.POINTER(_vp)]),
    ("bms_shard_lpt", C.c_int, [C.c_uint32, _u32p, _u32p, C.c_uint32, _u32p, C.POINTER(C.c_double)]),
    ("bms_create", C.c_int, [C.c_int, C.POINTER(_vp)]),
    ("bms_destroy", None, [_vp]),
    ("bms_set_stream", C.c_int, [_vp, _vp]),
    ("bms_set_expansion_budget", C.c_int, [_vp, C.c_uint64]),
    ("bms_set_logging", C.c_int, [_vp, C.c_int]),
    ("bms_set_option", C.c_int, [_vp, C.c_int, C.c_int64]),
    ("bms_load_graphs", C.c_int, [_vp, C.c_int, _vp]),
    ("bms_load_csr", C.c_int, [_vp, C.c_int, C.c_uint32, _u32p, _u32p, _u32p, _u8p, _u8p]),
    ("bms_signatures", C.c_int, [_vp, C.c_int]),
    ("bms_filter", C.c_int, [_vp]),
    ("bms_refine", C.c_int, [_vp, C.c_int]),
    ("bms_map", C.c_int, [_vp, _u64p]),
    ("bms_join", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _u64p]),
    ("bms_run", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _u64p]),
    ("bms_run_batches", C.c_int, [_vp, _vp, C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_int, _u64p, _u64p]),
    ("bms_load_resident", C.c_int, [_vp, _vp]),
    ("bms_run_resident", C.c_int, [_vp, C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_int, _u64p, _u64p]),
    ("bms_get_stats", C.c_int, [_vp, C.POINTER(Stats)]),
    ("bms_get_gmcr", C.c_int, [_vp, _u32p, _u32p, C.c_uint64]),
    ("bms_gmcr_offsets_static", C.c_int, [_vp, _vp, C.c_uint64, _vp]),
    ("bms_get_embeddings", C.c_int, [_vp, C.c_uint64, C.POINTER(C.c_uint8), C.c_uint64, _u64p]),
    ("bms_get_pair_counts", C.c_int, [_vp, _u64p, C.c_uint64]),
    ("bms_get_pair_expansions", C.c_int, [_vp, _u64p, C.c_uint64]),
    ("bms_get_pair_status", C.c_int, [_vp, _u8p, C.c_uint64]),
    ("bms_get_candidates", C.c_int, [_vp, _u32p, C.c_uint64]),
    ("bms_get_signatures", C.c_int, [_vp, C.c_int, _u64p, _u64p, _u16p, _u64p]),
    ("bms_feature_name", C.c_char_p, [C.c_int]),
    ("bms_query_features", C.c_int, [_vp, _f32p]),
    ("bms_vertex_expansions", C.c_int, [_vp, _u64p]),
    ("bms_model_train", C.c_int, [_vp, _f32p, _f32p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float, C.c_uint64,
                                  _f32p]),
    ("bms_model_grad", C.c_int, [_vp, _f32p, _f32p, _f32p, C.c_uint32, _f32p, _f32p, _f32p]),
    ("bms_model_get", C.c_int, [_vp, _f32p]),
    ("bms_model_set", C.c_int, [_vp, _f32p]),
    ("bms_model_save", C.c_int, [_vp, C.c_char_p]),
    ("bms_model_load", C.c_int, [_vp, C.c_char_p]),
    ("bms_model_predict", C.c_int, [_vp, _f32p, _u8p]),
    ("bms_set_query_order", C.c_int, [_vp, _u8p, C.c_uint64]),
    ("bms_get_schedule", C.c_int, [_vp, C.POINTER(Schedule)]),
    ("bms_set_schedule", C.c_int, [_vp, C.POINTER(Schedule)]),
    ("bms_autotune", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.POINTER(Schedule)]),
]

_lib = None


def lib() -> C.CDLL:
    """Load libbms.so (built by bms2_gb300.build); raises if it is missing."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise FileNotFoundError(f"{LIB_PATH} not found: build it with bms2_gb300.build.build()")
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a: np.ndarray | None, ct):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ct))


def _check(st: int, ctx=None) -> int:
    if st != BMS_OK:
        msg = lib().bms_last_error(ctx).decode(errors="replace")
        raise BmsError(st, msg)
    return st


# ---------------------------------------------------------------- graphs
class Graphs:
    """A host-side batched CSR owned by libbms."""

    def __init__(self, handle):
        self._h = handle

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h and _lib is not None:
            _lib.bms_graphs_free(h)

    @property
    def handle(self):
        return self._h

    @classmethod
    def parse_text(cls, text: str | bytes, max_graphs: int = 0, skip_invalid: bool = False) -> "Graphs":
        b = text.encode() if isinstance(text, str) else text
        h = _vp()
        _check(lib().bms_graphs_parse_text(b, len(b), max_graphs, int(skip_invalid), C.byref(h)))
        return cls(h)

    @classmethod
    def parse_file(cls, path, max_graphs: int = 0, skip_invalid: bool = False) -> "Graphs":
        h = _vp()
        _check(lib().bms_graphs_parse_file(str(path).encode(), max_graphs, int(skip_invalid), C.byref(h)))
        return cls(h)

    @classmethod
    def from_csr(cls, graph_offsets, row_offsets, column_indices, node_labels, edge_labels=None) -> "Graphs":
        go = np.ascontiguousarray(graph_offsets, dtype=np.uint32)
        ro = np.ascontiguousarray(row_offsets, dtype=np.uint32)
        ci = np.ascontiguousarray(column_indices, dtype=np.uint32)
        nl = np.ascontiguousarray(node_labels, dtype=np.uint8)
        el = None if edge_labels is None else np.ascontiguousarray(edge_labels, dtype=np.uint8)
        h = _vp()
        _check(lib().bms_graphs_from_csr(len(go) - 1, _ptr(go, C.c_uint32), _ptr(ro, C.c_uint32),
                                         _ptr(ci, C.c_uint32), _ptr(nl, C.c_uint8), _ptr(el, C.c_uint8), C.byref(h)))
        return cls(h)

    @classmethod
    def synth_molecules(cls, n_graphs: int, seed: int, size_dist: int = SIZE_UNIFORM, p0: float = 0.0,
                        p1: float = 0.0, min_nodes: int = 10, max_nodes: int = 40, min_rings: int = 1,
                        max_rings: int = 4) -> "Graphs":
        p = MolParams(n_graphs, size_dist, p0, p1, min_nodes, max_nodes, min_rings, max_rings)
        h = _vp()
        _check(lib().bms_synth_molecules(C.byref(p), seed, C.byref(h)))
        return cls(h)

    @classmethod
    def synth_queries(cls, source: "Graphs", n_queries: int, seed: int, min_nodes: int = 3, max_nodes: int = 12,
                      frac_carbon: float = 0.0, frac_adversarial: float = 0.0) -> "Graphs":
        p = QueryParams(n_queries, min_nodes, max_nodes, frac_carbon, frac_adversarial)
        h = _vp()
        _check(lib().bms_synth_queries(C.byref(p), source.handle, seed, C.byref(h)))
        return cls(h)

    def view(self) -> GraphsView:
        v = GraphsView()
        _check(lib().bms_graphs_view_of(self._h, C.byref(v)))
        return v

    def arrays(self) -> dict:
        """Copies of the CSR arrays as numpy arrays."""
        v = self.view()

        def arr(p, n, dt):
            if n == 0:
                return np.zeros(0, dtype=dt)
            return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True)

        return {
            "graph_offsets": arr(v.graph_offsets, v.n_graphs + 1, np.uint32),
            "row_offsets": arr(v.row_offsets, v.n_nodes + 1, np.uint32),
            "column_indices": arr(v.column_indices, v.n_entries, np.uint32),
            "node_labels": arr(v.node_labels, v.n_nodes, np.uint8),
            "edge_labels": arr(v.edge_labels, v.n_entries, np.uint8),
        }

    @property
    def n_graphs(self) -> int:
        return self.view().n_graphs

    @property
    def n_nodes(self) -> int:
        return self.view().n_nodes

    @property
    def max_nodes(self) -> int:
        return self.view().max_nodes

    def pin(self) -> None:
        """Page-lock the batch for asynchronous uploads (undone when freed)."""
        _check(lib().bms_graphs_pin(self._h))

    def unpin(self) -> None:
        _check(lib().bms_graphs_unpin(self._h))

    def write_file(self, path) -> None:
        _check(lib().bms_graphs_write_file(self._h, str(path).encode()))

    def filter_size(self, min_nodes: int, max_nodes: int) -> "Graphs":
        h = _vp()
        _check(lib().bms_graphs_filter_size(self._h, min_nodes, max_nodes, C.byref(h)))
        return Graphs(h)


# ---------------------------------------------------------------- context
class Context:
    """One libbms context (one CUDA device, one stream)."""

    def __init__(self, device: int = 0):
        h = _vp()
        _check(lib().bms_create(device, C.byref(h)))
        self._h = h

    def close(self) -> None:
        h, self._h = getattr(self, "_h", None), None
        if h and _lib is not None:
            _lib.bms_destroy(h)

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _c(self, st: int) -> int:
        return _check(st, self._h)

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: int | None) -> None:
        self._c(lib().bms_set_stream(self._h, stream_ptr))

    def set_expansion_budget(self, budget: int) -> None:
        self._c(lib().bms_set_expansion_budget(self._h, budget))

    def set_option(self, option: int, value: int) -> None:
        self._c(lib().bms_set_option(self._h, option, value))

    def set_logging(self, vertex_expansions: bool) -> None:
        self._c(lib().bms_set_logging(self._h, int(vertex_expansions)))

    def load(self, kind: int, g: Graphs) -> None:
        self._c(lib().bms_load_graphs(self._h, kind, g.handle))
        if kind == QUERY:
            v = g.view()
            self._qgoff = np.ctypeslib.as_array(v.graph_offsets, shape=(v.n_graphs + 1,)).astype(np.uint32)

    def query_graph_offsets(self) -> np.ndarray:
        """Node offsets of the loaded query batch."""
        return self._qgoff

    def load_csr(self, kind: int, graph_offsets, row_offsets, column_indices, node_labels, edge_labels=None) -> None:
        arrs = [np.ascontiguousarray(graph_offsets, dtype=np.uint32), np.ascontiguousarray(row_offsets, dtype=np.uint32),
                np.ascontiguousarray(column_indices, dtype=np.uint32), np.ascontiguousarray(node_labels, dtype=np.uint8)]
        el = None if edge_labels is None else np.ascontiguousarray(edge_labels, dtype=np.uint8)
        self._c(lib().bms_load_csr(self._h, kind, len(arrs[0]) - 1, _ptr(arrs[0], C.c_uint32), _ptr(arrs[1], C.c_uint32),
                                   _ptr(arrs[2], C.c_uint32), _ptr(arrs[3], C.c_uint8), _ptr(el, C.c_uint8)))
        if kind == QUERY:
            self._qgoff = arrs[0].copy()

    def load_csr_ptrs(self, kind: int, n_graphs: int, goff: int, rowp: int, col: int, lab: int, elab: int | None) -> None:
        """Upload from raw host pointers (e.g. pinned buffers)."""
        L = lib()
        self._c(L.bms_load_csr(self._h, kind, n_graphs, C.cast(goff, _u32p), C.cast(rowp, _u32p), C.cast(col, _u32p),
                               C.cast(lab, _u8p), C.cast(elab, _u8p) if elab else None))

    # staged pipeline
    def signatures(self, refine_steps: int) -> None:
        self._c(lib().bms_signatures(self._h, refine_steps))

    def filter(self) -> None:
        self._c(lib().bms_filter(self._h))

    def refine(self, step: int) -> None:
        self._c(lib().bms_refine(self._h, step))

    def map(self) -> int:
        n = C.c_uint64()
        self._c(lib().bms_map(self._h, C.byref(n)))
        return n.value

    def join(self, mode: int = COUNT_ALL, order: int = ORDER_GMCR, semantics: int = SEM_EXACT) -> int:
        t = C.c_uint64()
        self._c(lib().bms_join(self._h, mode, order, semantics, C.byref(t)))
        return t.value

    # fused pipeline
    def run(self, refine_steps: int, mode: int = COUNT_ALL, order: int = ORDER_GMCR, semantics: int = SEM_EXACT) -> int:
        t = C.c_uint64()
        self._c(lib().bms_run(self._h, refine_steps, mode, order, semantics, C.byref(t)))
        return t.value

    def load_resident(self, data: "Graphs") -> None:
        """Upload a data batch once and keep it in HBM for run_resident."""
        self._c(lib().bms_load_resident(self._h, data._h))

    def run_resident(self, window_graphs: int, refine_steps: int, mode: int = COUNT_ALL, order: int = ORDER_GMCR,
                     semantics: int = SEM_EXACT) -> tuple[int, np.ndarray]:
        """The loaded queries over the resident data in windows: (total, per-query matches)."""
        t = C.c_uint64()
        nq = self.stats()["n_query_graphs"]
        per_query = np.zeros(max(nq, 1), dtype=np.uint64)
        self._c(lib().bms_run_resident(self._h, window_graphs, refine_steps, mode, order, semantics, C.byref(t),
                                       _ptr(per_query, C.c_uint64)))
        return t.value, per_query[:nq]

    def run_batches(self, data: "Graphs", batch_graphs: int, refine_steps: int, mode: int = COUNT_ALL,
                    order: int = ORDER_GMCR, semantics: int = SEM_EXACT) -> tuple[int, np.ndarray]:
        """The loaded queries against `data` in slices of batch_graphs graphs: (total, per-query matches)."""
        t = C.c_uint64()
        per_query = np.zeros(max(self.stats()["n_query_graphs"], 1), dtype=np.uint64)
        self._c(lib().bms_run_batches(self._h, data._h, batch_graphs, refine_steps, mode, order, semantics,
                                      C.byref(t), _ptr(per_query, C.c_uint64)))
        return t.value, per_query[:self.stats()["n_query_graphs"]]

    # results
    def stats(self) -> dict:
        s = Stats()
        self._c(lib().bms_get_stats(self._h, C.byref(s)))
        return s.as_dict()

    def gmcr(self) -> tuple[np.ndarray, np.ndarray]:
        st = self.stats()
        off = np.zeros(st["n_data_graphs"] + 1, dtype=np.uint32)
        n = st["n_valid_pairs"]
        qidx = np.zeros(max(n, 1), dtype=np.uint32)
        self._c(lib().bms_get_gmcr(self._h, _ptr(off, C.c_uint32), _ptr(qidx, C.c_uint32), len(qidx)))
        return off, qidx[:n]

    def pair_counts(self) -> np.ndarray:
        n = self.stats()["n_valid_pairs"]
        out = np.zeros(max(n, 1), dtype=np.uint64)
        self._c(lib().bms_get_pair_counts(self._h, _ptr(out, C.c_uint64), len(out)))
        return out[:n]

    def embeddings(self, pair: int, max_embeddings: int | None = None) -> np.ndarray:
        """Every embedding of GMCR pair `pair` (count-all EXACT run): [k, n] local
        data ids per query vertex, sorted lexicographically."""
        found = C.c_uint64()
        self._c(lib().bms_get_embeddings(self._h, pair, None, 0, C.byref(found)))
        k = found.value if max_embeddings is None else min(found.value, max_embeddings)
        off, qidx = self.gmcr()
        qo = self.query_graph_offsets()
        n = int(qo[qidx[pair] + 1] - qo[qidx[pair]])
        out = np.zeros(max(k * n, 1), dtype=np.uint8)
        self._c(lib().bms_get_embeddings(self._h, pair, out.ctypes.data_as(C.POINTER(C.c_uint8)), k, C.byref(found)))
        return out[:k * n].reshape(k, n)

    def pair_expansions(self) -> np.ndarray:
        n = self.stats()["n_valid_pairs"]
        out = np.zeros(max(n, 1), dtype=np.uint64)
        self._c(lib().bms_get_pair_expansions(self._h, _ptr(out, C.c_uint64), len(out)))
        return out[:n]

    def pair_status(self) -> np.ndarray:
        n = self.stats()["n_valid_pairs"]
        out = np.zeros(max(n, 1), dtype=np.uint8)
        self._c(lib().bms_get_pair_status(self._h, _ptr(out, C.c_uint8), len(out)))
        return out[:n]

    def candidates(self) -> np.ndarray:
        st = self.stats()
        W = (st["n_data_nodes"] + 31) // 32
        out = np.zeros(max(st["n_query_nodes"] * W, 1), dtype=np.uint32)
        self._c(lib().bms_get_candidates(self._h, _ptr(out, C.c_uint32), len(out)))
        return out[: st["n_query_nodes"] * W].reshape(st["n_query_nodes"], W)

    def signatures_of(self, kind: int, steps: int) -> dict:
        st = self.stats()
        n = st["n_query_nodes"] if kind == QUERY else st["n_data_nodes"]
        lg = np.zeros(max(n, 1), dtype=np.uint64)
        path = np.zeros(max(4 * n, 1), dtype=np.uint64)
        cyc = np.zeros(max(4 * n, 1), dtype=np.uint16)
        sh = np.zeros(max(steps * n, 1), dtype=np.uint64)
        self._c(lib().bms_get_signatures(self._h, kind, _ptr(lg, C.c_uint64), _ptr(path, C.c_uint64),
                                         _ptr(cyc, C.c_uint16), _ptr(sh, C.c_uint64)))
        return {"label_gen": lg[:n], "path": path[: 4 * n].reshape(n, 4), "cycle": cyc[: 4 * n].reshape(n, 4),
                "shells": sh[: steps * n].reshape(steps, n)}

    # learned order
    def query_features(self) -> np.ndarray:
        n = self.stats()["n_query_nodes"]
        out = np.zeros(max(n * NUM_FEATURES, 1), dtype=np.float32)
        self._c(lib().bms_query_features(self._h, _ptr(out, C.c_float)))
        return out[: n * NUM_FEATURES].reshape(n, NUM_FEATURES)

    def vertex_expansions(self) -> np.ndarray:
        n = self.stats()["n_query_nodes"]
        out = np.zeros(max(n, 1), dtype=np.uint64)
        self._c(lib().bms_vertex_expansions(self._h, _ptr(out, C.c_uint64)))
        return out[:n]

    def model_train(self, x: np.ndarray, y: np.ndarray, epochs: int, batch: int, lr: float, seed: int) -> float:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        loss = C.c_float()
        self._c(lib().bms_model_train(self._h, _ptr(x, C.c_float), _ptr(y, C.c_float), len(y), epochs, batch, lr, seed,
                                      C.byref(loss)))
        return loss.value

    def model_grad(self, params: np.ndarray, x: np.ndarray, y: np.ndarray) -> tuple[np.ndarray, np.ndarray, float]:
        params = np.ascontiguousarray(params, dtype=np.float32)
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        yo = np.zeros(len(y), dtype=np.float32)
        g = np.zeros(MLP_PARAMS, dtype=np.float32)
        loss = C.c_float()
        self._c(lib().bms_model_grad(self._h, _ptr(params, C.c_float), _ptr(x, C.c_float), _ptr(y, C.c_float), len(y),
                                     _ptr(yo, C.c_float), _ptr(g, C.c_float), C.byref(loss)))
        return yo, g, loss.value

    def model_get(self) -> np.ndarray:
        p = np.zeros(MLP_PARAMS, dtype=np.float32)
        self._c(lib().bms_model_get(self._h, _ptr(p, C.c_float)))
        return p

    def model_set(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        assert p.size == MLP_PARAMS
        self._c(lib().bms_model_set(self._h, _ptr(p, C.c_float)))

    def model_save(self, path) -> None:
        self._c(lib().bms_model_save(self._h, str(path).encode()))

    def model_load(self, path) -> None:
        self._c(lib().bms_model_load(self._h, str(path).encode()))

    def model_predict(self) -> tuple[np.ndarray, np.ndarray]:
        n = self.stats()["n_query_nodes"]
        cost = np.zeros(max(n, 1), dtype=np.float32)
        order = np.zeros(max(n, 1), dtype=np.uint8)
        self._c(lib().bms_model_predict(self._h, _ptr(cost, C.c_float), _ptr(order, C.c_uint8)))
        return cost[:n], order[:n]

    def set_query_order(self, order: np.ndarray) -> None:
        """Explicit per-query search orders for ORDER_GIVEN (order[qoff + t] =
        the local vertex searched at depth t)."""
        o = np.ascontiguousarray(order, dtype=np.uint8)
        self._c(lib().bms_set_query_order(self._h, _ptr(o, C.c_uint8), len(o)))

    def schedule(self) -> dict:
        s = Schedule()
        self._c(lib().bms_get_schedule(self._h, C.byref(s)))
        return s.as_dict()

    def set_schedule(self, d: dict) -> None:
        s = Schedule()
        for k, _ in Schedule._fields_:
            if k in d:
                arr = getattr(s, k)
                for i, v in enumerate(d[k]):
                    arr[i] = v
        self._c(lib().bms_set_schedule(self._h, C.byref(s)))

    def autotune(self, refine_steps: int, mode: int = COUNT_ALL, order: int = ORDER_GMCR) -> dict:
        s = Schedule()
        self._c(lib().bms_autotune(self._h, refine_steps, mode, order, C.byref(s)))
        return s.as_dict()


def feature_names() -> list[str]:
    return [lib().bms_feature_name(i).decode() for i in range(NUM_FEATURES)]
