"""ctypes driver of liboracle.so: the reference pipeline of BMS2.cpp:131-234
(signatures, filter, refine steps 1..R, GMCR, join) run on the CPU.

Test infrastructure only (the checker).  See oracle.cpp for the file:line
citations of every restated kernel.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

_u32p = C.POINTER(C.c_uint32)
_u64p = C.POINTER(C.c_uint64)
_u16p = C.POINTER(C.c_uint16)
_u8p = C.POINTER(C.c_uint8)
_f32p = C.POINTER(C.c_float)

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from bms2_gb300 import build as _b

            _b.build_oracle()
        L = C.CDLL(str(LIB_PATH))
        L.orc_words_per_row.restype = C.c_uint64
        L.orc_words_per_row.argtypes = [C.c_uint64]
        L.orc_signatures.restype = C.c_int
        L.orc_signatures.argtypes = [C.c_uint32, _u32p, _u32p, _u32p, _u8p, C.c_int, C.c_int, C.c_int, _u64p, _u64p,
                                     _u16p, _u64p]
        L.orc_filter.restype = C.c_int
        L.orc_filter.argtypes = [C.c_uint64, _u32p, _u8p, _u64p, _u16p, C.c_uint64, _u32p, _u8p, _u64p, _u16p, C.c_int,
                                 _u32p]
        L.orc_refine.restype = C.c_int
        L.orc_refine.argtypes = [C.c_uint64, _u64p, C.c_uint64, _u64p, C.c_int, _u32p]
        L.orc_gmcr.restype = C.c_int
        L.orc_gmcr.argtypes = [C.c_uint32, _u32p, C.c_uint32, _u32p, C.c_uint64, _u32p, C.c_int, _u32p, _u32p,
                               C.c_uint64, _u64p]
        L.orc_join.restype = C.c_int
        L.orc_join.argtypes = [C.c_uint32, _u32p, _u32p, _u32p, C.c_uint32, _u32p, _u32p, _u32p, C.c_uint64, _u32p,
                               _u32p, _u32p, C.c_int, C.c_int, C.c_int, C.c_int, _u64p, _u64p]
        L.orc_join_cs.restype = C.c_int
        L.orc_join_cs.argtypes = [C.c_uint32, _u32p, _u32p, _u32p, C.c_uint32, _u32p, _u32p, _u32p, C.c_uint64,
                                  _u32p, _u32p, _u32p, C.c_int, C.c_int, C.c_int, _u64p, _u64p, _u64p, _u64p]
        L.orc_pair_embeddings.restype = C.c_int
        L.orc_pair_embeddings.argtypes = [_u32p, _u32p, _u32p, _u32p, _u32p, _u32p, C.c_uint64, _u32p, _u32p,
                                          C.c_uint32, _u32p, C.c_uint64, C.POINTER(C.c_uint8), C.c_uint64, _u64p]
        L.orc_mlp_grad.restype = C.c_float
        L.orc_mlp_grad.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p,
                                   _f32p, _f32p, _f32p, _f32p, _f32p]
        _lib = L
    return _lib


def _p(a, ct):
    return None if a is None else a.ctypes.data_as(C.POINTER(ct))


def _csr(g) -> dict:
    """Accepts a bms2_gb300.Graphs or a dict of CSR arrays."""
    if isinstance(g, dict):
        return {k: np.ascontiguousarray(v) for k, v in g.items()}
    return g.arrays()


@dataclass
class Signatures:
    label_gen: np.ndarray
    path: np.ndarray   # [n, 4] uint64
    cycle: np.ndarray  # [n, 4] uint16
    shells: np.ndarray  # [R, n] uint64


def signatures(g: dict, R: int, x86: bool = False, threads: int = 0) -> Signatures:
    L = load()
    n = int(g["graph_offsets"][-1])
    lg = np.zeros(max(n, 1), np.uint64)
    path = np.zeros(max(4 * n, 1), np.uint64)
    cyc = np.zeros(max(4 * n, 1), np.uint16)
    sh = np.zeros(max(R * n, 1), np.uint64)
    L.orc_signatures(len(g["graph_offsets"]) - 1, _p(g["graph_offsets"], C.c_uint32), _p(g["row_offsets"], C.c_uint32),
                     _p(g["column_indices"], C.c_uint32), _p(g["node_labels"], C.c_uint8), R, int(x86), threads,
                     _p(lg, C.c_uint64), _p(path, C.c_uint64), _p(cyc, C.c_uint16), _p(sh, C.c_uint64))
    return Signatures(lg[:n], path[: 4 * n].reshape(n, 4), cyc[: 4 * n].reshape(n, 4), sh[: R * n].reshape(R, n))


@dataclass
class OracleResult:
    q_sigs: Signatures
    d_sigs: Signatures
    cand_filter: np.ndarray | None
    cand_steps: list = field(default_factory=list)  # candidate matrix after each refine step
    offsets: np.ndarray | None = None
    qidx: np.ndarray | None = None
    counts: np.ndarray | None = None
    expansions: np.ndarray | None = None
    n_partial: int = 0      # clustered join: prototype matches over all data graphs
    partial_exps: int = 0   # clustered join: roots and pushes of its first step

    @property
    def cand(self) -> np.ndarray:
        return self.cand_steps[-1] if self.cand_steps else self.cand_filter

    def pair_counts_dense(self, n_queries: int) -> np.ndarray:
        """[Q, D] counts, zero for pairs outside the GMCR."""
        D = len(self.offsets) - 1
        out = np.zeros((n_queries, D), np.uint64)
        for d in range(D):
            for t in range(self.offsets[d], self.offsets[d + 1]):
                out[self.qidx[t], d] = self.counts[t]
        return out

    @property
    def total(self) -> int:
        return int(self.counts.sum()) if self.counts is not None else 0


def run_pipeline(query, data, R: int, find_first: bool = False, x86: bool = False, dfs_literal: bool = False,
                 threads: int = 0, keep_steps: bool = True, join: bool = True, cs: bool = False) -> OracleResult:
    """The reference driver's flow (BMS2.cpp:131-234) on the CPU; cs=True runs
    the clustered join of its --use-cs flag (BMS2.cpp:218-296, query 0 the
    prototype), falling back to the plain join when query 0 is empty."""
    if cs and x86:
        raise ValueError("the clustered join has the generalized reading only")
    L = load()
    q, d = _csr(query), _csr(data)
    qs = signatures(q, R, x86, threads)
    ds = signatures(d, R, x86, threads)
    Qn = int(q["graph_offsets"][-1])
    Dn = int(d["graph_offsets"][-1])
    W = int(L.orc_words_per_row(Dn))
    cand = np.zeros(max(Qn * W, 1), np.uint32)
    L.orc_filter(Qn, _p(q["row_offsets"], C.c_uint32), _p(q["node_labels"], C.c_uint8),
                 _p(np.ascontiguousarray(qs.path), C.c_uint64), _p(np.ascontiguousarray(qs.cycle), C.c_uint16), Dn,
                 _p(d["row_offsets"], C.c_uint32), _p(d["node_labels"], C.c_uint8),
                 _p(np.ascontiguousarray(ds.path), C.c_uint64), _p(np.ascontiguousarray(ds.cycle), C.c_uint16), threads,
                 _p(cand, C.c_uint32))
    res = OracleResult(qs, ds, cand[: Qn * W].reshape(Qn, W).copy())
    for k in range(1, R + 1):
        L.orc_refine(Qn, _p(np.ascontiguousarray(qs.shells[k - 1]), C.c_uint64), Dn,
                     _p(np.ascontiguousarray(ds.shells[k - 1]), C.c_uint64), threads, _p(cand, C.c_uint32))
        if keep_steps or k == R:
            res.cand_steps.append(cand[: Qn * W].reshape(Qn, W).copy())
    Qg = len(q["graph_offsets"]) - 1
    Dg = len(d["graph_offsets"]) - 1
    offsets = np.zeros(Dg + 1, np.uint32)
    total = C.c_uint64()
    L.orc_gmcr(Qg, _p(q["graph_offsets"], C.c_uint32), Dg, _p(d["graph_offsets"], C.c_uint32), Dn, _p(cand, C.c_uint32),
               threads, _p(offsets, C.c_uint32), None, 0, C.byref(total))
    T = total.value
    qidx = np.zeros(max(T, 1), np.uint32)
    L.orc_gmcr(Qg, _p(q["graph_offsets"], C.c_uint32), Dg, _p(d["graph_offsets"], C.c_uint32), Dn, _p(cand, C.c_uint32),
               threads, _p(offsets, C.c_uint32), _p(qidx, C.c_uint32), len(qidx), C.byref(total))
    res.offsets, res.qidx = offsets, qidx[:T]
    if join and cs:
        counts = np.zeros(max(T, 1), np.uint64)
        exps = np.zeros(max(T, 1), np.uint64)
        npart, pexps = C.c_uint64(), C.c_uint64()
        r = L.orc_join_cs(Qg, _p(q["graph_offsets"], C.c_uint32), _p(q["row_offsets"], C.c_uint32),
                          _p(q["column_indices"], C.c_uint32), Dg, _p(d["graph_offsets"], C.c_uint32),
                          _p(d["row_offsets"], C.c_uint32), _p(d["column_indices"], C.c_uint32), Dn,
                          _p(cand, C.c_uint32), _p(offsets, C.c_uint32), _p(qidx, C.c_uint32), int(find_first),
                          int(dfs_literal), threads, _p(counts, C.c_uint64), _p(exps, C.c_uint64), C.byref(npart),
                          C.byref(pexps))
        if r == 0:
            res.counts, res.expansions = counts[:T], exps[:T]
            res.n_partial, res.partial_exps = int(npart.value), int(pexps.value)
            return res
    if join:
        counts = np.zeros(max(T, 1), np.uint64)
        exps = np.zeros(max(T, 1), np.uint64)
        L.orc_join(Qg, _p(q["graph_offsets"], C.c_uint32), _p(q["row_offsets"], C.c_uint32),
                   _p(q["column_indices"], C.c_uint32), Dg, _p(d["graph_offsets"], C.c_uint32),
                   _p(d["row_offsets"], C.c_uint32), _p(d["column_indices"], C.c_uint32), Dn, _p(cand, C.c_uint32),
                   _p(offsets, C.c_uint32), _p(qidx, C.c_uint32), int(find_first), int(x86), int(dfs_literal), threads,
                   _p(counts, C.c_uint64), _p(exps, C.c_uint64))
        res.counts, res.expansions = counts[:T], exps[:T]
    return res


def mlp_grad(params: np.ndarray, x: np.ndarray, y: np.ndarray):
    """CPU forward/backward of the cost model (bf16-rounded weights, fp32 math)."""
    L = load()
    p = np.ascontiguousarray(params, np.float32)
    W1, b1 = p[0:768], p[768:832]
    W2, b2 = p[832:4928], p[4928:4992]
    w3, b3 = p[4992:5056], p[5056:5057]
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    B = len(y)
    pred = np.zeros(B, np.float32)
    g = np.zeros_like(p)
    gW1, gb1, gW2, gb2, gw3, gb3 = (g[0:768], g[768:832], g[832:4928], g[4928:4992], g[4992:5056], g[5056:5057])
    loss = L.orc_mlp_grad(B, _p(x, C.c_float), _p(y, C.c_float), _p(W1, C.c_float), _p(b1, C.c_float),
                          _p(W2, C.c_float), _p(b2, C.c_float), _p(w3, C.c_float), _p(b3, C.c_float),
                          _p(pred, C.c_float), _p(gW1, C.c_float), _p(gb1, C.c_float), _p(gW2, C.c_float),
                          _p(gb2, C.c_float), _p(gw3, C.c_float), _p(gb3, C.c_float))
    return pred, g, float(loss)


def cpu_threads() -> int:
    return os.cpu_count() or 1


def pair_embeddings(query, data, res: "OracleResult", t: int, cap: int = 1 << 20) -> np.ndarray:
    """Every embedding of GMCR pair t of a run_pipeline result (EXACT semantics,
    the candidate matrix of its last refine step): [k, n] local data ids per
    query vertex, sorted lexicographically."""
    L = load()
    q, d = _csr(query), _csr(data)
    qi = int(res.qidx[t])
    n = int(q["graph_offsets"][qi + 1] - q["graph_offsets"][qi])
    out = np.zeros(max(cap * n, 1), np.uint8)
    found = C.c_uint64()
    Dn = int(d["graph_offsets"][-1])
    cand = np.ascontiguousarray(res.cand)
    r = L.orc_pair_embeddings(_p(q["graph_offsets"], C.c_uint32), _p(q["row_offsets"], C.c_uint32),
                              _p(q["column_indices"], C.c_uint32), _p(d["graph_offsets"], C.c_uint32),
                              _p(d["row_offsets"], C.c_uint32), _p(d["column_indices"], C.c_uint32), Dn,
                              _p(cand, C.c_uint32), _p(res.offsets, C.c_uint32), len(d["graph_offsets"]) - 1,
                              _p(res.qidx, C.c_uint32), t, out.ctypes.data_as(C.POINTER(C.c_uint8)), cap,
                              C.byref(found))
    if r != 0:
        raise ValueError("pair index out of range")
    k = int(found.value)
    if k > cap:
        raise ValueError(f"{k} embeddings exceed cap {cap}")
    e = out[:k * n].reshape(k, n)
    return e[np.lexsort(e.T[::-1])] if k else e

