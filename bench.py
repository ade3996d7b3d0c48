#!/usr/bin/env python3
"""Benchmark: query x data-graph pairs per second of the batched engine on one GB300.

One step = one full pass of the fused pipeline over the whole workload with
inputs resident in HBM: signatures -> filter + 6 refinement steps -> GMCR ->
join (count-all, EXACT semantics, bit-exact counts), i.e. bms_run.  The
default workload is mol1m: 1,000,000 seeded synthetic molecular data graphs
(log-normal atom counts, median 25, clipped to 5-120) x 1,000 queries of 3-40
nodes — the batched configuration on which the learned order is trained (seed
A) and evaluated (seed B).  mol100k (100,000 graphs of N(28, 9) atoms x 600
queries of 5-30 nodes, 30% pure-carbon) is the plain-method GPU configuration.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--order learned|plain] [--workload mol100k|mol1m]
  python bench.py --workload mol1m-cs [--cluster-members M]   # the clustered join (--use-cs)
  python bench.py --impl reference ...   # the CPU restatement of the reference

With the learned order (the default) the cost model is first trained on a
seed-A workload of the same shape (every vertex's root-level search-tree size
logged by the join, GPU training); the timed steps run on seed-B inputs, and the plain GMCR order is
timed on the same inputs for the learned-over-plain ratio, with per-pair counts
compared.

With N > 1 (torchrun, one rank per GPU) the data batch is N times the
single-GPU batch, split across the ranks by the reference MPI driver's LPT
balancing; every rank runs the whole pipeline on its shard (weak scaling), and
the only collectives are the final sums and the maximum of the timed region.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = "mol1m"
REFINE_STEPS = 6
METRIC = "query x data-graph pairs/s, learned vs plain GMCR order (count-all, bit-exact counts)"
HBM_FALLBACK_GBS = 6800.0
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of the three fused
# filter launches per data graph, from one ncu capture of 100,000 graphs of the
# workload (traffic grows with the graphs processed).
FILTER_DRAM_BYTES_PER_GRAPH = {"mol1m": 1.4082e9 / 100_000}


def peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.skip = 0
        self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # the sampler takes a moment to start: wait for its first line so that
        # the samples cover the timed region
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            self.out.flush()
            if Path(self.out.name).stat().st_size > 0:
                break
            time.sleep(0.02)
        self.skip = Path(self.out.name).read_text().count("\n")

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.out.flush()
        rows = [r.split(",") for r in Path(self.out.name).read_text().strip().splitlines()[self.skip:] if r.strip()]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() in ("active", "1"):
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_filter_bytes(qn: int, dn: int, R: int) -> float:
    """Compulsory bytes of filter + refine: the Qn x Dn candidate bits written
    once plus the node signatures read (label 1 + row offset 4 + path 32 +
    cycle 8 bytes, and 8 bytes per refinement step) on both sides."""
    return qn * dn / 8.0 + (dn + qn) * (45.0 + 8.0 * R)


def graph_offsets(g) -> np.ndarray:
    """graph_offsets of a Graphs batch as a numpy view (no copy of the batch)."""
    v = g.view()
    if v.n_graphs == 0:
        return np.zeros(1, dtype=np.uint32)
    return np.ctypeslib.as_array(v.graph_offsets, shape=(v.n_graphs + 1,))


def outside_reference_domain(q_offsets, d_offsets) -> dict:
    """Share of a workload outside the reference's sizes: its bitsets and
    join arrays hold data graphs of <= 64 nodes and queries of <= 30 nodes
    (utils.hpp:90-120, isomorphism.hpp:248).  Pairs are the full cross
    product, so the pairs with either side beyond those sizes are
    1 - (data share inside) x (query share inside)."""
    dsz = np.diff(np.asarray(d_offsets, dtype=np.int64))
    qsz = np.diff(np.asarray(q_offsets, dtype=np.int64))
    d_in = float(np.mean(dsz <= 64)) if len(dsz) else 1.0
    q_in = float(np.mean(qsz <= 30)) if len(qsz) else 1.0
    return {"data_graphs_over_64_nodes": 1.0 - d_in, "queries_over_30_nodes": 1.0 - q_in,
            "pairs": 1.0 - d_in * q_in}


def algorithmic_signature_bytes(nodes: int, entries: int, R: int) -> float:
    """Compulsory bytes of the data and query signatures: row offsets and labels
    (4 + 1 per node) and the CSR column ids (4 per entry) read once, and per
    node the label (8), path (32), cycle (8) and R shell (8 R) signatures
    written once."""
    return nodes * (4.0 + 1.0) + entries * 4.0 + nodes * (8.0 + 32.0 + 8.0 + 8.0 * R)


def cpu_baseline(qa: dict, da: dict, threads: int, budget_s: float = 15.0, cs: bool = False) -> tuple[dict, object, int]:
    """The CPU restatement of the reference pipeline (OpenMP over nodes, words,
    pairs) on a bounded sample: all queries x the first k data graphs (cs: the
    clustered join of the driver's --use-cs).  Returns the baseline record, the
    oracle's result on the sample (its per-pair counts are the parity check of
    the GPU run) and k."""
    import oracle

    Q = len(qa["graph_offsets"]) - 1
    D = len(da["graph_offsets"]) - 1
    k = min(256, D)
    while True:
        sub = _head(da, k)
        t0 = time.perf_counter()
        res = oracle.run_pipeline(qa, sub, REFINE_STEPS, threads=threads, keep_steps=False, cs=cs)
        t_one = time.perf_counter() - t0
        if t_one > budget_s / 4 or k >= D:
            break
        k = min(k * 4, D)
    info = {"value": Q * k / t_one, "unit": "pairs/s", "cores": threads, "kind": "port",
            "sample": f"{Q} queries x first {k} of {D} data graphs, R={REFINE_STEPS}, "
                      f"count-all{', clustered join' if cs else ''}, {t_one:.2f} s", "matches": int(res.total)}
    return info, res, k


def sample_parity(gpu_offsets: np.ndarray, gpu_qidx: np.ndarray, gpu_counts: np.ndarray, res, k: int) -> dict:
    """The GPU run's GMCR rows and per-pair counts of the first k data graphs
    against the oracle's run on exactly those graphs (all queries)."""
    n = int(res.offsets[-1])
    ok_off = bool(len(gpu_offsets) > k and np.array_equal(gpu_offsets[:k + 1].astype(np.int64),
                                                           res.offsets.astype(np.int64)))
    ok_q = ok_off and bool(np.array_equal(gpu_qidx[:n], res.qidx))
    ok_c = ok_q and bool(np.array_equal(gpu_counts[:n], res.counts))
    return {"data_graphs": int(k), "pairs_compared": n, "gmcr_equal": ok_q, "counts_equal": ok_c,
            "matches": int(res.total)}


def _head(a: dict, k: int) -> dict:
    go = a["graph_offsets"][: k + 1]
    n = int(go[-1])
    ro = a["row_offsets"][: n + 1]
    e = int(ro[-1])
    return {"graph_offsets": go.copy(), "row_offsets": ro.copy(), "column_indices": a["column_indices"][:e].copy(),
            "node_labels": a["node_labels"][:n].copy(), "edge_labels": a["edge_labels"][:e].copy()}


def train_cost_model(ctx, workload: str, seed: int, n_data: int) -> dict:
    """Seed-A plain-order run with vertex logging -> features + targets -> GPU training."""
    from bms2_gb300 import COUNT_ALL, DATA, ORDER_GMCR, QUERY, SEM_EXACT, workloads
    from bms2_gb300.train import collect, train

    qa, da = workloads.make(workload, seed, n_data=n_data)
    ctx.load(QUERY, qa)
    ctx.load(DATA, da)
    x, y = collect(ctx, REFINE_STEPS, qa.arrays())
    loss = train(ctx, x, y, seed=seed)
    del COUNT_ALL, ORDER_GMCR, SEM_EXACT
    return {"train_samples": int(len(y)), "train_loss": float(loss), "train_seed": seed, "train_data_graphs": n_data,
            "train_workload": workload}


def run_ours(args) -> None:
    import torch
    import torch.distributed as dist

    from bms2_gb300 import (COUNT_ALL, DATA, FIND_FIRST, ORDER_GMCR, ORDER_LEARNED, QUERY, SEM_EXACT,
                            SEM_REFERENCE_DFS, Context, Graphs, shards, workloads)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = Context(local)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    order = ORDER_LEARNED if args.order == "learned" else ORDER_GMCR
    extra = {}
    if order == ORDER_LEARNED:
        extra.update(train_cost_model(ctx, args.workload, seed=101, n_data=args.train_graphs))
    schedule = None
    if args.tune_graphs != 0 and not args.once:
        # the join schedule per size bucket, tuned on seed-A inputs of the same shape
        tq, td = workloads.make(args.workload, 101, n_data=args.tune_graphs if args.tune_graphs > 0 else None)
        ctx.load(QUERY, tq)
        ctx.load(DATA, td)
        s = ctx.autotune(REFINE_STEPS, COUNT_ALL, order)
        schedule = [{"max_data_nodes": s["max_data_nodes"][k], "word_bits": s["word_bits"][k],
                     "split_depth": s["split_depth"][k], "blocks_per_sm": s["blocks_per_sm"][k],
                     "warps_per_block": s["warps_per_block"][k], "steps": s["steps"][k],
                     "refill": s["refill"][k], "lanes_per_pair": s["lanes_per_pair"][k],
                     "split_budget": s["split_budget"][k], "tuned_join_ms": round(s["ms"][k], 3)}
                    for k in range(3)]
        del tq, td
    # evaluation workload (seed B).  With N ranks the data batch is N blocks of
    # the single-GPU batch's size (block 0 is that batch; queries are the
    # single-GPU queries), split across the ranks by the reference MPI driver's
    # LPT balancing (BMS2_mpi.cpp:78-157): each rank holds about one block
    q, d = workloads.make(args.workload, 202, n_data=args.data_graphs)
    d_total = d.n_graphs
    if world > 1:
        full = workloads.make_data(args.workload, 202, n_data=world * d.n_graphs)
        fa = full.arrays()
        del full
        owners = shards.lpt_owners_native(fa, world)
        d = Graphs.from_csr(**shards.take_graphs(fa, np.nonzero(owners == rank)[0]))
        d_total = len(fa["graph_offsets"]) - 1
        del fa, owners
    Q, D = q.n_graphs, d.n_graphs
    qa, da = q.arrays(), d.arrays()
    ctx.load(QUERY, q)
    ctx.load(DATA, d)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def step(o=order, mode=COUNT_ALL, sem=SEM_EXACT):
        return ctx.run(REFINE_STEPS, mode, o, sem)

    def timed(o, k, mode=COUNT_ALL, sem=SEM_EXACT):
        """k steps of order o, each bracketed by CUDA events on the library's stream."""
        ms, stages = [], []
        for _ in range(k):
            flush.fill_(1)  # L2 flush between steps (outside the timed events)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            tot = step(o, mode, sem)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            stages.append(ctx.stats())
        return ms, stages, tot

    if args.once:  # one pipeline run, for profilers
        total = step()
        st = ctx.stats()
        e = np.sort(ctx.pair_expansions().astype(np.float64))[::-1]
        c = ctx.pair_counts()
        dist_ = {"pair_exp_max": float(e[0]) if len(e) else 0.0,
                 "pair_exp_p99": float(np.percentile(e, 99)) if len(e) else 0.0,
                 "pair_exp_top100_share": float(e[:100].sum() / max(e.sum(), 1.0)),
                 "pair_count_max": int(c.max()) if len(c) else 0,
                 "pairs_with_work": int((e > 0).sum())}
        print(json.dumps({"once": True, "order": args.order, "total": int(total), **st, **dist_}), flush=True)
        ctx.close()
        return
    for _ in range(args.warmup):
        step()
    plain = None
    if order == ORDER_LEARNED:
        # the plain GMCR order on the same inputs: per-pair counts must be equal,
        # and its timed steps give the learned-over-plain ratio
        plain_total = step(ORDER_GMCR)
        plain_counts, plain_exp = ctx.pair_counts(), ctx.stats()["expansions"]
        step()
        same_pairs = bool(np.array_equal(ctx.pair_counts(), plain_counts))
        for _ in range(args.warmup):
            step(ORDER_GMCR)
        p_ms, p_stage, _ = timed(ORDER_GMCR, args.steps)
        plain = {"plain_total_matches": int(plain_total), "plain_expansions": int(plain_exp),
                 "counts_equal_every_pair": same_pairs,
                 "plain_ms_per_step": float(np.mean(p_ms)),
                 "plain_join_ms": float(np.mean([s["ms_join"] for s in p_stage]))}
        for _ in range(args.warmup):
            step()
    clocks = Clocks(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    ms_steps, stage, total = timed(order, args.steps)
    launches = sum(s["kernel_launches"] for s in stage)
    torch.cuda.synchronize(dev)
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    t_total = float(np.sum(ms_steps)) / 1e3
    st = stage[-1]
    all_total, all_valid = int(total), int(st["n_valid_pairs"])
    # the timed run's GMCR and per-pair counts, for the oracle comparison below
    ca_counts = ctx.pair_counts()
    ca_off, ca_qidx = ctx.gmcr()
    # find-first (the reference driver's default mode) on the same inputs: one
    # 0/1 per pair, equal to "count-all found something" on every pair
    for _ in range(args.warmup):
        step(order, FIND_FIRST)
    ff_ms, ff_stage, ff_total = timed(order, args.steps, FIND_FIRST)
    find_first = {"find_first_value": Q * d_total / (float(np.mean(ff_ms)) / 1e3),
                  "find_first_ms_per_step": float(np.mean(ff_ms)),
                  "find_first_join_ms": float(np.mean([s["ms_join"] for s in ff_stage])),
                  "find_first_pairs_matched": int(ff_total),
                  "find_first_equals_count_all_nonzero": bool(np.array_equal(
                      ctx.pair_counts(), (ca_counts > 0).astype(np.uint64)))}
    # the reference's own DFS (REFERENCE_DFS: its literal frame bookkeeping,
    # isomorphism.hpp:401-448, in plain GMCR order) timed on the same inputs
    rd_steps = max(1, min(args.steps, 5))
    for _ in range(args.warmup):
        step(ORDER_GMCR, COUNT_ALL, SEM_REFERENCE_DFS)
    rd_ms, rd_stage, rd_total = timed(ORDER_GMCR, rd_steps, COUNT_ALL, SEM_REFERENCE_DFS)
    rd_counts = ctx.pair_counts()
    rd_off, rd_qidx = ctx.gmcr()
    reference_dfs = {"reference_dfs_value": Q * d_total / (float(np.mean(rd_ms)) / 1e3),
                     "reference_dfs_ms_per_step": float(np.mean(rd_ms)),
                     "reference_dfs_join_ms": float(np.mean([s_["ms_join"] for s_ in rd_stage])),
                     "reference_dfs_total_matches": int(rd_total), "reference_dfs_steps": rd_steps}
    for _ in range(args.warmup):
        step()
    if world > 1:  # shards: sum of counts, slowest rank's time
        all_total, all_valid, t_total = shards.reduce_totals(all_total, all_valid, t_total, device=dev)
    # e2e: host buffers in, counts out, through the C ABI
    pin = {k: torch.from_numpy(v).pin_memory() for k, v in da.items()}
    qpin = {k: torch.from_numpy(v).pin_memory() for k, v in qa.items()}
    T = st["n_valid_pairs"]
    out = torch.empty(max(T, 1), dtype=torch.int64).pin_memory()
    import ctypes

    from bms2_gb300 import native

    L = native.lib()
    e2e_ms = []
    # bytes the library copies (edge labels are accepted but never copied: matching ignores them)
    h2d = sum(int(v.numel() * v.element_size()) for p in (pin, qpin) for k, v in p.items() if k != "edge_labels")
    for i in range(args.warmup + args.steps):
        flush.fill_(1)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for kind, p in ((QUERY, qpin), (DATA, pin)):
            ctx.load_csr_ptrs(kind, len(p["graph_offsets"]) - 1, p["graph_offsets"].data_ptr(),
                              p["row_offsets"].data_ptr(), p["column_indices"].data_ptr(), p["node_labels"].data_ptr(),
                              p["edge_labels"].data_ptr())
        step()
        native._check(L.bms_get_pair_counts(ctx.handle, ctypes.cast(out.data_ptr(), native._u64p), out.numel()),
                      ctx.handle)
        torch.cuda.synchronize(dev)
        if i >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_s = float(np.mean(e2e_ms)) / 1e3
    pairs = Q * D
    value = Q * d_total * args.steps / t_total  # all ranks' pairs over the slowest rank's time
    peak, peak_kind = peaks()
    fbytes = algorithmic_filter_bytes(st["n_query_nodes"], st["n_data_nodes"], REFINE_STEPS)
    f_ms = float(np.mean([s["ms_filter"] for s in stage]))
    j_ms = float(np.mean([s["ms_join"] for s in stage]))
    achieved = fbytes / (f_ms / 1e3) / 1e9
    sig_bytes = algorithmic_signature_bytes(int(st["n_data_nodes"] + st["n_query_nodes"]),
                                            int(len(da["column_indices"]) + len(qa["column_indices"])), REFINE_STEPS)
    sig_ms = float(np.mean([s["ms_signatures"] for s in stage]))
    sig_gbs = sig_bytes / (sig_ms / 1e3) / 1e9
    per_graph = FILTER_DRAM_BYTES_PER_GRAPH.get(args.workload)
    traffic = per_graph * D if per_graph else None
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "pairs/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_total * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64",
        "data": "synthetic",
        "config": {"workload": f"{args.workload}: {D} data graphs x {Q} queries per GPU, refine steps {REFINE_STEPS}, "
                               f"count-all, EXACT semantics, order {args.order}",
                   "data_graphs_per_gpu": D, "queries": Q, "refine_steps": REFINE_STEPS, "order": args.order,
                   "l2": "flushed between steps (512 MiB write outside the timed events)",
                   "parallelism": f"data-graph shards x{world} (LPT, BMS2_mpi.cpp:78-157)",
                   "data_graphs_all_ranks": d_total,
                   "outside_reference_domain": outside_reference_domain(qa["graph_offsets"], da["graph_offsets"])},
        "e2e": {"value": Q * d_total / e2e_s, "unit": "pairs/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": int(T * 8)},
        "roofline": {"kernel": "sliced_filter (fused filter + refine + GMCR validity)", "bound": "hbm",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": f"{peak_kind} hbm_gbs",
                     "algorithmic_bytes": fbytes, "ms": f_ms, "equivalent": True,
                     "actual_gbs": traffic / (f_ms / 1e3) / 1e9 if traffic else None},
        "roofline_signatures": {"kernel": "signatures_kernel (data and query side)", "bound": "hbm",
                                "achieved": sig_gbs, "peak": peak, "unit": "GB/s", "frac": sig_gbs / peak,
                                "algorithmic_bytes": sig_bytes, "ms": sig_ms,
                                "note": "instruction-bound (ncu: lanes active per instruction, issue stalls)"},
        "join": {"kernel": "join_kernel (three size classes side by side)", "bound": "latency",
                 "ms": j_ms, "expansions_per_step": int(st["expansions"]),
                 "expansions_per_s": float(st["expansions"]) / max(j_ms / 1e3, 1e-9),
                 "note": "no HBM or tensor roofline: a DFS bound by latency and integer issue, "
                         "lanes active per instruction and stall reasons from ncu"},
        "stage_ms": {k: float(np.mean([s[k] for s in stage])) for k in
                     ("ms_signatures", "ms_filter", "ms_map", "ms_order", "ms_join", "ms_total")},
        "clocks": clk,
        "gpu_launches": int(launches),
        "results": {"total_matches": int(total), "valid_pairs": int(T), "expansions": int(st["expansions"]),
                    "total_matches_all_ranks": all_total, "valid_pairs_all_ranks": all_valid},
    }
    if plain is not None:
        line["results"].update(plain)
        line["results"]["plain_value"] = Q * d_total / (plain["plain_ms_per_step"] / 1e3)
        line["results"]["learned_over_plain"] = line["results"]["plain_value"] and value / line["results"]["plain_value"]
        line["results"]["expansion_ratio_plain_over_learned"] = float(plain["plain_expansions"]) / max(1, st["expansions"])
    line["results"].update(extra)
    line["results"].update(find_first)
    line["results"].update(reference_dfs)
    if schedule is not None:
        line["schedule"] = {"tuned_on": f"{args.workload} seed A, "
                                        f"{args.tune_graphs if args.tune_graphs > 0 else 'all'} data graphs",
                            "buckets": schedule}
    parity_ok = True
    if rank == 0:
        import oracle

        threads = os.cpu_count() or 1
        if not args.no_cpu:
            info, res, k = cpu_baseline(qa, da, threads, args.cpu_budget)
            line["cpu_baseline"] = info
        else:
            k = min(1024, D)
            res = oracle.run_pipeline(qa, _head(da, k), REFINE_STEPS, threads=threads, keep_steps=False)
        # the oracle's counts on the sample, pair by pair: EXACT for the timed
        # run, the literal restatement of the reference DFS for REFERENCE_DFS
        exact = sample_parity(ca_off, ca_qidx, ca_counts, res, k)
        k_lit = min(k, 4096)
        lit = oracle.run_pipeline(qa, _head(da, k_lit), REFINE_STEPS, threads=threads, keep_steps=False,
                                  dfs_literal=True)
        literal = sample_parity(rd_off, rd_qidx, rd_counts, lit, k_lit)
        line["results"]["oracle_sample"] = {"exact": exact, "reference_dfs": literal}
        line["results"]["oracle_sample_counts_equal"] = exact["counts_equal"]
        line["results"]["reference_dfs_oracle_counts_equal"] = literal["counts_equal"]
        parity_ok = exact["counts_equal"] and literal["counts_equal"]
    del ca_counts, rd_counts
    ctx.close()
    del flush
    torch.cuda.empty_cache()
    if rank == 0 and world == 1 and args.workload == "mol1m" and not args.no_configs:
        # the other GPU configurations, measured in the same run
        configs = {}
        for name, fn in (("mol100k", lambda: leg_mol100k(local, min(args.steps, 10), args.warmup, args.train_graphs)),
                         ("mol10m", lambda: leg_mol10m(local, 1, args.train_graphs))):
            t0 = time.perf_counter()
            try:
                configs[name] = fn()
            except Exception as e:  # recorded, not fatal: the headline stands on its own
                configs[name] = {"error": f"{type(e).__name__}: {e}"}
            configs[name]["wall_seconds"] = time.perf_counter() - t0
        line["configs"] = configs
        parity_ok = parity_ok and all(c.get("counts_equal", True) for c in configs.values())
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    if not parity_ok:
        sys.exit("per-pair counts differ from the oracle on the sample: the measurement is void")


def _ms_timed(ctx, stream, flush, k, fn):
    """k calls of fn, each bracketed by CUDA events on the library's stream
    (L2 flushed before each, outside the events); mean ms and the last stats."""
    import torch

    ms = []
    out = None
    for _ in range(k):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    return float(np.mean(ms)), ctx.stats(), out


def leg_mol100k(local: int, steps: int, warmup: int, train_graphs: int) -> dict:
    """The plain-method GPU configuration: 100,000 data graphs (N(28, 9) atoms,
    10-60) x 600 queries of 5-30 nodes (30% pure carbon); count-all and
    find-first in plain GMCR order, the reference's literal DFS, and the
    learned order, each compared pair by pair with the oracle on a sample."""
    import torch

    import oracle
    from bms2_gb300 import (COUNT_ALL, DATA, FIND_FIRST, ORDER_GMCR, ORDER_LEARNED, QUERY, SEM_EXACT,
                            SEM_REFERENCE_DFS, Context, workloads)

    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    out = {"workload": "mol100k: 100000 data graphs x 600 queries, refine steps 6"}
    with Context(local) as ctx:
        ctx.set_stream(stream.cuda_stream)
        out.update(train_cost_model(ctx, "mol100k", seed=101, n_data=train_graphs))
        tq, td = workloads.make("mol100k", 101)
        ctx.load(QUERY, tq)
        ctx.load(DATA, td)
        ctx.autotune(REFINE_STEPS, COUNT_ALL, ORDER_GMCR)
        q, d = workloads.make("mol100k", 202)
        Q, D = q.n_graphs, d.n_graphs
        ctx.load(QUERY, q)
        ctx.load(DATA, d)
        res = {}
        for name, mode, order, sem in (("plain", COUNT_ALL, ORDER_GMCR, SEM_EXACT),
                                       ("learned", COUNT_ALL, ORDER_LEARNED, SEM_EXACT),
                                       ("find_first", FIND_FIRST, ORDER_GMCR, SEM_EXACT),
                                       ("reference_dfs", COUNT_ALL, ORDER_GMCR, SEM_REFERENCE_DFS)):
            def run(mode=mode, order=order, sem=sem):
                return ctx.run(REFINE_STEPS, mode, order, sem)
            for _ in range(warmup):
                run()
            ms, st, total = _ms_timed(ctx, stream, flush, steps, run)
            off, qidx = ctx.gmcr()
            res[name] = {"value": Q * D / (ms / 1e3), "ms_per_step": ms, "ms_join": st["ms_join"],
                         "total": int(total), "expansions": int(st["expansions"]),
                         "_counts": ctx.pair_counts(), "_gmcr": (off, qidx)}
        qa, da = q.arrays(), d.arrays()
        k = 2048
        threads = os.cpu_count() or 1
        checks = {}
        for name, kw in (("plain", {}), ("find_first", {"find_first": True}), ("reference_dfs", {"dfs_literal": True})):
            want = oracle.run_pipeline(qa, _head(da, k), REFINE_STEPS, threads=threads, keep_steps=False, **kw)
            off, qidx = res[name]["_gmcr"]
            checks[name] = sample_parity(off, qidx, res[name]["_counts"], want, k)
        learned_equal = bool(np.array_equal(res["learned"]["_counts"], res["plain"]["_counts"]))
        for r in res.values():
            r.pop("_counts")
            r.pop("_gmcr")
        out.update({"data_graphs": D, "queries": Q, "runs": res, "oracle_sample": checks,
                    "learned_counts_equal_plain_every_pair": learned_equal,
                    "learned_over_plain": res["learned"]["value"] / res["plain"]["value"],
                    "expansion_ratio_plain_over_learned": res["plain"]["expansions"] / max(1, res["learned"]["expansions"]),
                    "counts_equal": all(c["counts_equal"] for c in checks.values()) and learned_equal})
    del flush
    torch.cuda.empty_cache()
    return out


def leg_mol10m(local: int, warmup: int, train_graphs: int, slice_graphs: int = 500_000,
               latency_sample: int = 16) -> dict:
    """The large mixed configuration: 10,000,000 data graphs resident in HBM x
    3,000 queries (20% adversarial).  One pass each in the learned and in the
    plain GMCR order (windows of slice_graphs data graphs), the batch driver
    from page-locked host memory (e2e), per-query latency over all resident
    graphs, and the engine against the oracle pair by pair on a prefix."""
    import torch

    import oracle
    from bms2_gb300 import (COUNT_ALL, DATA, OPT_RESIDENT_SIGNATURES, ORDER_GMCR, ORDER_LEARNED, QUERY, SEM_EXACT,
                            Context, Graphs, shards, workloads)

    dev = torch.device("cuda", local)
    out = {"workload": f"mol10m: 10000000 data graphs x 3000 queries (20% adversarial), resident in HBM, windows of "
                       f"{slice_graphs}, refine steps 6"}
    with Context(local) as ctx:
        out.update(train_cost_model(ctx, "mol10m", seed=101, n_data=train_graphs))
        t0 = time.perf_counter()
        q, d = workloads.make("mol10m", 202)
        out["synth_seconds"] = time.perf_counter() - t0
        Q, D = q.n_graphs, d.n_graphs
        ctx.load(QUERY, q)
        # pair by pair against the oracle on the first 1,024 data graphs
        qa = q.arrays()
        head = _head(d.arrays(), 1024)
        ctx.load(DATA, Graphs.from_csr(**head))
        ctx.run(REFINE_STEPS, COUNT_ALL, ORDER_LEARNED, SEM_EXACT)
        off, qidx = ctx.gmcr()
        want = oracle.run_pipeline(qa, head, REFINE_STEPS, threads=os.cpu_count() or 1, keep_steps=False)
        out["oracle_sample"] = sample_parity(off, qidx, ctx.pair_counts(), want, 1024)
        del head
        # e2e: the batch driver from page-locked host memory (after one sizing pass)
        d.pin()
        ctx.run_batches(d, slice_graphs, REFINE_STEPS, COUNT_ALL, ORDER_LEARNED, SEM_EXACT)
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        e2e_total, _ = ctx.run_batches(d, slice_graphs, REFINE_STEPS, COUNT_ALL, ORDER_LEARNED, SEM_EXACT)
        torch.cuda.synchronize(dev)
        e2e_s = time.perf_counter() - t
        d.unpin()
        ctx.load_resident(d)
        passes = {}
        for name, order in (("learned", ORDER_LEARNED), ("plain", ORDER_GMCR)):
            for _ in range(max(1, warmup)):
                ctx.run_resident(slice_graphs, REFINE_STEPS, COUNT_ALL, order, SEM_EXACT)
            torch.cuda.synchronize(dev)
            t = time.perf_counter()
            total, per_query = ctx.run_resident(slice_graphs, REFINE_STEPS, COUNT_ALL, order, SEM_EXACT)
            torch.cuda.synchronize(dev)
            sec = time.perf_counter() - t
            st = ctx.stats()
            passes[name] = {"value": Q * D / sec, "seconds_per_pass": sec, "total": int(total),
                            "expansions": int(st["expansions"]), "ms_join": st["ms_join"], "ms_filter": st["ms_filter"],
                            "ms_signatures": st["ms_signatures"], "_per_query": per_query}
        same = bool(np.array_equal(passes["learned"]["_per_query"], passes["plain"]["_per_query"]))
        per_query = passes["learned"]["_per_query"]
        rng = np.random.default_rng(7)
        sample = np.sort(rng.choice(Q, size=min(latency_sample, Q), replace=False))
        lat = []
        for qi in sample:
            ctx.load(QUERY, Graphs.from_csr(**shards.take_graphs(qa, np.array([qi]))))
            torch.cuda.synchronize(dev)
            t = time.perf_counter()
            one, _ = ctx.run_resident(slice_graphs, REFINE_STEPS, COUNT_ALL, ORDER_LEARNED, SEM_EXACT)
            torch.cuda.synchronize(dev)
            lat.append(time.perf_counter() - t)
            if one != int(per_query[qi]):
                raise AssertionError("single-query pass disagrees with the batched pass")
        ctx.set_option(OPT_RESIDENT_SIGNATURES, 1)
        ctx.run_resident(slice_graphs, REFINE_STEPS, COUNT_ALL, ORDER_LEARNED, SEM_EXACT)
        lat_c = []
        for qi in sample:
            ctx.load(QUERY, Graphs.from_csr(**shards.take_graphs(qa, np.array([qi]))))
            torch.cuda.synchronize(dev)
            t = time.perf_counter()
            ctx.run_resident(slice_graphs, REFINE_STEPS, COUNT_ALL, ORDER_LEARNED, SEM_EXACT)
            torch.cuda.synchronize(dev)
            lat_c.append(time.perf_counter() - t)
        ctx.set_option(OPT_RESIDENT_SIGNATURES, 0)
        for r in passes.values():
            r.pop("_per_query")
        fbytes = algorithmic_filter_bytes(int(qa["graph_offsets"][-1]), int(d.n_nodes), REFINE_STEPS)
        peak, peak_kind = peaks()
        f_ms = passes["learned"]["ms_filter"]
        out.update({"data_graphs": D, "queries": Q, "passes": passes,
                    "learned_over_plain": passes["learned"]["value"] / passes["plain"]["value"],
                    "expansion_ratio_plain_over_learned": passes["plain"]["expansions"] / max(1, passes["learned"]["expansions"]),
                    "per_query_totals_equal_across_orders": same,
                    "e2e": {"value": Q * D / e2e_s, "unit": "pairs/s", "seconds": e2e_s,
                            "total_equal_resident": int(e2e_total) == passes["learned"]["total"]},
                    "query_latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                                        "sample": int(len(lat))},
                    "query_latency_s_resident_signatures": {"p50": float(np.percentile(lat_c, 50)),
                                                            "p99": float(np.percentile(lat_c, 99))},
                    "roofline_filter": {"achieved": fbytes / (f_ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                                        "frac": fbytes / (f_ms / 1e3) / 1e9 / peak, "equivalent": True,
                                        "peak_kind": f"{peak_kind} hbm_gbs"},
                    "outside_reference_domain": outside_reference_domain(qa["graph_offsets"], graph_offsets(d)),
                    "counts_equal": out["oracle_sample"]["counts_equal"] and same and
                                    int(e2e_total) == passes["learned"]["total"]})
    torch.cuda.empty_cache()
    return out


def run_streamed(args) -> None:
    """mol10m: 10,000,000 data graphs x 3,000 queries (20% adversarial).  One
    pass over all pairs would need more candidate-row memory than HBM holds, so
    the data side is processed in windows of --slice graphs.  value: the data
    side resident in HBM (bms_load_resident once), a step = one pass of
    bms_run_resident over all windows.  e2e: one pass of the batch driver
    (bms_run_batches), every slice uploaded from host memory inside it.
    Per-query latency: single-query resident passes of a seeded sample."""
    import torch
    import torch.distributed as dist

    from bms2_gb300 import COUNT_ALL, ORDER_GMCR, ORDER_LEARNED, QUERY, SEM_EXACT, Context, Graphs, shards, workloads

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = Context(local)
    order = ORDER_LEARNED if args.order == "learned" else ORDER_GMCR
    extra = {}
    if order == ORDER_LEARNED:
        extra.update(train_cost_model(ctx, args.workload, seed=101, n_data=args.train_graphs))
    t0 = time.perf_counter()
    q, d = workloads.make(args.workload, 202 + rank, n_data=args.data_graphs)
    extra["synth_seconds"] = time.perf_counter() - t0
    Q, D = q.n_graphs, d.n_graphs
    ctx.load(QUERY, q)
    # e2e: the data side streamed from host memory through the batch driver,
    # from a page-locked host batch (bms_graphs_pin), after one untimed pass
    # that sizes the device buffers
    d.pin()
    ctx.run_batches(d, args.slice, REFINE_STEPS, COUNT_ALL, order, SEM_EXACT)
    torch.cuda.synchronize(dev)
    t = time.perf_counter()
    e2e_total, _ = ctx.run_batches(d, args.slice, REFINE_STEPS, COUNT_ALL, order, SEM_EXACT)
    torch.cuda.synchronize(dev)
    e2e_s = time.perf_counter() - t
    d.unpin()
    # value: the data side resident in HBM, processed in windows of --slice graphs
    ctx.load_resident(d)
    for _ in range(max(1, args.warmup)):
        ctx.run_resident(args.slice, REFINE_STEPS, COUNT_ALL, order, SEM_EXACT)
    clocks = Clocks(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    secs, total, per_query, st = [], 0, None, None
    for _ in range(args.steps):
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        total, per_query = ctx.run_resident(args.slice, REFINE_STEPS, COUNT_ALL, order, SEM_EXACT)
        torch.cuda.synchronize(dev)
        secs.append(time.perf_counter() - t)
        st = ctx.stats()
    assert total == e2e_total, "resident and streamed passes disagree"
    clk = clocks.stop()
    t_step = float(np.mean(secs))
    all_total, _, t_max = int(total), 0, t_step
    if world > 1:
        all_total, _, t_max = shards.reduce_totals(int(total), 0, t_step, device=dev)
    # per-query latency over the whole resident data set, one query per pass
    rng = np.random.default_rng(7)
    sample = np.sort(rng.choice(Q, size=min(args.latency_sample, Q), replace=False))
    qa = q.arrays()
    lat = []
    for qi in sample:
        ctx.load(QUERY, Graphs.from_csr(**shards.take_graphs(qa, np.array([qi]))))
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        one, _ = ctx.run_resident(args.slice, REFINE_STEPS, COUNT_ALL, order, SEM_EXACT)
        torch.cuda.synchronize(dev)
        lat.append(time.perf_counter() - t)
        assert one == int(per_query[qi]), "single-query pass disagrees with the batched pass"
    # serving: the data side's signatures computed once for the resident batch
    # (BMS_OPT_RESIDENT_SIGNATURES) and reused by every later single-query pass
    from bms2_gb300 import OPT_RESIDENT_SIGNATURES

    ctx.set_option(OPT_RESIDENT_SIGNATURES, 1)
    ctx.load(QUERY, Graphs.from_csr(**shards.take_graphs(qa, np.array([int(sample[0])]))))
    torch.cuda.synchronize(dev)
    t = time.perf_counter()
    ctx.run_resident(args.slice, REFINE_STEPS, COUNT_ALL, order, SEM_EXACT)
    torch.cuda.synchronize(dev)
    sig_once_s = time.perf_counter() - t
    lat_c = []
    for qi in sample:
        ctx.load(QUERY, Graphs.from_csr(**shards.take_graphs(qa, np.array([qi]))))
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        one, _ = ctx.run_resident(args.slice, REFINE_STEPS, COUNT_ALL, order, SEM_EXACT)
        torch.cuda.synchronize(dev)
        lat_c.append(time.perf_counter() - t)
        assert one == int(per_query[qi]), "single-query pass with resident signatures disagrees"
    ctx.set_option(OPT_RESIDENT_SIGNATURES, 0)
    peak, peak_kind = peaks()
    fbytes = algorithmic_filter_bytes(int(q.arrays()["graph_offsets"][-1]), int(d.arrays()["graph_offsets"][-1]),
                                      REFINE_STEPS)
    achieved = fbytes / (st["ms_filter"] / 1e3) / 1e9
    pairs = Q * D
    value = world * pairs / t_max
    a = d.arrays()
    h2d = int(sum(v.nbytes for k, v in a.items() if k != "edge_labels"))
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {D} data graphs x {Q} queries per GPU, resident in HBM, in windows "
                               f"of {args.slice}, refine steps {REFINE_STEPS}, count-all, EXACT, order {args.order}",
                   "data_graphs_per_gpu": D, "queries": Q, "slice_graphs": args.slice, "order": args.order,
                   "l2": "inputs far larger than L2 (every window is processed once per pass)",
                   "parallelism": f"data-graph shards x{world}",
                   "outside_reference_domain": outside_reference_domain(graph_offsets(q), graph_offsets(d))},
        "e2e": {"value": world * pairs / e2e_s, "unit": "pairs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 8 * Q,
                "note": "one pass through bms_run_batches: every slice uploaded from page-locked host memory "
                        "inside it (after one untimed pass)"},
        "roofline": {"kernel": "sliced_filter (fused filter + refine + GMCR validity), all slices", "bound": "hbm",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "peak_kind": f"{peak_kind} hbm_gbs", "algorithmic_bytes": fbytes, "ms": st["ms_filter"],
                     "equivalent": True},
        "stage_ms": {k: float(st[k]) for k in ("ms_signatures", "ms_filter", "ms_map", "ms_order", "ms_join",
                                                  "ms_total")},
        "clocks": clk,
        "gpu_launches": int(st["kernel_launches"]),
        "results": {"total_matches": int(total), "total_matches_all_ranks": all_total,
                    "expansions": int(st["expansions"]), "incomplete_pairs": int(st["n_incomplete"]),
                    "query_latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                                        "max": float(np.max(lat)), "sample": int(len(lat)),
                                        "definition": "one query alone over all resident data graphs"},
                    "query_latency_s_resident_signatures": {
                        "p50": float(np.percentile(lat_c, 50)), "p99": float(np.percentile(lat_c, 99)),
                        "max": float(np.max(lat_c)), "sample": int(len(lat_c)),
                        "first_pass_s": sig_once_s,
                        "definition": "the same queries after one pass has computed the data side's signatures "
                                      "for the whole resident batch (BMS_OPT_RESIDENT_SIGNATURES)"},
                    "per_query_matches": {"p50": float(np.percentile(per_query, 50)),
                                          "p99": float(np.percentile(per_query, 99)),
                                          "max": int(per_query.max())}},
    }
    line["results"].update(extra)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


def run_clustered(args) -> None:
    """mol1m-cs: the reference driver's --use-cs phase (run.sh: -i 6 --find-all,
    one cluster file per run, BMS2.cpp:218-296) on GB300.  One seeded cluster
    (query 0 the prototype of 5-8 nodes, --cluster-members members listing its
    nodes first) against the mol1m seed-B data graphs.  value: steps of bms_run
    with the clustered join (count-all, EXACT, GMCR order); results.plain_*: the
    plain join on the same inputs and settings, timed the same way."""
    import ctypes

    import torch
    import torch.distributed as dist

    from bms2_gb300 import (COUNT_ALL, DATA, OPT_USE_CS, ORDER_GMCR, QUERY, SEM_EXACT, Context, native, shards,
                            workloads)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = Context(local)
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    _, d = workloads.make("mol1m", 202 + rank, n_data=args.data_graphs)
    q = workloads.make_cluster(d, args.cluster_members, 303, proto_nodes=(5, 8), proto=args.cluster_proto)
    Q, D = q.n_graphs, d.n_graphs
    qa, da = q.arrays(), d.arrays()
    ctx.load(QUERY, q)
    ctx.load(DATA, d)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def step(cs=True, R=REFINE_STEPS):
        ctx.set_option(OPT_USE_CS, int(cs))
        return ctx.run(R, COUNT_ALL, ORDER_GMCR, SEM_EXACT)

    def timed(cs, k):
        ms, stages = [], []
        for _ in range(k):
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            tot = step(cs)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            stages.append(ctx.stats())
        return ms, stages, tot

    # at two refinement steps every filter is sound for induced embeddings and
    # both joins count the same embeddings, pair by pair
    step(False, 2)
    r2_plain = ctx.pair_counts()
    step(True, 2)
    r2_equal = bool(np.array_equal(ctx.pair_counts(), r2_plain))
    for _ in range(args.warmup):
        step(False)
    p_ms, p_stage, p_total = timed(False, args.steps)
    p_counts = ctx.pair_counts()
    for _ in range(args.warmup):
        step(True)
    clocks = Clocks(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    ms_steps, stage, total = timed(True, args.steps)
    torch.cuda.synchronize(dev)
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    launches = sum(s["kernel_launches"] for s in stage)
    st = stage[-1]
    c_counts = ctx.pair_counts()
    c_off, c_qidx = ctx.gmcr()
    t_total = float(np.sum(ms_steps)) / 1e3
    all_total, all_valid = int(total), int(st["n_valid_pairs"])
    if world > 1:
        all_total, all_valid, t_total = shards.reduce_totals(all_total, all_valid, t_total, device=dev)
    # e2e: pinned host CSR in, per-pair counts out, through the C ABI
    pin = {k: torch.from_numpy(v).pin_memory() for k, v in da.items()}
    qpin = {k: torch.from_numpy(v).pin_memory() for k, v in qa.items()}
    T = st["n_valid_pairs"]
    out = torch.empty(max(T, 1), dtype=torch.int64).pin_memory()
    L = native.lib()
    # bytes the library copies (edge labels are accepted but never copied: matching ignores them)
    h2d = sum(int(v.numel() * v.element_size()) for p in (pin, qpin) for k, v in p.items() if k != "edge_labels")
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        flush.fill_(1)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for kind, p in ((QUERY, qpin), (DATA, pin)):
            ctx.load_csr_ptrs(kind, len(p["graph_offsets"]) - 1, p["graph_offsets"].data_ptr(),
                              p["row_offsets"].data_ptr(), p["column_indices"].data_ptr(), p["node_labels"].data_ptr(),
                              p["edge_labels"].data_ptr())
        step(True)
        native._check(L.bms_get_pair_counts(ctx.handle, ctypes.cast(out.data_ptr(), native._u64p), out.numel()),
                      ctx.handle)
        torch.cuda.synchronize(dev)
        if i >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_s = float(np.mean(e2e_ms)) / 1e3
    pairs = Q * D
    value = world * pairs * args.steps / t_total
    plain_value = world * pairs / (float(np.mean(p_ms)) / 1e3)
    peak, peak_kind = peaks()
    fbytes = algorithmic_filter_bytes(st["n_query_nodes"], st["n_data_nodes"], REFINE_STEPS)
    f_ms = float(np.mean([s["ms_filter"] for s in stage]))
    achieved = fbytes / (f_ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_total * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": f"mol1m-cs: {D} data graphs x one cluster of {Q} queries ({args.cluster_proto} "
                               f"prototype of {int(qa['graph_offsets'][1])} atoms + {Q - 1} members) per GPU, "
                               f"refine steps {REFINE_STEPS}, count-all, EXACT, clustered join (--use-cs)",
                   "data_graphs_per_gpu": D, "queries": Q, "refine_steps": REFINE_STEPS, "order": "plain",
                   "l2": "flushed between steps (512 MiB write outside the timed events)",
                   "parallelism": f"data-graph shards x{world} (LPT, BMS2_mpi.cpp:78-157)",
                   "data_graphs_all_ranks": d_total,
                   "outside_reference_domain": outside_reference_domain(qa["graph_offsets"], da["graph_offsets"])},
        "e2e": {"value": Q * d_total / e2e_s, "unit": "pairs/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": int(T * 8)},
        "roofline": {"kernel": "sliced_filter (fused filter + refine + GMCR validity)", "bound": "hbm",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "peak_kind": f"{peak_kind} hbm_gbs", "algorithmic_bytes": fbytes, "ms": f_ms,
                     "equivalent": True},
        "stage_ms": {k: float(np.mean([s[k] for s in stage])) for k in
                     ("ms_signatures", "ms_filter", "ms_map", "ms_order", "ms_join", "ms_total")},
        "clocks": clk,
        "gpu_launches": int(launches),
        "results": {"total_matches": int(total), "valid_pairs": int(T), "expansions": int(st["expansions"]),
                    "partial_matches": int(st["n_partial_matches"]),
                    "total_matches_all_ranks": all_total, "valid_pairs_all_ranks": all_valid,
                    "plain_value": plain_value, "clustered_over_plain": value / plain_value,
                    "plain_total_matches": int(p_total), "plain_expansions": int(p_stage[-1]["expansions"]),
                    "plain_ms_per_step": float(np.mean(p_ms)),
                    "plain_join_ms": float(np.mean([s["ms_join"] for s in p_stage])),
                    "counts_equal_every_pair": bool(np.array_equal(c_counts, p_counts)),
                    "counts_equal_every_pair_at_2_refine_steps": r2_equal},
    }
    parity_ok = True
    if rank == 0:
        import oracle

        threads = os.cpu_count() or 1
        if not args.no_cpu:
            info, res, k = cpu_baseline(qa, da, threads, args.cpu_budget, cs=True)
            line["cpu_baseline"] = info
        else:
            k = min(1024, D)
            res = oracle.run_pipeline(qa, _head(da, k), REFINE_STEPS, threads=threads, keep_steps=False, cs=True)
        par = sample_parity(c_off, c_qidx, c_counts, res, k)
        line["results"]["oracle_sample"] = {"exact": par}
        line["results"]["oracle_sample_counts_equal"] = par["counts_equal"]
        parity_ok = par["counts_equal"]
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()
    if not parity_ok:
        sys.exit("per-pair counts differ from the oracle on the sample: the measurement is void")


def run_reference(args) -> None:
    """The reference's CPU path.  Its SYCL CPU build cannot be built here (no
    SYCL compiler or runtime), so the oracle — the C++ restatement of the
    reference kernels, OpenMP over all host threads — runs on a bounded sample
    of the same workload.  Nothing of the GPU engine is loaded in this arm: the
    inputs come from the generator's own CPU-only build (oracle/synth.py),
    byte-identical to the engine arm's."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import synth

    from bms2_gb300.workloads import make_cluster_arrays

    cs = args.workload == "mol1m-cs"
    if cs:
        _, da = synth.make("mol1m", 202)
        qa = make_cluster_arrays(da, args.cluster_members, 303, proto_nodes=(5, 8), proto=args.cluster_proto)
    else:
        qa, da = synth.make(args.workload, 202)
    threads = os.cpu_count() or 1
    cb = None
    vals = []
    for i in range(args.warmup + args.steps):
        cb, _, _ = cpu_baseline(qa, da, threads, budget_s=args.cpu_budget if i >= args.warmup else 4.0, cs=cs)
        if i >= args.warmup:
            vals.append(cb["value"])
    v = float(np.mean(vals))
    cb["value"] = v
    cb["implementation"] = "oracle restatement of the reference kernels (the reference's SYCL build is unavailable)"
    Q, D = len(qa["graph_offsets"]) - 1, len(da["graph_offsets"]) - 1
    line = {"metric": METRIC, "value": v, "unit": "pairs/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic", "impl": "reference",
            "config": {"workload": f"{args.workload}: {D} data graphs x {Q} queries (bounded sample per "
                                   f"step), refine steps {REFINE_STEPS}, count-all", "order": "plain",
                       "sample_scaling": "pairs/s of all queries x a prefix of the data graphs; the prefix grows "
                                         "until one pass takes about a quarter of the CPU budget"},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--order", choices=["learned", "plain"], default="learned")
    ap.add_argument("--workload", choices=["mol100k", "mol1m", "mol10m", "mol1m-cs"], default=WORKLOAD)
    ap.add_argument("--cluster-members", type=int, default=100, help="mol1m-cs: members of the query cluster")
    ap.add_argument("--cluster-proto", choices=["ring", "grow"], default="ring",
                    help="mol1m-cs: a carbon-ring prototype or a grown 5-8 atom fragment")
    ap.add_argument("--slice", type=int, default=500_000, help="mol10m: data graphs per streamed slice")
    ap.add_argument("--latency-sample", type=int, default=16, help="mol10m: queries timed alone")
    ap.add_argument("--train-graphs", type=int, default=20000)
    ap.add_argument("--tune-graphs", type=int, default=-1,
                    help="seed-A data graphs for the join autotuner (-1: the workload's full size, 0: off)")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="mol1m: skip the mol100k and mol10m measurements that follow the headline")
    ap.add_argument("--data-graphs", type=int, default=None, help="shrink the workload (profiling)")
    ap.add_argument("--once", action="store_true", help="one untimed pipeline run (profiling)")
    args = ap.parse_args()
    from bms2_gb300 import build

    if args.impl == "reference":
        build.build_cpu_side()  # the oracle and the generator only
        run_reference(args)
        return
    build.build()
    if args.workload == "mol10m":
        run_streamed(args)
    elif args.workload == "mol1m-cs":
        run_clustered(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
