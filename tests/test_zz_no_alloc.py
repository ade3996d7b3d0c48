"""bms_gmcr_offsets_static: the allocation-free GMCR offsets entry point.

It is for callers that must not allocate device memory while they run (their
device memory belongs to their own pool allocator, or they cannot take the
device-wide synchronisation of cudaMalloc/cudaFree), so its scan scratch is a
fixed array inside libbms.  The test feeds it the per-data-graph pair counts of
two real runs, one after the other, and compares its offsets with the offsets
bms_run produced through the library's allocating path.  This file sorts last
so that a run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from bms2_gb300 import COUNT_ALL, DATA, ORDER_GMCR, QUERY, SEM_EXACT, Context, native, workloads

pytestmark = pytest.mark.gpu


def _offsets_static(counts: np.ndarray) -> np.ndarray:
    import torch

    dev = torch.device("cuda", 0)
    c = torch.from_numpy(counts.astype(np.int32)).to(dev)  # uint32 bits in an int32 tensor
    out = torch.full((len(counts) + 1,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    st = native.lib().bms_gmcr_offsets_static(ctypes.c_void_p(c.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                              len(counts), ctypes.c_void_p(stream.cuda_stream))
    native._check(st)
    stream.synchronize()
    return out.cpu().numpy().view(np.uint32)


def _run_offsets(n_data: int, n_queries: int, seed: int) -> np.ndarray:
    q, d = workloads.make("mol1k", seed, n_data=n_data, n_queries=n_queries)
    with Context(0) as ctx:
        ctx.load(QUERY, q)
        ctx.load(DATA, d)
        ctx.run(2, COUNT_ALL, ORDER_GMCR, SEM_EXACT)
        off, _ = ctx.gmcr()
    return off


def test_static_offsets_match_the_allocating_path_twice_in_a_row():
    big = _run_offsets(20000, 8, 31)     # 20,000 data graphs: a multi-block scan
    small = _run_offsets(700, 12, 32)    # then a smaller one over the same scratch
    for want in (big, small):
        got = _offsets_static(np.diff(want).astype(np.uint32))
        assert np.array_equal(got, want)


def test_static_offsets_reject_oversized_input():
    st = native.lib().bms_gmcr_offsets_static(ctypes.c_void_p(16), ctypes.c_void_p(16), 200_000_000, None)
    assert st == -6
    assert b"exceed" in native.lib().bms_last_error(None)
