"""The CUDA engine against outputs of the reference's own code.

The fixtures (tests/golden/ref_*.npz) hold what the reference's headers
compute on seeded inputs; see tests/ref_golden.py.  The staged pipeline's
signatures, candidate matrix after the filter and after every refinement
step, GMCR and per-pair join counts (REFERENCE_DFS, the reference's literal
DFS) must equal them bit for bit, and so must the fused pipeline's GMCR and
per-pair counts, eager and replayed from its CUDA graph.
"""
import numpy as np
import pytest

from bms2_gb300 import COUNT_ALL, DATA, FIND_FIRST, ORDER_GMCR, QUERY, SEM_REFERENCE_DFS, Graphs
from tests import ref_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=ref_golden.CASES)
def case(request):
    f = ref_golden.load(request.param)
    qt, dt = ref_golden.texts(f)
    return f, Graphs.parse_text(qt), Graphs.parse_text(dt)


def _load(ctx, q, d):
    ctx.load(QUERY, q)
    ctx.load(DATA, d)


def test_staged_pipeline_equals_the_reference(ctx, case):
    f, q, d = case
    R = int(f["refine_steps"][0])
    _load(ctx, q, d)
    ctx.signatures(R)
    for kind, side in ((QUERY, "q"), (DATA, "d")):
        got = ctx.signatures_of(kind, R)
        assert np.array_equal(got["label_gen"], f[f"{side}_label_gen"])
        assert np.array_equal(got["path"].ravel(), f[f"{side}_path"])
        assert np.array_equal(got["cycle"].ravel(), f[f"{side}_cycle"])
        for k in range(1, R + 1):
            assert np.array_equal(got["shells"][k - 1], f[f"{side}_shell_{k}"]), f"{side} shell {k}"
    ctx.filter()
    assert np.array_equal(ctx.candidates(), ref_golden.candidates(f, "cand_filter"))
    for k in range(1, R + 1):
        ctx.refine(k)
        assert np.array_equal(ctx.candidates(), ref_golden.candidates(f, f"cand_step_{k}")), f"step {k}"
    ctx.map()
    off, qidx = ctx.gmcr()
    assert np.array_equal(off, f["gmcr_offsets"])
    assert np.array_equal(qidx, f["gmcr_query_indices"])
    for mode, key in ((FIND_FIRST, "find_first"), (COUNT_ALL, "find_all")):
        total = ctx.join(mode, ORDER_GMCR, SEM_REFERENCE_DFS)
        assert np.array_equal(ctx.pair_counts(), f[f"join_pair_{key}"]), key
        assert total == int(f[f"join_total_{key}"][0])


@pytest.mark.parametrize("mode,key", [(FIND_FIRST, "find_first"), (COUNT_ALL, "find_all")])
def test_fused_pipeline_equals_the_reference(ctx, case, mode, key):
    f, q, d = case
    R = int(f["refine_steps"][0])
    _load(ctx, q, d)
    for _ in range(3):  # eager, capture + launch, replay
        total = ctx.run(R, mode, ORDER_GMCR, SEM_REFERENCE_DFS)
        off, qidx = ctx.gmcr()
        assert np.array_equal(off, f["gmcr_offsets"])
        assert np.array_equal(qidx, f["gmcr_query_indices"])
        assert np.array_equal(ctx.pair_counts(), f[f"join_pair_{key}"])
        assert total == int(f[f"join_total_{key}"][0])
