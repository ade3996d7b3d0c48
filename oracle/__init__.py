"""CPU oracle of the bms2_gb300 path (test infrastructure only).

The C++ restatement of the reference kernels lives in oracle.cpp and is built
into oracle/_build/liboracle.so by bms2_gb300.build.build_oracle().  Only the
tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the
checker.  Parity status: unpinned by the reference itself (it cannot be built
here and ships no tests or golden vectors); pinned by hand-derived known-answer
tests and an independent networkx cross-check (tests/golden/).
"""
from .pipeline import OracleResult, Signatures, load, mlp_grad, pair_embeddings, run_pipeline, signatures  # noqa: F401
