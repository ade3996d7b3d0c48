"""CPU oracle of the bms2_gb300 path (test infrastructure only).

The C++ restatement of the reference kernels lives in oracle.cpp and is built
into oracle/_build/liboracle.so by bms2_gb300.build.build_oracle().  Only the
tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the
checker.  Parity status: pinned to the reference's own code — its headers,
compiled on the CPU against a host-only SYCL stand-in (oracle/ref/), produced
tests/golden/ref_*.npz, which every stage of the oracle equals bit for bit —
and further by hand-derived known-answer tests and an independent networkx
cross-check (tests/golden/nx_*.json).
"""
from .pipeline import OracleResult, Signatures, load, mlp_grad, pair_embeddings, run_pipeline, signatures  # noqa: F401
