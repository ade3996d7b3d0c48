"""bms2_gb300 — GB300-native batched subgraph-isomorphism engine.

The engine is libbms.so (C ABI in include/bms.h); this package holds its CUDA
and C++ sources (csrc/), the build recipe (build.py), the seeded workload
presets (workloads.py) and the ctypes binding (native.py).
"""
from .native import (COUNT_ALL, DATA, FIND_FIRST, OPT_CUDA_GRAPH, OPT_FILTER_KERNEL, OPT_JOIN_STEPS,  # noqa: F401
                     OPT_RESIDENT_SIGNATURES, OPT_SPLIT_BUDGET, OPT_SUBTREE_CAP, OPT_USE_CS, ORDER_GIVEN, ORDER_GMCR, ORDER_LEARNED, QUERY, SEM_EXACT,
                     SEM_REFERENCE_DFS, BmsError, Context, Graphs, lib)
