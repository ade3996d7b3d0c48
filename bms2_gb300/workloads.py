"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference measures on converted public SMARTS sets; those cannot be
converted here (no rdkit), so seeded synthetic molecular graphs with the stated
distributions stand in for them.  Every workload is a pure function of its seed.

  mol1k     1,000 data graphs of 10-40 atoms (uniform), 20 queries of 3-12 nodes
  mol100k   100,000 data graphs, N(28, 9) atoms clipped to 10-60, 600 queries of
            5-30 nodes of which 30% are pure-carbon chains or rings
  mol1m     1,000,000 data graphs, log-normal atoms (median 25, sigma 0.55)
            clipped to 5-120, 1,000 queries of 3-40 nodes
  mol10m    10,000,000 data graphs as mol1m (about 290M atoms), 3,000 queries of
            3-40 nodes of which 20% are adversarial symmetric patterns
Element mix C 72%, N 12%, O 11%, S 2%, F 1.5%, Cl 1%, Br 0.5%; degree <= 4;
1-4 rings per molecule; bonds single/double/triple/aromatic 60/20/2/18%.
"""
from __future__ import annotations

from dataclasses import dataclass

from .native import SIZE_LOGNORMAL, SIZE_NORMAL, SIZE_UNIFORM, Graphs


@dataclass(frozen=True)
class Workload:
    name: str
    n_data: int
    size_dist: int
    p0: float
    p1: float
    min_atoms: int
    max_atoms: int
    n_queries: int
    q_min: int
    q_max: int
    frac_carbon: float
    frac_adversarial: float


WORKLOADS = {
    "mol1k": Workload("mol1k", 1_000, SIZE_UNIFORM, 0, 0, 10, 40, 20, 3, 12, 0.0, 0.0),
    "mol100k": Workload("mol100k", 100_000, SIZE_NORMAL, 28.0, 9.0, 10, 60, 600, 5, 30, 0.3, 0.0),
    "mol1m": Workload("mol1m", 1_000_000, SIZE_LOGNORMAL, 25.0, 0.55, 5, 120, 1_000, 3, 40, 0.0, 0.0),
    "mol10m": Workload("mol10m", 10_000_000, SIZE_LOGNORMAL, 25.0, 0.55, 5, 120, 3_000, 3, 40, 0.0, 0.2),
}


def make(name: str, seed: int = 1, n_data: int | None = None, n_queries: int | None = None) -> tuple[Graphs, Graphs]:
    """(queries, data) of a named workload; n_data / n_queries shrink it."""
    w = WORKLOADS[name]
    data = Graphs.synth_molecules(n_data or w.n_data, seed, w.size_dist, w.p0, w.p1, w.min_atoms, w.max_atoms, 1, 4)
    queries = Graphs.synth_queries(data, n_queries or w.n_queries, seed + 1000003, w.q_min, w.q_max, w.frac_carbon,
                                   w.frac_adversarial)
    return queries, data
