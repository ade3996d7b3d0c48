"""Small hand-built graphs with hand-derived answers (known-answer tests).

Labels use the reference converter's ids (generate_data.py:8): N=0, O=7, C=8.
"""
from __future__ import annotations

C, N, O = 8, 0, 7
WILD = 255


def line(labels: list[int], edges: list[tuple[int, int]]) -> str:
    """One graph in the reference text format (graph.hpp:150-202)."""
    parts = [f"n#{len(labels)}", "l#11"]
    for i, l in enumerate(labels):
        parts += [str(i), str(l)]
    parts.append(f"e#{len(edges)}")
    for u, v in edges:
        parts += [str(u), str(v), "1"]
    return " ".join(parts)


def ring(n: int, labels=None):
    labels = labels or [C] * n
    return labels, [(i, (i + 1) % n) for i in range(n)]


def chain(n: int, labels=None):
    labels = labels or [C] * n
    return labels, [(i, i + 1) for i in range(n - 1)]


def star(leaves: int, center=C, leaf=C):
    return [center] + [leaf] * leaves, [(0, i + 1) for i in range(leaves)]
