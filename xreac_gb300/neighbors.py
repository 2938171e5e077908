"""Validation of caller-supplied neighbour lists ``(i, j, S)`` with xreac's rules and messages.

Restates the checks of ``Neighbors.__init__`` and ``_edge_order`` (src/xreac/neighbors.py:65-131):
a tuple of three integer arrays of shapes (M,), (M,), (M, 3); indices in range; zero shifts in
non-periodic directions; no zero-shift self edge; no duplicate edge; both directions present.
"""

from __future__ import annotations

import numpy as np


def check_supplied(neighbors, n, flags):
    if not isinstance(neighbors, (tuple, list)) or len(neighbors) != 3:
        raise ValueError("neighbors must be a tuple (i, j, S)")
    i, j, s = (np.asarray(v) for v in neighbors)
    if i.ndim != 1 or j.shape != i.shape or s.shape != (len(i), 3):
        raise ValueError("neighbors require i and j with shape (M,) and S with shape (M, 3)")
    if any(v.dtype.kind not in "iu" for v in (i, j, s)):
        raise ValueError("Neighbor indices and lattice shifts must be integers")
    if np.any(i < 0) or np.any(j < 0) or np.any(i >= n) or np.any(j >= n):
        raise ValueError("Neighbor atom indices are out of range")
    if np.any(s[:, ~np.asarray(flags, dtype=bool)] != 0):
        raise ValueError("Neighbor shifts must be zero in nonperiodic directions")
    if np.any((i == j) & np.all(s == 0, axis=1)):
        raise ValueError("Zero-shift self neighbors are not allowed")
    keys = [tuple(int(v) for v in row) for row in zip(i, j, s[:, 0], s[:, 1], s[:, 2])]
    ordered = sorted(keys)
    if any(a == b for a, b in zip(ordered, ordered[1:])):
        raise ValueError("Duplicate neighbor edges are not allowed")
    if sorted((b, a, -x, -y, -z) for a, b, x, y, z in ordered) != ordered:
        raise ValueError("neighbors must include both directions: (i, j, S) and (j, i, -S)")
