"""Caller-supplied neighbour lists ``(i, j, S)``: the checks that concern the Python objects.

xreac validates a supplied list in ``Neighbors.__init__`` and ``_edge_order``
(src/xreac/neighbors.py:65-131): a tuple of three integer arrays of shapes (M,), (M,), (M, 3);
indices in range; zero shifts in non-periodic directions; no zero-shift self edge; no duplicate
edge; both directions present. The first four checks (which need the Python objects, and the range
check before the indices are narrowed to 32 bits) run here; the library runs the rest, in xreac's
order and with its messages, while it puts the list in canonical order (``xr_eval_neighbors``).
"""

from __future__ import annotations

import numpy as np

_I32 = np.iinfo(np.int32)


def supplied_arrays(neighbors, n):
    """``(i, j, S)`` as C-contiguous int32 arrays, after xreac's structural and range checks."""
    if not isinstance(neighbors, (tuple, list)) or len(neighbors) != 3:
        raise ValueError("neighbors must be a tuple (i, j, S)")
    i, j, s = (np.asarray(v) for v in neighbors)
    if i.ndim != 1 or j.shape != i.shape or s.shape != (len(i), 3):
        raise ValueError("neighbors require i and j with shape (M,) and S with shape (M, 3)")
    if any(v.dtype.kind not in "iu" for v in (i, j, s)):
        raise ValueError("Neighbor indices and lattice shifts must be integers")
    if len(i) and (i.min() < 0 or j.min() < 0 or i.max() >= n or j.max() >= n):
        raise ValueError("Neighbor atom indices are out of range")
    if len(s) and (s.min() < _I32.min or s.max() > _I32.max):
        raise ValueError("An image shift exceeds the supported range of +-255 cells; wrap the positions into the cell")
    return tuple(np.ascontiguousarray(v, dtype=np.int32) for v in (i, j, s))
