"""Host-side cell and input validation with xreac's semantics and error messages.

Mirrors ``Boundary`` (src/xreac/geometry.py:15-79) and ``validate_input`` /
``validate_total_charge`` (src/xreac/calculator.py:45-66): same accepted forms of ``cell`` and
``pbc``, same ``ValueError`` texts, and the same small-cell replication count and memory limit,
so that ``cell_repetitions`` and the ``max_expanded_atoms`` error agree with the reference. The
device evaluates small cells directly from image shifts; the replication count is reported for
compatibility only. The coincident-atom check runs on the device as part of the neighbour search.
"""

from __future__ import annotations

import math
from numbers import Real

import numpy as np


def validate_expansion_limit(value):
    if isinstance(value, bool) or not isinstance(value, (int, np.integer)) or value < 1:
        raise ValueError("max_expanded_atoms must be a positive integer")


def validate_total_charge(total_charge):
    if isinstance(total_charge, (bool, np.bool_)) or not isinstance(total_charge, Real) or not np.isfinite(total_charge):
        raise ValueError("total_charge must be a finite real scalar")


def boundary(cell, pbc):
    """Validated ``(pbc flags (3,), cell matrix or None)``."""
    if pbc is None:
        pbc = cell is not None
    flags = np.asarray(pbc)
    if flags.shape not in ((), (3,)) or flags.dtype.kind not in "biu" or not ((flags == 0) | (flags == 1)).all():
        raise ValueError("pbc must be a boolean or three boolean flags")
    flags = np.broadcast_to(flags.astype(bool), (3,)).copy()
    if not flags.any():
        return flags, None
    if cell is None:
        raise ValueError("A cell is required when pbc is enabled")
    m = np.array(cell, dtype=float, copy=True)
    if m.shape == (3,):
        if np.any(m <= 0):
            raise ValueError("Cell lengths must be positive")
        m = np.diag(m)
    if m.shape != (3, 3) or not np.isfinite(m).all():
        raise ValueError("cell must contain three finite lengths or a finite (3, 3) matrix")
    if np.linalg.det(m) <= 1e-12 * np.prod(np.linalg.norm(m, axis=1)):
        raise ValueError("Periodic cells must be nonsingular and right-handed")
    return flags, m


def cell_repetitions(cutoff, flags, m, atoms, max_expanded_atoms=512):
    """Replication counts of xreac's neighbour search and its memory limit (src/xreac/geometry.py:58-79)."""
    validate_expansion_limit(max_expanded_atoms)
    reps = np.ones(3, dtype=int)
    if m is None:
        return (1, 1, 1)
    heights = 1.0 / np.linalg.norm(np.linalg.inv(m), axis=0)
    required = np.floor(cutoff * (1 + 1e-12) / heights[flags]) + 1
    copies = float(np.prod(required))
    if copies > 1 and copies * atoms > max_expanded_atoms:
        raise ValueError(
            f"Small-cell replication needs {copies * atoms:g} internal atoms, "
            f"exceeding max_expanded_atoms={max_expanded_atoms}; "
            "increase this limit explicitly if memory permits"
        )
    reps[flags] = required.astype(int)
    return tuple(int(v) for v in reps)


_ALL_PBC = np.ones(3, dtype=bool)
_ALL_PBC.flags.writeable = False


def periodic_cell(cell, pbc, cutoff, atoms, max_expanded_atoms):
    """``(pbc flags, cell matrix, repetitions)`` of a fully periodic cell given as three lengths or a (3, 3)
    matrix with ``pbc`` True (or None), computed with scalar arithmetic, which for a 3 x 3 cell is
    several times cheaper than the general path; None for any other input or any input the general
    path would reject, which then gives the same result or error through ``boundary`` and
    ``cell_repetitions``. Face heights are volume / area of the opposite face, the same quantity as
    the inverse of the reciprocal vectors' norms."""
    if not (pbc is True or (pbc is None and cell is not None)):
        return None
    try:
        m = np.array(cell, dtype=np.float64)
    except (TypeError, ValueError):
        return None
    if m.shape == (3,):
        if not (m > 0).all():
            return None
        m = np.diag(m)
    if m.shape != (3, 3):
        return None
    a, b, c = m.tolist()
    if not all(math.isfinite(v) for v in a + b + c):
        return None
    bc = (b[1] * c[2] - b[2] * c[1], b[2] * c[0] - b[0] * c[2], b[0] * c[1] - b[1] * c[0])
    ca = (c[1] * a[2] - c[2] * a[1], c[2] * a[0] - c[0] * a[2], c[0] * a[1] - c[1] * a[0])
    ab = (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])
    det = a[0] * bc[0] + a[1] * bc[1] + a[2] * bc[2]
    norms = [math.sqrt(sum(v * v for v in r)) for r in (a, b, c)]
    if not det > 1e-12 * norms[0] * norms[1] * norms[2]:
        return None
    reps = []
    for face in (bc, ca, ab):
        ratio = cutoff * (1 + 1e-12) * math.sqrt(face[0] ** 2 + face[1] ** 2 + face[2] ** 2) / det
        if abs(ratio - round(ratio)) < 1e-9:
            return None  # on a boundary the general path's rounding decides
        reps.append(int(math.floor(ratio)) + 1)
    copies = reps[0] * reps[1] * reps[2]
    if copies > 1 and copies * atoms > max_expanded_atoms:
        return None
    return _ALL_PBC, m, tuple(reps)


def validate_input(symbols, positions, total_charge=0, cell=None, pbc=None):
    """Symbols, float64 positions and the validated cell (src/xreac/calculator.py:55-66)."""
    symbols = tuple(symbols)
    if not symbols or any(not isinstance(s, str) or not s for s in symbols):
        raise ValueError("A nonempty sequence of parameter-file atom labels is required")
    validate_total_charge(total_charge)
    x = np.array(positions, dtype=np.float64, copy=True)
    if x.shape != (len(symbols), 3) or not np.isfinite(x).all():
        raise ValueError("positions must be a finite (N, 3) array in Angstrom")
    flags, m = boundary(cell, pbc)
    return symbols, x, flags, m
