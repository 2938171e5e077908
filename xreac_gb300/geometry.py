"""Host-side cell and input validation with xreac's semantics and error messages.

Mirrors ``Boundary`` (src/xreac/geometry.py:15-79) and ``validate_input`` /
``validate_total_charge`` (src/xreac/calculator.py:45-66): same accepted forms of ``cell`` and
``pbc``, same ``ValueError`` texts, and the same small-cell replication count and memory limit,
so that ``cell_repetitions`` and the ``max_expanded_atoms`` error agree with the reference. The
device evaluates small cells directly from image shifts; the replication count is reported for
compatibility only. The coincident-atom check runs on the device as part of the neighbour search.
"""

from __future__ import annotations

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
