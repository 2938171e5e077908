"""Energy + force loss and its gradient with respect to force-field parameters.

For a system with reference energy E_ref and forces F_ref (e.g. from the unperturbed force field),

    L = w_E (E - E_ref)^2 + w_F sum_k (F_k - F_ref,k)^2,

and for the bond, angle and vdW parameters theta (``Calculator.parameter_gradient``):

    dL/dtheta = 2 w_E (E - E_ref) dE/dtheta + 2 w_F sum_k (F - F_ref)_k dF_k/dtheta.

With F = -dE/dx, the force term is -2 w_F d/de [dE/dtheta (x + e v)] at e = 0 for v = F - F_ref: the
directional derivative of the adjoint parameter gradient along v, taken here by a central difference
in positions (two more adjoint evaluations; error O(h^2)). The position gradient of the energy is
the force itself. xreac has no parameter derivatives; this serves the differentiation workload
(perturbed copies of a TiO2/water slab) on top of the device adjoint.
"""

from __future__ import annotations

import numpy as np

from .calculator import ParameterGradient


def _combine(a, b, ca, cb):
    pairs = {}
    for key, d in a.pairs.items():
        pairs[key] = {n: ca * v + cb * b.pairs[key][n] for n, v in d.items()}
    angles = {key: [ca * x + cb * y for x, y in zip(recs, b.angles[key])] for key, recs in a.angles.items()}
    return ParameterGradient(pairs, angles)


def energy_force_loss(calc, symbols, positions, reference_energy, reference_forces, *, cell=None, pbc=None,
                      total_charge=0, w_energy=1.0, w_force=1.0, step=1e-4):
    """``(L, dL/dtheta, evaluation)`` for one system; ``step`` is the largest atomic displacement (A)
    of the central difference along F - F_ref."""
    kw = dict(cell=cell, pbc=pbc, total_charge=total_charge)
    x = np.asarray(positions, dtype=np.float64)
    ev, g0 = calc.parameter_gradient(symbols, x, **kw)
    v = ev.forces - np.asarray(reference_forces, dtype=np.float64)
    de = ev.energy - float(reference_energy)
    loss = w_energy * de * de + w_force * float(np.sum(v * v))
    grad = _combine(g0, g0, 2 * w_energy * de, 0.0)
    vmax = float(np.abs(v).max())
    if w_force != 0.0 and vmax > 0.0:
        h = step / vmax  # displacement x +- h v moves no atom by more than `step`
        _, gp = calc.parameter_gradient(symbols, x + h * v, initial_charges=ev.charges, **kw)
        _, gm = calc.parameter_gradient(symbols, x - h * v, initial_charges=ev.charges, **kw)
        dd = _combine(gp, gm, 1.0 / (2 * h), -1.0 / (2 * h))  # d/de dE/dtheta(x + e v)
        grad = _combine(grad, dd, 1.0, -2.0 * w_force)
    return loss, grad, ev
