"""Differentiation on the device adjoint: an energy + force loss, a flat parameter vector, the
batched loss of many perturbed force-field copies, and ``torch.autograd.Function`` wrappers.

xreac has no parameter derivatives; it differentiates energies with HIPS autograd
(``make_vjp`` at src/xreac/calculator.py:141-148). Here every derivative comes from the device's
hand-written adjoint kernels: forces (positions) and dE/dtheta for the bond, angle and vdW
parameters (``Calculator.parameter_gradient``).

Loss of the differentiation workload. For a system with reference energy E_ref and forces F_ref
(e.g. from the unperturbed force field),

    L = w_E (E - E_ref)^2 + w_F sum_k (F_k - F_ref,k)^2,
    dL/dtheta = 2 w_E (E - E_ref) dE/dtheta + 2 w_F sum_k (F - F_ref)_k dF_k/dtheta.

With F = -dE/dx, the force term is -2 w_F d/de [dE/dtheta (x + e v)] at e = 0 for v = F - F_ref:
the directional derivative of the adjoint parameter gradient along v, taken by a central
difference (error O(h^2)) whose two displaced geometries are evaluated in one device call with a
gradient per system.
"""

from __future__ import annotations

import operator
from typing import NamedTuple

import numpy as np

from .calculator import GRADIENT_PAIR_COLUMNS, ParameterGradient


def _combine(a, b, ca, cb):
    pairs = {}
    for key, d in a.pairs.items():
        pairs[key] = {n: ca * v + cb * b.pairs[key][n] for n, v in d.items()}
    angles = {key: [ca * x + cb * y for x, y in zip(recs, b.angles[key])] for key, recs in a.angles.items()}
    return ParameterGradient(pairs, angles)


def energy_force_loss(calc, symbols, positions, reference_energy, reference_forces, *, cell=None, pbc=None,
                      total_charge=0, w_energy=1.0, w_force=1.0, step=1e-4):
    """``(L, dL/dtheta, evaluation)`` for one system with ``calc``'s force field; ``step`` is the
    largest atomic displacement (A) of the central difference along F - F_ref. Two device calls:
    the evaluation at x, then x + h v and x - h v together."""
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
        pts = [dict(symbols=symbols, positions=x + sgn * h * v, initial_charges=ev.charges, **kw) for sgn in (1, -1)]
        _, (gp, gm) = calc.parameter_gradient_many(pts, per_system=True)
        dd = _combine(gp, gm, 1.0 / (2 * h), -1.0 / (2 * h))  # d/de dE/dtheta(x + e v)
        grad = _combine(grad, dd, 1.0, -2.0 * w_force)
    return loss, grad, ev


class ParameterVector:
    """The force-field parameters that have a device adjoint gradient, as one flat float64 vector:
    the bond, bond-order, over-coordination weight and vdW columns of every distinct pair record
    (``GRADIENT_PAIR_COLUMNS``) and the seven entries of every distinct angle record. A record the
    force field shares between keys (a pair's two orders, an angle's two ends) is one entry.

    Each entry also knows the table entries that hold it (``ForceField.tables()``: pair rows
    ``s*T+t`` x 28 columns, then angle rows x 7), so parameter vectors become device tables, and
    raw per-table-entry gradients become vector gradients, by array indexing alone."""

    def __init__(self, force_field):
        from .forcefield import PAIR_COLUMNS

        names = list(force_field.elements)
        T = len(names)
        self.ntypes = T
        self.entries = []
        self._pair_records = []   # (key, column names) per distinct pair record, in entry order
        self._angle_records = []  # (key, record index) per distinct angle record, in entry order
        index_of = {}             # id(record) -> first entry of the record
        for key, prm in force_field.pairs.items():
            if id(prm) in index_of:
                continue
            cols = [name for name in GRADIENT_PAIR_COLUMNS if name in prm]
            index_of[id(prm)] = len(self.entries)
            self._pair_records.append((key, cols))
            self.entries += [("pair", key, name) for name in cols]
        for key, records in force_field.angles.items():
            for q, rec in enumerate(records):
                if id(rec) in index_of:
                    continue
                index_of[id(rec)] = len(self.entries)
                self._angle_records.append((key, q))
                self.entries += [("angle", key, q, k) for k in range(7)]
        # table positions of every entry: flat index into [pair table (T*T*28) | angle table (R*7)]
        npair = T * T * 28
        positions = [[] for _ in self.entries]
        for si, s in enumerate(names):
            for ti, t in enumerate(names):
                prm = force_field.pairs.get((s, t))
                if prm is None or id(prm) not in index_of:
                    continue
                first = index_of[id(prm)]
                for c, name in enumerate(name for name in GRADIENT_PAIR_COLUMNS if name in prm):
                    positions[first + c].append((si * T + ti) * 28 + PAIR_COLUMNS.index(name))
        rows = force_field.angle_row_keys()
        for r, (key, q) in enumerate(rows):
            first = index_of[id(force_field.angles[key][q])]
            for k in range(7):
                positions[first + k].append(npair + 7 * r + k)
        self.npair, self.nangle_rows = npair, len(rows)
        width = max((len(p) for p in positions), default=1)
        sentinel = npair + 7 * len(rows)  # a zero column appended to the raw gradients
        self._pos = np.full((len(self.entries), max(width, 1)), sentinel, dtype=np.int64)
        for n, p in enumerate(positions):
            self._pos[n, :len(p)] = p
        # the summation (table position -> entry) as a sparse matrix, split at the pair/angle boundary
        from scipy.sparse import csr_matrix

        rows_, cols_ = [], []
        for n, p in enumerate(positions):
            rows_ += p
            cols_ += [n] * len(p)
        rows_, cols_ = np.asarray(rows_, dtype=np.int64), np.asarray(cols_, dtype=np.int64)
        total = csr_matrix((np.ones(len(rows_)), (rows_, cols_)), shape=(npair + 7 * len(rows), len(self.entries)))
        self._sum_pair, self._sum_angle = total[:npair], total[npair:]
        self._getters = [(key, operator.itemgetter(*cols) if cols else None, len(cols))
                         for key, cols in self._pair_records]

    def __len__(self):
        return len(self.entries)

    def values(self, force_field):
        """This vector's parameters read from ``force_field`` (the same elements and records)."""
        out = []
        pairs, angles = force_field.pairs, force_field.angles
        for key, get, n in self._getters:
            if n == 1:
                out.append(get(pairs[key]))
            elif n:
                out.extend(get(pairs[key]))
        vals = np.asarray(out, dtype=np.float64)
        if not self._angle_records:
            return vals
        return np.concatenate([vals] + [np.asarray(angles[key][q], dtype=np.float64) for key, q in self._angle_records])

    def apply(self, force_field, theta):
        """A copy of ``force_field`` with these parameters set to ``theta``."""
        import copy

        ff = copy.deepcopy(force_field)
        for n, e in enumerate(self.entries):
            if e[0] == "pair":
                ff.pairs[e[1]][e[2]] = float(theta[n])
            else:
                ff.angles[e[1]][e[2]][e[3]] = float(theta[n])
        return ff

    def tables(self, base_tables, thetas):
        """Pair and angle tables ``(G, T*T, 28)``, ``(G, R, 7)`` of G parameter vectors ``thetas``
        (G, n): ``base_tables`` (``ForceField.tables()`` of the force field this vector was made
        from) with every entry's table positions set to its value."""
        thetas = np.atleast_2d(np.asarray(thetas, dtype=np.float64))
        G = len(thetas)
        flat = np.concatenate([np.asarray(base_tables["pair"], dtype=np.float64).ravel(),
                               np.asarray(base_tables["angle"], dtype=np.float64).ravel(), [0.0]])
        out = np.repeat(flat[None, :], G, axis=0)
        for c in range(self._pos.shape[1]):
            out[:, self._pos[:, c]] = thetas
        pair = out[:, :self.npair].reshape(G, self.ntypes * self.ntypes, 28)
        angle = out[:, self.npair:-1].reshape(G, self.nangle_rows, 7)
        return pair, angle

    def gradient_rows(self, pair_rows, angle_rows):
        """Vector gradients ``(G, n)`` from raw per-table-entry gradients: ``pair_rows`` (G, T*T, 28)
        and ``angle_rows`` (G, R, 7) as ``Calculator.parameter_gradient_many(..., raw=True)`` gives
        them; each entry sums the rows of every table position that holds it."""
        G = len(pair_rows)
        out = np.asarray(self._sum_pair.T @ np.asarray(pair_rows, dtype=np.float64).reshape(G, -1).T).T
        if self.nangle_rows:
            out = out + np.asarray(self._sum_angle.T @ np.asarray(angle_rows, dtype=np.float64).reshape(G, -1).T).T
        return np.ascontiguousarray(out)

    def gradient(self, grad):
        """A ``ParameterGradient`` as a vector in this order."""
        out = np.empty(len(self.entries))
        for n, e in enumerate(self.entries):
            out[n] = grad.pairs[e[1]][e[2]] if e[0] == "pair" else grad.angles[e[1]][e[2]][e[3]]
        return out


class CopiesLoss(NamedTuple):
    """Losses of G copies and their gradients in ``vector`` order."""

    losses: np.ndarray     # (G,)
    gradients: np.ndarray  # (G, len(vector)) dL/dtheta
    vector: ParameterVector


def perturbed_copies_loss(copies, reference_ff, device=0, *, w_energy=1.0, w_force=1.0, step=1e-4, calculator=None):
    """The differentiation workload as one batch: for every ``(system, perturbed force field)``, the
    loss ``energy_force_loss`` defines against ``reference_ff``'s energy and forces of the same
    system, and its parameter gradient.

    Every copy's force field becomes a parameter set of one device force field (set 0 is
    ``reference_ff``), so the whole workload is three batched device calls: the reference
    evaluations, the copies at x with a gradient per system, and the copies at x +- h v (the force
    term's central difference) with a gradient per system. A copy enters through the parameters of
    ``ParameterVector`` (bond, bond-order, over-coordination weight, vdW and valence-angle values);
    its other parameters are taken to be ``reference_ff``'s. ``calculator`` may pass a
    ``Calculator`` of ``reference_ff`` to reuse.
    """
    from .calculator import Calculator

    copies = list(copies)
    calc = calculator if calculator is not None else Calculator(reference_ff, device=device)
    vec = ParameterVector(reference_ff)
    for _, ff in copies:
        if tuple(ff.elements) != tuple(reference_ff.elements):
            raise ValueError("every copy must have the reference force field's elements and parameter records")
    thetas = np.stack([vec.values(ff) for _, ff in copies])
    return copies_loss(calc, vec, [s for s, _ in copies], thetas, w_energy=w_energy, w_force=w_force, step=step)


def copies_loss(calc, vec, systems, thetas, *, w_energy=1.0, w_force=1.0, step=1e-4):
    """``perturbed_copies_loss`` for parameter vectors: system k with ``calc``'s force field
    modified to ``thetas[k]`` (in ``vec`` order), against ``calc``'s own force field on system k."""
    G = len(systems)
    pair, angle = vec.tables(calc._tables0(), thetas)
    calc.load_parameter_tables(pair=pair, angle=angle, count=G)
    items = [dict(symbols=s.symbols, positions=s.positions, cell=s.cell, pbc=s.pbc, total_charge=s.total_charge)
             for s in systems]
    refs = calc.evaluate_many(items)
    sets = np.arange(1, G + 1, dtype=np.int32)
    # the reference charges of the same geometry start each copy's QEq solve
    evs, p0, a0 = calc.parameter_gradient_many([dict(d, initial_charges=r.charges) for d, r in zip(items, refs)],
                                               parameter_sets=sets, raw=True)
    g0 = vec.gradient_rows(p0, a0)
    de = np.array([e.energy - r.energy for e, r in zip(evs, refs)])
    vs = [e.forces - r.forces for e, r in zip(evs, refs)]
    losses = w_energy * de * de + w_force * np.array([float(np.sum(v * v)) for v in vs])
    grads = (2 * w_energy * de)[:, None] * g0
    vmax = np.array([float(np.abs(v).max()) for v in vs])
    moved = np.nonzero((vmax > 0.0) & (w_force != 0.0))[0]
    if len(moved):
        h = step / vmax[moved]
        pts = []
        for sgn in (1, -1):
            for k, hk in zip(moved, h):
                x = np.asarray(items[k]["positions"], dtype=np.float64) + sgn * hk * vs[k]
                pts.append(dict(items[k], positions=x, initial_charges=evs[k].charges))
        _, pp, ap = calc.parameter_gradient_many(pts, parameter_sets=np.concatenate([sets[moved]] * 2), raw=True)
        gpm = vec.gradient_rows(pp, ap)
        n = len(moved)
        dd = (gpm[:n] - gpm[n:]) / (2 * h)[:, None]  # d/de dE/dtheta(x + e v)
        grads[moved] -= 2.0 * w_force * dd
    return CopiesLoss(losses, grads, vec)


class DeviceModel:
    """One system on a device ``Calculator`` as a function of positions and force-field parameters,
    for the ``torch.autograd`` wrappers below. A parameter vector is evaluated as parameter set 1 of
    the calculator's device force field (written by array indexing, no force-field copy).

    Forces are the charge-response forces (``full_derivative=True``): the exact derivative of the
    energy, QEq charges included, which is what automatic differentiation of the energy gives.
    """

    def __init__(self, calc, symbols, *, cell=None, pbc=None, total_charge=0):
        self.calc = calc
        self.base = calc.force_field
        self.vector = ParameterVector(self.base)
        self.symbols = list(symbols)
        self.kw = dict(cell=cell, pbc=pbc, total_charge=total_charge)

    def theta0(self):
        """The force field's own parameter vector (a float64 tensor)."""
        import torch

        return torch.tensor(self.vector.values(self.base), dtype=torch.float64)

    def _set(self, theta):
        pair, angle = self.vector.tables(self.calc._tables0(), np.asarray(theta, dtype=np.float64)[None])
        self.calc.load_parameter_tables(pair=pair, angle=angle, count=1)

    def _run(self, positions_list, theta):
        self._set(theta)
        pts = [dict(symbols=self.symbols, positions=x, **self.kw) for x in positions_list]
        evs, pr, ar = self.calc.parameter_gradient_many(pts, full_derivative=True, raw=True,
                                                        parameter_sets=np.ones(len(pts), dtype=np.int32))
        return evs, self.vector.gradient_rows(pr, ar)

    def evaluate(self, positions, theta):
        """(energy, forces, dE/dtheta vector) at one point."""
        (ev,), g = self._run([positions], theta)
        return ev.energy, np.array(ev.forces), g[0]

    def evaluate_pair(self, positions, direction, h, theta):
        """Forces and dE/dtheta at positions +- h direction, in one device call."""
        evs, g = self._run([positions + h * direction, positions - h * direction], theta)
        return [np.array(e.forces) for e in evs], [g[0], g[1]]

    def energy(self, positions, theta):
        return DeviceEnergy.apply(positions, theta, self)

    def energy_forces(self, positions, theta, step=1e-4):
        return DeviceEnergyForces.apply(positions, theta, self, step)


def _torch_function_classes():
    import torch

    class _DeviceEnergy(torch.autograd.Function):
        """E(positions, theta) with its gradient from the device adjoint: dE/dx = -F, dE/dtheta."""

        @staticmethod
        def forward(ctx, positions, theta, model):
            x = positions.detach().cpu().numpy().astype(np.float64)
            e, f, g = model.evaluate(x, theta.detach().cpu().numpy())
            ctx.save_for_backward(torch.as_tensor(-f), torch.as_tensor(g))
            return torch.tensor(e, dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad_e):
            dx, dth = ctx.saved_tensors
            return grad_e * dx, grad_e * dth, None

    class _DeviceEnergyForces(torch.autograd.Function):
        """(E, F)(positions, theta). The backward pass needs second derivatives: for an output
        gradient (g_E, g_F) it is

            dL/dx = -g_E F - H g_F,        dL/dtheta = g_E dE/dtheta - d/de dE/dtheta(x + e g_F),

        with H g_F = -d/de F(x + e g_F); both directional derivatives are one central difference
        along g_F (displacement at most `step` A), the two points evaluated in one device call."""

        @staticmethod
        def forward(ctx, positions, theta, model, step):
            x = positions.detach().cpu().numpy().astype(np.float64)
            th = theta.detach().cpu().numpy()
            e, f, g = model.evaluate(x, th)
            ctx.model, ctx.step, ctx.x, ctx.th = model, step, x, th
            ctx.f, ctx.g = f, g
            return torch.tensor(e, dtype=torch.float64), torch.as_tensor(f)

        @staticmethod
        def backward(ctx, grad_e, grad_f):
            ge = 0.0 if grad_e is None else float(grad_e)
            dx = -ge * ctx.f
            dth = ge * ctx.g
            if grad_f is not None:
                v = grad_f.detach().cpu().numpy().astype(np.float64)
                vmax = float(np.abs(v).max())
                if vmax > 0.0:
                    h = ctx.step / vmax
                    (fp, fm), (gp, gm) = ctx.model.evaluate_pair(ctx.x, v, h, ctx.th)
                    dx = dx + (fp - fm) / (2 * h)  # -H v
                    dth = dth - (gp - gm) / (2 * h)
            return torch.as_tensor(dx), torch.as_tensor(dth), None, None

    return _DeviceEnergy, _DeviceEnergyForces


class _Lazy:
    """The torch classes are made on first use, so importing this module needs no torch."""

    def __init__(self, index):
        self.index = index
        self.cls = None

    def apply(self, *args):
        if self.cls is None:
            self.cls = _torch_function_classes()[self.index]
        return self.cls.apply(*args)


DeviceEnergy = _Lazy(0)
DeviceEnergyForces = _Lazy(1)
