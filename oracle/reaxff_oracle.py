"""CPU oracle: a restatement of xreac's E+F+QEq evaluation (TEST INFRASTRUCTURE ONLY).

This module restates hsulab/xreac v0.10.0's ``Calculator.evaluate`` path
(``src/xreac/calculator.py:76-165``) in float64 on the CPU so the CUDA path can be
checked against it on the GPU machine, where the reference itself is not available.
It is the checker and the timed CPU baseline -- never the product: the
``xreac_gb300`` package does not import it.

- Neighbour search, canonical edge order, reverse map, half flags and rows restate
  ``src/xreac/neighbors.py:17-141`` and ``src/xreac/geometry.py:15-99``.
- Charges restate the dense KKT QEq solve (``src/xreac/energy.py:89-103``) in numpy.
- Bond orders, the 14 energy components, angles, torsions and hydrogen bonds
  restate ``src/xreac/energy.py:105-370`` in torch float64.
- Forces are ``-dE/dx`` from torch autograd, with charges held fixed by default
  (the reference's ``make_vjp`` at ``src/xreac/calculator.py:141-148``) and the
  same near-collinear angle rule (``src/xreac/energy.py:49-55``); with
  ``full_derivative`` the QEq solve is differentiated too.
- Properties restate ``src/xreac/energy.py:167-178``.

Parity of this restatement is pinned against fixtures written by the unmodified
reference (``tests/golden/make_golden.py``) and against the reference's published
known answers (monomer energy -248.34420920633704 kcal/mol).
"""

from __future__ import annotations

from itertools import product
from numbers import Real

import numpy as np
import torch

# Constants of src/xreac/energy.py:17-25.
C_ELE = 332.06371
QEQ_COULOMB = 14.4
SELF_CONVERSION = 23.02
THB_CUT = 0.001
THB_PRODUCT_CUT = 0.00001
BOND_CUT = 5.0
HBOND_CUT = 7.5
HBOND_THRESHOLD = 0.01
BOND_GRAPH_CUT = 0.3
COMPONENTS = (
    "bond",
    "atom",
    "lone_pair",
    "molecule",
    "angle",
    "penalty",
    "angle_conjugation",
    "hydrogen_bond",
    "torsion",
    "conjugation",
    "vdw",
    "coulomb",
    "electric_field",
    "qeq",
)
F64 = torch.float64


# ----------------------------------------------------------------------------- cells
def boundary(cell, pbc):
    """Validate a cell; returns ``(pbc flags (3,), matrix or None)`` (src/xreac/geometry.py:18-46)."""
    if pbc is None:
        pbc = cell is not None
    flags = np.asarray(pbc)
    if flags.shape not in ((), (3,)) or flags.dtype.kind not in "biu" or not np.isin(flags, [0, 1]).all():
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


def repetitions(cutoff, flags, m, atoms, max_expanded_atoms=512):
    """Small-cell replication counts and their memory check (src/xreac/geometry.py:58-79)."""
    if isinstance(max_expanded_atoms, bool) or not isinstance(max_expanded_atoms, (int, np.integer)) or max_expanded_atoms < 1:
        raise ValueError("max_expanded_atoms must be a positive integer")
    reps = np.ones(3, dtype=int)
    if m is None:
        return tuple(int(v) for v in reps)
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


# ------------------------------------------------------------------------- neighbours
def neighbor_list(x, cutoff, cell=None, pbc=None, chunk=256):
    """All directed image edges ``(i, j, S)`` with ``|x_j - x_i + S @ cell| <= cutoff``.

    The edge set of ``replicated_neighbors`` (src/xreac/neighbors.py:17-53): every
    image of every atom within the cutoff, zero-shift self edges excluded, with
    the distance test ``sum(v * v) <= cutoff**2`` on ``v = (x_j - x_i) + S @ cell``.
    Instead of replicating the cell, each pair scans the integer shifts around
    its nearest image, ``floor(cutoff / height) + 1`` cells each way, which
    reaches every image within the cutoff (only the nearest image when every
    periodic height exceeds twice the cutoff). Returned in canonical order.
    """
    x = np.asarray(x, dtype=float)
    flags, m = boundary(cell, pbc)
    n = len(x)
    lattice = m if m is not None else np.eye(3)
    if m is not None:
        inv = np.linalg.inv(m)
        heights = 1.0 / np.linalg.norm(inv, axis=0)
        reach = np.where(flags, np.floor(cutoff / heights) + 1, 0).astype(int)
        # When every periodic height exceeds twice the cutoff, an image within the cutoff has
        # |fractional offset| < 1/2 in each periodic direction, so it is the nearest image.
        if np.all(heights[flags] > 2 * cutoff * (1 + 1e-9)):
            reach = np.zeros(3, dtype=int)
    else:
        reach = np.zeros(3, dtype=int)
    offsets = np.array(list(product(*[range(-r, r + 1) for r in reach])), dtype=np.int64)
    rc2 = cutoff * cutoff
    out_i, out_j, out_s = [], [], []
    cols = np.arange(n)
    for start in range(0, n, chunk):
        rows = np.arange(start, min(n, start + chunk))
        delta = x[None, :, :] - x[rows, None, :]
        if m is not None:
            base = -np.rint(delta @ inv).astype(np.int64) * flags
        else:
            base = np.zeros(delta.shape, dtype=np.int64)
        self_pair = rows[:, None] == cols[None, :]
        for off in offsets:
            s = base + off
            v = delta + s @ lattice
            hit = np.sum(v * v, axis=-1) <= rc2
            hit &= ~(self_pair & np.all(s == 0, axis=-1))
            a, b = np.nonzero(hit)
            out_i.append(rows[a])
            out_j.append(b)
            out_s.append(s[a, b])
    i = np.concatenate(out_i).astype(np.int64)
    j = np.concatenate(out_j).astype(np.int64)
    s = np.concatenate(out_s).astype(np.int64).reshape(-1, 3)
    order = np.lexsort((s[:, 2], s[:, 1], s[:, 0], j, i))
    return i[order], j[order], s[order]


class Edges:
    """Validated canonical directed list with reverse map, half flags and rows.

    Restates ``Neighbors`` and ``_edge_order`` (src/xreac/neighbors.py:65-131).
    """

    def __init__(self, neighbors, n, flags, m):
        if not isinstance(neighbors, (tuple, list)) or len(neighbors) != 3:
            raise ValueError("neighbors must be a tuple (i, j, S)")
        i, j, s = (np.asarray(v) for v in neighbors)
        if i.ndim != 1 or j.shape != i.shape or s.shape != (len(i), 3):
            raise ValueError("neighbors require i and j with shape (M,) and S with shape (M, 3)")
        if any(v.dtype.kind not in "iu" for v in (i, j, s)):
            raise ValueError("Neighbor indices and lattice shifts must be integers")
        if np.any(i < 0) or np.any(j < 0) or np.any(i >= n) or np.any(j >= n):
            raise ValueError("Neighbor atom indices are out of range")
        if np.any(s[:, ~flags] != 0):
            raise ValueError("Neighbor shifts must be zero in nonperiodic directions")
        if np.any((i == j) & np.all(s == 0, axis=1)):
            raise ValueError("Zero-shift self neighbors are not allowed")
        # Python-int sort keys: exact for any shift magnitude.
        i = i.astype(object) if i.dtype == np.uint64 else i.astype(np.int64)
        j = j.astype(object) if j.dtype == np.uint64 else j.astype(np.int64)
        s = s.astype(object) if s.dtype == np.uint64 else s.astype(np.int64)
        keys = [tuple(int(v) for v in row) for row in zip(i, j, s[:, 0], s[:, 1], s[:, 2])]
        order = sorted(range(len(keys)), key=keys.__getitem__)
        sorted_keys = [keys[k] for k in order]
        for a, b in zip(sorted_keys, sorted_keys[1:]):
            if a == b:
                raise ValueError("Duplicate neighbor edges are not allowed")
        rkeys = [(b, a, -x, -y, -z) for a, b, x, y, z in sorted_keys]
        reverse = sorted(range(len(rkeys)), key=rkeys.__getitem__)
        if sorted_keys != [rkeys[k] for k in reverse]:
            raise ValueError("neighbors must include both directions: (i, j, S) and (j, i, -S)")
        arr = np.array(sorted_keys, dtype=np.int64).reshape(-1, 5)
        self.i, self.j, self.shifts = arr[:, 0].copy(), arr[:, 1].copy(), arr[:, 2:].copy()
        self.reverse = np.array(reverse, dtype=np.int64)
        self.n = n
        lattice = m if m is not None else np.eye(3)
        self.offsets = self.shifts @ lattice
        self.half = np.arange(len(self.i)) < self.reverse
        counts = np.bincount(self.i, minlength=n)
        self.starts = np.concatenate(([0], np.cumsum(counts)[:-1])).astype(np.int64)
        self.counts = counts

    @classmethod
    def from_sorted(cls, i, j, s, n, m):
        """Fast path for lists that are canonical by construction."""
        self = cls.__new__(cls)
        self.i, self.j, self.shifts, self.n = i, j, s, n
        order = np.lexsort((-s[:, 2], -s[:, 1], -s[:, 0], i, j))
        self.reverse = order.astype(np.int64)
        lattice = m if m is not None else np.eye(3)
        self.offsets = self.shifts @ lattice
        self.half = np.arange(len(i)) < self.reverse
        counts = np.bincount(i, minlength=n)
        self.starts = np.concatenate(([0], np.cumsum(counts)[:-1])).astype(np.int64)
        self.counts = counts
        return self


# --------------------------------------------------------------------------- physics
class _LammpsAngle(torch.autograd.Function):
    """arccos with LAMMPS's regularised derivative -1/max(sin, 1e-5) (src/xreac/energy.py:49-55)."""

    @staticmethod
    def forward(ctx, c):
        theta = torch.arccos(torch.clamp(c, -1.0, 1.0))
        ctx.save_for_backward(theta)
        return theta

    @staticmethod
    def backward(ctx, g):
        (theta,) = ctx.saved_tensors
        return -g / torch.clamp(torch.sin(theta), min=1e-5)


def _positive_power(x, p):
    # x**p for x > 0 and 0 otherwise, with finite derivatives (src/xreac/energy.py:44-46).
    return torch.where(x > 0, torch.where(x > 0, x, torch.ones_like(x)) ** p, torch.zeros_like(x))


def _t(a):
    return torch.as_tensor(np.asarray(a, dtype=float), dtype=F64)


class _Model:
    """Per-system parameter views (src/xreac/energy.py:65-87)."""

    def __init__(self, ff, symbols, edges):
        self.ff, self.symbols, self.n, self.e = ff, tuple(symbols), len(symbols), edges
        self.g = np.asarray(ff.general, dtype=float)
        labels = tuple(dict.fromkeys(symbols))
        self.labels = labels
        tix = {s: k for k, s in enumerate(labels)}
        self.t = np.array([tix[s] for s in symbols], dtype=np.int64)
        self.T = len(labels)
        self.a = {k: np.array([float(ff.atoms[s][k]) for s in labels])[self.t] for k in ff.atoms[labels[0]]}
        self.pair_keys = tuple(ff.pairs[labels[0], labels[0]].keys())
        self.pair_table = {k: np.array([ff.pairs[s, u][k] for s in labels for u in labels], dtype=float) for k in self.pair_keys}
        T = self.T
        self.tor = np.full(T**4, -1, dtype=np.int64)
        self.tor_prm = []
        for (a, b, c, d), prm in ff.torsions.items():
            if all(s in tix for s in (a, b, c, d)) and np.any(np.asarray(prm)[[0, 1, 2, 4]] != 0):
                self.tor[((tix[a] * T + tix[b]) * T + tix[c]) * T + tix[d]] = len(self.tor_prm)
                self.tor_prm.append(np.asarray(prm, dtype=float))
        self.tor_prm = np.array(self.tor_prm, dtype=float).reshape(-1, 5)
        self.ang_first = np.zeros(T**3, dtype=np.int64)
        self.ang_count = np.zeros(T**3, dtype=np.int64)
        rows = []
        for (a, b, c), recs in ff.angles.items():
            if all(s in tix for s in (a, b, c)):
                k = (tix[a] * T + tix[b]) * T + tix[c]
                self.ang_first[k], self.ang_count[k] = len(rows), len(recs)
                rows.extend(np.asarray(r, dtype=float) for r in recs)
        self.ang_prm = np.array(rows, dtype=float).reshape(-1, 7)
        self.hb = np.full(T**3, -1, dtype=np.int64)
        hb_rows = []
        for (a, b, c), prm in ff.hydrogen_bonds.items():
            if all(s in tix for s in (a, b, c)):
                self.hb[(tix[a] * T + tix[b]) * T + tix[c]] = len(hb_rows)
                hb_rows.append(np.asarray(prm, dtype=float))
        self.hb_prm = np.array(hb_rows, dtype=float).reshape(-1, 4)

    def pair(self, key, edge_ids):
        e = self.e
        return self.pair_table[key][self.t[e.i[edge_ids]] * self.T + self.t[e.j[edge_ids]]]


def _shield_taper(model, r):
    """Taper polynomial and shielded-Coulomb kernel (src/xreac/energy.py:90-92)."""
    rc = model.g[12]
    u = torch.clamp(r / rc, max=1.0)
    taper = torch.where(r < rc, 1 + u**4 * (-35 + u * (84 + u * (-70 + 20 * u))), torch.zeros_like(r))
    gamma = _t(model.pair("gamma", np.arange(len(model.e.i))))
    shield = taper / (r**3 + gamma) ** (1.0 / 3.0)
    return taper, shield


def qeq_charges(model, r_np, total_charge):
    """Dense KKT QEq solve outside the derivative (src/xreac/energy.py:95-103)."""
    e, n = model.e, model.n
    with torch.no_grad():
        _, shield = _shield_taper(model, _t(r_np))
    shield = shield.numpy()
    h = np.bincount(e.i * n + e.j, weights=QEQ_COULOMB * shield, minlength=n * n).astype(float).reshape(n, n)
    # QEQ_COULOMB * pair_sum(shield) in the reference multiplies after summing; both orders
    # agree to rounding, well inside the charge tolerance.
    h[np.diag_indices(n)] += model.a["eta"]
    kkt = np.zeros((n + 1, n + 1))
    kkt[:n, :n] = h
    kkt[:n, n] = 1.0
    kkt[n, :n] = 1.0
    rhs = np.concatenate((-model.a["chi"], [float(total_charge)]))
    try:
        return np.linalg.solve(kkt, rhs)[:n]
    except np.linalg.LinAlgError as exc:
        raise ValueError("Singular QEq system; check the geometry and parameters") from exc


def _bond_orders(model, r):
    """Corrected bond orders per directed edge (src/xreac/energy.py:105-165)."""
    a, g, e = model.a, model.g, model.e
    M = len(e.i)
    sel = np.flatnonzero(r.detach().numpy() <= min(BOND_CUT, g[12]))
    rs = r[sel]
    ii, jj = e.i[sel], e.j[sel]
    P = {k: model.pair(k, sel) for k in (
        "p_bo1", "p_bo2", "p_bo3", "p_bo4", "p_bo5", "p_bo6", "r_s", "r_p", "r_pp", "ovc", "v13cor",
        "p_boc3", "p_boc4", "p_boc5")}
    cut = 0.01 * g[29]
    sig_ok = (a["r_s"][ii] > 0) & (a["r_s"][jj] > 0)
    pi_ok = (a["r_pi"][ii] > 0) & (a["r_pi"][jj] > 0)
    pp_ok = (a["r_pi_pi"][ii] > 0) & (a["r_pi_pi"][jj] > 0)
    zero = torch.zeros_like(rs)
    sig = torch.where(_t(sig_ok).bool(), (1 + cut) * torch.exp(_t(P["p_bo1"]) * (rs / _t(np.where(sig_ok, P["r_s"], 1))) ** _t(P["p_bo2"])), zero)
    pi = torch.where(_t(pi_ok).bool(), torch.exp(_t(P["p_bo3"]) * (rs / _t(np.where(pi_ok, P["r_p"], 1))) ** _t(P["p_bo4"])), zero)
    pp = torch.where(_t(pp_ok).bool(), torch.exp(_t(P["p_bo5"]) * (rs / _t(np.where(pp_ok, P["r_pp"], 1))) ** _t(P["p_bo6"])), zero)
    raw = sig + pi + pp
    mask = raw.detach().numpy() >= cut
    corrected = mask & ((P["ovc"] >= 0.001) | (P["v13cor"] >= 0.001))
    for key in ("p_boc3", "p_boc4", "p_boc5"):
        if np.any(corrected & ~np.isfinite(P[key])):
            raise ValueError(f"Invalid {key} mixing for an active bond-order correction")
        P[key] = np.where(corrected, P[key], 0.0)
    mt = torch.as_tensor(mask)
    bo = torch.where(mt, raw - cut, zero)
    pi, pp = torch.where(mt, pi, zero), torch.where(mt, pp, zero)
    ii_t, jj_t = torch.as_tensor(ii), torch.as_tensor(jj)
    total = torch.zeros(model.n, dtype=F64).index_add(0, ii_t, bo)
    d = total - _t(a["valency"])
    db = total - _t(a["valency_val"])
    f2 = torch.exp(-g[0] * d[ii_t]) + torch.exp(-g[0] * d[jj_t])
    f3 = -torch.log(0.5 * (torch.exp(-g[1] * d[ii_t]) + torch.exp(-g[1] * d[jj_t]))) / g[1]
    vi, vj = _t(a["valency"][ii]), _t(a["valency"][jj])
    f1 = torch.where(_t(P["ovc"] >= 0.001).bool(), 0.5 * ((vi + f2) / (vi + f2 + f3) + (vj + f2) / (vj + f2 + f3)), torch.ones_like(rs))
    b3, b4, b5 = _t(P["p_boc3"]), _t(P["p_boc4"]), _t(P["p_boc5"])
    f4 = 1 / (1 + torch.exp(-(b4 * bo**2 - db[ii_t]) * b3 + b5))
    f5 = 1 / (1 + torch.exp(-(b4 * bo**2 - db[jj_t]) * b3 + b5))
    corr = f1 * torch.where(_t(P["v13cor"] >= 0.001).bool(), f4 * f5, torch.ones_like(rs))
    bo, pi, pp = bo * corr, pi * corr * f1, pp * corr * f1
    sel_t = torch.as_tensor(sel)
    out = []
    for v in (bo, bo - pi - pp, pi, pp):
        kept = torch.where(v >= 1e-10, v, torch.zeros_like(v))
        out.append(torch.zeros(M, dtype=F64).index_add(0, sel_t, kept))
    return tuple(out)


def _components(model, x, q, total_charge, lammps_forces):
    """The 14 energy components (src/xreac/energy.py:180-229); returns (E dict, bond state)."""
    a, g, e, n = model.a, model.g, model.e, model.n
    i_t, j_t = torch.as_tensor(e.i), torch.as_tensor(e.j)
    vectors = x[j_t] - x[i_t] + _t(e.offsets)
    r = torch.sqrt(torch.sum(vectors * vectors, dim=1))
    taper, shield = _shield_taper(model, r)
    if q is None:  # charge-response derivative: QEq inside the derivative
        h = torch.zeros(n * n, dtype=F64).index_add(0, torch.as_tensor(e.i * n + e.j), shield).reshape(n, n)
        h = QEQ_COULOMB * h + torch.diag(_t(a["eta"]))
        ones = torch.ones((n, 1), dtype=F64)
        kkt = torch.cat((torch.cat((h, ones), 1), torch.cat((ones.T, torch.zeros((1, 1), dtype=F64)), 1)), 0)
        rhs = torch.cat((-_t(a["chi"]), _t([float(total_charge)])))
        q = torch.linalg.solve(kkt, rhs)[:n]
    else:
        q = _t(q)
    bo, sigma, pi, pp = _bond_orders(model, r)
    total = torch.zeros(n, dtype=F64).index_add(0, i_t, bo)
    d = total - _t(a["valency"])
    db = total - _t(a["valency_boc"])
    de = total - _t(a["valency_e"])
    half = np.trunc(de.detach().numpy() / 2)
    vlpex = de - 2 * _t(half)
    nlp = torch.exp(-g[15] * (2 + vlpex) ** 2) - _t(half)
    dlp = 0.5 * _t(a["valency_e"] - a["valency"]) - nlp
    dlpt = torch.where(_t(a["mass"] > 21).bool(), torch.zeros_like(dlp), dlp)
    E = {k: torch.zeros((), dtype=F64) for k in COMPONENTS}
    # Edges carrying any nonzero bond-order part; every other edge adds exactly zero below.
    cand = np.flatnonzero((bo.detach().numpy() != 0) | (sigma.detach().numpy() != 0) | (pi.detach().numpy() != 0) | (pp.detach().numpy() != 0))
    c_t = torch.as_tensor(cand)
    E["bond"] = -0.5 * torch.sum(
        _t(model.pair("De_s", cand)) * sigma[c_t] * torch.exp(_t(model.pair("p_be1", cand)) * (1 - _positive_power(sigma[c_t], _t(model.pair("p_be2", cand)))))
        + _t(model.pair("De_p", cand)) * pi[c_t]
        + _t(model.pair("De_pp", cand)) * pp[c_t]
    )
    E["lone_pair"] = torch.sum(_t(a["p_lp2"]) * dlp / (1 + torch.exp(-75 * dlp)))
    _special_corrections(model, E, bo, total, d)
    dfvl = _t((a["mass"] <= 21).astype(float))
    ov1 = torch.zeros(n, dtype=F64).index_add(0, i_t[c_t], _t(model.pair("p_ovun1", cand) * model.pair("De_s", cand)) * bo[c_t])
    ov2 = torch.zeros(n, dtype=F64).index_add(0, i_t[c_t], (d[j_t[c_t]] - dfvl[i_t[c_t]] * dlpt[j_t[c_t]]) * (pi[c_t] + pp[c_t]))
    dc = d - dfvl * dlpt / (1 + g[32] * torch.exp(g[31] * ov2))
    val = _t(a["valency"])
    over = ov1 * dc / (dc + val + 1e-8) / (1 + torch.exp(_t(a["p_ovun2"]) * dc))
    under = (
        -_t(a["p_ovun5"]) * (1 - torch.exp(g[6] * dc)) / (1 + torch.exp(-_t(a["p_ovun2"]) * dc)) / (1 + g[8] * torch.exp(g[9] * ov2))
    )
    E["atom"] = torch.sum(over + under)
    allm = np.arange(len(e.i))
    vdw_type = model.ff.vdw_type
    if vdw_type in (1, 3):
        f13 = (r ** g[28] + _t((1 / model.pair("gamma_w", allm)) ** g[28])) ** (1 / g[28])
    else:
        f13 = r
    ev = torch.exp(0.5 * _t(model.pair("alpha", allm)) * (1 - f13 / _t(model.pair("r_vdW", allm))))
    E["vdw"] = 0.5 * torch.sum(taper * _t(model.pair("D", allm)) * (ev**2 - 2 * ev))
    if vdw_type in (2, 3):
        E["vdw"] = E["vdw"] + 0.5 * torch.sum(
            taper * _t(model.pair("ecore", allm)) * torch.exp(_t(model.pair("acore", allm)) * (1 - r / _t(model.pair("rcore", allm))))
        )
    E["coulomb"] = 0.5 * C_ELE * torch.sum(q[i_t] * q[j_t] * shield)
    E["qeq"] = SELF_CONVERSION * torch.sum(_t(a["chi"]) * q + 0.5 * _t(a["eta"]) * q * q)
    bo_np = bo.detach().numpy()
    keep = np.flatnonzero(bo_np > THB_CUT)  # bonded rows (src/xreac/energy.py:220)
    fcount = np.bincount(e.i[keep], minlength=n)
    fstart = np.concatenate(([0], np.cumsum(fcount)[:-1]))
    ctx = dict(vectors=vectors, r=r, bo=bo, pi=pi, pp=pp, total=total, d=d, db=db, nlp=nlp, vlpex=vlpex,
               keep=keep, fcount=fcount, fstart=fstart, bo_np=bo_np)
    _angles(model, E, ctx, lammps_forces)
    _torsions(model, E, ctx)
    _hydrogen_bonds(model, E, ctx)
    return E, q, (bo_np, total.detach().numpy(), nlp.detach().numpy()), r.detach().numpy()


def _special_corrections(model, E, bo, total, d):
    """C2 over-bond and triple-bond stabilisation (src/xreac/energy.py:231-246)."""
    a, g, e = model.a, model.g, model.e
    carbon = np.array([s.upper() == "C" for s in model.symbols])
    if g[5] > 0.001 and np.any(carbon):
        cc = np.flatnonzero(carbon[e.i] & carbon[e.j])
        if len(cc):
            c_t = torch.as_tensor(cc)
            di = d[torch.as_tensor(e.i[cc])]
            vov3 = bo[c_t] - di - 0.040 * di**4
            mask = torch.as_tensor(vov3.detach().numpy() > 3)
            E["lone_pair"] = E["lone_pair"] + torch.sum(torch.where(mask, g[5] * (vov3 - 3) ** 2, torch.zeros_like(vov3)))
    mass = a["mass"]
    co = ((mass[e.i] == 12.0) & (mass[e.j] == 15.999)) | ((mass[e.j] == 12.0) & (mass[e.i] == 15.999))
    allowed = co if int(g[37]) != 2 else np.ones(len(e.i), dtype=bool)
    sel = np.flatnonzero(allowed & (bo.detach().numpy() >= 1.0) & e.half)
    if len(sel):
        s_t = torch.as_tensor(sel)
        ii, jj = torch.as_tensor(e.i[sel]), torch.as_tensor(e.j[sel])
        b = bo[s_t]
        stab = g[10] * torch.exp(-g[7] * (b - 2.5) ** 2) / (1 + 25 * torch.exp(g[4] * (d[ii] + d[jj])))
        stab = stab * (torch.exp(-g[3] * (total[ii] - b)) + torch.exp(-g[3] * (total[jj] - b)))
        E["bond"] = E["bond"] + torch.sum(stab)


def _angles(model, E, c, lammps_forces):
    """Valence angle, penalty and angle conjugation (src/xreac/energy.py:278-318)."""
    a, g, e = model.a, model.g, model.e
    keep, fcount, fstart, bv = c["keep"], c["fcount"], c["fstart"], c["bo_np"]
    lefts, rights = [], []
    for cnt in np.unique(fcount[fcount >= 2]):
        centres = np.flatnonzero(fcount == cnt)
        p, q = np.triu_indices(cnt, 1)
        lefts.append((fstart[centres][:, None] + p[None, :]).ravel())
        rights.append((fstart[centres][:, None] + q[None, :]).ravel())
    if not lefts:
        return
    L = np.concatenate(lefts)
    R = np.concatenate(rights)
    order = np.lexsort((R, L))
    left, right = keep[L[order]], keep[R[order]]
    ok = bv[left] * bv[right] > THB_PRODUCT_CUT
    left, right = left[ok], right[ok]
    T = model.T
    key = (model.t[e.j[left]] * T + model.t[e.i[left]]) * T + model.t[e.j[right]]
    cnt = model.ang_count[key]
    rep = np.repeat(np.arange(len(left)), cnt)
    rec = model.ang_first[key][rep] + (np.arange(len(rep)) - np.repeat(np.cumsum(cnt) - cnt, cnt))
    prm = model.ang_prm[rec].reshape(-1, 7)
    ok = np.abs(prm[:, 1]) > 0.001
    left, right, prm = left[rep][ok], right[rep][ok], prm[ok]
    if not len(left):
        return
    lt, rt = torch.as_tensor(left), torch.as_tensor(right)
    it, jt, kt = torch.as_tensor(e.j[left]), torch.as_tensor(e.i[left]), torch.as_tensor(e.j[right])
    theta00, v1, v2, coa1, v7, pen1, v4 = (_t(prm[:, k]) for k in range(7))
    bo, pi, pp, total, d, db, nlp, vlpex = (c[k] for k in ("bo", "pi", "pp", "total", "d", "db", "nlp", "vlpex"))
    i_all = torch.as_tensor(e.i)
    prod = torch.exp(-torch.zeros(model.n, dtype=F64).index_add(0, i_all, bo**8))
    sum_pi = torch.zeros(model.n, dtype=F64).index_add(0, i_all, pi + pp)
    lp_term = torch.where(torch.as_tensor(vlpex.detach().numpy() >= 0), torch.zeros_like(nlp), nlp)
    sbo = sum_pi + (1 - prod) * (-db - g[33] * lp_term)
    sbo2 = torch.where(
        sbo <= 0,
        torch.zeros_like(sbo),
        torch.where(sbo <= 1, _positive_power(sbo, g[16]), torch.where(sbo < 2, 2 - _positive_power(2 - sbo, g[16]), 2 * torch.ones_like(sbo))),
    )
    theta0 = (180 - theta00 * (1 - torch.exp(-g[17] * (2 - sbo2[jt])))) * (3.14159265 / 180)
    vec, r = c["vectors"], c["r"]
    cos = torch.sum(vec[lt] * vec[rt], dim=1) / (r[lt] * r[rt])
    theta = _LammpsAngle.apply(cos) if lammps_forces else torch.arccos(torch.clamp(cos, -1 + 1e-14, 1 - 1e-14))
    bij, bjk = bo[lt] - THB_CUT, bo[rt] - THB_CUT
    pv3 = _t(a["p_val3"])[jt]
    f7 = (1 - torch.exp(-pv3 * bij**v4)) * (1 - torch.exp(-pv3 * bjk**v4))
    ex6, ex7 = torch.exp(g[14] * db[jt]), torch.exp(-v7 * db[jt])
    pv5 = _t(a["p_val5"])[jt]
    f8 = pv5 - (pv5 - 1) * (2 + ex6) / (1 + ex6 + ex7)
    exangle = torch.exp(-v2 * (theta0 - theta) ** 2)
    E["angle"] = torch.sum(f7 * f8 * v1 * torch.where(v1 >= 0, 1 - exangle, -exangle))
    ex3, ex4 = torch.exp(-g[20] * d[jt]), torch.exp(g[21] * d[jt])
    E["penalty"] = torch.sum(pen1 * (2 + ex3) / (1 + ex3 + ex4) * torch.exp(-g[19] * ((bij - 2) ** 2 + (bjk - 2) ** 2)))
    E["angle_conjugation"] = torch.sum(
        coa1
        / (1 + torch.exp(g[2] * (total[jt] - _t(a["valency_val"])[jt])))
        * torch.exp(-g[38] * ((total[it] - bij) ** 2 + (total[kt] - bjk) ** 2))
        * torch.exp(-g[30] * ((bij - 1.5) ** 2 + (bjk - 1.5) ** 2))
    )


def _torsions(model, E, c):
    """Torsion and four-body conjugation (src/xreac/energy.py:320-370)."""
    g, e = model.g, model.e
    keep, fcount, fstart, bv = c["keep"], c["fcount"], c["fstart"], c["bo_np"]
    mids = np.flatnonzero(e.half & (bv > THB_CUT))
    if not len(mids) or not len(model.tor_prm):
        return
    jm, km = e.i[mids], e.j[mids]
    nl, nr = fcount[jm], fcount[km]
    tot = nl * nr
    which = np.repeat(np.arange(len(mids)), tot)
    q = np.arange(tot.sum()) - np.repeat(np.cumsum(tot) - tot, tot)
    li, ri = q // nr[which], q % nr[which]
    left = keep[fstart[jm[which]] + li]
    right = keep[fstart[km[which]] + ri]
    middle = mids[which]
    T = model.T
    t = model.t
    key = ((t[e.j[left]] * T + t[e.i[middle]]) * T + t[e.j[middle]]) * T + t[e.j[right]]
    prm_row = model.tor[key]
    ok = (left != middle) & (prm_row >= 0) & (right != e.reverse[middle]) & (bv[left] * bv[middle] * bv[right] > THB_CUT)
    same = (e.j[left] == e.j[right]) & np.all(e.shifts[left] == e.shifts[middle] + e.shifts[right], axis=1)
    ok &= ~same
    left, middle, right, prm_row = left[ok], middle[ok], right[ok], prm_row[ok]
    if not len(left):
        return
    lt, mt, rt = (torch.as_tensor(v) for v in (left, middle, right))
    jt, kt = torch.as_tensor(e.i[middle]), torch.as_tensor(e.j[middle])
    prm = model.tor_prm[prm_row]
    v1, v2, v3, tor1, cot1 = (_t(prm[:, k]) for k in range(5))
    vec, r, bo, pi, db = c["vectors"], c["r"], c["bo"], c["pi"], c["db"]
    u, v, w = vec[lt], vec[mt], vec[rt]
    n1, n2 = torch.linalg.cross(u, v, dim=1), torch.linalg.cross(w, v, dim=1)
    area1, area2 = torch.sum(n1**2, dim=1), torch.sum(n2**2, dim=1)
    s1 = area1 / (r[lt] * r[mt]) ** 2
    s2 = area2 / (r[mt] * r[rt]) ** 2
    if np.any(s1.detach().numpy() < 1e-20) or np.any(s2.detach().numpy() < 1e-20):
        raise ValueError("Collinear atoms in an active torsion: the dihedral derivative is undefined; perturb the geometry")
    sinprod = torch.sqrt(s1 * s2)
    cw = torch.sum(n1 * n2, dim=1) / torch.sqrt(area1 * area2)
    b1, b2, b3 = bo[lt] - THB_CUT, bo[mt] - THB_CUT, bo[rt] - THB_CUT
    ds = db[jt] + db[kt]
    ex3, ex4 = torch.exp(-g[24] * ds), torch.exp(g[25] * ds)
    f11 = (2 + ex3) / (1 + ex3 + ex4)
    ex1 = torch.exp(tor1 * (2 - pi[mt] - f11) ** 2)
    fn10 = (1 - torch.exp(-g[23] * b1)) * (1 - torch.exp(-g[23] * b2)) * (1 - torch.exp(-g[23] * b3))
    cv = 0.5 * (v1 * (1 + cw) + v2 * ex1 * (2 - 2 * cw * cw) + v3 * (1 + 4 * cw**3 - 3 * cw))
    E["torsion"] = torch.sum(fn10 * sinprod * cv)
    fn12 = torch.exp(-g[27] * ((b1 - 1.5) ** 2 + (b2 - 1.5) ** 2 + (b3 - 1.5) ** 2))
    E["conjugation"] = torch.sum(cot1 * fn12 * (1 + (cw * cw - 1) * sinprod))


def _hydrogen_bonds(model, E, c):
    """Hydrogen bonds, ordered by H, donor edge, acceptor edge (src/xreac/energy.py:248-276)."""
    a, g, e = model.a, model.g, model.e
    roles = a["p_hbond"].astype(int)
    bv, rv = c["bo_np"], c["r"].detach().numpy()
    hs = np.flatnonzero(roles == 1)
    if not len(hs) or not len(model.hb_prm):
        return
    rows = np.concatenate([np.arange(e.starts[h], e.starts[h] + e.counts[h]) for h in hs]) if len(hs) else np.zeros(0, int)
    heavy = rows[roles[e.j[rows]] == 2]
    donors = heavy[bv[heavy] >= HBOND_THRESHOLD]
    accs = heavy[rv[heavy] <= min(HBOND_CUT, g[12])]
    hd, ha = e.i[donors], e.i[accs]
    # All donor/acceptor edge pairs of the same H, in (H, donor, acceptor) order.
    order_a = np.argsort(ha, kind="stable")
    accs, ha = accs[order_a], ha[order_a]
    a_start = np.searchsorted(ha, hd, side="left")
    a_end = np.searchsorted(ha, hd, side="right")
    cnt = a_end - a_start
    dd = np.repeat(donors, cnt)
    aa = accs[np.repeat(a_start, cnt) + (np.arange(cnt.sum()) - np.repeat(np.cumsum(cnt) - cnt, cnt))]
    ok = dd != aa
    dd, aa = dd[ok], aa[ok]
    T, t = model.T, model.t
    key = (t[e.j[dd]] * T + t[e.i[dd]]) * T + t[e.j[aa]]
    row = model.hb[key]
    ok = row >= 0
    dd, aa, row = dd[ok], aa[ok], row[ok]
    prm = model.hb_prm[row]
    ok = prm[:, 0] > 0
    dd, aa, prm = dd[ok], aa[ok], prm[ok]
    if not len(dd):
        return
    dt, at = torch.as_tensor(dd), torch.as_tensor(aa)
    r0, hb1, hb2, hb3 = (_t(prm[:, k]) for k in range(4))
    vec, r, bo = c["vectors"], c["r"], c["bo"]
    dist = r[at]
    cos = torch.sum(vec[dt] * vec[at], dim=1) / (r[dt] * dist)
    sin4 = 0.25 * (1 - torch.clamp(cos, -1.0, 1.0)) ** 2
    E["hydrogen_bond"] = torch.sum(hb1 * (1 - torch.exp(-hb2 * bo[dt])) * torch.exp(-hb3 * (r0 / dist + dist / r0 - 2)) * sin4)


# --------------------------------------------------------------------------- driver
def evaluate(ff, symbols, positions, *, total_charge=0, cell=None, pbc=None, full_derivative=False,
             neighbors=None, max_expanded_atoms=512, dense_bond_orders=True, need_forces=True):
    """Energy, components, charges, forces and properties of one system.

    Returns a dict with the fields of xreac's ``Evaluation``
    (src/xreac/calculator.py:15-33) plus internals used by parity tests:
    ``neighbors`` (canonical i, j, S), per-edge ``bo``/``sigma``/``pi``/``pp``.
    """
    symbols = tuple(symbols)
    if not symbols or any(not isinstance(s, str) or not s for s in symbols):
        raise ValueError("A nonempty sequence of parameter-file atom labels is required")
    if isinstance(total_charge, (bool, np.bool_)) or not isinstance(total_charge, Real) or not np.isfinite(total_charge):
        raise ValueError("total_charge must be a finite real scalar")
    x = np.array(positions, dtype=np.float64, copy=True)
    if x.shape != (len(symbols), 3) or not np.isfinite(x).all():
        raise ValueError("positions must be a finite (N, 3) array in Angstrom")
    flags, m = boundary(cell, pbc)
    ff.validate_model(symbols)
    n = len(symbols)
    cutoff = float(ff.general[12])
    if neighbors is None:
        reps = repetitions(cutoff, flags, m, n, max_expanded_atoms)
        i, j, s = neighbor_list(x, cutoff, cell, pbc)
        edges = Edges.from_sorted(i, j, s, n, m)
        backend = "replicated"
    else:
        reps = (1, 1, 1)
        edges = Edges(neighbors, n, flags, m)
        backend = "provided"
    model = _Model(ff, symbols, edges)
    v = x[edges.j] - x[edges.i] + edges.offsets
    r0 = np.sqrt(np.sum(v * v, axis=1))
    if np.any(r0 < 1e-6):
        raise ValueError("Coincident atoms are not supported")
    q_fixed = None if full_derivative else qeq_charges(model, r0, total_charge)
    xt = torch.tensor(x, dtype=F64, requires_grad=need_forces)
    E, q, bond_state, _ = _components(model, xt, q_fixed, total_charge, lammps_forces=not full_derivative)
    comps = torch.stack([E[k] for k in COMPONENTS])
    total = comps.sum()
    if need_forces:
        (grad,) = torch.autograd.grad(total, xt, allow_unused=True)
        forces = -(grad.numpy() if grad is not None else np.zeros_like(x))
    else:
        forces = None
    charges = q.detach().numpy().copy()
    comps_np = comps.detach().numpy()
    if not (np.isfinite(comps_np).all() and np.isfinite(charges).all() and (forces is None or np.isfinite(forces).all())):
        raise ValueError("Non-finite energy, charges, or forces; check the geometry")
    if abs(charges.sum() - total_charge) > 1e-8:
        raise ValueError("QEq charge constraint failed")
    bo, tbo, nlp = bond_state
    mass = model.a["mass"]
    centre = np.sum(x * mass[:, None], axis=0) / np.sum(mass)
    out = dict(
        energy=float(comps_np.sum()),
        forces=forces,
        charges=charges,
        components=dict(zip(COMPONENTS, map(float, comps_np))),
        full_derivative=full_derivative,
        total_bond_orders=tbo,
        lone_pairs=nlp,
        bond_counts=np.bincount(edges.i, weights=(bo > BOND_GRAPH_CUT).astype(float), minlength=n).astype(float).astype(int),
        dipole=np.sum((x - centre) * charges[:, None], axis=0),
        cell_repetitions=reps,
        neighbor_backend=backend,
        neighbors=(edges.i, edges.j, edges.shifts),
        edge_bo=bo,
    )
    if dense_bond_orders:
        out["bond_orders"] = np.bincount(edges.i * n + edges.j, weights=bo, minlength=n * n).astype(float).reshape(n, n)
    return out
