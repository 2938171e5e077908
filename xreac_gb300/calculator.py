"""Device-backed ``Calculator`` / ``Evaluation``: a drop-in for xreac's public evaluation API.

Mirrors src/xreac/calculator.py:15-165: ``Calculator(force_field, *, max_expanded_atoms=512)``
and ``Calculator.evaluate(symbols, positions, *, total_charge=0, cell=None, pbc=None,
full_derivative=False, neighbors=None)`` returning an ``Evaluation`` with the same fields and
units (energy and 14 components in kcal/mol, forces in kcal/mol/A, QEq charges in e, bond orders).
Invalid input raises ``ValueError`` with xreac's messages. The computation itself runs in the
CUDA library (include/xreac_gb300.h); there is no CPU path.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _native as nat
from .geometry import cell_repetitions, validate_expansion_limit, validate_input

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

_ERRORS = {
    nat.XR_ECOINCIDENT: "Coincident atoms are not supported",
    nat.XR_ESINGULAR: "Singular QEq system; check the geometry and parameters",
    nat.XR_ENONFINITE: "Non-finite energy, charges, or forces; check the geometry",
    nat.XR_ECHARGE: "QEq charge constraint failed",
}


@dataclass(frozen=True)
class Evaluation:
    """Result fields of xreac's ``Evaluation`` (src/xreac/calculator.py:15-33).

    ``bond_orders`` is the dense (N, N) matrix summed over images; it is assembled from the
    sparse per-bond list on first access, so large systems pay for it only when asked.
    """

    energy: float
    forces: np.ndarray
    charges: np.ndarray
    components: dict
    full_derivative: bool
    total_bond_orders: np.ndarray
    lone_pairs: np.ndarray
    bond_counts: np.ndarray
    dipole: np.ndarray
    cell_repetitions: tuple = (1, 1, 1)
    neighbor_backend: str = "replicated"
    bonds: tuple = field(default=None, repr=False, compare=False)  # (i, j, S, bo) per bond-order candidate

    @property
    def force_convention(self):
        """Name of the derivative used for ``forces``."""
        return "charge_response" if self.full_derivative else "fixed_charge"

    @property
    def bond_orders(self):
        n = len(self.charges)
        i, j, _, bo = self.bonds
        dense = np.zeros((n, n))
        np.add.at(dense, (i, j), bo)
        np.add.at(dense, (j, i), bo)
        return dense


def _guess(initial_charges, n):
    if initial_charges is None:
        return None
    g = np.ascontiguousarray(initial_charges, dtype=np.float64)
    if g.shape != (n,) or not np.isfinite(g).all():
        raise ValueError("initial_charges must be a finite array with one charge per atom")
    return g


def _is_carbon(ff):
    return np.array([s.upper() == "C" for s in ff.elements], dtype=np.int32)


class Calculator:
    """GB300 ReaxFF calculator with xreac's constructor and ``evaluate`` signature."""

    def __init__(self, force_field, *, max_expanded_atoms=512, device=0):
        force_field.validate_model()
        validate_expansion_limit(max_expanded_atoms)
        self.force_field = force_field
        self.max_expanded_atoms = max_expanded_atoms
        self._ff = nat.ForceFieldHandle(force_field.tables(), _is_carbon(force_field), force_field.vdw_type)
        self._ctx = nat.Context(device)
        self._lib = nat.load()

    def set_qeq(self, tolerance=1e-13, max_iterations=2000):
        """QEq solver tolerance and iteration limit.

        ``tolerance`` bounds the preconditioned projected residual relative to its value at the
        uniform start q = Q/n (also for warm starts from ``initial_charges``). The default 1e-13
        keeps charges within about 1e-12 e of the exact KKT solution, which holds fixed-charge
        forces of ionic systems (Ti/O) within 2e-8 kcal/mol/A of the reference.
        """
        if self._lib.xr_ctx_set_qeq(self._ctx.handle, float(tolerance), int(max_iterations)) != nat.XR_OK:
            raise ValueError("QEq tolerance must be positive and the iteration limit at least 1")

    def reserve(self, atoms, systems=1, edges_per_atom=450, bonds_per_atom=30):
        """Pre-size the device buffers for batches of up to ``atoms`` atoms in ``systems`` systems.

        Buffers otherwise grow on demand, and a growth reallocates device memory, which
        synchronises the whole device (a stall for every other stream, e.g. other server workers).
        ``edges_per_atom`` bounds the directed neighbours within the cutoff per atom (about 420 at
        liquid water density with a 10 A cutoff); ``bonds_per_atom`` the bond candidates within 5 A.
        """
        code = self._lib.xr_ctx_reserve(self._ctx.handle, int(atoms), int(systems), int(atoms * edges_per_atom),
                                        int(atoms * bonds_per_atom))
        if code != nat.XR_OK:
            raise RuntimeError(self._ctx.last_error())

    def _prepare(self, symbols, positions, total_charge, cell, pbc, full_derivative):
        if not isinstance(full_derivative, bool):
            raise ValueError("full_derivative must be a boolean")
        symbols, x, flags, m = validate_input(symbols, positions, total_charge, cell, pbc)
        ff = self.force_field
        ff.validate_model(symbols)
        reps = cell_repetitions(float(ff.general[12]), flags, m, len(symbols), self.max_expanded_atoms)
        types = np.ascontiguousarray(ff.type_indices(symbols))
        cellm = None if m is None else np.ascontiguousarray(m, dtype=np.float64)
        return symbols, np.ascontiguousarray(x), types, flags, cellm, reps

    def _raise(self, code):
        if code in _ERRORS:
            raise ValueError(_ERRORS[code])
        msg = self._ctx.last_error()
        if code in (nat.XR_ECUDA,):
            raise RuntimeError(msg)
        raise ValueError(msg)

    def evaluate(self, symbols, positions, *, total_charge=0, cell=None, pbc=None, full_derivative=False,
                 neighbors=None, initial_charges=None):
        """Energy, QEq charges and fixed-charge forces of one system (src/xreac/calculator.py:76-165).

        ``initial_charges`` (an extension; xreac has no such argument) starts the QEq solve from
        given charges, e.g. those of the previous step of a relaxation or MD run. The result meets
        the same tolerance; only the iteration count changes.
        """
        symbols, x, types, flags, cellm, reps = self._prepare(symbols, positions, total_charge, cell, pbc,
                                                              full_derivative)
        backend = "replicated"
        if neighbors is not None:
            from .neighbors import check_supplied

            check_supplied(neighbors, len(symbols), flags)
            reps, backend = (1, 1, 1), "provided"
        guess = _guess(initial_charges, len(symbols))
        return self._run([(types, x, flags, cellm, float(total_charge), guess)], full_derivative, [reps], backend)[0]

    def evaluate_many(self, systems, *, full_derivative=False):
        """Evaluate independent systems in one ragged device batch.

        ``systems`` is a sequence of dicts with the keyword arguments of :meth:`evaluate`
        (``symbols``, ``positions`` and optionally ``total_charge``, ``cell``, ``pbc``,
        ``initial_charges``). Returns a list of :class:`Evaluation` in the same order.
        """
        batch, reps = [], []
        for s in systems:
            sym, x, types, flags, cellm, rp = self._prepare(s["symbols"], s["positions"], s.get("total_charge", 0),
                                                            s.get("cell"), s.get("pbc"), full_derivative)
            guess = _guess(s.get("initial_charges"), len(sym))
            batch.append((types, x, flags, cellm, float(s.get("total_charge", 0)), guess))
            reps.append(rp)
        return self._run(batch, full_derivative, reps, "replicated")

    def _run(self, batch, full_derivative, reps, backend):
        lib = self._lib
        n_sys = len(batch)
        sizes = [len(b[0]) for b in batch]
        total = sum(sizes)
        # one allocation per kind for the whole batch; each Evaluation gets views
        energy = np.zeros((n_sys, 15))
        dipole = np.zeros((n_sys, 3))
        forces = np.zeros((total, 3))
        per_atom = np.zeros((3, total))  # charges, total bond orders, lone pairs
        counts = np.zeros(total, dtype=np.int32)
        sys_arr = (nat.System * n_sys)()
        res_arr = (nat.Result * n_sys)()
        offsets = np.concatenate(([0], np.cumsum(sizes))).astype(int)
        keep = []
        for k, (types, x, flags, cellm, q, guess) in enumerate(batch):
            a0 = offsets[k]
            keep.append((types, x, cellm, guess))
            s = sys_arr[k]
            s.natoms = sizes[k]
            s.types = nat.ptr(types, nat.c_int)
            s.positions = nat.ptr(x, nat.c_double)
            s.cell = nat.ptr(cellm, nat.c_double) if cellm is not None else None
            for d in range(3):
                s.pbc[d] = int(flags[d])
            s.total_charge = q
            s.charges_guess = nat.ptr(guess, nat.c_double)
            r = res_arr[k]
            r.energy = nat.ptr(energy[k], nat.c_double)
            r.forces = nat.ptr(forces[a0:], nat.c_double)
            r.charges = nat.ptr(per_atom[0, a0:], nat.c_double)
            r.total_bond_orders = nat.ptr(per_atom[1, a0:], nat.c_double)
            r.lone_pairs = nat.ptr(per_atom[2, a0:], nat.c_double)
            r.bond_counts = nat.ptr(counts[a0:], nat.c_int)
            r.dipole = nat.ptr(dipole[k], nat.c_double)
        flags_ = nat.XR_FLAG_FULL_DERIVATIVE if full_derivative else 0
        code = lib.xr_eval_batch(self._ctx.handle, self._ff.handle, n_sys, sys_arr, flags_, res_arr)
        if code != nat.XR_OK:
            self._raise(code)
        counts64 = counts.astype(int)
        results = []
        for k in range(n_sys):
            a0, a1 = offsets[k], offsets[k + 1]
            e = energy[k]
            results.append(
                Evaluation(
                    energy=float(e[14]),
                    forces=forces[a0:a1],
                    charges=per_atom[0, a0:a1],
                    components=dict(zip(COMPONENTS, e[:14].tolist())),
                    full_derivative=full_derivative,
                    total_bond_orders=per_atom[1, a0:a1],
                    lone_pairs=per_atom[2, a0:a1],
                    bond_counts=counts64[a0:a1],
                    dipole=dipole[k],
                    cell_repetitions=reps[k],
                    neighbor_backend=backend,
                    bonds=self._bonds(k),
                )
            )
        return results

    def _bonds(self, index):
        lib, h = self._lib, self._ctx.handle
        count = nat.c_longlong()
        lib.xr_get_bonds(h, index, None, None, None, None, 0, nat.byref(count))
        m = count.value
        i = np.zeros(m, dtype=np.int32)
        j = np.zeros(m, dtype=np.int32)
        S = np.zeros((m, 3), dtype=np.int32)
        bo = np.zeros(m)
        lib.xr_get_bonds(h, index, nat.ptr(i, nat.c_int), nat.ptr(j, nat.c_int), nat.ptr(S, nat.c_int),
                         nat.ptr(bo, nat.c_double), m, nat.byref(count))
        return i, j, S, bo

    def neighbor_list(self, index=0):
        """Canonical directed neighbour list ``(i, j, S)`` of the last evaluation (system ``index``)."""
        lib, h = self._lib, self._ctx.handle
        count = nat.c_longlong()
        lib.xr_get_neighbors(h, index, None, None, None, 0, nat.byref(count))
        m = count.value
        i = np.zeros(m, dtype=np.int32)
        j = np.zeros(m, dtype=np.int32)
        S = np.zeros((m, 3), dtype=np.int32)
        lib.xr_get_neighbors(h, index, nat.ptr(i, nat.c_int), nat.ptr(j, nat.c_int), nat.ptr(S, nat.c_int), m,
                             nat.byref(count))
        return i, j, S

    @property
    def last_launches(self):
        return int(self._lib.xr_last_launches(self._ctx.handle))
