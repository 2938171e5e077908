"""Device-backed ``Calculator`` / ``Evaluation``: a drop-in for xreac's public evaluation API.

Mirrors src/xreac/calculator.py:15-165: ``Calculator(force_field, *, max_expanded_atoms=512)``
and ``Calculator.evaluate(symbols, positions, *, total_charge=0, cell=None, pbc=None,
full_derivative=False, neighbors=None)`` returning an ``Evaluation`` with the same fields and
units (energy and 14 components in kcal/mol, forces in kcal/mol/A, QEq charges in e, bond orders).
Invalid input raises ``ValueError`` with xreac's messages. The computation itself runs in the
CUDA library (include/xreac_gb300.h); there is no CPU path.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from numbers import Real
from typing import NamedTuple

import numpy as np

from . import _native as nat
from .geometry import (boundary, cell_repetitions, periodic_cell, validate_expansion_limit, validate_input,
                       validate_total_charge)

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

try:  # the host-side batch packing module (built with the CUDA library; optional)
    from ._lib import _xr_host as _host
except ImportError:
    _host = None

_NO_PBC = np.zeros(3, dtype=bool)
_NO_PBC.flags.writeable = False
_SYSTEM_DTYPE = np.dtype(nat.System)
_RESULT_DTYPE = np.dtype(nat.Result)
_SYSTEM_P = nat.POINTER(nat.System)
_RESULT_P = nat.POINTER(nat.Result)

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

    def __getattr__(self, name):
        # Only reached for a field that is not set yet: an evaluation of a batch makes its array
        # fields (views of the batch's result arrays) on first access.
        batch = self.__dict__.get("_batch")
        if batch is None or name not in _BATCH_FIELDS:
            raise AttributeError(name)
        value = batch.field(name, self.__dict__["_index"])
        object.__setattr__(self, name, value)
        return value

    @property
    def bond_orders(self):
        n = len(self.charges)
        i, j, _, bo = self.bonds
        dense = np.zeros((n, n))
        np.add.at(dense, (i, j), bo)
        np.add.at(dense, (j, i), bo)
        return dense


# A batch's evaluations make these fields on first access. ``bonds`` has a default in the dataclass;
# its class attribute is removed below (the default stays in ``__init__``) so that the lookup of a
# missing value reaches ``__getattr__``.
# Skin of the device neighbour list during a native relaxation (A), ASE's default.
RELAX_SKIN = 0.3

_BATCH_FIELDS = frozenset(("forces", "charges", "components", "total_bond_orders", "lone_pairs", "bond_counts",
                           "dipole", "bonds"))
del Evaluation.bonds


class _BatchResults:
    """The result arrays of one ``xr_eval_batch`` call; the fields of its k-th system are views."""

    __slots__ = ("energy", "forces", "per_atom", "counts", "dipole", "offsets", "bonds", "cut")

    def __init__(self, energy, forces, per_atom, counts, dipole, offsets, bonds, cut):
        self.energy, self.forces, self.per_atom, self.counts = energy, forces, per_atom, counts
        self.dipole, self.offsets, self.bonds, self.cut = dipole, offsets, bonds, cut

    def field(self, name, k):
        a0, a1 = self.offsets[k], self.offsets[k + 1]
        if name == "forces":
            return self.forces[a0:a1]
        if name == "charges":
            return self.per_atom[0, a0:a1]
        if name == "total_bond_orders":
            return self.per_atom[1, a0:a1]
        if name == "lone_pairs":
            return self.per_atom[2, a0:a1]
        if name == "bond_counts":
            return self.counts[a0:a1].astype(np.int64)
        if name == "dipole":
            return self.dipole[k]
        if name == "bonds":
            c0, c1 = self.cut[k], self.cut[k + 1]
            return tuple(a[c0:c1] for a in self.bonds)
        return dict(zip(COMPONENTS, self.energy[k, :14].tolist()))  # components


# Pair-table columns (xreac_gb300.forcefield.PAIR_COLUMNS order) with a parameter gradient, and the
# angle record entries (src/xreac/forcefield.py angle block order).
GRADIENT_PAIR_COLUMNS = ("De_s", "De_p", "De_pp", "p_be1", "p_be2", "p_ovun1", "p_bo1", "p_bo2", "p_bo3", "p_bo4",
                         "p_bo5", "p_bo6", "r_s", "r_p", "r_pp", "D", "alpha", "gamma_w", "r_vdW", "rcore", "ecore",
                         "acore")
ANGLE_PARAMETERS = ("theta_00", "p_val1", "p_val2", "p_coa1", "p_val7", "p_pen1", "p_val4")
# QEq parameters with a gradient (through the adjoint QEq solve): atom-table and pair-table columns.
QEQ_ATOM_COLUMNS = ("chi", "eta")
QEQ_PAIR_COLUMNS = ("gamma",)


@dataclass
class Relaxation:
    """Result of :meth:`Calculator.relax` (src/xreac/calculator.py:37-42): final positions, the
    evaluation at them, whether the force tolerance was reached, iterations taken, a message."""

    positions: np.ndarray
    evaluation: Evaluation
    converged: bool
    iterations: int
    message: str


@dataclass(frozen=True)
class ParameterGradient:
    """dE/dtheta keyed like ``ForceField.pairs`` and ``ForceField.angles``.

    ``pairs[(s, t)][name]`` and ``angles[(a, b, c)][record][k]`` (k in ``ANGLE_PARAMETERS`` order).
    A parameter the force field stores once for several keys (a pair's two orders, an angle's two
    ends) appears under each of them with the summed gradient of all its table rows, i.e. the
    derivative with respect to that single stored value. With the QEq parameters (``qeq=True``),
    ``atoms[s]["chi"]``, ``atoms[s]["eta"]`` and ``pairs[(s, t)]["gamma"]`` (the pair table's shielding
    parameter) hold their total derivatives, charges' response included.
    """

    pairs: dict
    angles: dict
    atoms: dict = field(default_factory=dict)

    @classmethod
    def from_rows(cls, ff, pair_rows, angle_rows, angle_keys, atom_rows=None):
        from .forcefield import ATOM_COLUMNS, PAIR_COLUMNS

        names = ff.elements
        T = len(names)
        pair_names = GRADIENT_PAIR_COLUMNS + (QEQ_PAIR_COLUMNS if atom_rows is not None else ())
        cols = [PAIR_COLUMNS.index(c) for c in pair_names]
        by_obj = {}
        for si, s in enumerate(names):
            for ti, t in enumerate(names):
                key = (s, t)
                if key not in ff.pairs:
                    continue
                by_obj.setdefault(id(ff.pairs[key]), [np.zeros(len(cols)), []])
                acc = by_obj[id(ff.pairs[key])]
                acc[0] += pair_rows[si * T + ti, cols]
                acc[1].append(key)
        pairs = {}
        for vec, keys in by_obj.values():
            d = dict(zip(pair_names, map(float, vec)))
            for key in keys:
                pairs[key] = d
        rec = {}
        for row, (key, q) in enumerate(angle_keys):
            obj = id(ff.angles[key][q])
            rec.setdefault(obj, np.zeros(7))
            rec[obj] += angle_rows[row]
        angles = {}
        for key, records in ff.angles.items():
            angles[key] = [rec.get(id(r), np.zeros(7)).copy() for r in records]
        atoms = {}
        if atom_rows is not None:
            acols = [ATOM_COLUMNS.index(c) for c in QEQ_ATOM_COLUMNS]
            for k, s_ in enumerate(names):
                atoms[s_] = dict(zip(QEQ_ATOM_COLUMNS, map(float, atom_rows[k, acols])))
        return cls(pairs, angles, atoms)


class _GuessAddresses(NamedTuple):
    """Initial charges of a packed batch: one address per system (0: none) and the converted arrays
    that some of them point into (held until the call returns)."""

    addr: np.ndarray
    keep: list


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
        self._type_pos = {s: k for k, s in enumerate(force_field.elements) if isinstance(s, str) and s}
        self._angle_rows = force_field.angle_row_keys()
        # When every labelled element passes the model checks together, so does every subset of them
        # (the checks are per element and per pair), and requests need no per-call check.
        try:
            force_field.validate_model(tuple(self._type_pos))
            self._all_valid = True
        except (ValueError, KeyError):
            self._all_valid = False

    def update_force_field(self, force_field):
        """Evaluate with another parameter set of the same force field from now on (an extension).

        ``force_field`` must have the same elements and parameter records as the current one
        (e.g. a copy with perturbed or fitted values); its tables are written into the device
        tables in place (``xr_ff_update``), so the device context, its buffers and any kept
        neighbour list stay as they are.
        """
        if tuple(force_field.elements) != tuple(self.force_field.elements):
            raise ValueError("an updated force field must have the same elements and parameter records")
        force_field.validate_model()
        if force_field.angle_row_keys() != self._angle_rows:
            raise ValueError("an updated force field must have the same elements and parameter records")
        self._ff.update(force_field.tables(), _is_carbon(force_field), force_field.vdw_type)
        self.force_field = force_field
        self._base_tables = None

    # ------------------------------------------------------------------ parameter sets
    @property
    def parameter_set_count(self):
        """Parameter sets on the device: 1 (the calculator's force field) plus those loaded."""
        return self._ff.nsets

    def _tables0(self):
        t = getattr(self, "_base_tables", None)
        if t is None:
            t = self._base_tables = self.force_field.tables()
        return t

    def load_parameter_sets(self, force_fields):
        """Load variants of the force field as parameter sets 1 .. len(force_fields) (an extension;
        xreac evaluates one force field per call). Each must have the calculator's elements, general
        parameters and parameter records; its atom, pair, angle, torsion and hydrogen-bond values
        may differ. Set 0 stays the calculator's own force field. ``evaluate_many`` and
        ``parameter_gradient_many`` then take ``parameter_sets=[...]``, one set per system, and
        evaluate every system with its own set in one device batch."""
        force_fields = list(force_fields)
        base = self._tables0()
        stacks = {k: [] for k in ("atom", "pair", "angle", "torsion", "hbond")}
        for ff in force_fields:
            if tuple(ff.elements) != tuple(self.force_field.elements):
                raise ValueError("parameter sets must have the calculator's elements and parameter records")
            ff.validate_model()
            t = ff.tables()
            if not np.array_equal(np.asarray(t["general"]), np.asarray(base["general"])):
                raise ValueError("parameter sets share the general parameters of the calculator's force field")
            for k in ("angle_index", "torsion_index", "hbond_index"):
                if not np.array_equal(t[k], base[k]):
                    raise ValueError("parameter sets must have the calculator's elements and parameter records")
            for k in stacks:
                stacks[k].append(t[k])
        self.load_parameter_tables(**{k: (np.stack(v) if v else None) for k, v in stacks.items()},
                                   count=len(force_fields))

    def load_parameter_tables(self, atom=None, pair=None, angle=None, torsion=None, hbond=None, *, count=None):
        """``load_parameter_sets`` from stacked tables: each argument None (every set takes the
        calculator's own values for it) or an array of ``count`` tables in the shapes of
        ``ForceField.tables()``; the values are used as given. Replaces any sets loaded before."""
        given = [a for a in (atom, pair, angle, torsion, hbond) if a is not None]
        if count is None:
            if not given:
                raise ValueError("the number of parameter sets is required when no table is given")
            count = len(given[0])
        count = int(count)
        if count < 0 or count + 1 > nat.XR_MAX_PARAMETER_SETS:
            raise ValueError(f"between 0 and {nat.XR_MAX_PARAMETER_SETS - 1} parameter sets can be loaded")
        self._ff.set_count(count + 1)
        if count:
            self._ff.update_sets(1, count, atom=atom, pair=pair, angle=angle, torsion=torsion, hbond=hbond)

    def _sets(self, parameter_sets, n_sys):
        if parameter_sets is None:
            return None
        sets = np.ascontiguousarray(parameter_sets, dtype=np.int32)
        if sets.shape != (n_sys,):
            raise ValueError("parameter_sets must give one parameter set per system")
        if len(sets) and (sets.min() < 0 or sets.max() >= self._ff.nsets):
            raise ValueError("parameter set index out of range")
        return sets

    def set_qeq(self, tolerance=1e-13, max_iterations=2000):
        """QEq solver tolerance and iteration limit.

        ``tolerance`` bounds the preconditioned projected residual relative to its value at the
        uniform start q = Q/n (also for warm starts from ``initial_charges``). The default 1e-13
        keeps charges within about 1e-12 e of the exact KKT solution, which holds fixed-charge
        forces of ionic systems (Ti/O) within 2e-8 kcal/mol/A of the reference.
        """
        if self._lib.xr_ctx_set_qeq(self._ctx.handle, float(tolerance), int(max_iterations)) != nat.XR_OK:
            raise ValueError("QEq tolerance must be positive and the iteration limit at least 1")

    def set_neighbor_skin(self, skin):
        """Reuse the device neighbour list across calls (``xr_ctx_set_skin``), ASE's skin rule.

        With ``skin`` > 0 (A) each call keeps a list of every image within cutoff + 2 skin on the
        device, and a later call on the same systems (atom counts, labels, cell, pbc) reuses it while
        no atom has moved more than ``skin`` from where it was at the build. The edges within the
        cutoff are re-selected from it by exact distance tests each call, so results equal those of
        a fresh list. 0 (the default) scans every call.
        """
        if isinstance(skin, bool) or not isinstance(skin, Real) or not math.isfinite(skin) or skin < 0:
            raise ValueError("neighbor_skin must be a finite nonnegative number")
        if self._lib.xr_ctx_set_skin(self._ctx.handle, float(skin)) != nat.XR_OK:
            raise ValueError("neighbor_skin must be a finite nonnegative number")
        self._skin = float(skin)

    @property
    def neighbor_skin(self):
        return getattr(self, "_skin", 0.0)

    def list_info(self):
        """(how the last call got its neighbour rows: "scan", "built", "reused", "supplied", "cells"
        (a cell-list search) or "built-cells" (a skin list built from the cell list), skin lists built
        so far)."""
        mode = nat.c_int()
        builds = nat.c_longlong()
        self._lib.xr_last_list_info(self._ctx.handle, nat.byref(mode), nat.byref(builds))
        return ("scan", "built", "reused", "supplied", "cells", "built-cells")[mode.value], int(builds.value)

    def set_graphs(self, enabled=True):
        """CUDA graphs for repeated launch sequences (``xr_ctx_set_graphs``, an extension; on by
        default): the second call with given system sizes and settings records its kernels as a
        graph, and later such calls replay it (the 128 most recently used graphs are kept)."""
        self._lib.xr_ctx_set_graphs(self._ctx.handle, 1 if enabled else 0)

    @property
    def last_graph(self):
        """How the last call launched its kernels after the neighbour count: "direct", "recorded"
        or "replayed"."""
        return ("direct", "recorded", "replayed")[self._lib.xr_last_graph(self._ctx.handle)]

    def set_cell_list(self, enabled=None):
        """Neighbour search by cell list (``xr_ctx_set_cell_list``, an extension): None chooses per
        call (large systems where it halves the image tests), True always, False never. The list and
        the results are the same either way."""
        mode = 0 if enabled is None else (1 if enabled else -1)
        if enabled is not None and not isinstance(enabled, bool):
            raise ValueError("enabled must be None, True or False")
        self._lib.xr_ctx_set_cell_list(self._ctx.handle, mode)

    def set_wait_test(self, polls=0, fail_at=0):
        """For tests of the QEq solver's failure path (``xr_ctx_set_wait_test``): ``polls`` > 0
        replaces the poll limits of the bounded team waits, and ``fail_at`` > 0 makes team wait number
        ``fail_at`` of every solve wait for an arrival that never comes, so the call raises
        ``RuntimeError`` while the context stays usable. ``set_wait_test()`` restores the defaults."""
        if self._lib.xr_ctx_set_wait_test(self._ctx.handle, int(polls), int(fail_at)) != nat.XR_OK:
            raise ValueError("polls and fail_at must be non-negative")

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

    def _prepare(self, symbols, positions, total_charge, cell, pbc, full_derivative, replicate=True):
        """Validated ``(symbols, positions, types, pbc flags, cell or None, repetitions)``.

        The positions are float64 and C-contiguous, but not copied when they already are, and not
        yet checked for finite values: ``_run`` checks the whole batch at once. ``replicate=False``
        (a caller-supplied list) skips xreac's small-cell replication count and its
        ``max_expanded_atoms`` limit, as xreac does when it is given neighbours, and reports
        (1, 1, 1).
        """
        if full_derivative is not True and full_derivative is not False:
            raise ValueError("full_derivative must be a boolean")
        ff = self.force_field
        symbols = tuple(symbols)
        # Fast path: every label maps to an element of the force field (str keys only, so a
        # non-string or empty label falls through to the full validation and its message).
        try:
            types = np.fromiter(map(self._type_pos.__getitem__, symbols), dtype=np.int32, count=len(symbols))
        except (KeyError, TypeError):
            types = None
        if types is None or not symbols:
            symbols, x, flags, m = validate_input(symbols, positions, total_charge, cell, pbc)
            ff.validate_model(symbols)
            types = ff.type_indices(symbols)
        else:
            if type(total_charge) not in (int, float) or not math.isfinite(total_charge):
                validate_total_charge(total_charge)
            x = np.ascontiguousarray(positions, dtype=np.float64)
            if x.shape != (len(symbols), 3):
                raise ValueError("positions must be a finite (N, 3) array in Angstrom")
            if (pbc is None and cell is None) or pbc is False:
                flags, m = _NO_PBC, None
            else:
                limit = self.max_expanded_atoms if replicate else 1 << 62
                fast = periodic_cell(cell, pbc, float(ff.general[12]), len(symbols), limit)
                if fast is not None:
                    if not self._all_valid:
                        ff.validate_model(symbols)
                    return symbols, x, types, fast[0], fast[1], fast[2] if replicate else (1, 1, 1)
                flags, m = boundary(cell, pbc)
            if not self._all_valid:
                ff.validate_model(symbols)
        if m is None:
            return symbols, x, types, flags, None, (1, 1, 1)
        reps = (cell_repetitions(float(ff.general[12]), flags, m, len(symbols), self.max_expanded_atoms) if replicate
                else (1, 1, 1))
        return symbols, x, types, flags, np.ascontiguousarray(m, dtype=np.float64), reps

    def _raise(self, code):
        if code in _ERRORS:
            raise ValueError(_ERRORS[code])
        msg = self._ctx.last_error()
        if code in (nat.XR_ECUDA, nat.XR_EWAIT):
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
                                                              full_derivative, replicate=neighbors is None)
        guess = _guess(initial_charges, len(symbols))
        if neighbors is not None:
            from .neighbors import supplied_arrays

            # exactly the caller's edges (their validation, canonical order and reduction to the
            # cutoff run in the library: xr_eval_neighbors)
            i, j, shifts = supplied_arrays(neighbors, len(symbols))
            nb = nat.Neighbors(len(i), nat.addr(i), nat.addr(j), nat.addr(shifts))
            return self._run([(types, x, flags, cellm, float(total_charge), guess)], full_derivative, [(1, 1, 1)],
                             "provided", supplied=nb)[0]
        return self._run_one(types, x, flags, cellm, float(total_charge), guess, full_derivative, reps, "replicated")

    def _evaluate_backend(self, symbols, positions, *, total_charge=0, cell=None, pbc=None, full_derivative=False,
                          backend="replicated"):
        """``evaluate`` for the ASE adapter. ``backend="ase"`` evaluates as xreac does with ASE's image
        lists: no small-cell replication count or ``max_expanded_atoms`` limit, ``cell_repetitions``
        (1, 1, 1) and the result labelled "ase"; the device list (and its skin reuse) is the same."""
        if backend != "ase":
            return self.evaluate(symbols, positions, total_charge=total_charge, cell=cell, pbc=pbc,
                                 full_derivative=full_derivative)
        symbols, x, types, flags, cellm, _ = self._prepare(symbols, positions, total_charge, cell, pbc,
                                                           full_derivative, replicate=False)
        return self._run([(types, x, flags, cellm, float(total_charge), None)], full_derivative, [(1, 1, 1)], "ase")[0]

    def parameter_gradient(self, symbols, positions, *, total_charge=0, cell=None, pbc=None, initial_charges=None,
                           full_derivative=False, qeq=False):
        """Energy, forces and dE/dtheta for the bond, angle and vdW parameters (an extension; xreac
        has no parameter derivatives). Returns ``(Evaluation, ParameterGradient)``.

        The gradient comes from the same hand-written adjoint as the forces: each energy kernel adds
        its parameter sensitivities, the bond-order parameters get theirs through the bond-order
        chain's adjoints. Charges do not depend on these parameters, so it is the total derivative.
        ``full_derivative`` selects the charge-response forces, as in :meth:`evaluate`. ``qeq``
        adds the QEq parameters (chi, eta per element, the pair table's gamma), which change the
        charges: their total derivatives take one adjoint QEq solve more.
        """
        return self.parameter_gradient_many([dict(symbols=symbols, positions=positions, total_charge=total_charge,
                                                  cell=cell, pbc=pbc, initial_charges=initial_charges)],
                                            full_derivative=full_derivative, qeq=qeq)

    def parameter_gradient_many(self, systems, *, per_system=False, full_derivative=False, parameter_sets=None,
                                raw=False, qeq=False):
        """As :meth:`parameter_gradient` for a batch, in one device call: the evaluations, and the
        gradient of their summed energy, or (``per_system``) one gradient per system. With
        ``parameter_sets`` (see :meth:`load_parameter_sets`) system k is evaluated with set
        ``parameter_sets[k]`` and its gradient is with respect to that set. ``raw`` returns the
        gradients as table rows instead: ``(evaluations, pair (S, T*T, 28), angle (S, R, 7))``, one
        block per system, each row the derivative with respect to that table entry, and with ``qeq``
        the atom-table rows ``(S, T, 24)`` as a fourth item. ``qeq``: see :meth:`parameter_gradient`."""
        sets = self._sets(parameter_sets, len(systems))
        flags_ = nat.XR_FLAG_PARAM_GRADIENT | (nat.XR_FLAG_QEQ_GRADIENT if qeq else 0)
        results = self._evaluate_items([(s["symbols"], s["positions"], s.get("total_charge", 0), s.get("cell"),
                                         s.get("pbc"), s.get("initial_charges")) for s in systems], full_derivative,
                                       flags_, sets)
        T = len(self.force_field.elements)
        if raw:
            np_, na, nat_ = T * T * 28, 7 * len(self._angle_rows), T * 24
            blocks = np.empty((len(systems), np_ + na + nat_))
            code = self._lib.xr_get_param_gradient_blocks(self._ctx.handle, nat.ptr(blocks, nat.c_double), blocks.size)
            if code != nat.XR_OK:
                raise RuntimeError("parameter gradient unavailable")
            out = (results, blocks[:, :np_].reshape(-1, T * T, 28), blocks[:, np_:np_ + na].reshape(-1, na // 7, 7))
            return out + (blocks[:, np_ + na:].reshape(-1, T, 24),) if qeq else out
        grads = []
        for index in (range(len(systems)) if per_system else (-1,)):
            pair = np.zeros(T * T * 28)
            angle = np.zeros(7 * len(self._angle_rows))
            code = self._lib.xr_get_param_gradient_system(self._ctx.handle, index, nat.ptr(pair, nat.c_double),
                                                          len(pair), nat.ptr(angle, nat.c_double) if len(angle) else None,
                                                          len(angle))
            atom = None
            if code == nat.XR_OK and qeq:
                atom = np.zeros(T * 24)
                code = self._lib.xr_get_param_gradient_atoms(self._ctx.handle, index, nat.ptr(atom, nat.c_double),
                                                             len(atom))
                atom = atom.reshape(T, 24)
            if code != nat.XR_OK:
                raise RuntimeError("parameter gradient unavailable")
            grads.append(ParameterGradient.from_rows(self.force_field, pair.reshape(T * T, 28), angle.reshape(-1, 7),
                                                     self._angle_rows, atom))
        if per_system:
            return results, grads
        return (results[0] if len(systems) == 1 else results), grads[0]

    def evaluate_many(self, systems, *, full_derivative=False, parameter_sets=None):
        """Evaluate independent systems in one ragged device batch.

        ``systems`` is a sequence of dicts with the keyword arguments of :meth:`evaluate`
        (``symbols``, ``positions`` and optionally ``total_charge``, ``cell``, ``pbc``,
        ``initial_charges``). Returns a list of :class:`Evaluation` in the same order.
        ``parameter_sets`` (an extension): one parameter set per system, see
        :meth:`load_parameter_sets`.
        """
        sets = self._sets(parameter_sets, len(systems))
        return self._evaluate_items([(s["symbols"], s["positions"], s.get("total_charge", 0), s.get("cell"),
                                      s.get("pbc"), s.get("initial_charges")) for s in systems], full_derivative,
                                    0, sets)

    def _evaluate_items(self, items, full_derivative=False, extra_flags=0, sets=None):
        """``evaluate_many`` on tuples (symbols, positions, total_charge, cell, pbc, initial_charges)."""
        if _host is not None and self._all_valid and type(items) is list and items:
            packed = self._pack(items, full_derivative)
            if packed is not None:
                return self._run_packed(*packed, full_derivative, "replicated", extra_flags, sets=sets)
        batch, reps = [], []
        prepare = self._prepare
        for symbols, positions, total_charge, cell, pbc, initial in items:
            sym, x, types, flags, cellm, rp = prepare(symbols, positions, total_charge, cell, pbc, full_derivative)
            guess = None if initial is None else _guess(initial, len(sym))
            batch.append((types, x, flags, cellm, float(total_charge), guess))
            reps.append(rp)
        return self._run(batch, full_derivative, reps, "replicated", extra_flags, sets=sets)

    def _pack(self, items, full_derivative):
        """The batch's types and positions packed by the host module (one C pass over the requests);
        requests it leaves (any input the fast path does not take as is) go through ``_prepare``,
        and cells, periodicity and initial charges through the Python checks. None when the batch
        needs the general path."""
        if full_derivative is not True and full_derivative is not False:
            raise ValueError("full_derivative must be a boolean")
        try:
            sizes = [len(it[0]) for it in items]
        except TypeError:
            return None
        total = sum(sizes)
        types = np.empty(total, dtype=np.int32)
        x = np.empty((total, 3))
        slow = _host.fill(items, self._type_pos, types, x)
        n_sys = len(items)
        flags_l = [_NO_PBC] * n_sys
        cells = [None] * n_sys
        reps = [(1, 1, 1)] * n_sys
        # initial charges: the host module takes float64 arrays of finite charges as they are; the
        # rest get the Python checks (and a converted copy, held with the addresses)
        guess_addr = np.zeros(n_sys, dtype=np.uint64)
        keep = []
        for k in _host.guesses(items, guess_addr):
            g = _guess(items[k][5], sizes[k])
            if g is not None:
                keep.append(g)
                guess_addr[k] = nat.addr(g)
        offsets = np.zeros(n_sys + 1, dtype=np.int64)
        np.cumsum(sizes, out=offsets[1:])
        for k in slow:
            sym, xk, tk, fk, ck, rk = self._prepare(*items[k][:5], full_derivative)
            a0, a1 = int(offsets[k]), int(offsets[k + 1])
            if len(tk) != a1 - a0:
                return None
            types[a0:a1] = tk
            x[a0:a1] = xk
            flags_l[k], cells[k], reps[k] = fk, ck, rk
        cutoff = None
        slow_set = set(slow)
        for k, it in enumerate(items):
            cell, pbc = it[3], it[4]
            if k not in slow_set and not ((pbc is None and cell is None) or pbc is False):
                if cutoff is None:
                    cutoff = float(self.force_field.general[12])
                fast = periodic_cell(cell, pbc, cutoff, sizes[k], self.max_expanded_atoms)
                if fast is not None:
                    flags_l[k], cells[k], reps[k] = fast
                else:
                    flags, m = boundary(cell, pbc)
                    if m is not None:
                        reps[k] = cell_repetitions(cutoff, flags, m, sizes[k], self.max_expanded_atoms)
                        cells[k] = np.ascontiguousarray(m, dtype=np.float64)
                    flags_l[k] = flags
        charges = [float(it[2]) for it in items]
        return types, x, offsets, flags_l, cells, charges, _GuessAddresses(guess_addr, keep), reps

    def _run_one(self, types, x, flags, cellm, total_charge, guess, full_derivative, rep, backend):
        """``_run`` for one system (``xr_eval``) with a reused pair of C descriptors and one output
        block, instead of the batch's structured arrays: the plain path's host cost."""
        n = len(types)
        if not np.isfinite(x).all():
            raise ValueError("positions must be a finite (N, 3) array in Angstrom")
        one = self.__dict__.get("_one")
        if one is None:
            one = self._one = (nat.System(), nat.Result())
        sd, rd = one
        sd.natoms = n
        sd.types = nat.addr(types)
        sd.positions = nat.addr(x)
        sd.cell = None if cellm is None else nat.addr(cellm)
        sd.pbc[0], sd.pbc[1], sd.pbc[2] = int(flags[0]), int(flags[1]), int(flags[2])
        sd.total_charge = total_charge
        sd.charges_guess = None if guess is None else nat.addr(guess)
        # one block: energy (15) | dipole (3) | forces (3n) | charges, total bond orders, lone pairs (3n)
        block = np.empty(18 + 6 * n)
        counts = np.empty(n, dtype=np.int32)
        base = nat.addr(block)
        rd.energy = base
        rd.dipole = base + 120
        rd.forces = base + 144
        rd.charges = base + 144 + 24 * n
        rd.total_bond_orders = base + 144 + 32 * n
        rd.lone_pairs = base + 144 + 40 * n
        rd.bond_counts = nat.addr(counts)
        code = self._lib.xr_eval(self._ctx.handle, self._ff.handle, nat.byref(sd),
                                 nat.XR_FLAG_FULL_DERIVATIVE if full_derivative else 0, nat.byref(rd))
        if code != nat.XR_OK:
            self._raise(code)
        bonds = self._bonds(0)
        held = _BatchResults(block[:15].reshape(1, 15), block[18:18 + 3 * n].reshape(n, 3),
                             block[18 + 3 * n:].reshape(3, n), counts, block[15:18].reshape(1, 3), [0, n], bonds,
                             [0, len(bonds[0])])
        ev = object.__new__(Evaluation)
        ev.__dict__.update(energy=float(block[14]), full_derivative=full_derivative, cell_repetitions=rep,
                           neighbor_backend=backend, _batch=held, _index=0)
        return ev

    def _run(self, batch, full_derivative, reps, backend, extra_flags=0, supplied=None, sets=None):
        """One ``xr_eval_batch`` call over ``batch`` = [(types, positions, pbc flags, cell, total
        charge, initial charges)]: the inputs are packed into one array per kind, then as
        ``_run_packed`` (``xr_eval_neighbors`` with a supplied list for a single system)."""
        n_sys = len(batch)
        types_l, xs, flags_l, cells, charges, guesses = zip(*batch)
        sizes = np.fromiter(map(len, types_l), dtype=np.int64, count=n_sys)
        offsets = np.zeros(n_sys + 1, dtype=np.int64)
        np.cumsum(sizes, out=offsets[1:])
        types = np.concatenate(types_l) if n_sys > 1 else types_l[0]
        x = np.concatenate(xs) if n_sys > 1 else xs[0]
        return self._run_packed(types, x, offsets, flags_l, cells, charges, guesses, reps, full_derivative, backend,
                                extra_flags, supplied, sets)

    def _run_packed(self, types, x, offsets, flags_l, cells, charges, guesses, reps, full_derivative, backend,
                    extra_flags=0, supplied=None, sets=None):
        """One ``xr_eval_batch`` call: the per-system descriptors are filled column-wise over the
        packed types and positions, so the host cost per system is a handful of numpy operations;
        each ``Evaluation`` gets views of the batch's result arrays."""
        lib = self._lib
        n_sys = len(offsets) - 1
        sizes = np.diff(offsets)
        total = int(offsets[-1])
        if not np.isfinite(x).all():
            raise ValueError("positions must be a finite (N, 3) array in Angstrom")
        sys_arr = np.zeros(n_sys, dtype=_SYSTEM_DTYPE)
        sys_arr["natoms"] = sizes
        sys_arr["types"] = nat.addr(types) + 4 * offsets[:-1]
        sys_arr["positions"] = nat.addr(x) + 24 * offsets[:-1]
        periodic = [k for k, f in enumerate(flags_l) if f is not _NO_PBC]
        if periodic:
            pbc = sys_arr["pbc"]
            for k in periodic:
                pbc[k] = flags_l[k]
        sys_arr["total_charge"] = charges
        if any(c is not None for c in cells):
            sys_arr["cell"] = [0 if c is None else nat.addr(c) for c in cells]
        if isinstance(guesses, _GuessAddresses):
            if guesses.addr.any():
                sys_arr["charges_guess"] = guesses.addr
        elif any(g is not None for g in guesses):
            sys_arr["charges_guess"] = [0 if g is None else nat.addr(g) for g in guesses]
        # one allocation per kind for the whole batch, every element written by the call; each
        # Evaluation gets views
        energy = np.empty((n_sys, 15))
        dipole = np.empty((n_sys, 3))
        forces = np.empty((total, 3))
        per_atom = np.empty((3, total))  # charges, total bond orders, lone pairs
        counts = np.empty(total, dtype=np.int32)
        res_arr = np.empty(n_sys, dtype=_RESULT_DTYPE)
        ks = np.arange(n_sys, dtype=np.int64)
        a0s = offsets[:-1]
        q_base = nat.addr(per_atom)
        res_arr["energy"] = nat.addr(energy) + 120 * ks
        res_arr["forces"] = nat.addr(forces) + 24 * a0s
        res_arr["charges"] = q_base + 8 * a0s
        res_arr["total_bond_orders"] = q_base + 8 * (total + a0s)
        res_arr["lone_pairs"] = q_base + 8 * (2 * total + a0s)
        res_arr["bond_counts"] = nat.addr(counts) + 4 * a0s
        res_arr["dipole"] = nat.addr(dipole) + 24 * ks
        flags_ = (nat.XR_FLAG_FULL_DERIVATIVE if full_derivative else 0) | extra_flags
        if supplied is not None:
            code = lib.xr_eval_neighbors(self._ctx.handle, self._ff.handle, sys_arr.ctypes.data_as(_SYSTEM_P),
                                         nat.byref(supplied), flags_, res_arr.ctypes.data_as(_RESULT_P))
        elif sets is not None:
            code = lib.xr_eval_batch_sets(self._ctx.handle, self._ff.handle, n_sys, sys_arr.ctypes.data_as(_SYSTEM_P),
                                          nat.ptr(sets, nat.c_int), flags_, res_arr.ctypes.data_as(_RESULT_P))
        else:
            code = lib.xr_eval_batch(self._ctx.handle, self._ff.handle, n_sys, sys_arr.ctypes.data_as(_SYSTEM_P),
                                     flags_, res_arr.ctypes.data_as(_RESULT_P))
        if code != nat.XR_OK:
            self._raise(code)
        bi, bj, bS, bbo = self._bonds(-1)
        cut = np.searchsorted(bi, offsets)  # bonds are grouped by system, in pair order
        if len(bi):
            shift = np.repeat(a0s.astype(np.int32), np.diff(cut))
            bi -= shift
            bj -= shift
        held = _BatchResults(energy, forces, per_atom, counts, dipole, offsets.tolist(), (bi, bj, bS, bbo),
                             cut.tolist())
        etot = energy[:, 14].tolist()
        results = []
        new = object.__new__
        for k in range(n_sys):
            # a frozen dataclass: set without the per-field checks; the array fields follow on access
            ev = new(Evaluation)
            ev.__dict__.update(energy=etot[k], full_derivative=full_derivative, cell_repetitions=reps[k],
                               neighbor_backend=backend, _batch=held, _index=k)
            results.append(ev)
        return results

    def _bonds(self, index):
        lib, h = self._lib, self._ctx.handle
        count = nat.c_longlong()
        lib.xr_get_bonds(h, index, None, None, None, None, 0, nat.byref(count))
        m = count.value
        ints = np.empty(5 * m, dtype=np.int32)  # i | j | S
        bo = np.empty(m)
        base = nat.addr(ints)
        lib.xr_get_bonds(h, index, base, base + 4 * m, base + 8 * m, nat.addr(bo), m, nat.byref(count))
        return ints[:m], ints[m:2 * m], ints[2 * m:].reshape(m, 3), bo

    def relax(self, symbols, positions, *, force_tolerance=1e-4, max_iterations=500, total_charge=0, cell=None,
              pbc=None, backend="ase"):
        """Relax with fixed-charge forces by FIRE (src/xreac/calculator.py:167-246); the cell stays fixed.

        Convergence requires the largest absolute Cartesian force component to be at most
        ``force_tolerance`` (kcal/mol/A). ``backend="native"`` runs xreac's own FIRE: unit masses,
        dt = 0.02 growing by 1.1 up to 0.2 after more than five steps with positive power, halved
        (and the velocity reset) otherwise, mixing alpha = 0.1 decaying by 0.99, and the largest
        atomic step capped at 0.1 A (Bitzek et al., Phys. Rev. Lett. 97, 170201, 2006). Every step
        is one device evaluation whose QEq starts from the previous step's charges and whose
        neighbour list is the device's skin list (0.3 A, rebuilt only when an atom has moved that
        far); the returned evaluation is a plain one at the final positions, identical to
        :meth:`evaluate` there. ``backend="ase"`` runs ASE's FIRE through
        :class:`xreac_gb300.ase.ReaxFFCalculator`, which needs ASE installed, as xreac's does.
        """
        symbols, x, _, _ = validate_input(symbols, positions, total_charge, cell, pbc)
        if isinstance(force_tolerance, bool) or not isinstance(force_tolerance, Real) \
                or not np.isfinite(force_tolerance) or force_tolerance <= 0:
            raise ValueError("force_tolerance must be positive and finite")
        if isinstance(max_iterations, bool) or not isinstance(max_iterations, (int, np.integer)) or max_iterations < 1:
            raise ValueError("max_iterations must be a positive integer")
        if backend not in ("ase", "native"):
            raise ValueError("backend must be 'ase' or 'native'")
        kw = dict(total_charge=total_charge, cell=cell, pbc=pbc)
        if backend == "ase":
            from .ase import relax_with_ase

            flags, _ = boundary(cell, pbc)
            x, result, converged, iterations = relax_with_ase(self, symbols, x, force_tolerance, max_iterations,
                                                              cell=cell, pbc=flags, total_charge=total_charge)
            message = "Fixed-charge force tolerance reached" if converged else "Maximum relaxation iterations reached"
            return Relaxation(x, result, converged, iterations, message)
        skin = self.neighbor_skin
        self.set_neighbor_skin(RELAX_SKIN)
        try:
            return self._fire(symbols, x, force_tolerance, max_iterations, kw)
        finally:
            self.set_neighbor_skin(skin)

    def _fire(self, symbols, x, force_tolerance, max_iterations, kw):
        """xreac's native FIRE recurrence (src/xreac/calculator.py:213-246) on device evaluations."""
        velocity = np.zeros_like(x)
        dt, dt_max, alpha = 0.02, 0.2, 0.1
        positive_steps = 0
        result = self.evaluate(symbols, x, **kw)
        warm = result
        iteration = 0
        while True:
            force = warm.forces
            if np.max(np.abs(force)) <= force_tolerance:
                if warm is not result:  # confirm on the plain evaluation that is returned
                    result = self.evaluate(symbols, x, **kw)
                    warm = result
                    continue
                return Relaxation(x, result, True, iteration, "Fixed-charge force tolerance reached")
            if iteration == max_iterations:
                if warm is not result:
                    result = self.evaluate(symbols, x, **kw)
                return Relaxation(x, result, False, max_iterations, "Maximum relaxation iterations reached")
            power = float(np.sum(velocity * force))
            if power > 0:
                velocity = (1 - alpha) * velocity + alpha * np.linalg.norm(velocity) / np.linalg.norm(force) * force
                positive_steps += 1
                if positive_steps > 5:
                    dt = min(dt * 1.1, dt_max)
                    alpha *= 0.99
            else:
                velocity.fill(0.0)
                positive_steps = 0
                alpha = 0.1
                if iteration > 0:
                    dt *= 0.5
            velocity += dt * force
            step = dt * velocity
            largest = float(np.max(np.linalg.norm(step, axis=1)))
            if largest > 0.1:
                step *= 0.1 / largest
            x = x + step
            iteration += 1
            warm = self.evaluate(symbols, x, initial_charges=warm.charges, **kw)

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
        """Kernels launched by the last evaluation call."""
        return int(self._lib.xr_last_launches(self._ctx.handle))

    def qeq_work(self):
        """(CG iterations summed over the last call's systems, their matrix-free algorithmic bytes)."""
        its = nat.c_longlong()
        b = nat.c_double()
        self._lib.xr_last_qeq_work(self._ctx.handle, nat.byref(its), nat.byref(b))
        return int(its.value), float(b.value)

    def transfer_bytes(self):
        """(host-to-device, device-to-host) bytes moved by the last evaluation call."""
        h2d = nat.c_longlong()
        d2h = nat.c_longlong()
        self._lib.xr_last_transfer_bytes(self._ctx.handle, nat.byref(h2d), nat.byref(d2h))
        return int(h2d.value), int(d2h.value)

    def set_profiling(self, enable=True):
        """Per-stage CUDA-event timing of later calls (resets the accumulators)."""
        self._lib.xr_ctx_set_profiling(self._ctx.handle, 1 if enable else 0)

    def stage_times(self):
        """(summed milliseconds of the 8 stages, number of calls) since profiling was enabled."""
        ms = (nat.c_double * 8)()
        calls = nat.c_longlong()
        self._lib.xr_ctx_stage_times(self._ctx.handle, ms, 8, nat.byref(calls))
        return np.array(ms[:8]), int(calls.value)

    def memory(self):
        """The context's device memory (``xr_ctx_memory``): bytes held and the capacities a call can
        use without allocating (atoms, systems, directed edges, pairs, bonds, candidate edges)."""
        b = nat.c_longlong()
        caps = (nat.c_longlong * 6)()
        self._lib.xr_ctx_memory(self._ctx.handle, nat.byref(b), caps, 6)
        names = ("atoms", "systems", "edges", "pairs", "bonds", "candidates")
        return dict(device_bytes=int(b.value), **{k: int(v) for k, v in zip(names, caps)})

    @staticmethod
    def footprint_bytes(atoms, systems=1, edges=0, bonds=0):
        """Device bytes a context needs for calls of up to these sizes (``xr_footprint_bytes``)."""
        v = nat.load().xr_footprint_bytes(int(atoms), int(systems), int(edges), int(bonds))
        if v < 0:
            raise ValueError("atoms and systems must be positive, edges and bonds nonnegative")
        return int(v)

    def list_sizes(self):
        """Sizes of the last call's lists: directed edges, pairs, bond candidates, bond-row entries,
        active bonds, torsion middles (summed over its systems)."""
        out = (nat.c_longlong * 6)()
        self._lib.xr_last_list_sizes(self._ctx.handle, out, 6)
        return tuple(int(v) for v in out)
