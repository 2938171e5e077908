"""ASE calculator adapter over the device ``Calculator`` (src/xreac/ase.py:1-200).

Needs ASE, as xreac's adapter does; importing this module without ASE raises ``ImportError``. The
adapter keeps xreac's parameters, units (eV, eV/A; charges in e, dipole in e A) and its topology
reuse: with ``neighbor_backend="ase"`` an ASE ``PrimitiveNeighborList`` with per-atom radius rc/2 and
``neighbor_skin`` is updated before each evaluation (ASE rebuilds it after any atom moved more than
the skin, or the cell or periodicity changed) and handed to the evaluator as the directed list
``(i, j, S)``. The device evaluator validates a supplied list and evaluates every pair within rc,
which any complete list yields, so topology reuse changes the count of list builds
(``neighbor_list_builds``), not the result.
"""

from __future__ import annotations

from dataclasses import replace
from numbers import Real

import numpy as np

try:
    from ase.calculators.calculator import Calculator as _AseCalculator
    from ase.calculators.calculator import all_changes
    from ase.neighborlist import PrimitiveNeighborList
    from ase.units import kcal, mol
except ImportError as exc:  # the adapter is optional, as in xreac
    raise ImportError("Install ASE to use the ASE calculator (xreac_gb300.ase)") from exc

from .calculator import Calculator
from .geometry import boundary, validate_expansion_limit, validate_total_charge

KCAL_MOL_TO_EV = kcal / mol


def directed_neighbors(half_list):
    """(i, j, S) with both directions from an ASE half list (``neighbors``/``displacements`` per atom)."""
    counts = np.fromiter((len(row) for row in half_list.neighbors), dtype=np.int64, count=len(half_list.neighbors))
    i = np.repeat(np.arange(len(counts), dtype=np.int64), counts)
    if counts.sum():
        j = np.concatenate(half_list.neighbors).astype(np.int64)
        s = np.concatenate(half_list.displacements).reshape(-1, 3).astype(np.int64)
    else:
        j = np.empty(0, dtype=np.int64)
        s = np.empty((0, 3), dtype=np.int64)
    return np.concatenate((i, j)), np.concatenate((j, i)), np.concatenate((s, -s))


class ReaxFFCalculator(_AseCalculator):
    """ReaxFF for ASE ``Atoms`` on the GPU: energy, forces, charges and dipole.

    ``evaluation`` keeps the last :class:`~xreac_gb300.calculator.Evaluation` (kcal/mol units).
    Fixed-charge forces by default; ``full_derivative=True`` gives charge-response forces.
    """

    implemented_properties = ["energy", "forces", "charges", "dipole"]
    default_parameters = {
        "full_derivative": False,
        "total_charge": 0,
        "max_expanded_atoms": 512,
        "neighbor_backend": "ase",
        "neighbor_skin": 0.3,
    }

    def __init__(self, force_field, *, full_derivative=False, total_charge=0, max_expanded_atoms=512,
                 neighbor_backend="ase", neighbor_skin=0.3, **kwargs):
        self.core = Calculator(force_field, max_expanded_atoms=max_expanded_atoms)
        self.evaluation = None
        self.neighbor_list_builds = 0
        self._half_list = None
        self._half_key = None
        self._directed = None
        super().__init__(full_derivative=full_derivative, total_charge=total_charge,
                         max_expanded_atoms=max_expanded_atoms, neighbor_backend=neighbor_backend,
                         neighbor_skin=neighbor_skin, **kwargs)

    def set(self, **kwargs):
        unknown = set(kwargs) - set(self.default_parameters)
        if unknown:
            raise ValueError(f"Unknown ReaxFF calculator parameters: {sorted(unknown)}")
        if "full_derivative" in kwargs and not isinstance(kwargs["full_derivative"], bool):
            raise ValueError("full_derivative must be a boolean")
        if "total_charge" in kwargs:
            validate_total_charge(kwargs["total_charge"])
        if "max_expanded_atoms" in kwargs:
            validate_expansion_limit(kwargs["max_expanded_atoms"])
        if kwargs.get("neighbor_backend", "ase") not in ("ase", "replicated"):
            raise ValueError("neighbor_backend must be 'replicated' or 'ase'")
        if "neighbor_skin" in kwargs:
            skin = kwargs["neighbor_skin"]
            if isinstance(skin, bool) or not isinstance(skin, Real) or not np.isfinite(skin) or skin < 0:
                raise ValueError("neighbor_skin must be a finite nonnegative number")
        changed = super().set(**kwargs)
        if changed:
            self.core.max_expanded_atoms = self.parameters.max_expanded_atoms
            self.reset()
        return changed

    def reset(self):
        super().reset()
        self.evaluation = None
        self._half_list = None
        self._half_key = None
        self._directed = None

    def _topology(self):
        atoms = self.atoms
        boundary(atoms.cell.array, atoms.pbc)  # the same cell validation (and errors) as evaluate
        cutoff = np.nextafter(float(self.core.force_field.general[12]), np.inf)
        skin = self.parameters.neighbor_skin
        key = (cutoff, skin, tuple(atoms.numbers))
        if self._half_list is None or key != self._half_key or skin == 0:
            # pair cutoff = two radii of rc/2 plus twice the skin
            self._half_list = PrimitiveNeighborList(np.full(len(atoms), cutoff / 2), skin=skin,
                                                    self_interaction=False, bothways=False)
            self._half_key = key
        try:
            rebuilt = self._half_list.update(atoms.pbc, atoms.cell, atoms.positions)
        except Exception:
            self._half_list = None
            self._directed = None
            raise
        if rebuilt:
            self._directed = directed_neighbors(self._half_list)
            self.neighbor_list_builds += 1
        return self._directed

    def calculate(self, atoms=None, properties=("energy", "forces"), system_changes=all_changes):
        super().calculate(atoms, properties, system_changes)
        self.results = {}
        self.evaluation = None
        if self.atoms is None:
            raise ValueError("An ASE Atoms object is required")
        start = self.atoms.get_initial_charges()
        if self.atoms.has("initial_charges") and (
                not np.isfinite(start).all() or abs(start.sum() - self.parameters.total_charge) > 1e-8):
            raise ValueError("Initial charges must be finite and sum to total_charge")
        neighbors = self._topology() if self.parameters.neighbor_backend == "ase" else None
        result = self.core.evaluate(self.atoms.get_chemical_symbols(), self.atoms.positions,
                                    cell=self.atoms.cell.array, pbc=self.atoms.pbc,
                                    total_charge=self.parameters.total_charge,
                                    full_derivative=self.parameters.full_derivative, neighbors=neighbors)
        result = replace(result, neighbor_backend=self.parameters.neighbor_backend)
        self.evaluation = result
        self.results = {
            "energy": result.energy * KCAL_MOL_TO_EV,
            "forces": result.forces * KCAL_MOL_TO_EV,
            "charges": result.charges.copy(),
            "dipole": result.dipole.copy(),
        }


def relax_with_ase(core, symbols, positions, force_tolerance, max_iterations, *, cell=None, pbc=False,
                   total_charge=0):
    """ASE FIRE on ``core`` with xreac's stop rule (largest Cartesian force component, kcal/mol/A).

    Returns ``(positions, evaluation, converged, iterations)``."""
    from ase import Atoms
    from ase.optimize import FIRE

    atoms = Atoms(symbols, positions=positions, cell=cell, pbc=pbc)
    adapter = ReaxFFCalculator(core.force_field, total_charge=total_charge, max_expanded_atoms=core.max_expanded_atoms)
    adapter.core = core  # the caller's calculator, with its device context
    atoms.calc = adapter
    with FIRE(atoms, logfile=None, downhill_check=False) as optimizer:
        for _ in optimizer.irun(fmax=force_tolerance * KCAL_MOL_TO_EV, steps=max_iterations):
            if np.max(np.abs(adapter.evaluation.forces)) <= force_tolerance:
                return atoms.positions.copy(), adapter.evaluation, True, optimizer.nsteps
        return atoms.positions.copy(), adapter.evaluation, False, optimizer.nsteps
