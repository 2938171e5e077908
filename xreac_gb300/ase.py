"""ASE calculator over the device evaluator (the counterpart of xreac's src/xreac/ase.py:30-188).

Needs ASE, as xreac's adapter does: importing this module without it raises ``ImportError``.

Parameters, defaults, units and messages are xreac's: energy in eV, forces in eV/A, charges in e,
the dipole in e A, and ``evaluation`` holding the last result in kcal/mol units. What differs is
where the neighbour topology lives. xreac builds an ASE ``PrimitiveNeighborList`` on the host and
hands its arrays to the evaluator on every call; here the list never leaves the GPU:

- ``neighbor_backend="ase"`` (the default) evaluates without small-cell replication (no
  ``max_expanded_atoms`` limit, ``cell_repetitions`` (1, 1, 1)), as ASE's image lists do, and
  keeps the device list across calls with ``neighbor_skin`` (``Calculator.set_neighbor_skin``):
  a list of every image within cutoff + 2 skin, reused until an atom has moved more than the skin
  from its position at the build, or the cell, periodicity or atoms change. Reuse skips the
  neighbour search on the device; the edges within the cutoff are re-selected from the kept list
  each call, so results equal those of a fresh list. A skin of 0 searches every call.
- ``neighbor_backend="replicated"`` is xreac's native search: a fresh search every call, the
  ``max_expanded_atoms`` limit and the replication count reported.

``neighbor_list_builds`` counts the calls that searched for neighbours (a skin list built, or a
search without a skin) under the "ase" backend, the quantity xreac's adapter counts.
"""

from __future__ import annotations

from numbers import Real

import numpy as np

try:
    from ase.calculators.calculator import Calculator as _AseCalculator
    from ase.calculators.calculator import all_changes
    from ase.units import kcal, mol
except ImportError as exc:  # the adapter is optional, as in xreac
    raise ImportError("Install ASE to use the ASE calculator (xreac_gb300.ase)") from exc

from .calculator import Calculator
from .geometry import validate_expansion_limit, validate_total_charge

KCAL_MOL_TO_EV = kcal / mol
BACKENDS = ("ase", "replicated")


def _check_skin(value):
    if isinstance(value, bool) or not isinstance(value, Real) or not np.isfinite(value) or value < 0:
        raise ValueError("neighbor_skin must be a finite nonnegative number")


def _check_derivative(value):
    if not isinstance(value, bool):
        raise ValueError("full_derivative must be a boolean")


def _check_backend(value):
    if value not in BACKENDS:
        raise ValueError("neighbor_backend must be 'replicated' or 'ase'")


# Each parameter's check, with xreac's messages; applied to every value handed to set().
_CHECKS = {
    "full_derivative": _check_derivative,
    "total_charge": validate_total_charge,
    "max_expanded_atoms": validate_expansion_limit,
    "neighbor_backend": _check_backend,
    "neighbor_skin": _check_skin,
}


class ReaxFFCalculator(_AseCalculator):
    """ReaxFF for ASE ``Atoms`` on the GPU, with a net charge and a fixed cell.

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
        self._bind(Calculator(force_field, max_expanded_atoms=max_expanded_atoms))
        super().__init__(full_derivative=full_derivative, total_charge=total_charge,
                         max_expanded_atoms=max_expanded_atoms, neighbor_backend=neighbor_backend,
                         neighbor_skin=neighbor_skin, **kwargs)

    @classmethod
    def around(cls, core, **parameters):
        """An adapter that evaluates through an existing device ``Calculator`` (its context and
        force field) instead of making a new one; ``relax_with_ase`` uses the caller's."""
        self = cls.__new__(cls)
        self._bind(core)
        params = dict(max_expanded_atoms=core.max_expanded_atoms)
        params.update(parameters)
        _AseCalculator.__init__(self, **params)
        return self

    def _bind(self, core):
        self.core = core
        self.evaluation = None
        self.neighbor_list_builds = 0

    def set(self, **kwargs):
        unknown = sorted(set(kwargs) - set(self.default_parameters))
        if unknown:
            raise ValueError(f"Unknown ReaxFF calculator parameters: {unknown}")
        for name, value in kwargs.items():
            _CHECKS[name](value)
        changed = super().set(**kwargs)
        if changed:
            self.core.max_expanded_atoms = self.parameters.max_expanded_atoms
            self.reset()
        return changed

    def reset(self):
        super().reset()
        self.evaluation = None
        # drop the kept device list; the next "ase" evaluation builds one with the current skin
        skin = float(self.parameters.get("neighbor_skin", 0.0))
        self.core.set_neighbor_skin(skin if self.parameters.get("neighbor_backend") == "ase" else 0.0)

    def calculate(self, atoms=None, properties=("energy", "forces"), system_changes=all_changes):
        super().calculate(atoms, properties, system_changes)
        self.results = {}
        self.evaluation = None
        if self.atoms is None:
            raise ValueError("An ASE Atoms object is required")
        p = self.parameters
        if self.atoms.has("initial_charges"):
            q0 = self.atoms.get_initial_charges()
            if not np.isfinite(q0).all() or abs(q0.sum() - p.total_charge) > 1e-8:
                raise ValueError("Initial charges must be finite and sum to total_charge")
        ase_lists = p.neighbor_backend == "ase"
        if self.core.neighbor_skin != (p.neighbor_skin if ase_lists else 0.0):
            self.core.set_neighbor_skin(p.neighbor_skin if ase_lists else 0.0)
        result = self.core._evaluate_backend(
            self.atoms.get_chemical_symbols(), self.atoms.positions, cell=self.atoms.cell.array, pbc=self.atoms.pbc,
            total_charge=p.total_charge, full_derivative=p.full_derivative, backend=p.neighbor_backend)
        if ase_lists and self.core.list_info()[0] in ("built", "scan"):
            self.neighbor_list_builds += 1
        self.evaluation = result
        self.results = {
            "energy": result.energy * KCAL_MOL_TO_EV,
            "forces": np.asarray(result.forces) * KCAL_MOL_TO_EV,
            "charges": np.array(result.charges, copy=True),
            "dipole": np.array(result.dipole, copy=True),
        }


def relax_with_ase(core, symbols, positions, force_tolerance, max_iterations, *, cell=None, pbc=False, total_charge=0):
    """ASE FIRE on fixed-charge forces of ``core``, stopped by xreac's rule: the largest absolute
    Cartesian force component at most ``force_tolerance`` (kcal/mol/A), checked before each step.
    Returns (positions, evaluation, converged, steps taken). The core's skin setting is restored."""
    from ase import Atoms
    from ase.optimize import FIRE

    atoms = Atoms(symbols, positions=positions, cell=cell, pbc=pbc)
    skin = core.neighbor_skin
    adapter = ReaxFFCalculator.around(core, total_charge=total_charge)
    atoms.calc = adapter
    try:
        with FIRE(atoms, logfile=None, downhill_check=False) as fire:
            steps = 0
            while True:
                atoms.get_forces()  # one evaluation per geometry (ASE caches it for the step)
                result = adapter.evaluation
                if np.max(np.abs(result.forces)) <= force_tolerance:
                    return atoms.positions.copy(), result, True, steps
                if steps == max_iterations:
                    return atoms.positions.copy(), result, False, steps
                fire.step()
                steps += 1
    finally:
        core.set_neighbor_skin(skin)
