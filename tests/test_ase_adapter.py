"""The ASE adapter's own logic on CPU, with ASE (absent here) replaced by a minimal stand-in.

The stand-in provides what xreac_gb300.ase uses: a calculator base class with ASE's parameter
handling, ``all_changes``, a ``PrimitiveNeighborList`` that rebuilds after any atom moved more than
the skin (ASE's rule), and ``kcal``/``mol``. The device ``Calculator`` is replaced by a recorder, so
the test covers parameter validation, topology reuse and rebuild counting, the directed list handed
to the evaluator, unit conversion and the initial-charge check (src/xreac/ase.py:50-175).
"""

import importlib
import sys
import types

import numpy as np
import pytest


class _Params(dict):
    def __getattr__(self, k):
        return self[k]


class _AseCalculator:
    default_parameters = {}

    def __init__(self, **kwargs):
        self.parameters = _Params(self.default_parameters)
        self.atoms = None
        self.results = {}
        self.set(**kwargs)

    def set(self, **kwargs):
        changed = {k: v for k, v in kwargs.items() if self.parameters.get(k) != v}
        self.parameters.update(kwargs)
        return changed

    def reset(self):
        self.results = {}

    def calculate(self, atoms=None, properties=None, system_changes=None):
        if atoms is not None:
            self.atoms = atoms


class _HalfList:
    def __init__(self, radii, skin, self_interaction, bothways):
        assert not self_interaction and not bothways
        self.cut = 2 * float(radii[0]) + 2 * skin
        self.skin = skin
        self.x0 = None

    def update(self, pbc, cell, positions):
        x = np.asarray(positions, dtype=float)
        if self.x0 is not None and self.skin > 0 and np.max(np.linalg.norm(x - self.x0, axis=1)) <= self.skin:
            return False
        self.x0 = x.copy()
        n = len(x)
        d = np.linalg.norm(x[:, None] - x[None], axis=2)
        self.neighbors = [np.array([j for j in range(i + 1, n) if d[i, j] < self.cut], dtype=int) for i in range(n)]
        self.displacements = [np.zeros((len(r), 3), dtype=int) for r in self.neighbors]
        return True


class _Atoms:
    def __init__(self, symbols, positions):
        self.symbols = list(symbols)
        self.positions = np.array(positions, dtype=float)
        self.numbers = np.array([8 if s == "O" else 1 for s in symbols])
        self.cell = types.SimpleNamespace(array=np.zeros((3, 3)))
        self.pbc = np.zeros(3, dtype=bool)
        self.charges = None

    def __len__(self):
        return len(self.symbols)

    def get_chemical_symbols(self):
        return self.symbols

    def get_initial_charges(self):
        return np.zeros(len(self.symbols)) if self.charges is None else self.charges

    def has(self, name):
        return name == "initial_charges" and self.charges is not None


class _Core:
    def __init__(self, force_field, max_expanded_atoms=512):
        self.force_field = force_field
        self.max_expanded_atoms = max_expanded_atoms
        self.calls = []

    def evaluate(self, symbols, positions, **kw):
        from xreac_gb300.calculator import Evaluation

        self.calls.append(kw)
        n = len(symbols)
        return Evaluation(energy=-10.0, forces=np.ones((n, 3)), charges=np.zeros(n), components={},
                          full_derivative=kw["full_derivative"], total_bond_orders=np.zeros(n),
                          lone_pairs=np.zeros(n), bond_counts=np.zeros(n, dtype=int), dipole=np.zeros(3))


@pytest.fixture()
def adapter(monkeypatch):
    mods = {
        "ase": types.ModuleType("ase"),
        "ase.calculators": types.ModuleType("ase.calculators"),
        "ase.calculators.calculator": types.ModuleType("ase.calculators.calculator"),
        "ase.neighborlist": types.ModuleType("ase.neighborlist"),
        "ase.units": types.ModuleType("ase.units"),
    }
    mods["ase.calculators.calculator"].Calculator = _AseCalculator
    mods["ase.calculators.calculator"].all_changes = ["positions"]
    mods["ase.neighborlist"].PrimitiveNeighborList = _HalfList
    mods["ase.units"].kcal = 4.184e3 / 96485.33212 / 1e3 * 1e3
    mods["ase.units"].mol = 1.0
    for k, v in mods.items():
        monkeypatch.setitem(sys.modules, k, v)
    monkeypatch.delitem(sys.modules, "xreac_gb300.ase", raising=False)
    mod = importlib.import_module("xreac_gb300.ase")
    monkeypatch.setattr(mod, "Calculator", _Core)
    yield mod
    sys.modules.pop("xreac_gb300.ase", None)


def _water():
    return _Atoms(["O", "H", "H"], [[0, 0, 0], [0.96, 0, 0], [-0.24, 0.93, 0]])


def test_topology_reuse_and_rebuilds(adapter):
    from xreac_gb300 import ForceField

    calc = adapter.ReaxFFCalculator(ForceField.bundled("ffield.reax.HO.2015"), neighbor_skin=0.3)
    atoms = _water()
    calc.calculate(atoms)
    assert calc.neighbor_list_builds == 1
    i, j, s = calc.core.calls[-1]["neighbors"]
    assert len(i) == 6 and set(zip(i.tolist(), j.tolist())) == {(0, 1), (1, 0), (0, 2), (2, 0), (1, 2), (2, 1)}
    assert s.shape == (6, 3)
    atoms.positions[1, 0] += 0.2  # within the skin: the topology is reused
    calc.calculate(atoms)
    assert calc.neighbor_list_builds == 1
    atoms.positions[1, 0] += 0.2  # 0.4 A from the build positions: rebuilt
    calc.calculate(atoms)
    assert calc.neighbor_list_builds == 2
    calc.set(neighbor_skin=0.0)  # a changed parameter resets; a zero skin rebuilds every time
    calc.calculate(atoms)
    calc.calculate(atoms)
    assert calc.neighbor_list_builds == 4
    calc.set(neighbor_backend="replicated")
    calc.calculate(atoms)
    assert calc.core.calls[-1]["neighbors"] is None
    assert calc.evaluation.neighbor_backend == "replicated"


def test_results_in_ase_units(adapter):
    from xreac_gb300 import ForceField

    calc = adapter.ReaxFFCalculator(ForceField.bundled("ffield.reax.HO.2015"))
    calc.calculate(_water())
    assert calc.results["energy"] == pytest.approx(-10.0 * adapter.KCAL_MOL_TO_EV)
    np.testing.assert_allclose(calc.results["forces"], adapter.KCAL_MOL_TO_EV)
    assert calc.evaluation.neighbor_backend == "ase"
    assert calc.core.calls[-1]["full_derivative"] is False


@pytest.mark.parametrize("kwargs", [{"neighbor_backend": "x"}, {"neighbor_skin": -1.0}, {"neighbor_skin": True},
                                    {"full_derivative": 1}, {"total_charge": float("nan")}, {"unknown": 1},
                                    {"max_expanded_atoms": 0}])
def test_invalid_parameters(adapter, kwargs):
    from xreac_gb300 import ForceField

    with pytest.raises(ValueError):
        adapter.ReaxFFCalculator(ForceField.bundled("ffield.reax.HO.2015"), **kwargs)


def test_initial_charges_must_sum_to_total(adapter):
    from xreac_gb300 import ForceField

    calc = adapter.ReaxFFCalculator(ForceField.bundled("ffield.reax.HO.2015"))
    atoms = _water()
    atoms.charges = np.array([0.1, 0.0, 0.0])
    with pytest.raises(ValueError):
        calc.calculate(atoms)
