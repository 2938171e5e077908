"""A minimal stand-in for the parts of ASE that xreac_gb300.ase imports (ASE is absent here and on the
GPU host): a calculator base class with ASE's parameter handling, ``all_changes`` and the units. Test
infrastructure only: ``install`` registers it under the ``ase`` module names for one test."""

import importlib
import sys
import types

import numpy as np


class Params(dict):
    def __getattr__(self, k):
        return self[k]


class AseCalculator:
    """ASE's Calculator parameter protocol: defaults, ``set`` returning the changed values, ``reset``."""

    default_parameters = {}

    def __init__(self, **kwargs):
        self.parameters = Params(self.default_parameters)
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


class Atoms:
    """The Atoms attributes the adapter reads."""

    def __init__(self, symbols, positions, cell=None, pbc=False):
        self.symbols = list(symbols)
        self.positions = np.array(positions, dtype=float)
        self.cell = types.SimpleNamespace(array=np.zeros((3, 3)) if cell is None else np.array(cell, dtype=float))
        self.pbc = np.broadcast_to(np.asarray(pbc, dtype=bool), (3,)).copy()
        self.charges = None

    def __len__(self):
        return len(self.symbols)

    def get_chemical_symbols(self):
        return list(self.symbols)

    def get_initial_charges(self):
        return np.zeros(len(self.symbols)) if self.charges is None else self.charges

    def has(self, name):
        return name == "initial_charges" and self.charges is not None


KCAL = 4.184 / 96.48533212  # eV per kcal/mol (ase.units.kcal / ase.units.mol)


def install(monkeypatch):
    """Register the stand-in as ``ase`` and import xreac_gb300.ase afresh against it."""
    mods = {name: types.ModuleType(name) for name in ("ase", "ase.calculators", "ase.calculators.calculator",
                                                      "ase.units")}
    mods["ase.calculators.calculator"].Calculator = AseCalculator
    mods["ase.calculators.calculator"].all_changes = ["positions", "numbers", "cell", "pbc"]
    mods["ase.units"].kcal = KCAL
    mods["ase.units"].mol = 1.0
    for k, v in mods.items():
        monkeypatch.setitem(sys.modules, k, v)
    monkeypatch.delitem(sys.modules, "xreac_gb300.ase", raising=False)
    return importlib.import_module("xreac_gb300.ase")
