"""The ASE adapter on the device's neighbour lists, with ASE (absent here and on the GPU host)
replaced by a minimal stand-in (tests/ase_standin.py) for its calculator protocol. Mirrors the skin
tests of the reference (tests/test_neighbors.py:345-409): topology reused over displacements
measured from the build, rebuilt once an atom moves more than the skin or the system changes, and
the physics recomputed every call (results equal a fresh evaluation)."""

import numpy as np
import pytest

from ase_standin import Atoms, install
from conftest import load_golden

pytestmark = pytest.mark.gpu


def _same(a, b):
    assert a.energy == b.energy
    np.testing.assert_array_equal(a.charges, b.charges)
    np.testing.assert_allclose(a.forces, b.forces, atol=1e-9, rtol=0)


@pytest.fixture()
def ase_mod(monkeypatch):
    return install(monkeypatch)


@pytest.mark.parametrize("name", ["small_water_4A", "small_zinc_chain", "periodic_partial_pbc_water"])
def test_skin_reuses_topology_and_recomputes_physics(ase_mod, name):
    from xreac_gb300 import Calculator, ForceField

    g = load_golden(name)
    x = np.asarray(g["positions"], dtype=float)
    atoms = Atoms(g["symbols"], x, g["cell"], g["pbc"])
    calc = ase_mod.ReaxFFCalculator(ForceField.bundled(g["ff"]))
    fresh = Calculator(ForceField.bundled(g["ff"]))
    calc.calculate(atoms)
    assert calc.neighbor_list_builds == 1
    for displacement, builds in ((0.04, 1), (0.2, 1), (0.31, 2)):
        atoms.positions[0, 0] = x[0, 0] + displacement
        calc.calculate(atoms)
        assert calc.neighbor_list_builds == builds
        assert calc.evaluation.neighbor_backend == "ase" and calc.evaluation.cell_repetitions == (1, 1, 1)
        _same(calc.evaluation, fresh._evaluate_backend(g["symbols"], atoms.positions, cell=g["cell"], pbc=g["pbc"],
                                                       backend="ase"))


def test_skin_invalidation(ase_mod):
    from xreac_gb300 import Calculator, ForceField

    g = load_golden("small_water_4A")
    atoms = Atoms(g["symbols"], g["positions"], g["cell"], g["pbc"])
    calc = ase_mod.ReaxFFCalculator(ForceField.bundled(g["ff"]))
    fresh = Calculator(ForceField.bundled(g["ff"]))

    def check(builds):
        calc.calculate(atoms)
        assert calc.neighbor_list_builds == builds
        _same(calc.evaluation, fresh._evaluate_backend(atoms.get_chemical_symbols(), atoms.positions,
                                                       cell=atoms.cell.array, pbc=atoms.pbc, backend="ase"))

    check(1)
    check(1)
    atoms.cell.array[0, 0] += 0.1
    check(2)
    atoms.pbc[2] = False
    check(3)
    atoms.positions[0] += atoms.cell.array[0]
    check(4)
    atoms = Atoms([atoms.symbols[k] for k in (1, 0, 2)], atoms.positions[[1, 0, 2]], atoms.cell.array, atoms.pbc)
    check(5)
    atoms = Atoms(atoms.symbols[:2], atoms.positions[:2], atoms.cell.array, atoms.pbc)
    check(6)
    calc.set(neighbor_skin=0.1)
    check(7)
    calc.reset()
    check(8)
    calc.set(neighbor_backend="replicated")
    check(8)
    calc.set(neighbor_backend="ase")
    check(9)
    calc.set(neighbor_skin=0)
    check(10)
    check(11)


def test_pair_enters_cutoff_without_rebuild(ase_mod):
    from xreac_gb300 import ForceField

    calc = ase_mod.ReaxFFCalculator(ForceField.bundled("ffield.reax.ZnOH.2010"))
    rc = float(calc.core.force_field.general[12])
    atoms = Atoms(["Zn", "O"], [[0, 0, 0], [rc + 0.5, 0, 0]])
    calc.calculate(atoms)
    atoms.positions[:, 0] += [0.29, -0.29]
    calc.calculate(atoms)
    assert calc.neighbor_list_builds == 1
    assert calc.evaluation.energy != 0
    _same(calc.evaluation, calc.core.evaluate(["Zn", "O"], atoms.positions))
