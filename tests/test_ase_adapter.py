"""The ASE adapter's own logic on CPU, with ASE (absent here) replaced by a minimal stand-in
(tests/ase_standin.py) and the device Calculator by a recorder.

Covered: parameter validation with xreac's messages (src/xreac/ase.py:75-96), the skin handed to
the device list and dropped by a reset or a changed parameter, the count of list builds taken
from the device's report, the backends, unit conversion and the initial-charge check
(src/xreac/ase.py:133-166). The device side of the lists is covered by tests/test_gpu_lists.py and
tests/test_gpu_ase_adapter.py.
"""

import numpy as np
import pytest

from ase_standin import KCAL, Atoms, install


class Recorder:
    """Stands in for xreac_gb300.Calculator: records calls, reports scripted list modes."""

    def __init__(self, force_field, max_expanded_atoms=512):
        self.force_field = force_field
        self.max_expanded_atoms = max_expanded_atoms
        self.calls, self.skins, self.modes = [], [], []
        self.neighbor_skin = 0.0
        self._mode = "scan"

    def set_neighbor_skin(self, skin):
        self.neighbor_skin = skin
        self.skins.append(skin)

    def list_info(self):
        return self._mode, 0

    def _evaluate_backend(self, symbols, positions, **kw):
        from xreac_gb300.calculator import Evaluation

        self.calls.append(kw)
        self._mode = self.modes.pop(0) if self.modes else "reused"
        n = len(symbols)
        return Evaluation(energy=-10.0, forces=np.ones((n, 3)), charges=np.zeros(n), components={},
                          full_derivative=kw["full_derivative"], total_bond_orders=np.zeros(n),
                          lone_pairs=np.zeros(n), bond_counts=np.zeros(n, dtype=int), dipole=np.zeros(3),
                          neighbor_backend=kw["backend"])


@pytest.fixture()
def adapter(monkeypatch):
    mod = install(monkeypatch)
    monkeypatch.setattr(mod, "Calculator", Recorder)
    return mod


def _water():
    return Atoms(["O", "H", "H"], [[0, 0, 0], [0.96, 0, 0], [-0.24, 0.93, 0]])


def _ff():
    from xreac_gb300 import ForceField

    return ForceField.bundled("ffield.reax.HO.2015")


def test_builds_follow_the_device_report_and_resets_drop_the_list(adapter):
    calc = adapter.ReaxFFCalculator(_ff(), neighbor_skin=0.3)
    atoms = _water()
    calc.core.modes = ["built", "reused", "built"]
    for _ in range(3):
        calc.calculate(atoms)
    assert calc.neighbor_list_builds == 2
    assert calc.core.neighbor_skin == 0.3 and calc.core.calls[-1]["backend"] == "ase"
    n = len(calc.core.skins)
    calc.reset()  # drops the device list: the skin is set again
    assert calc.core.skins[n:] == [0.3]
    calc.set(neighbor_skin=0.1)  # a changed parameter resets too
    assert calc.core.skins[-1] == 0.1
    calc.set(neighbor_skin=0.0)  # no skin: a search on every call, each counted
    calc.core.modes = ["scan", "scan"]
    calc.calculate(atoms)
    calc.calculate(atoms)
    assert calc.neighbor_list_builds == 4
    calc.set(neighbor_backend="replicated")
    calc.core.modes = ["scan"]
    calc.calculate(atoms)
    assert calc.core.calls[-1]["backend"] == "replicated" and calc.core.neighbor_skin == 0.0
    assert calc.neighbor_list_builds == 4  # builds count under the "ase" backend only
    assert calc.evaluation.neighbor_backend == "replicated"


def test_results_in_ase_units(adapter):
    calc = adapter.ReaxFFCalculator(_ff())
    calc.calculate(_water())
    assert calc.results["energy"] == pytest.approx(-10.0 * KCAL)
    np.testing.assert_allclose(calc.results["forces"], KCAL)
    assert calc.evaluation.neighbor_backend == "ase"
    assert calc.core.calls[-1]["full_derivative"] is False


@pytest.mark.parametrize("kwargs,message", [
    ({"neighbor_backend": "x"}, "neighbor_backend"), ({"neighbor_backend": None}, "neighbor_backend"),
    ({"neighbor_skin": -1.0}, "neighbor_skin"), ({"neighbor_skin": True}, "neighbor_skin"),
    ({"neighbor_skin": float("inf")}, "neighbor_skin"), ({"full_derivative": 1}, "full_derivative"),
    ({"total_charge": float("nan")}, "total_charge"), ({"unknown": 1}, "Unknown ReaxFF"),
    ({"max_expanded_atoms": 0}, "max_expanded_atoms")])
def test_invalid_parameters(adapter, kwargs, message):
    with pytest.raises(ValueError, match=message):
        adapter.ReaxFFCalculator(_ff(), **kwargs)


def test_initial_charges_must_sum_to_total(adapter):
    calc = adapter.ReaxFFCalculator(_ff())
    atoms = _water()
    atoms.charges = np.array([0.1, 0.0, 0.0])
    with pytest.raises(ValueError, match="Initial charges"):
        calc.calculate(atoms)
    atoms.charges = np.array([0.1, -0.1, 0.0])
    calc.calculate(atoms)


def test_an_adapter_around_an_existing_core(adapter):
    core = Recorder(_ff(), max_expanded_atoms=77)
    calc = adapter.ReaxFFCalculator.around(core, total_charge=1)
    assert calc.core is core and calc.parameters.max_expanded_atoms == 77 and calc.parameters.total_charge == 1
    calc.calculate(_water())
    assert core.calls[-1]["total_charge"] == 1
