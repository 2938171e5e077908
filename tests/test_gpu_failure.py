"""Failure paths of the QEq solver, in forms that fault and hang nothing.

- An iteration limit too small for the system ends the solve with the non-convergence error
  (``ValueError``), as a singular system does in the reference's direct solve
  (src/xreac/calculator.py:149-150).
- A bounded team wait that runs out (a test knob makes one wait for an arrival that never comes,
  after a small number of polls) ends the call with ``RuntimeError``; the same context then gives the
  normal result on the next call.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _water(n_mol, seed):
    from xreac_gb300 import workloads

    box = (n_mol / 64.0) ** (1.0 / 3.0) * 12.0
    return workloads.water_cluster(n_mol=n_mol, box=box, seed=seed)


def test_iteration_limit_raises_and_the_next_call_recovers():
    from xreac_gb300 import Calculator, ForceField

    ff = ForceField.bundled("ffield.reax.HO.2015")
    system = _water(64, 11)
    calc = Calculator(ff)
    want = calc.evaluate(system.symbols, system.positions)
    calc.set_qeq(max_iterations=1)
    with pytest.raises(ValueError, match="did not converge"):
        calc.evaluate(system.symbols, system.positions)
    calc.set_qeq()
    got = calc.evaluate(system.symbols, system.positions)
    assert got.energy == want.energy
    np.testing.assert_array_equal(got.charges, want.charges)


@pytest.mark.parametrize("n_mol", [70, 240])  # 210 atoms: a thread-block cluster; 720 atoms: a grid-wide team
@pytest.mark.parametrize("fail_at", [1, 12])  # the first team wait, and one inside the solve
def test_team_wait_that_runs_out_raises_and_the_context_recovers(n_mol, fail_at):
    from xreac_gb300 import Calculator, ForceField

    ff = ForceField.bundled("ffield.reax.HO.2015")
    system = _water(n_mol, 12)
    calc = Calculator(ff)
    want = calc.evaluate(system.symbols, system.positions)
    calc.set_wait_test(polls=2000, fail_at=fail_at)
    with pytest.raises(RuntimeError, match="gave up"):
        calc.evaluate(system.symbols, system.positions)
    calc.set_wait_test()
    got = calc.evaluate(system.symbols, system.positions)
    assert got.energy == want.energy
    np.testing.assert_array_equal(got.charges, want.charges)
    np.testing.assert_allclose(got.forces, want.forces, atol=1e-9, rtol=0)
