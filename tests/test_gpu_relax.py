"""Fixed-charge relaxation (``Calculator.relax``), after xreac's tests/test_calculator.py:67-101.

The native backend's trajectory is also checked step by step against the same FIRE recurrence
driven by the CPU oracle's forces (oracle/reaxff_oracle.py) on a 20-atom Zn/O cluster.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ZNO = (["Zn", "O"], [[0, 0, 0], [1.9, 0, 0]])


def _cluster20():
    # the reference's 20-atom validation cluster recipe (tests/cases.py:6-12): a cubic lattice of
    # alternating Zn/O at 2.15 A with 0.025 A seeded noise
    side = 3
    ijk = np.array(list(np.ndindex(side, side, side)))[:20]
    rng = np.random.default_rng(1729 + 20)
    symbols = ["Zn" if row.sum() % 2 == 0 else "O" for row in ijk]
    return symbols, ijk * 2.15 + rng.normal(0, 0.025, (20, 3))


@pytest.fixture(scope="module")
def calc():
    from xreac_gb300 import Calculator, ForceField

    return Calculator(ForceField.bundled("ffield.reax.ZnOH.2010"))


def test_relaxation_native(calc):
    symbols, x = ZNO
    x = np.array(x, dtype=float)
    initial = calc.evaluate(symbols, x)
    result = calc.relax(symbols, x, force_tolerance=1e-5, backend="native")
    assert result.converged, result.message
    assert result.evaluation.full_derivative is False
    assert result.evaluation.force_convention == "fixed_charge"
    assert result.evaluation.energy < initial.energy
    assert np.max(abs(result.evaluation.forces)) <= 1e-5
    np.testing.assert_array_equal(result.evaluation.forces, calc.evaluate(symbols, result.positions).forces)
    short = calc.relax(symbols, x, force_tolerance=1e-12, max_iterations=1, backend="native")
    assert not short.converged
    assert short.iterations == 1
    assert short.evaluation.full_derivative is False
    assert np.max(abs(short.evaluation.forces)) > 1e-12
    np.testing.assert_array_equal(x, [[0, 0, 0], [1.9, 0, 0]])


def test_relaxation_already_converged(calc):
    result = calc.relax(["Zn"], [[1.0, 2.0, 3.0]], max_iterations=1, backend="native")
    assert result.converged and result.iterations == 0
    assert result.evaluation.full_derivative is False
    np.testing.assert_array_equal(result.positions, [[1.0, 2.0, 3.0]])


@pytest.mark.parametrize(
    "kwargs",
    [
        {"force_tolerance": 0},
        {"force_tolerance": float("nan")},
        {"max_iterations": 0},
        {"max_iterations": 1.5},
        {"max_iterations": True},
        {"backend": "unknown"},
    ],
)
def test_invalid_relaxation_settings(calc, kwargs):
    with pytest.raises(ValueError):
        calc.relax(*ZNO, **kwargs)


def test_ase_backend_needs_ase(calc):
    try:
        import ase  # noqa: F401
    except ImportError:
        with pytest.raises(ImportError):
            calc.relax(*ZNO, backend="ase")
    else:
        result = calc.relax(*ZNO, force_tolerance=1e-5, backend="ase")
        assert result.converged


def test_native_trajectory_matches_oracle_fire(calc):
    """Ten FIRE steps on the device against the same recurrence on the oracle's forces."""
    from oracle import evaluate as oracle_evaluate
    from xreac_gb300 import ForceField

    ff = ForceField.bundled("ffield.reax.ZnOH.2010")
    symbols, x0 = _cluster20()
    steps = 10
    res = calc.relax(symbols, x0, force_tolerance=1e-12, max_iterations=steps, backend="native")
    assert not res.converged and res.iterations == steps
    # the FIRE recurrence of xreac's native backend (src/xreac/calculator.py:213-246) on oracle forces
    x = np.array(x0, dtype=float)
    v = np.zeros_like(x)
    dt, alpha, positive = 0.02, 0.1, 0
    for it in range(steps):
        f = oracle_evaluate(ff, symbols, x)["forces"]
        power = float(np.sum(v * f))
        if power > 0:
            v = (1 - alpha) * v + alpha * np.linalg.norm(v) / np.linalg.norm(f) * f
            positive += 1
            if positive > 5:
                dt = min(dt * 1.1, 0.2)
                alpha *= 0.99
        else:
            v[:] = 0
            positive = 0
            alpha = 0.1
            if it > 0:
                dt *= 0.5
        v += dt * f
        d = dt * v
        big = np.max(np.linalg.norm(d, axis=1))
        if big > 0.1:
            d *= 0.1 / big
        x = x + d
    np.testing.assert_allclose(res.positions, x, atol=1e-9, rtol=0)
    ref = oracle_evaluate(ff, symbols, x)
    assert res.evaluation.energy == pytest.approx(ref["energy"], rel=1e-8)
