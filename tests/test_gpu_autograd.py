"""Differentiation through the device adjoint: force-field updates in place, per-system parameter
gradients, the batched loss of the differentiation workload (its copies as parameter sets), and the
torch.autograd wrappers checked by torch.autograd.gradcheck in float64.

xreac differentiates its energy with HIPS autograd (src/xreac/calculator.py:141-148); here the
gradients come from the device's hand-written adjoint, so gradcheck compares them with central
differences of the device energy itself.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dimer():
    from xreac_gb300 import workloads

    return workloads.water_cluster(n_mol=2, box=4.5, min_oo=2.7, seed=3, jitter=0.05)


def test_force_field_update_in_place_equals_a_fresh_calculator():
    from xreac_gb300 import Calculator, workloads

    copies = list(workloads.perturbed_copies(n_copies=3))
    calc = Calculator(copies[0][1])
    for system, ff in copies[::-1]:
        calc.update_force_field(ff)
        got = calc.evaluate(system.symbols, system.positions, cell=system.cell, pbc=system.pbc)
        want = Calculator(ff).evaluate(system.symbols, system.positions, cell=system.cell, pbc=system.pbc)
        assert got.energy == want.energy
        np.testing.assert_array_equal(got.charges, want.charges)
        np.testing.assert_allclose(got.forces, want.forces, atol=1e-9, rtol=0)


def test_update_rejects_another_force_field():
    from xreac_gb300 import Calculator, ForceField

    calc = Calculator(ForceField.bundled("ffield.reax.HO.2015"))
    with pytest.raises(ValueError, match="same elements"):
        calc.update_force_field(ForceField.bundled("ffield.reax.CHO.2008"))


def test_per_system_gradients_equal_single_calls():
    from xreac_gb300 import Calculator, ForceField, workloads
    from xreac_gb300.differentiation import ParameterVector

    ff = ForceField.bundled("ffield.reax.HO.2015")
    calc = Calculator(ff)
    vec = ParameterVector(ff)
    systems = [workloads.water_cluster(n_mol=n, box=7.0, seed=30 + n, jitter=0.05) for n in (3, 5, 8)]
    items = [dict(symbols=s.symbols, positions=s.positions) for s in systems]
    evs, grads = calc.parameter_gradient_many(items, per_system=True)
    _, total = calc.parameter_gradient_many(items)
    acc = np.zeros(len(vec))
    for d, ev, g in zip(items, evs, grads):
        e1, g1 = calc.parameter_gradient(d["symbols"], d["positions"])
        assert ev.energy == e1.energy
        np.testing.assert_allclose(vec.gradient(g), vec.gradient(g1), rtol=1e-12, atol=1e-10)
        acc += vec.gradient(g)
    np.testing.assert_allclose(vec.gradient(total), acc, rtol=1e-12, atol=1e-10)


def test_batched_loss_of_perturbed_copies_matches_fresh_calculators():
    """perturbed_copies_loss (the copies as parameter sets of one device force field, three batched
    calls) against the same loss with a new calculator per copy and one system per call."""
    from xreac_gb300 import Calculator, ForceField, workloads
    from xreac_gb300.differentiation import energy_force_loss, perturbed_copies_loss

    base = ForceField.bundled("ffield.reax.TiOH.Kim2013")
    copies = list(workloads.perturbed_copies(n_copies=3))
    got = perturbed_copies_loss(copies, base)
    assert got.gradients.shape == (3, len(got.vector))
    ref = Calculator(base)
    for (s, ff), loss, grad in zip(copies, got.losses, got.gradients):
        r = ref.evaluate(s.symbols, s.positions, cell=s.cell, pbc=s.pbc)
        l1, g1, _ = energy_force_loss(Calculator(ff), s.symbols, s.positions, r.energy, r.forces, cell=s.cell,
                                      pbc=s.pbc)
        assert loss == pytest.approx(l1, rel=1e-10)
        np.testing.assert_allclose(grad, got.vector.gradient(g1), rtol=1e-7, atol=1e-6)


def test_energy_function_passes_gradcheck():
    """dE/dx (charge-response forces) and dE/dtheta (bond, angle, vdW parameters) of a water dimer
    against central differences of the device energy: torch.autograd.gradcheck in float64."""
    import torch
    from xreac_gb300 import Calculator, ForceField
    from xreac_gb300.differentiation import DeviceModel

    s = _dimer()
    model = DeviceModel(Calculator(ForceField.bundled("ffield.reax.HO.2015")), s.symbols)
    x = torch.tensor(s.positions, dtype=torch.float64, requires_grad=True)
    theta = model.theta0().requires_grad_(True)
    # h = 1e-5: the difference's truncation error (h^2 f''') and the energy's rounding over 2h
    # (about 1e-13 relative of ~500 kcal/mol) both stay below the tolerances
    assert torch.autograd.gradcheck(lambda a, b: model.energy(a, b), (x, theta), eps=1e-5, atol=2e-5, rtol=1e-4)
    e = model.energy(x, theta)
    e.backward()
    ev = model.calc.evaluate(s.symbols, s.positions, full_derivative=True)
    np.testing.assert_allclose(x.grad.numpy(), -ev.forces, atol=1e-12, rtol=0)


def test_energy_and_forces_function_passes_gradcheck():
    """(E, F)(x, theta): the backward pass's second derivatives (Hessian-vector products by one central
    difference of forces and parameter gradients) against gradcheck's own differences of the forward
    forces. Both are differences, so the tolerance is that of two O(h^2) estimates."""
    import torch
    from xreac_gb300 import Calculator, ForceField
    from xreac_gb300.differentiation import DeviceModel

    s = _dimer()
    model = DeviceModel(Calculator(ForceField.bundled("ffield.reax.HO.2015")), s.symbols)
    x = torch.tensor(s.positions, dtype=torch.float64, requires_grad=True)
    theta = model.theta0()
    idx = [k for k, e in enumerate(model.vector.entries) if e[0] == "pair" and e[1] in (("O", "H"), ("H", "O"))
           and e[2] in ("De_s", "p_bo1", "r_vdW", "alpha")]
    sub = theta[idx].clone().requires_grad_(True)

    def f(a, b):
        full = theta.clone()
        full[idx] = b
        return model.energy_forces(a, full, 1e-4)

    assert torch.autograd.gradcheck(f, (x, sub), eps=1e-5, atol=2e-3, rtol=2e-3)
