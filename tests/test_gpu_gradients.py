"""Force-field parameter gradients (device adjoint) against central finite differences.

dE/dtheta for bond, angle and vdW parameters and the gradient of an energy + force squared-error
loss are checked against central differences of the device energies with the parameter moved by
+-h (relative h = 1e-6), on a water cluster and on the TiO2/water slab of the differentiation
workload (ffield.reax.TiOH.Kim2013), and against central differences of the CPU oracle's energies
(the reference's algorithm restated and pinned to reference-written fixtures) under the same
modified force field.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _water(n_mol=6, seed=8):
    from xreac_gb300.workloads import water_cluster

    return water_cluster(n_mol=n_mol, box=7.0, min_oo=2.6, seed=seed, jitter=0.05)


def _fd(ff_name, system, setter, h, quantity):
    from xreac_gb300 import Calculator, ForceField

    vals = []
    for sgn in (1, -1):
        ff = ForceField.bundled(ff_name)
        setter(ff, sgn * h)
        r = Calculator(ff).evaluate(system.symbols, system.positions, cell=system.cell, pbc=system.pbc)
        vals.append(quantity(r))
    return (vals[0] - vals[1]) / (2 * h)


def _pair_setter(s, t, name, base):
    def setter(ff, d):
        ff.pairs[s, t][name] = base + d
    return setter


def _angle_setter(key, q, k, base):
    def setter(ff, d):
        ff.angles[key][q][k] = base + d
    return setter


PAIRS_HO = [("O", "H", n) for n in ("De_s", "De_p", "p_be1", "p_be2", "p_ovun1", "p_bo1", "p_bo2", "r_s", "D",
                                     "alpha", "gamma_w", "r_vdW")]
PAIRS_HO += [("O", "O", "D"), ("O", "O", "r_vdW"), ("H", "H", "alpha"), ("O", "O", "p_bo1"), ("O", "O", "p_bo3"),
             ("O", "O", "r_p")]


@pytest.mark.parametrize("s,t,name", PAIRS_HO)
def test_pair_parameter_gradient_water(s, t, name):
    from xreac_gb300 import Calculator, ForceField

    system = _water()
    ff = ForceField.bundled(system.force_field)
    _, grad = Calculator(ff).parameter_gradient(system.symbols, system.positions)
    base = ff.pairs[s, t][name]
    h = 1e-6 * max(abs(base), 1e-3)
    fd = _fd(system.force_field, system, _pair_setter(s, t, name, base), h, lambda r: r.energy)
    assert grad.pairs[s, t][name] == pytest.approx(fd, rel=2e-5, abs=2e-6)


def test_angle_parameter_gradient_water():
    from xreac_gb300 import Calculator, ForceField

    system = _water()
    ff = ForceField.bundled(system.force_field)
    _, grad = Calculator(ff).parameter_gradient(system.symbols, system.positions)
    key = ("H", "O", "H")
    checked = 0
    for k in range(7):
        base = float(ff.angles[key][0][k])
        if base == 0.0:
            continue
        h = 1e-6 * abs(base)
        fd = _fd(system.force_field, system, _angle_setter(key, 0, k, base), h, lambda r: r.energy)
        assert grad.angles[key][0][k] == pytest.approx(fd, rel=2e-5, abs=2e-6), k
        checked += 1
    assert checked >= 4


def test_parameter_gradient_anatase_slab():
    from xreac_gb300 import Calculator, ForceField
    from xreac_gb300.workloads import anatase_slab_water

    system = anatase_slab_water(displacement=0.05)
    ff = ForceField.bundled(system.force_field)
    _, grad = Calculator(ff).parameter_gradient(system.symbols, system.positions, cell=system.cell, pbc=system.pbc)
    for s, t, name in (("Ti", "O", "De_s"), ("Ti", "O", "p_bo2"), ("Ti", "O", "D"), ("Ti", "O", "r_vdW"),
                       ("O", "H", "p_be2")):
        base = ff.pairs[s, t][name]
        h = 1e-6 * max(abs(base), 1e-3)
        fd = _fd(system.force_field, system, _pair_setter(s, t, name, base), h, lambda r: r.energy)
        assert grad.pairs[s, t][name] == pytest.approx(fd, rel=2e-5, abs=1e-5), (s, t, name)
    # an angle record that the slab uses
    key = next(k for k in (("O", "Ti", "O"), ("Ti", "O", "Ti")) if k in ff.angles)
    for k in (1, 2):
        base = float(ff.angles[key][0][k])
        h = 1e-6 * max(abs(base), 1e-3)
        fd = _fd(system.force_field, system, _angle_setter(key, 0, k, base), h, lambda r: r.energy)
        assert grad.angles[key][0][k] == pytest.approx(fd, rel=2e-5, abs=1e-5), (key, k)


def test_energy_force_loss_gradient():
    """The differentiation workload's loss: perturbed parameters against the unperturbed result."""
    from xreac_gb300 import Calculator, ForceField
    from xreac_gb300.differentiation import energy_force_loss

    system = _water(n_mol=5, seed=9)
    ref = Calculator(ForceField.bundled(system.force_field)).evaluate(system.symbols, system.positions)
    perturb = {("O", "H", "De_s"): 1.02, ("O", "H", "p_bo1"): 0.98, ("O", "O", "D"): 1.02, ("H", "H", "r_vdW"): 0.98}

    def make_ff(extra=None):
        ff = ForceField.bundled(system.force_field)
        for (s, t, n), f in perturb.items():
            ff.pairs[s, t][n] *= f
        if extra:
            extra(ff)
        return ff

    def loss_of(ff):
        r = Calculator(ff).evaluate(system.symbols, system.positions)
        return (r.energy - ref.energy) ** 2 + float(np.sum((r.forces - ref.forces) ** 2))

    loss, grad, _ = energy_force_loss(Calculator(make_ff()), system.symbols, system.positions, ref.energy, ref.forces)
    assert loss == pytest.approx(loss_of(make_ff()), rel=1e-10)
    for s, t, name in (("O", "H", "De_s"), ("O", "H", "p_bo1"), ("O", "O", "D"), ("H", "H", "r_vdW"),
                       ("O", "H", "alpha")):
        base = make_ff().pairs[s, t][name]
        h = 1e-5 * abs(base)

        def shifted(d):
            def f(ff):
                ff.pairs[s, t][name] = base + d
            return f

        fd = (loss_of(make_ff(shifted(h))) - loss_of(make_ff(shifted(-h)))) / (2 * h)
        assert grad.pairs[s, t][name] == pytest.approx(fd, rel=1e-4, abs=1e-4 * max(1.0, abs(fd))), (s, t, name)


def _oracle_fd(system, setter, h):
    """Central difference of the oracle's energy with a force-field parameter moved by +-h."""
    import oracle
    from xreac_gb300 import ForceField

    vals = []
    for sgn in (1, -1):
        ff = ForceField.bundled(system.force_field)
        setter(ff, sgn * h)
        vals.append(oracle.evaluate(ff, system.symbols, system.positions, cell=system.cell, pbc=system.pbc,
                                    need_forces=False, dense_bond_orders=False)["energy"])
    return (vals[0] - vals[1]) / (2 * h)


ORACLE_PAIRS = [("O", "H", "De_s"), ("O", "H", "p_be1"), ("O", "H", "p_ovun1"), ("O", "H", "p_bo1"),
                ("O", "H", "p_bo2"), ("O", "H", "r_s"), ("O", "H", "D"), ("O", "H", "alpha"), ("O", "H", "gamma_w"),
                ("O", "O", "r_vdW"), ("O", "O", "p_bo3"), ("H", "H", "alpha")]


@pytest.mark.parametrize("s,t,name", ORACLE_PAIRS)
def test_pair_parameter_gradient_against_oracle(s, t, name):
    """The device adjoint dE/dtheta against central differences of the oracle on 5 H2O (15 atoms)."""
    from xreac_gb300 import Calculator, ForceField

    system = _water(n_mol=5, seed=9)
    ff = ForceField.bundled(system.force_field)
    _, grad = Calculator(ff).parameter_gradient(system.symbols, system.positions)
    base = ff.pairs[s, t][name]
    h = 1e-6 * max(abs(base), 1e-3)
    fd = _oracle_fd(system, _pair_setter(s, t, name, base), h)
    assert grad.pairs[s, t][name] == pytest.approx(fd, rel=2e-5, abs=2e-6), (s, t, name)


def test_angle_parameter_gradient_against_oracle():
    from xreac_gb300 import Calculator, ForceField

    system = _water(n_mol=5, seed=9)
    ff = ForceField.bundled(system.force_field)
    _, grad = Calculator(ff).parameter_gradient(system.symbols, system.positions)
    key = ("H", "O", "H")
    checked = 0
    for k in range(7):
        base = float(ff.angles[key][0][k])
        if base == 0.0:
            continue
        fd = _oracle_fd(system, _angle_setter(key, 0, k, base), 1e-6 * abs(base))
        assert grad.angles[key][0][k] == pytest.approx(fd, rel=2e-5, abs=2e-6), k
        checked += 1
    assert checked >= 4


def _atom_setter(s, name, base):
    def setter(ff, d):
        ff.atoms[s][name] = base + d
    return setter


@pytest.mark.parametrize("periodic", [False, True])
def test_qeq_parameter_gradients_against_oracle(periodic):
    """chi and eta of each element and the pair table's gamma (qeq=True: the charges' response
    through an adjoint QEq solve) against central differences of the oracle's energies, whose dense
    KKT solve re-solves the charges for every modified force field. A charged water cluster, and a
    periodic water box."""
    from xreac_gb300 import Calculator, ForceField, workloads
    from xreac_gb300.workloads import System

    if periodic:
        system = workloads.water_box(n_mol=64, box=12.4, seed=11)
    else:
        base_sys = _water(n_mol=5, seed=9)
        system = System(base_sys.symbols, base_sys.positions, None, False, 1.0, base_sys.force_field)
    ff = ForceField.bundled(system.force_field)
    calc = Calculator(ff)
    ev, grad = calc.parameter_gradient(system.symbols, system.positions, cell=system.cell, pbc=system.pbc,
                                       total_charge=system.total_charge, qeq=True)
    _, plain = calc.parameter_gradient(system.symbols, system.positions, cell=system.cell, pbc=system.pbc,
                                       total_charge=system.total_charge)
    assert plain.atoms == {} and "gamma" not in plain.pairs["O", "H"]

    def oracle_fd(setter, h):
        import oracle

        vals = []
        for sgn in (1, -1):
            f = ForceField.bundled(system.force_field)
            setter(f, sgn * h)
            vals.append(oracle.evaluate(f, system.symbols, system.positions, cell=system.cell, pbc=system.pbc,
                                        total_charge=system.total_charge, need_forces=False,
                                        dense_bond_orders=False)["energy"])
        return (vals[0] - vals[1]) / (2 * h)

    for s in ("O", "H"):
        for name in ("chi", "eta"):
            base = ff.atoms[s][name]
            fd = oracle_fd(_atom_setter(s, name, base), 1e-6 * abs(base))
            assert grad.atoms[s][name] == pytest.approx(fd, rel=1e-5, abs=1e-5), (s, name)
    for s, t in (("O", "H"), ("O", "O"), ("H", "H")):
        base = ff.pairs[s, t]["gamma"]
        fd = oracle_fd(_pair_setter(s, t, "gamma", base), 1e-6 * abs(base))
        assert grad.pairs[s, t]["gamma"] == pytest.approx(fd, rel=1e-5, abs=1e-5), (s, t)
    # the other parameters' gradients do not change with qeq=True
    assert grad.pairs["O", "H"]["De_s"] == pytest.approx(plain.pairs["O", "H"]["De_s"], rel=1e-12)
