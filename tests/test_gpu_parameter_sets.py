"""Parameter sets: many variants of one force field in one device batch (an extension; xreac
evaluates one force field per call, src/xreac/calculator.py:99-160). Every system evaluated with its
own set must give what a calculator built from that variant alone gives, for energies, forces,
charges and parameter gradients; the per-set tables cover the atom (QEq chi and eta included), pair,
angle, torsion and hydrogen-bond values."""

import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ATOM_SCALED = ("chi", "eta", "p_lp2", "p_ovun2", "p_ovun5", "p_val3", "p_val5", "valency_boc")
PAIR_SCALED = ("De_s", "De_p", "De_pp", "p_be1", "p_be2", "p_ovun1", "p_bo1", "p_bo2", "p_bo3", "p_bo4", "p_bo5",
               "p_bo6", "D", "alpha", "gamma_w", "r_vdW", "p_boc3", "p_boc4", "p_boc5")


def perturb_everything(ff, seed, relative=0.03):
    """A copy of ``ff`` with atom, pair, angle, torsion and hydrogen-bond values scaled by
    1 +- ``relative`` (each shared record once)."""
    rng = np.random.default_rng(seed)
    out = copy.deepcopy(ff)
    seen = set()
    for prm in out.atoms.values():
        for name in ATOM_SCALED:
            if name in prm and prm[name] != 0:
                prm[name] *= 1.0 + rng.uniform(-relative, relative)
    for prm in out.pairs.values():
        if id(prm) in seen:
            continue
        seen.add(id(prm))
        for name in PAIR_SCALED:
            if name in prm and prm[name] != 0:
                prm[name] *= 1.0 + rng.uniform(-relative, relative)
    for table in (out.angles,):
        for records in table.values():
            for rec in records:
                if id(rec) not in seen:
                    seen.add(id(rec))
                    rec *= 1.0 + rng.uniform(-relative, relative, rec.shape)
    for table in (out.torsions, out.hydrogen_bonds):
        for rec in table.values():
            if id(rec) not in seen:
                seen.add(id(rec))
                rec *= 1.0 + rng.uniform(-relative, relative, np.shape(rec))
    return out


def _water_systems():
    from xreac_gb300 import workloads

    return [workloads.water_cluster(n_mol=40, box=11.0, seed=8, jitter=0.05),
            workloads.water_box(n_mol=64, box=12.4, seed=4),
            workloads.water_cluster(n_mol=6, box=6.0, seed=2, jitter=0.05)]


def _items(systems):
    return [dict(symbols=s.symbols, positions=s.positions, cell=s.cell, pbc=s.pbc, total_charge=s.total_charge)
            for s in systems]


def _close(got, want, n):
    assert got.energy == pytest.approx(want.energy, abs=1e-9 * n)
    np.testing.assert_allclose(got.charges, want.charges, atol=1e-10, rtol=0)
    np.testing.assert_allclose(got.forces, want.forces, atol=1e-8, rtol=0)


def test_every_table_per_set_matches_a_calculator_of_that_variant():
    from xreac_gb300 import Calculator, ForceField

    base = ForceField.bundled("ffield.reax.HO.2015")
    variants = [perturb_everything(base, seed) for seed in (1, 2, 3)]
    calc = Calculator(base)
    calc.load_parameter_sets(variants)
    assert calc.parameter_set_count == 4
    systems = _water_systems()
    # every system with every set, in one batch (set 0 is the calculator's own force field)
    items, sets = [], []
    for k in range(4):
        items += _items(systems)
        sets += [k] * len(systems)
    batch = calc.evaluate_many(items, parameter_sets=sets)
    for k, ff in enumerate([base] + variants):
        fresh = Calculator(ff)
        for q, s in enumerate(systems):
            got = batch[k * len(systems) + q]
            want = fresh.evaluate(s.symbols, s.positions, cell=s.cell, pbc=s.pbc)
            _close(got, want, len(s.symbols))
            if k:
                assert abs(got.energy - batch[q].energy) > 1e-3  # the variant changed the energy


def test_perturbed_copies_of_the_slab_in_one_batch():
    """The differentiation workload's copies (288-atom TiO2 slab + water, bond/angle/vdW values
    perturbed): one batch with a set per copy against a calculator per copy, full-derivative forces."""
    from xreac_gb300 import Calculator, ForceField, workloads

    base = ForceField.bundled("ffield.reax.TiOH.Kim2013")
    copies = list(workloads.perturbed_copies(n_copies=3))
    calc = Calculator(base)
    calc.load_parameter_sets([ff for _, ff in copies])
    items = _items([s for s, _ in copies])
    batch = calc.evaluate_many(items, parameter_sets=[1, 2, 3], full_derivative=True)
    for (s, ff), got in zip(copies, batch):
        want = Calculator(ff).evaluate(s.symbols, s.positions, cell=s.cell, pbc=s.pbc, full_derivative=True)
        _close(got, want, len(s.symbols))


def test_parameter_gradients_are_per_set():
    from xreac_gb300 import Calculator, ForceField
    from xreac_gb300.differentiation import ParameterVector

    base = ForceField.bundled("ffield.reax.HO.2015")
    variants = [perturb_everything(base, seed) for seed in (4, 5)]
    calc = Calculator(base)
    calc.load_parameter_sets(variants)
    vec = ParameterVector(base)
    systems = _water_systems()[:2]
    items = _items(systems) * 2
    sets = [1, 1, 2, 2]
    evs, grads = calc.parameter_gradient_many(items, per_system=True, parameter_sets=sets)
    _, pr, ar = calc.parameter_gradient_many(items, parameter_sets=sets, raw=True)
    rows = vec.gradient_rows(pr, ar)
    for k, (d, g) in enumerate(zip(items, grads)):
        fresh = Calculator(variants[sets[k] - 1])
        ev1, g1 = fresh.parameter_gradient(d["symbols"], d["positions"], cell=d["cell"], pbc=d["pbc"])
        want = vec.gradient(g1)
        np.testing.assert_allclose(vec.gradient(g), want, rtol=1e-10, atol=1e-8)
        np.testing.assert_allclose(rows[k], want, rtol=1e-10, atol=1e-8)


def test_parameter_set_arguments_are_checked():
    from xreac_gb300 import Calculator, ForceField

    base = ForceField.bundled("ffield.reax.HO.2015")
    calc = Calculator(base)
    s = _water_systems()[2]
    with pytest.raises(ValueError, match="out of range"):
        calc.evaluate_many(_items([s]), parameter_sets=[1])
    with pytest.raises(ValueError, match="one parameter set per system"):
        calc.evaluate_many(_items([s]), parameter_sets=[0, 0])
    other = copy.deepcopy(base)
    other.general[0] *= 1.01  # a new array of the copy, changed in place
    with pytest.raises(ValueError, match="general parameters"):
        calc.load_parameter_sets([other])
    with pytest.raises(ValueError, match="elements"):
        calc.load_parameter_sets([ForceField.bundled("ffield.reax.CHO.2008")])
    # update_force_field returns the device force field to a single set
    calc.load_parameter_sets([perturb_everything(base, 9)])
    assert calc.parameter_set_count == 2
    calc.update_force_field(perturb_everything(base, 10))
    assert calc.parameter_set_count == 1
    with pytest.raises(ValueError, match="out of range"):
        calc.evaluate_many(_items([s]), parameter_sets=[1])
