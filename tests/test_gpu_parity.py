"""Parity of the CUDA path (through the C ABI) with the reference and the CPU oracle.

Tolerances: the reference's own strict backend-equivalence limits (xreac scripts/validate.py:122-146:
energy and components per atom 1e-9, forces 2e-8, charges and bond orders 1e-10, counts exact,
dipole 1e-9), the stated limits of the evaluation path (energy 1e-8 relative, forces 1e-6
kcal/mol/A, charges 1e-8 e), and exact neighbour lists.
"""

import hashlib

import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

COMP = ("bond atom lone_pair molecule angle penalty angle_conjugation hydrogen_bond torsion conjugation vdw coulomb "
        "electric_field qeq").split()
_CALCS = {}


def calc(ff_name):
    from xreac_gb300 import Calculator, ForceField

    if ff_name not in _CALCS:
        _CALCS[ff_name] = Calculator(ForceField.bundled(ff_name))
    return _CALCS[ff_name]


def check_strict(r, g, n):
    E = float(g["energy"])
    assert abs(r.energy - E) / n <= 1e-9
    assert abs(r.energy - E) <= 1e-8 * max(1.0, abs(E))
    comps = np.array([r.components[k] for k in COMP])
    assert np.max(np.abs(comps - g["components"])) / n <= 1e-9
    np.testing.assert_allclose(r.forces, g["forces"], atol=2e-8, rtol=0)
    np.testing.assert_allclose(r.charges, g["charges"], atol=1e-10, rtol=0)
    np.testing.assert_allclose(r.total_bond_orders, g["total_bond_orders"], atol=1e-10, rtol=0)
    np.testing.assert_allclose(r.lone_pairs, g["lone_pairs"], atol=1e-10, rtol=0)
    np.testing.assert_array_equal(r.bond_counts, g["bond_counts"])
    np.testing.assert_allclose(r.dipole, g["dipole"], atol=1e-9, rtol=0)
    assert tuple(r.cell_repetitions) == tuple(int(v) for v in g["cell_repetitions"])
    assert abs(r.charges.sum() - g["total_charge"]) <= 1e-8


def canonical_bonds(r):
    i, j, S, bo = r.bonds
    # both directions of every bond, in canonical (i, j, S) order, nonzero only
    ii = np.concatenate((i, j))
    jj = np.concatenate((j, i))
    SS = np.concatenate((S, -S))
    bb = np.concatenate((bo, bo))
    keep = bb != 0
    ii, jj, SS, bb = ii[keep], jj[keep], SS[keep], bb[keep]
    order = np.lexsort((SS[:, 2], SS[:, 1], SS[:, 0], jj, ii))
    return ii[order], jj[order], SS[order], bb[order]


@pytest.mark.parametrize("name", [n for n in golden_names() if not n.endswith("_full") and not n.startswith("supplied_")])
def test_reference_fixture(name):
    g = load_golden(name)
    c = calc(g["ff"])
    r = c.evaluate(g["symbols"], g["positions"], cell=g["cell"], pbc=g["pbc"], total_charge=g["total_charge"])
    check_strict(r, g, len(g["symbols"]))
    # neighbour list: the reference's canonical (i, j, S), exactly
    i, j, S = c.neighbor_list()
    canon = np.column_stack((i, j, S)).astype(np.int32)
    assert len(canon) == int(g["edge_count"])
    assert hashlib.sha256(np.ascontiguousarray(canon).tobytes()).hexdigest() == str(g["edge_sha256"])
    # per-edge corrected bond orders
    bi, bj, bS, bo = canonical_bonds(r)
    np.testing.assert_allclose(bo, g["bo_value"], atol=1e-10, rtol=0)
    if "bond_orders" in g:
        np.testing.assert_allclose(r.bond_orders, g["bond_orders"], atol=1e-10, rtol=0)
    assert c.last_launches > 0


def test_release_known_answers():
    """The reference's release check (.github/workflows/release.yml:77-87)."""
    c = calc("ffield.reax.HO.2015")
    r = c.evaluate(["O", "H", "H"], [[0, 0, 0], [0.97, 0, 0], [-0.243, 0.94, 0]])
    assert abs(r.energy - (-248.34420920633704)) < 1e-8
    assert np.isfinite(r.forces).all() and abs(r.charges.sum()) < 1e-12
    ion = c.evaluate(["O", "H"], [[0, 0, 0], [0.97, 0, 0]], total_charge=-1)
    assert abs(ion.charges.sum() + 1) < 1e-12


@pytest.fixture(scope="module")
def water_4608():
    from xreac_gb300 import workloads

    return workloads.water_box()


@pytest.mark.parametrize("name", [n for n in golden_names() if n.endswith("_full")])
def test_reference_fixture_charge_response(name):
    """full_derivative=True: forces through the QEq solve (adjoint solve on the device)."""
    g = load_golden(name)
    c = calc(g["ff"])
    r = c.evaluate(g["symbols"], g["positions"], cell=g["cell"], pbc=g["pbc"], total_charge=g["total_charge"],
                   full_derivative=True)
    assert r.full_derivative and r.force_convention == "charge_response"
    check_strict(r, g, len(g["symbols"]))


def test_fixed_and_charge_response_forces_differ():
    """tests/test_calculator.py:14-28 and 109-119 of the reference: the two conventions differ by more
    than 0.03 kcal/mol/A on a distorted water dimer, and the charge-response forces match central
    finite differences of the energy."""
    g = load_golden("water_distorted_dimer")
    c = calc(g["ff"])
    fixed = c.evaluate(g["symbols"], g["positions"])
    full = c.evaluate(g["symbols"], g["positions"], full_derivative=True)
    assert np.abs(fixed.forces - full.forces).max() > 0.03
    h = 1e-5
    x = np.array(g["positions"], dtype=float)
    for a, d in ((0, 0), (1, 2), (3, 1)):
        xp, xm = x.copy(), x.copy()
        xp[a, d] += h
        xm[a, d] -= h
        fd = -(c.evaluate(g["symbols"], xp).energy - c.evaluate(g["symbols"], xm).energy) / (2 * h)
        assert abs(full.forces[a, d] - fd) < 1e-5


def test_full_size_water_box_against_oracle(water_4608):
    """The 1,536-H2O (4,608-atom) periodic water box against the CPU oracle."""
    from oracle import evaluate as oracle_evaluate
    from xreac_gb300 import ForceField

    s = water_4608
    c = calc(s.force_field)
    r = c.evaluate(s.symbols, s.positions, cell=s.cell, pbc=s.pbc)
    o = oracle_evaluate(ForceField.bundled(s.force_field), s.symbols, s.positions, cell=s.cell, pbc=s.pbc,
                        dense_bond_orders=False)
    n = len(s.symbols)
    assert abs(r.energy - o["energy"]) <= 1e-8 * abs(o["energy"])
    comps = np.array([r.components[k] for k in COMP])
    ocomps = np.array([o["components"][k] for k in COMP])
    assert np.max(np.abs(comps - ocomps)) / n <= 1e-9
    np.testing.assert_allclose(r.forces, o["forces"], atol=1e-6, rtol=0)
    np.testing.assert_allclose(r.charges, o["charges"], atol=1e-8, rtol=0)
    np.testing.assert_allclose(r.total_bond_orders, o["total_bond_orders"], atol=1e-10, rtol=0)
    np.testing.assert_array_equal(r.bond_counts, o["bond_counts"])
    i, j, S = c.neighbor_list()
    oi, oj, oS = o["neighbors"]
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(j, oj)
    np.testing.assert_array_equal(S, oS)


def test_full_size_properties(water_4608):
    """Size-independent properties at full size: momentum, charge, determinism, invariances."""
    s = water_4608
    c = calc(s.force_field)
    a = c.evaluate(s.symbols, s.positions, cell=s.cell, pbc=s.pbc)
    b = c.evaluate(s.symbols, s.positions, cell=s.cell, pbc=s.pbc)
    assert a.energy == b.energy  # deterministic reductions
    np.testing.assert_array_equal(a.charges, b.charges)
    # forces repeat to the last bits only (the many-body kernels add with atomics): a few ulps
    np.testing.assert_allclose(a.forces, b.forces, atol=1e-12, rtol=1e-13)
    assert abs(a.charges.sum()) < 1e-10
    np.testing.assert_allclose(a.forces.sum(axis=0), 0.0, atol=1e-8)
    # periodic wrapping and translation leave the physics unchanged
    rng = np.random.default_rng(900)
    shift = rng.integers(-2, 3, s.positions.shape) @ s.cell
    w = c.evaluate(s.symbols, s.positions + shift + [0.37, -1.1, 2.3], cell=s.cell, pbc=s.pbc)
    assert w.energy == pytest.approx(a.energy, rel=1e-11)
    np.testing.assert_allclose(w.forces, a.forces, atol=1e-8, rtol=0)
    np.testing.assert_allclose(w.charges, a.charges, atol=1e-10, rtol=0)
    # permutation
    order = rng.permutation(len(s.symbols))
    p = c.evaluate([s.symbols[k] for k in order], s.positions[order], cell=s.cell, pbc=s.pbc)
    assert p.energy == pytest.approx(a.energy, rel=1e-11)
    np.testing.assert_allclose(p.forces, a.forces[order], atol=1e-8, rtol=0)


def test_cho_mixture_full_size_against_oracle():
    """The 3,300-atom C/H/O mixture box (300 CH4, 300 O2, 300 H2O, 100 CO2 at 0.6 g/cm3, CHO.2008)
    against the CPU oracle at the evaluation path's stated limits (energy 1e-8 relative, components
    1e-9 per atom, forces 1e-6 kcal/mol/A, charges 1e-8 e, exact neighbour arrays); every term active."""
    from oracle import evaluate as oracle_evaluate
    from xreac_gb300 import ForceField, workloads

    s = workloads.cho_mixture()
    c = calc(s.force_field)
    r = c.evaluate(s.symbols, s.positions, cell=s.cell, pbc=s.pbc)
    o = oracle_evaluate(ForceField.bundled(s.force_field), s.symbols, s.positions, cell=s.cell, pbc=s.pbc,
                        dense_bond_orders=False)
    n = len(s.symbols)
    assert n == 3300
    assert abs(r.energy - o["energy"]) <= 1e-8 * abs(o["energy"])
    comps = np.array([r.components[k] for k in COMP])
    ocomps = np.array([o["components"][k] for k in COMP])
    assert np.max(np.abs(comps - ocomps)) / n <= 1e-9
    np.testing.assert_allclose(r.forces, o["forces"], atol=1e-6, rtol=0)
    np.testing.assert_allclose(r.charges, o["charges"], atol=1e-8, rtol=0)
    np.testing.assert_allclose(r.total_bond_orders, o["total_bond_orders"], atol=1e-10, rtol=0)
    np.testing.assert_array_equal(r.bond_counts, o["bond_counts"])
    i, j, S = c.neighbor_list()
    oi, oj, oS = o["neighbors"]
    np.testing.assert_array_equal(i, oi)
    np.testing.assert_array_equal(j, oj)
    np.testing.assert_array_equal(S, oS)
    for k in ("angle", "torsion", "hydrogen_bond", "bond", "lone_pair", "atom", "vdw", "coulomb", "penalty",
              "conjugation"):
        assert r.components[k] != 0.0, k
    assert abs(r.charges.sum()) < 1e-10
    np.testing.assert_allclose(r.forces.sum(axis=0), 0.0, atol=1e-7)


def test_cho_mixture_charge_response_forces_by_finite_differences():
    """Central differences of the device energy (charges re-solved at every point) against the
    charge-response forces of the 3,300-atom box, on a C, an O and an H coordinate. h = 1e-4 A; the
    difference's own error (h^2 times the third derivative, plus energy rounding over 2h) stays below
    the 1e-4 kcal/mol/A allowed."""
    from xreac_gb300 import workloads

    s = workloads.cho_mixture()
    c = calc(s.force_field)
    full = c.evaluate(s.symbols, s.positions, cell=s.cell, pbc=s.pbc, full_derivative=True)
    x = np.array(s.positions, dtype=float)
    picks = [s.symbols.index("C"), s.symbols.index("O") + 1, s.symbols.index("H") + 2]
    h = 1e-4
    for a, d in zip(picks, (0, 1, 2)):
        xp, xm = x.copy(), x.copy()
        xp[a, d] += h
        xm[a, d] -= h
        fd = -(c.evaluate(s.symbols, xp, cell=s.cell, pbc=s.pbc).energy
               - c.evaluate(s.symbols, xm, cell=s.cell, pbc=s.pbc).energy) / (2 * h)
        assert abs(full.forces[a, d] - fd) < 1e-4, (a, d, full.forces[a, d], fd)


def test_batch_matches_single_evaluations():
    """A ragged batch gives each system the result it has alone."""
    names = ["cluster_water_192", "periodic_partial_pbc_water", "charged_water_4A", "water_monomer", "stream_08",
             "periodic_boundary_dimer"]
    cases = [load_golden(n) for n in names]
    c = calc("ffield.reax.HO.2015")
    systems = [dict(symbols=g["symbols"], positions=g["positions"], cell=g["cell"], pbc=g["pbc"],
                    total_charge=g["total_charge"]) for g in cases if g["ff"] == "ffield.reax.HO.2015"]
    batch = c.evaluate_many(systems)
    for s, rb in zip(systems, batch):
        r1 = c.evaluate(**s)
        assert rb.energy == pytest.approx(r1.energy, abs=1e-9 * len(s["symbols"]))
        np.testing.assert_allclose(rb.forces, r1.forces, atol=1e-9, rtol=0)
        np.testing.assert_allclose(rb.charges, r1.charges, atol=1e-11, rtol=0)


def test_batch_solver_layouts_agree():
    """The same systems through every QEq layout: alone, a 1,000-atom periodic box is solved by a
    grid-wide team and a 300-atom cluster by one thread-block cluster; in a batch the box goes to a
    cluster whose blocks' FP32 rows exceed shared memory (rows from global memory), and a small
    system to a single block. Charges agree to the solver tolerance, energies and forces to rounding."""
    from xreac_gb300 import workloads

    box = workloads.water_box(n_mol=334, box=21.6, seed=21)
    clus = workloads.water_cluster(n_mol=100, box=14.0, seed=5)
    small = workloads.water_cluster(n_mol=8, box=6.0, seed=5)
    c = calc("ffield.reax.HO.2015")
    systems = [dict(symbols=s.symbols, positions=s.positions, cell=s.cell, pbc=s.pbc) for s in (box, clus, small)]
    assert len(box.symbols) == 1002 and len(clus.symbols) == 300
    batch = c.evaluate_many(systems)
    for s, rb in zip(systems, batch):
        r1 = c.evaluate(**s)
        n = len(s["symbols"])
        assert rb.energy == pytest.approx(r1.energy, abs=1e-9 * n)
        np.testing.assert_allclose(rb.charges, r1.charges, atol=1e-10, rtol=0)
        np.testing.assert_allclose(rb.forces, r1.forces, atol=1e-8, rtol=0)
        assert abs(rb.charges.sum()) < 1e-10


def test_symmetries_cluster():
    """Rotation, translation and permutation (tests/test_calculator.py:77-90 of the reference)."""
    g = load_golden("zno_cluster20")
    c = calc(g["ff"])
    x = g["positions"]
    sym = g["symbols"]
    rot, _ = np.linalg.qr(np.random.default_rng(33).normal(size=(3, 3)))
    r = c.evaluate(sym, x)
    moved = c.evaluate(sym, x @ rot + [4.2, -3.1, 7])
    assert moved.energy == pytest.approx(r.energy, abs=1e-10)
    np.testing.assert_allclose(moved.forces, r.forces @ rot, atol=1e-9)
    order = np.random.default_rng(33).permutation(len(x))
    perm = c.evaluate([sym[k] for k in order], x[order])
    assert perm.energy == pytest.approx(r.energy, abs=1e-10)
    np.testing.assert_allclose(perm.charges, r.charges[order], atol=1e-12)
    np.testing.assert_allclose(perm.forces, r.forces[order], atol=1e-9)


@pytest.mark.parametrize(
    "symbols,x,kwargs",
    [
        ([], [], {}),
        (["He"], [[0, 0, 0]], {}),
        (["He"], [[0, 0, 0]], {"cell": [4.0] * 3}),
        (["Zn", "O"], [[0, 0, 0], [0, 0, 0]], {}),
        (["Zn"], [[np.nan, 0, 0]], {}),
        (["Zn"], [[0, 0]], {}),
        (["Zn"], [[0, 0, 0]], {"total_charge": float("nan")}),
        (["Zn"], [[0, 0, 0]], {"cell": np.eye(3)}),
        (["Zn"], [[0, 0, 0]], {"full_derivative": "false"}),
    ],
)
def test_invalid_input(symbols, x, kwargs):
    """Invalid inputs raise ValueError (tests/test_calculator.py:93-109 of the reference)."""
    c = calc("ffield.reax.ZnOH.2010")
    with pytest.raises(ValueError):
        c.evaluate(symbols, x, **kwargs)


def test_coincident_atoms_in_periodic_image():
    c = calc("ffield.reax.HO.2015")
    with pytest.raises(ValueError, match="Coincident"):
        c.evaluate(["O", "H"], [[0.0, 0, 0], [12.0, 0, 0]], cell=[12.0] * 3)


def test_collinear_active_torsion():
    """tests/test_general.py:545-562 of the reference."""
    c = calc("ffield.reax.CHO.2008")
    with pytest.raises(ValueError, match="Collinear atoms in an active torsion"):
        c.evaluate(["C"] * 4, [[0, 0, 0], [1.5, 0, 0], [3, 0, 0], [4.5, 0.3, 0]])


def test_small_cell_memory_limit():
    """tests/test_small_cells.py:200-204 of the reference."""
    from xreac_gb300 import Calculator, ForceField

    g = load_golden("water_monomer")
    with pytest.raises(ValueError, match="max_expanded_atoms"):
        Calculator(ForceField.bundled("ffield.reax.HO.2015"), max_expanded_atoms=80).evaluate(
            g["symbols"], g["positions"], cell=[4.0] * 3)


def test_identical_atoms_need_no_qeq_iterations():
    """Three O2 molecules: by symmetry of the element the QEq solution is q = 0 exactly, and the
    start point already solves it (the projected start gradient is pure rounding noise)."""
    import oracle
    from xreac_gb300 import ForceField

    x = np.array([[3.50123, 2.24014, 1.17288], [4.30737, 1.30776, 1.52977], [0.98644, 0.98603, 4.08601],
                  [2.17758, 1.10723, 3.7871], [2.28101, 3.78692, 3.64103], [3.19255, 3.38801, 3.9615]])
    c = calc("ffield.reax.CHO.2008")
    r = c.evaluate(["O"] * 6, x)
    np.testing.assert_allclose(r.charges, 0.0, atol=1e-12)
    ref = oracle.evaluate(ForceField.bundled("ffield.reax.CHO.2008"), ["O"] * 6, x)
    assert abs(r.energy - ref["energy"]) <= 1e-9 * 6
    np.testing.assert_allclose(r.forces, ref["forces"], atol=2e-8, rtol=0)


def test_batch_charge_response_forces_match_single():
    """full_derivative=True in a batch (the adjoint QEq solve on 4-block clusters and single blocks)
    against the same systems alone (8-block clusters, single blocks)."""
    from xreac_gb300 import workloads

    systems = [workloads.water_cluster(n_mol=100, box=14.0, seed=5), workloads.water_cluster(n_mol=8, box=6.0, seed=5),
               workloads.water_cluster(n_mol=60, box=12.0, seed=6)]
    c = calc("ffield.reax.HO.2015")
    items = [dict(symbols=s.symbols, positions=s.positions) for s in systems]
    batch = c.evaluate_many(items, full_derivative=True)
    for d, rb in zip(items, batch):
        r1 = c.evaluate(d["symbols"], d["positions"], full_derivative=True)
        assert rb.full_derivative and rb.force_convention == "charge_response"
        assert rb.energy == pytest.approx(r1.energy, abs=1e-9 * len(d["symbols"]))
        np.testing.assert_allclose(rb.forces, r1.forces, atol=1e-8, rtol=0)
        np.testing.assert_allclose(rb.charges, r1.charges, atol=1e-10, rtol=0)
