"""Neighbour lists on the device: exact evaluation of caller-supplied lists, and skin lists kept
across calls (the reference's semantics: src/xreac/calculator.py:113-120 and src/xreac/ase.py:107-131,
pinned by tests/test_neighbors.py:317-409 of the reference).

Tolerances: the reference's strict backend limits (energy and components per atom 1e-9, forces
2e-8 kcal/mol/A, charges and bond orders 1e-10, counts exact). A reused skin list gives the same
edges in the same order as a fresh scan, so its results are those of a fresh evaluation to the last
bit, except forces, whose many-body parts are added with atomics (1e-9 here).
"""

import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

SUPPLIED = [n for n in golden_names() if n.startswith("supplied_")]


def _calc(ff_name, **kw):
    from xreac_gb300 import Calculator, ForceField

    return Calculator(ForceField.bundled(ff_name), **kw)


def _same(a, b):
    """A reused list gives a fresh evaluation's results."""
    assert a.energy == b.energy
    assert a.components == b.components
    np.testing.assert_array_equal(a.charges, b.charges)
    np.testing.assert_allclose(a.forces, b.forces, atol=1e-9, rtol=0)
    np.testing.assert_array_equal(a.total_bond_orders, b.total_bond_orders)
    np.testing.assert_array_equal(a.bond_counts, b.bond_counts)


@pytest.mark.parametrize("name", SUPPLIED)
def test_supplied_list_gives_the_reference_result(name):
    """Skin lists (equal to the replicated result) and thinned lists (pairs left out contribute
    nothing), handed over in shuffled order, against the reference's own evaluation of each list."""
    from test_gpu_parity import check_strict

    g = load_golden(name)
    c = _calc(g["ff"])
    r = c.evaluate(g["symbols"], g["positions"], cell=g["cell"], pbc=g["pbc"], total_charge=g["total_charge"],
                   neighbors=(g["sup_i"], g["sup_j"], g["sup_S"]))
    assert r.neighbor_backend == "provided" and tuple(r.cell_repetitions) == (1, 1, 1)
    check_strict(r, g, len(g["symbols"]))
    assert c.list_info()[0] == "supplied"
    # the device keeps exactly the supplied edges within the cutoff, in canonical order
    x = np.asarray(g["positions"], dtype=float)
    lat = np.eye(3) if g["cell"] is None else np.asarray(g["cell"], dtype=float)
    i, j, S = (np.asarray(g[k], dtype=np.int64) for k in ("sup_i", "sup_j", "sup_S"))
    v = x[j] - x[i] + S @ lat
    rc = float(c.force_field.general[12])
    keep = np.sum(v * v, axis=1) <= rc * rc
    i, j, S = i[keep], j[keep], S[keep]
    order = np.lexsort((S[:, 2], S[:, 1], S[:, 0], j, i))
    di, dj, dS = c.neighbor_list()
    np.testing.assert_array_equal(di, i[order])
    np.testing.assert_array_equal(dj, j[order])
    np.testing.assert_array_equal(dS, S[order])


def test_partial_list_differs_from_the_full_one():
    g = load_golden("supplied_partial_cluster_water_192")
    full = load_golden("cluster_water_192")
    assert abs(float(g["energy"]) - float(full["energy"])) > 100.0  # the fixture really is partial


@pytest.mark.parametrize("neighbors,message", [
    (([0], [1]), "tuple"),
    (([0], [1, 0], [[0, 0, 0]]), "shape"),
    (([0.0, 1.0], [1, 0], [[0, 0, 0], [0, 0, 0]]), "integers"),
    (([-1, 1], [1, 0], [[0, 0, 0], [0, 0, 0]]), "out of range"),
    (([0, 1], [1, 0], [[1, 0, 0], [-1, 0, 0]]), "nonperiodic"),
    (([0], [0], [[0, 0, 0]]), "self neighbors"),
    (([0, 0, 1], [1, 1, 0], [[0, 0, 0]] * 3), "Duplicate"),
    (([0], [1], [[0, 0, 0]]), "both directions"),
])
def test_supplied_neighbor_validation(neighbors, message):
    """tests/test_neighbors.py:317-342 of the reference, through Calculator.evaluate."""
    c = _calc("ffield.reax.ZnOH.2010")
    with pytest.raises(ValueError, match=message):
        c.evaluate(["Zn", "O"], [[0, 0, 0], [1.9, 0, 0]], neighbors=neighbors)


def test_supplied_list_of_a_single_atom_chain():
    """tests/test_neighbors.py:300-314 of the reference: a Zn atom with its own images along x."""
    c = _calc("ffield.reax.ZnOH.2010")
    shifts = np.array([[s, 0, 0] for s in (-4, -3, -2, -1, 1, 2, 3, 4)])
    nb = (np.zeros(8, dtype=int), np.zeros(8, dtype=int), shifts)
    got = c.evaluate(["Zn"], [[0, 0, 0]], cell=[2.5, 12, 12], pbc=[True, False, False], neighbors=nb)
    want = c.evaluate(["Zn"], [[0, 0, 0]], cell=[2.5, 12, 12], pbc=[True, False, False])
    assert abs(got.energy - want.energy) < 1e-10
    assert got.bond_counts.tolist() == [2]


def test_coincident_atoms_are_found_whatever_list_is_supplied():
    """xreac checks every pair's minimum image before it looks at the list."""
    c = _calc("ffield.reax.HO.2015")
    x = [[0, 0, 0], [0.97, 0, 0], [0.97, 0, 0]]
    nb = ([0, 1], [1, 0], [[0, 0, 0], [0, 0, 0]])  # the coincident pair (1, 2) is not in the list
    with pytest.raises(ValueError, match="Coincident"):
        c.evaluate(["O", "H", "H"], x, neighbors=nb)


def _small_water_4A():
    g = load_golden("small_water_4A")
    return g["ff"], g["symbols"], np.asarray(g["positions"], dtype=float), g["cell"], g["pbc"]


@pytest.mark.parametrize("name", ["small_water_4A", "small_zinc_chain", "periodic_partial_pbc_water"])
def test_skin_list_is_reused_until_an_atom_moves_more_than_the_skin(name):
    """tests/test_neighbors.py:345-362 of the reference: displacements of 0.04 and 0.2 A from the
    build reuse the list, 0.31 A rebuilds it (skin 0.3 A); physics is recomputed every call."""
    g = load_golden(name)
    ff, s, x, cell, pbc = g["ff"], g["symbols"], np.asarray(g["positions"], dtype=float), g["cell"], g["pbc"]
    c = _calc(ff)
    fresh = _calc(ff)
    c.set_neighbor_skin(0.3)
    c.evaluate(s, x, cell=cell, pbc=pbc)
    assert c.list_info() == ("built", 1)
    for displacement, mode, builds in ((0.04, "reused", 1), (0.2, "reused", 1), (0.31, "built", 2)):
        y = x.copy()
        y[0, 0] += displacement
        got = c.evaluate(s, y, cell=cell, pbc=pbc)
        assert c.list_info() == (mode, builds)
        _same(got, fresh.evaluate(s, y, cell=cell, pbc=pbc))


def test_skin_list_is_rebuilt_when_the_system_changes():
    """tests/test_neighbors.py:365-395 of the reference: a changed cell, pbc, a wrapped atom, a new
    atom order or count, and a changed skin each rebuild the list."""
    ff, s, x, cell, pbc = _small_water_4A()
    c = _calc(ff)
    fresh = _calc(ff)
    c.set_neighbor_skin(0.3)
    cell = np.array(cell, dtype=float)
    pbc = np.array(pbc, dtype=bool)
    builds = 0

    def run(sym, y, cl, pb, mode):
        nonlocal builds
        got = c.evaluate(sym, y, cell=cl, pbc=pb)
        builds += mode == "built"
        assert c.list_info() == (mode, builds)
        _same(got, fresh.evaluate(sym, y, cell=cl, pbc=pb))

    run(s, x, cell, pbc, "built")
    run(s, x, cell, pbc, "reused")
    cell2 = cell.copy()
    cell2[0, 0] += 0.1
    run(s, x, cell2, pbc, "built")
    pbc2 = pbc.copy()
    pbc2[2] = False
    run(s, x, cell2, pbc2, "built")
    y = x.copy()
    y[0] += cell2[0]  # an atom wrapped by a lattice vector: a jump far beyond the skin
    run(s, y, cell2, pbc2, "built")
    run([s[1], s[0], s[2]], y[[1, 0, 2]], cell2, pbc2, "built")
    run(s[:2], y[:2], cell2, pbc2, "built")
    c.set_neighbor_skin(0.1)
    run(s[:2], y[:2], cell2, pbc2, "built")
    c.set_neighbor_skin(0.0)
    got = c.evaluate(s[:2], y[:2], cell=cell2, pbc=pbc2)
    assert c.list_info() == ("scan", builds)
    _same(got, fresh.evaluate(s[:2], y[:2], cell=cell2, pbc=pbc2))


def test_pair_enters_the_cutoff_without_a_rebuild():
    """tests/test_neighbors.py:398-409 of the reference: two atoms 0.5 A beyond the cutoff move 0.29 A
    towards each other each; the list, built with 2 x 0.3 A of skin, already holds the pair."""
    c = _calc("ffield.reax.ZnOH.2010")
    fresh = _calc("ffield.reax.ZnOH.2010")
    c.set_neighbor_skin(0.3)
    rc = float(c.force_field.general[12])
    x = np.array([[0.0, 0.0, 0.0], [rc + 0.5, 0.0, 0.0]])
    far = c.evaluate(["Zn", "O"], x)
    x[:, 0] += [0.29, -0.29]
    near = c.evaluate(["Zn", "O"], x)
    assert c.list_info() == ("reused", 1)
    assert near.energy != 0 and near.energy != far.energy
    _same(near, fresh.evaluate(["Zn", "O"], x))


def test_skin_list_of_a_batch_and_of_the_water_box():
    """A batch keeps one list for all its systems; the 4,608-atom periodic box reuses its list over a
    small displacement of every atom and gives the fresh evaluation's results."""
    from xreac_gb300 import workloads

    c = _calc("ffield.reax.HO.2015")
    fresh = _calc("ffield.reax.HO.2015")
    c.set_neighbor_skin(0.3)
    box = workloads.water_box()
    rng = np.random.default_rng(5)
    first = c.evaluate(box.symbols, box.positions, cell=box.cell, pbc=box.pbc)
    y = box.positions + rng.uniform(-0.1, 0.1, box.positions.shape)
    got = c.evaluate(box.symbols, y, cell=box.cell, pbc=box.pbc)
    assert c.list_info() == ("reused", 1)
    _same(got, fresh.evaluate(box.symbols, y, cell=box.cell, pbc=box.pbc))
    assert got.energy != first.energy
    systems = [dict(symbols=s.symbols, positions=s.positions) for s in
               (workloads.water_cluster(n_mol=n, box=(n / 64) ** (1 / 3) * 12, seed=20 + n) for n in (5, 40, 90))]
    c.evaluate_many(systems)
    assert c.list_info() == ("built", 2)
    moved = [dict(d, positions=d["positions"] + 0.05) for d in systems]
    got = c.evaluate_many(moved)
    assert c.list_info() == ("reused", 2)
    for a, b in zip(got, fresh.evaluate_many(moved)):
        _same(a, b)
