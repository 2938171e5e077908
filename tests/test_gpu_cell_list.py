"""Cell-list neighbour search: the list (every directed edge, in canonical order) and every result
must equal those of the image scan, which the parity tests pin to xreac's replicated_neighbors
(src/xreac/neighbors.py:17-53). Covers cubic and triclinic periodic cells, cells thinner than the
cutoff, partly periodic and open systems, ragged batches, and skin lists built from the cell list."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _calc(ff_name, cells):
    from xreac_gb300 import Calculator, ForceField

    c = Calculator(ForceField.bundled(ff_name))
    c.set_cell_list(cells)
    return c


def _same(a, b, n):
    """Results of the same list in the same order: energies and charges bit for bit (fixed-order
    reductions), forces to the last bits (the many-body kernels add with atomics)."""
    assert a.energy == b.energy
    assert a.components == b.components
    np.testing.assert_array_equal(a.charges, b.charges)
    np.testing.assert_allclose(a.forces, b.forces, atol=1e-10 * max(1.0, np.abs(b.forces).max()), rtol=0)


def _compare(ff_name, systems, full_derivative=False):
    scan, cell = _calc(ff_name, False), _calc(ff_name, True)
    items = [dict(symbols=s.symbols, positions=s.positions, cell=s.cell, pbc=s.pbc, total_charge=s.total_charge)
             for s in systems]
    a = scan.evaluate_many(items, full_derivative=full_derivative)
    assert scan.list_info()[0] == "scan"
    b = cell.evaluate_many(items, full_derivative=full_derivative)
    assert cell.list_info()[0] == "cells"
    for k, (ra, rb) in enumerate(zip(a, b)):
        _same(rb, ra, len(items[k]["symbols"]))
        la, lb = scan.neighbor_list(k), cell.neighbor_list(k)
        for xa, xb in zip(la, lb):
            np.testing.assert_array_equal(np.asarray(xb), np.asarray(xa))
    return a


def test_water_box_full_size():
    from xreac_gb300 import workloads

    _compare("ffield.reax.HO.2015", [workloads.water_box()])


def test_auto_choice_uses_cells_for_the_water_box_only():
    from xreac_gb300 import Calculator, ForceField, workloads

    c = Calculator(ForceField.bundled("ffield.reax.HO.2015"))
    box = workloads.water_box()
    c.evaluate(box.symbols, box.positions, cell=box.cell, pbc=box.pbc)
    assert c.list_info()[0] == "cells"
    small = workloads.water_cluster(n_mol=20, box=9.0, seed=4)
    c.evaluate(small.symbols, small.positions)
    assert c.list_info()[0] == "scan"


def test_cho_box_full_derivative():
    from xreac_gb300 import workloads

    _compare("ffield.reax.CHO.2008", [workloads.cho_mixture()], full_derivative=True)


def test_triclinic_and_thin_cells():
    """A sheared cell, and a cell with a face height below the cutoff (several images per pair)."""
    from xreac_gb300 import workloads
    from xreac_gb300.workloads import System

    base = workloads.water_box(n_mol=400, box=23.0, seed=6)
    shear = np.array([[23.0, 0.0, 0.0], [5.5, 22.0, 0.0], [-3.0, 4.0, 21.5]])
    frac = base.positions @ np.linalg.inv(np.diag([23.0, 23.0, 23.0]))
    tri = System(base.symbols, frac @ shear, shear, True, 0.0, base.force_field)
    thin_src = workloads.water_box(n_mol=60, box=12.0, seed=7)
    thin_cell = np.array([[12.0, 0.0, 0.0], [0.0, 12.0, 0.0], [0.0, 0.0, 6.0]])
    keep = thin_src.positions[:, 2] < 5.8
    keep = np.repeat(keep.reshape(-1, 3).all(axis=1), 3)  # whole molecules
    thin = System([s for s, k in zip(thin_src.symbols, keep) if k], thin_src.positions[keep], thin_cell, True, 0.0,
                  thin_src.force_field)
    _compare("ffield.reax.HO.2015", [tri, thin])


def test_partly_periodic_and_open_systems_in_one_batch():
    from xreac_gb300 import workloads
    from xreac_gb300.workloads import System

    slab = workloads.anatase_slab_water(displacement=0.05)  # jittered: the ideal crystal has collinear torsions
    partial = System(slab.symbols, slab.positions, slab.cell, (True, True, False), 0.0, slab.force_field)
    _compare("ffield.reax.TiOH.Kim2013", [partial, slab])
    cluster = workloads.water_cluster(n_mol=300, box=30.0, seed=9, jitter=0.05)
    far = workloads.water_cluster(n_mol=4, box=6.0, seed=10)
    spread = System(cluster.symbols + far.symbols, np.vstack([cluster.positions, far.positions + 80.0]), None, False,
                    0.0, cluster.force_field)
    small = workloads.water_cluster(n_mol=3, box=5.0, seed=11)
    _compare("ffield.reax.HO.2015", [spread, small, cluster])


def test_skin_list_built_from_cells():
    from xreac_gb300 import workloads

    box = workloads.water_box(n_mol=700, box=27.6, seed=12)
    scan, cell = _calc("ffield.reax.HO.2015", False), _calc("ffield.reax.HO.2015", True)
    for c in (scan, cell):
        c.set_neighbor_skin(1.0)
    rng = np.random.default_rng(1)
    x = box.positions
    for step in range(3):
        a = scan.evaluate(box.symbols, x, cell=box.cell, pbc=True)
        b = cell.evaluate(box.symbols, x, cell=box.cell, pbc=True)
        assert cell.list_info()[0] == ("built-cells" if step == 0 else "reused")
        _same(b, a, len(box.symbols))
        for xa, xb in zip(scan.neighbor_list(0), cell.neighbor_list(0)):
            np.testing.assert_array_equal(np.asarray(xb), np.asarray(xa))
        x = x + rng.normal(0.0, 0.05, x.shape)
