"""Pin the CPU oracle to fixtures written by the unmodified xreac reference.

The tolerances are the reference's own strict backend-equivalence limits
(scripts/validate.py:122-146 of xreac: energy per atom 1e-9, forces 2e-8,
charges and bond orders 1e-10, counts exact), plus exact neighbour lists.
"""

import hashlib

import numpy as np
import pytest

from conftest import golden_names
from oracle import COMPONENTS, evaluate
from xreac_gb300.forcefield import ForceField

NAMES = golden_names()


def check_neighbors(g, i, j, s):
    """Canonical (i, j, S) arrays equal to the reference's (stored in full, or by count and SHA-256)."""
    canon = np.column_stack((i, j, s)).astype(np.int32)
    assert len(canon) == int(g["edge_count"])
    if "edge_i" in g:
        np.testing.assert_array_equal(canon[:, 0], g["edge_i"])
        np.testing.assert_array_equal(canon[:, 1], g["edge_j"])
        np.testing.assert_array_equal(canon[:, 2:], g["edge_S"])
    else:
        assert hashlib.sha256(np.ascontiguousarray(canon).tobytes()).hexdigest() == str(g["edge_sha256"])


def run_oracle(g):
    ff = ForceField.bundled(g["ff"])
    supplied = (g["sup_i"], g["sup_j"], g["sup_S"]) if "sup_i" in g else None
    return evaluate(
        ff, g["symbols"], g["positions"], cell=g["cell"], pbc=g["pbc"], total_charge=g["total_charge"],
        full_derivative=g["full_derivative"], dense_bond_orders="bond_orders" in g, neighbors=supplied,
    )


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference(name, golden):
    g = golden(name)
    o = run_oracle(g)
    n = len(g["symbols"])
    assert abs(o["energy"] - float(g["energy"])) / n <= 1e-9
    comps = np.array([o["components"][k] for k in COMPONENTS])
    assert np.max(np.abs(comps - g["components"])) / n <= 1e-9
    np.testing.assert_allclose(o["forces"], g["forces"], atol=2e-8, rtol=0)
    np.testing.assert_allclose(o["charges"], g["charges"], atol=1e-10, rtol=0)
    np.testing.assert_allclose(o["total_bond_orders"], g["total_bond_orders"], atol=1e-10, rtol=0)
    np.testing.assert_allclose(o["lone_pairs"], g["lone_pairs"], atol=1e-10, rtol=0)
    np.testing.assert_array_equal(o["bond_counts"], g["bond_counts"])
    np.testing.assert_allclose(o["dipole"], g["dipole"], atol=1e-9, rtol=0)
    assert tuple(o["cell_repetitions"]) == tuple(int(v) for v in g["cell_repetitions"])
    if "bond_orders" in g:
        np.testing.assert_allclose(o["bond_orders"], g["bond_orders"], atol=1e-10, rtol=0)
    # Neighbour list: identical canonical arrays, hence identical sets.
    i, j, s = o["neighbors"]
    check_neighbors(g, i, j, s)
    nz = np.flatnonzero(o["edge_bo"])
    np.testing.assert_allclose(o["edge_bo"][nz], g["bo_value"], atol=1e-10, rtol=0)


def test_release_known_answers():
    """The reference's release check (.github/workflows/release.yml:77-87)."""
    ff = ForceField.bundled("ffield.reax.HO.2015")
    r = evaluate(ff, ["O", "H", "H"], [[0, 0, 0], [0.97, 0, 0], [-0.243, 0.94, 0]])
    assert abs(r["energy"] - (-248.34420920633704)) < 1e-8
    assert np.isfinite(r["forces"]).all()
    assert abs(r["charges"].sum()) < 1e-12
    ion = evaluate(ff, ["O", "H"], [[0, 0, 0], [0.97, 0, 0]], total_charge=-1)
    assert abs(ion["charges"].sum() + 1) < 1e-12


def test_reference_test_known_answers(golden):
    """Values the reference's tests assert (tests/test_reference.py:98-108, tests/test_neighbors.py:56-61)."""
    g = golden("small_water_4A")
    hb = g["components"][list(COMPONENTS).index("hydrogen_bond")]
    assert hb == pytest.approx(-0.3700520183, abs=1e-9)
    g = golden("carbon_dimer")
    assert g["components"][list(COMPONENTS).index("lone_pair")] > 50
    g = golden("periodic_carbon_chain")
    assert abs(g["components"][list(COMPONENTS).index("torsion")]) > 0.1
    g = golden("small_zinc_chain")
    assert g["bond_counts"].tolist() == [2] and g["bond_orders"][0, 0] > 1


def test_collinear_active_torsion_raises():
    """tests/test_general.py:142-159 of the reference: a straight C4 chain is rejected."""
    ff = ForceField.bundled("ffield.reax.CHO.2008")
    with pytest.raises(ValueError, match="Collinear atoms in an active torsion"):
        evaluate(ff, ["C"] * 4, [[0, 0, 0], [1.5, 0, 0], [3, 0, 0], [4.5, 0.3, 0]])


def test_fixed_charge_forces_match_finite_differences():
    """Fixed-charge forces against a central difference of the energy at fixed q."""
    from oracle.reaxff_oracle import Edges, _Model, _components, boundary, neighbor_list, qeq_charges
    import torch

    ff = ForceField.bundled("ffield.reax.HO.2015")
    from conftest import load_golden

    g = load_golden("water_distorted_dimer")
    x = g["positions"]
    r = evaluate(ff, g["symbols"], x)
    flags, m = boundary(None, None)
    i, j, s = neighbor_list(x, ff.general[12])
    model = _Model(ff, g["symbols"], Edges.from_sorted(i, j, s, len(x), m))
    direction = np.random.default_rng(21).normal(size=x.shape)
    direction /= np.linalg.norm(direction)

    def energy(y):
        E, *_ = _components(model, torch.tensor(y), r["charges"], 0.0, True)
        return float(sum(E.values()))

    h = 1e-5
    fd = -(energy(x + h * direction) - energy(x - h * direction)) / (2 * h)
    assert fd == pytest.approx(np.sum(r["forces"] * direction), abs=1e-6, rel=0)
