"""CUDA-graph replay of the launch sequence: the kernels after the neighbour count are recorded as a
graph the second time a launch key occurs, and later calls with that key replay it. Every
replayed result must equal that of direct launches on the same inputs (xreac's Calculator.evaluate,
src/xreac/calculator.py:76-165, has no such state): energies and charges bit for bit, forces to the
last bits (atomics), including steps whose lists change size between replays."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pair(ff_name):
    from xreac_gb300 import Calculator, ForceField

    ff = ForceField.bundled(ff_name)
    on, off = Calculator(ff), Calculator(ff)
    off.set_graphs(False)
    return on, off


def _same(a, b):
    assert a.energy == b.energy
    assert a.components == b.components
    np.testing.assert_array_equal(a.charges, b.charges)
    np.testing.assert_allclose(a.forces, b.forces, atol=1e-10 * max(1.0, np.abs(b.forces).max()), rtol=0)
    np.testing.assert_array_equal(a.bond_counts, b.bond_counts)
    np.testing.assert_array_equal(a.total_bond_orders, b.total_bond_orders)


def _steps(x, n, scale, seed=0):
    rng = np.random.default_rng(seed)
    out = [x]
    for _ in range(n - 1):
        out.append(out[-1] + rng.normal(0.0, scale, x.shape))
    return out


@pytest.mark.parametrize("full_derivative", [False, True])
def test_repeated_steps_record_then_replay(full_derivative):
    from xreac_gb300 import workloads

    s = workloads.water_cluster(n_mol=60, box=12.0, seed=5, jitter=0.05)
    on, off = _pair("ffield.reax.HO.2015")
    modes = []
    # steps of 0.05 A: the lists change size between replays
    for x in _steps(s.positions, 6, 0.05):
        a = on.evaluate(s.symbols, x, full_derivative=full_derivative)
        modes.append(on.last_graph)
        b = off.evaluate(s.symbols, x, full_derivative=full_derivative)
        assert off.last_graph == "direct"
        _same(a, b)
    assert modes[0] == "direct" and modes[1] == "recorded" and set(modes[2:]) == {"replayed"}
    assert on.last_launches == off.last_launches


def test_batches_periodic_systems_and_a_changed_shape():
    from xreac_gb300 import workloads

    systems = [workloads.water_cluster(n_mol=n, box=9.0 + n / 20, seed=n, jitter=0.05) for n in (4, 30, 90)]
    box = workloads.water_box(n_mol=64, box=12.4, seed=3)
    on, off = _pair("ffield.reax.HO.2015")
    rng = np.random.default_rng(2)
    items = [dict(symbols=s.symbols, positions=s.positions) for s in systems]
    items.append(dict(symbols=box.symbols, positions=box.positions, cell=box.cell, pbc=True))
    seen = []
    for step in range(5):
        moved = [dict(d, positions=d["positions"] + rng.normal(0.0, 0.02, d["positions"].shape)) for d in items]
        a = on.evaluate_many(moved)
        seen.append(on.last_graph)
        for ra, rb in zip(a, off.evaluate_many(moved)):
            _same(ra, rb)
    assert seen[2:] == ["replayed"] * 3
    # another shape: direct again, then recorded on its repeat
    one = items[:2]
    on.evaluate_many(one)
    assert on.last_graph == "direct"
    on.evaluate_many(one)
    assert on.last_graph == "recorded"


def test_skin_lists_and_parameter_gradients_under_replay():
    from xreac_gb300 import workloads

    s = workloads.water_cluster(n_mol=40, box=11.0, seed=8, jitter=0.05)
    on, off = _pair("ffield.reax.HO.2015")
    for c in (on, off):
        c.set_neighbor_skin(1.0)
    for k, x in enumerate(_steps(s.positions, 6, 0.01, seed=4)):
        a = on.evaluate(s.symbols, x)
        b = off.evaluate(s.symbols, x)
        _same(a, b)
        if k >= 3:
            assert on.list_info()[0] == "reused" and on.last_graph == "replayed"
    ga = [on.parameter_gradient(s.symbols, s.positions)[1] for _ in range(3)]
    gb = off.parameter_gradient(s.symbols, s.positions)[1]
    assert on.last_graph == "replayed"
    for key, d in gb.pairs.items():
        for name, v in d.items():
            assert ga[-1].pairs[key][name] == pytest.approx(v, rel=1e-12, abs=1e-12)


def test_graphs_off_and_profiling_launch_directly():
    from xreac_gb300 import Calculator, ForceField, workloads

    s = workloads.water_cluster(n_mol=10, box=8.0, seed=1)
    c = Calculator(ForceField.bundled("ffield.reax.HO.2015"))
    c.set_profiling(True)
    for _ in range(3):
        c.evaluate(s.symbols, s.positions)
        assert c.last_graph == "direct"
    c.set_profiling(False)
    c.set_graphs(False)
    for _ in range(3):
        c.evaluate(s.symbols, s.positions)
        assert c.last_graph == "direct"
