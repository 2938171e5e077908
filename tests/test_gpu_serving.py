"""Serving path: continuous batching gives every request the result it gets alone; warm starts.

Tolerances are the evaluation path's stated limits (energy 1e-8 relative, forces 1e-6 kcal/mol/A,
charges 1e-8 e); in practice batch and single evaluations agree to rounding.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FFS = ("ffield.reax.HO.2015", "ffield.reax.CHO.2008")


def _requests(n=64, seed=4):
    from xreac_gb300 import workloads
    from xreac_gb300.serving import Request

    stream = workloads.request_stream(n_requests=n, seed=seed)
    reqs = [Request(r.system.symbols, r.system.positions, r.system.force_field, r.system.cell, r.system.pbc,
                    r.system.total_charge, session=r.index if r.repeat_of is None else r.repeat_of) for r in stream]
    return stream, reqs


def _close(a, b):
    assert abs(a.energy - b.energy) <= 1e-8 * max(1.0, abs(b.energy))
    np.testing.assert_allclose(a.forces, b.forces, atol=1e-6, rtol=0)
    np.testing.assert_allclose(a.charges, b.charges, atol=1e-8, rtol=0)
    np.testing.assert_allclose(a.total_bond_orders, b.total_bond_orders, atol=1e-8, rtol=0)
    np.testing.assert_array_equal(a.bond_counts, b.bond_counts)


def test_each_request_alone_equals_in_the_mix():
    from xreac_gb300 import Calculator, ForceField
    from xreac_gb300.serving import Server, replay

    stream, reqs = _requests()
    ffs = {n: ForceField.bundled(n) for n in FFS}
    alone = {n: Calculator(f) for n, f in ffs.items()}
    with Server(ffs, workers=2, max_batch_atoms=4096) as srv:
        served, _ = replay(srv, reqs)
        batches = list(srv.batches)
    assert len(batches) < len(reqs)  # requests really were batched
    assert max(b.requests for b in batches) > 1
    for req, out in zip(reqs, served):
        assert not isinstance(out, Exception), out
        ref = alone[req.force_field].evaluate(req.symbols, req.positions, cell=req.cell, pbc=req.pbc,
                                              total_charge=req.total_charge)
        _close(out.evaluation, ref)
        assert out.latency >= 0


def test_requests_arriving_during_a_batch_join_later_batches():
    from xreac_gb300 import ForceField
    from xreac_gb300.serving import Server, replay

    stream, reqs = _requests(n=48, seed=7)
    ffs = {n: ForceField.bundled(n) for n in FFS}
    arrivals = np.array([r.arrival for r in stream])
    with Server(ffs, workers=2) as srv:
        served, wall = replay(srv, reqs, arrivals=arrivals - arrivals[0])
        nb = len(srv.batches)
    assert all(not isinstance(o, Exception) for o in served)
    assert 1 < nb <= len(reqs)
    assert wall >= arrivals[-1] - arrivals[0]


def test_warm_start_reaches_the_same_charges_in_fewer_iterations():
    from xreac_gb300 import Calculator, ForceField
    from xreac_gb300 import _native as nat
    from xreac_gb300.workloads import water_box

    s = water_box(n_mol=256, box=19.7, seed=12)
    calc = Calculator(ForceField.bundled(s.force_field))
    lib = nat.load()
    first = calc.evaluate(s.symbols, s.positions, cell=s.cell, pbc=s.pbc)
    rng = np.random.default_rng(3)
    x2 = s.positions + rng.normal(0.0, 0.01, s.positions.shape)
    cold = calc.evaluate(s.symbols, x2, cell=s.cell, pbc=s.pbc)
    it_cold = lib.xr_last_qeq_iterations(calc._ctx.handle)
    warm = calc.evaluate(s.symbols, x2, cell=s.cell, pbc=s.pbc, initial_charges=first.charges)
    it_warm = lib.xr_last_qeq_iterations(calc._ctx.handle)
    assert it_warm < it_cold
    np.testing.assert_allclose(warm.charges, cold.charges, atol=1e-10, rtol=0)
    np.testing.assert_allclose(warm.forces, cold.forces, atol=1e-7, rtol=0)
    assert abs(warm.energy - cold.energy) <= 1e-9 * abs(cold.energy)
    # a guess that does not sum to the total charge is shifted onto the constraint
    off = calc.evaluate(s.symbols, x2, cell=s.cell, pbc=s.pbc, initial_charges=first.charges + 0.01)
    np.testing.assert_allclose(off.charges, cold.charges, atol=1e-10, rtol=0)
    with pytest.raises(ValueError):
        calc.evaluate(s.symbols, x2, cell=s.cell, pbc=s.pbc, initial_charges=first.charges[:-1])


def test_many_workers_and_small_batches_give_the_same_results():
    """Six workers with 2,048-atom batches: many batches in flight on the device at once (their QEq
    clusters, grid teams and single blocks interleaved), each request still matching its result alone."""
    from xreac_gb300 import Calculator, ForceField
    from xreac_gb300.serving import Server, replay

    stream, reqs = _requests(n=96, seed=11)
    ffs = {n: ForceField.bundled(n) for n in FFS}
    alone = {n: Calculator(f) for n, f in ffs.items()}
    with Server(ffs, workers=6, max_batch_atoms=2048) as srv:
        served, _ = replay(srv, reqs)
        assert len(srv.batches) >= 4
    for req, out in zip(reqs, served):
        assert not isinstance(out, Exception), out
        ref = alone[req.force_field].evaluate(req.symbols, req.positions, cell=req.cell, pbc=req.pbc,
                                              total_charge=req.total_charge)
        _close(out.evaluation, ref)


def test_batches_are_deterministic():
    """The same batch twice: bit-identical energies and charges (fixed-order reductions, including the
    thread-block-cluster exchanges of the QEq solve); forces to the last bits, since the many-body
    kernels add their contributions to other atoms with atomics."""
    from xreac_gb300 import Calculator, ForceField

    stream, _ = _requests(n=64, seed=13)
    ff = "ffield.reax.CHO.2008"
    systems = [dict(symbols=r.system.symbols, positions=r.system.positions, cell=r.system.cell, pbc=r.system.pbc,
                    total_charge=r.system.total_charge) for r in stream if r.system.force_field == ff]
    calc = Calculator(ForceField.bundled(ff))
    a = calc.evaluate_many(systems)
    b = calc.evaluate_many(systems)
    for x, y in zip(a, b):
        assert x.energy == y.energy
        np.testing.assert_array_equal(x.charges, y.charges)
        np.testing.assert_allclose(x.forces, y.forces, rtol=1e-13, atol=1e-12)


def test_footprint_admission_keeps_dense_periodic_batches_within_the_reservation():
    """Dense periodic requests (liquid water at 1 g/cm^3, about 400 directed edges per atom) served
    within a device-memory budget: the contexts' reservations fit the budget, no batch reallocates
    device memory, and each result equals its evaluation alone."""
    from xreac_gb300 import Calculator, ForceField, workloads
    from xreac_gb300.serving import Request, Server, replay

    ff = ForceField.bundled("ffield.reax.HO.2015")
    boxes = [workloads.water_box(n_mol=100, box=14.42, seed=40 + k) for k in range(12)]
    reqs = [Request(b.symbols, b.positions, "ff", b.cell, True) for b in boxes]
    budget = 2 * Calculator.footprint_bytes(1200, 64, 1200 * 450, 1200 * 30)
    with Server({"ff": ff}, workers=2, max_batch_atoms=8192, max_batch_requests=64, memory_budget=budget) as srv:
        assert srv.max_batch_atoms <= 1200
        served, _ = replay(srv, reqs)
        report = srv.memory_report()
        batches = list(srv.batches)
    assert report["reallocations"] == 0
    assert sum(c["device_bytes"] for c in report["contexts"]) <= budget
    assert max(b.requests for b in batches) >= 2 and all(b.edges <= 1.25 * b.est_edges for b in batches)
    alone = Calculator(ff)
    for req, out in zip(reqs, served):
        assert not isinstance(out, Exception), out
        _close(out.evaluation, alone.evaluate(req.symbols, req.positions, cell=req.cell, pbc=True))


def test_footprint_bytes_match_a_reservation():
    from xreac_gb300 import Calculator, ForceField

    calc = Calculator(ForceField.bundled("ffield.reax.HO.2015"))
    before = calc.memory()["device_bytes"]
    calc.reserve(4096, 128, edges_per_atom=450, bonds_per_atom=30)
    m = calc.memory()
    est = Calculator.footprint_bytes(4096, 128, 4096 * 450, 4096 * 30)
    assert m["atoms"] >= 4096 and m["systems"] >= 128 and m["edges"] >= 4096 * 450 and m["bonds"] >= 4096 * 30
    assert 0.8 * est <= m["device_bytes"] - before <= 1.2 * est
