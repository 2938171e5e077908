"""Server host logic on CPU: batching, error isolation, worker failures, warm-start hand-off.

The device calculator is replaced by a recorder (no GPU): each result's energy is the request's atom
count, so every request can be matched to its own result.
"""

import threading

import numpy as np
import pytest

import xreac_gb300.serving as serving


class _Eval:
    def __init__(self, n, charges):
        self.energy = float(n)
        self.charges = charges


class _Calc:
    fail_next_batch = threading.Event()

    def __init__(self, force_field, device=0, max_expanded_atoms=512):
        self.batches = []
        self.last_launches = 1

    def reserve(self, atoms, systems, **kw):
        pass

    def _evaluate_items(self, items):
        self.batches.append(len(items))
        out = []
        for symbols, positions, q, cell, pbc, initial in items:
            if symbols[0] == "Bad":
                raise ValueError("unknown element")
            n = len(symbols)
            out.append(_Eval(n, np.full(n, 0.5) if initial is None else initial + 1.0))
        return out

    def qeq_work(self):
        if _Calc.fail_next_batch.is_set():
            _Calc.fail_next_batch.clear()
            raise RuntimeError("device fault report")
        return 0, 0.0

    def transfer_bytes(self):
        return 0, 0


@pytest.fixture()
def server(monkeypatch):
    monkeypatch.setattr(serving, "Calculator", _Calc)
    srv = serving.Server({"ff": object()}, workers=2)
    yield srv
    srv.close()


def _req(n, session=None, bad=False):
    symbols = ["Bad"] * n if bad else ["H"] * n
    return serving.Request(symbols, np.zeros((n, 3)), "ff", session=session)


def test_every_request_gets_its_own_result(server):
    reqs = [_req(1 + k % 7) for k in range(200)]
    out, _ = serving.replay(server, reqs)
    assert [o.evaluation.energy for o in out] == [float(r.natoms) for r in reqs]
    assert len(server.batches) < len(reqs)
    assert all(o.batch_size >= 1 and o.latency >= 0 for o in out)


def test_a_bad_request_fails_alone(server):
    reqs = [_req(3), _req(2, bad=True), _req(4)]
    out, _ = serving.replay(server, reqs)
    assert isinstance(out[1], ValueError)
    assert out[0].evaluation.energy == 3.0 and out[2].evaluation.energy == 4.0


def test_worker_failure_fails_the_batch_and_serving_continues(server):
    _Calc.fail_next_batch.set()
    first = server.submit(_req(2))
    with pytest.raises(RuntimeError):
        first.result(timeout=10)
    assert first.done() and isinstance(first.exception(), RuntimeError)
    later = server.submit(_req(5))
    assert later.result(timeout=10).evaluation.energy == 5.0


def test_sessions_hand_charges_to_the_next_step(server):
    a = server.submit(_req(3, session="traj")).result(timeout=10)
    b = server.submit(_req(3, session="traj")).result(timeout=10)
    np.testing.assert_array_equal(a.evaluation.charges, 0.5)
    np.testing.assert_array_equal(b.evaluation.charges, 1.5)  # started from a's charges
    c = server.submit(_req(4, session="traj")).result(timeout=10)  # another size: no warm start
    np.testing.assert_array_equal(c.evaluation.charges, 0.5)


def test_a_failed_step_keeps_the_session_charges(server):
    server.submit(_req(3, session="traj")).result(timeout=10)  # charges 0.5
    bad = server.submit(_req(3, session="traj", bad=True))
    with pytest.raises(ValueError):
        bad.result(timeout=10)
    c = server.submit(_req(3, session="traj")).result(timeout=10)
    np.testing.assert_array_equal(c.evaluation.charges, 1.5)  # from the last good step


def test_unknown_force_field_and_closed_server(server):
    with pytest.raises(ValueError):
        server.submit(serving.Request(["H"], np.zeros((1, 3)), "other"))
    server.close()
    with pytest.raises(RuntimeError):
        server.submit(_req(1))


def test_submit_many_matches_single_submits(server):
    reqs = [_req(1 + k % 5) for k in range(50)]
    futs = server.submit_many(reqs)
    assert [f.result(timeout=10).evaluation.energy for f in futs] == [float(r.natoms) for r in reqs]
    with pytest.raises(ValueError):
        server.submit_many([_req(1), serving.Request(["H"], np.zeros((1, 3)), "other")])


def test_batches_respect_the_atom_and_request_budgets(monkeypatch):
    monkeypatch.setattr(serving, "Calculator", _Calc)
    sizes = (3, 3, 3, 3, 12, 2, 2, 2, 2, 1)
    with serving.Server({"ff": object()}, workers=1, max_batch_atoms=10, max_batch_requests=3) as srv:
        reqs = [_req(n) for n in sizes]
        out, _ = serving.replay(srv, reqs)
        batches = [(b.requests, b.atoms) for b in srv.batches]
    assert [o.evaluation.energy for o in out] == [float(n) for n in sizes]
    assert sum(r for r, _ in batches) == len(sizes)
    assert all(r <= 3 for r, _ in batches)
    assert all(a <= 10 or r == 1 for r, a in batches)  # a request above the budget is a batch alone
    assert (1, 12) in batches


class _MemCalc(_Calc):
    """A stand-in that reports device capacities and list sizes, as the device calculator does."""

    edges_per_atom = 100  # directed edges each request really has per atom

    def __init__(self, force_field, device=0, max_expanded_atoms=512):
        super().__init__(force_field, device, max_expanded_atoms)
        self.caps = dict(device_bytes=0, atoms=0, systems=0, edges=0, pairs=0, bonds=0, candidates=0)
        self.last = (0, 0, 0, 0, 0, 0)

    def reserve(self, atoms, systems, edges_per_atom=450, bonds_per_atom=30):
        self.caps.update(atoms=atoms, systems=systems, edges=int(atoms * edges_per_atom),
                         bonds=int(atoms * bonds_per_atom), device_bytes=atoms * 1000)

    def memory(self):
        return dict(self.caps)

    def list_sizes(self):
        return self.last

    def _evaluate_items(self, items):
        out = super()._evaluate_items(items)
        e = sum(len(it[0]) * self.edges_per_atom for it in items)
        self.last = (e, e // 2, e // 20, 0, 0, 0)
        if e > self.caps["edges"]:  # the device would grow its buffers
            self.caps["edges"] = e
            self.caps["device_bytes"] += e
        return out


def _periodic(n):
    return serving.Request(["H"] * n, np.zeros((n, 3)), "ff", cell=np.eye(3) * 20.0, pbc=True)


def test_batches_are_cut_by_estimated_footprint(monkeypatch):
    monkeypatch.setattr(serving, "Calculator", _MemCalc)
    # 1,000 atoms and 100 k directed edges per context: periodic requests of 100 atoms are estimated
    # at 100 x 450 edges, so two fit a batch by edges although ten would fit by atoms
    srv = serving.Server({"ff": object()}, workers=1, max_batch_atoms=1000, max_batch_requests=64,
                         edges_per_atom=450, bonds_per_atom=30)
    try:
        srv._caps[0]["ff"] = (1000, 64, 100_000, 30_000)
        with srv._cv:
            for _ in range(6):
                srv._queues["ff"].append((_periodic(100), serving.Pending(srv._done_cv)))
            name, batch, est = srv._take_batch(0)
        assert name == "ff" and len(batch) == 2 and est[0] == 2 * 100 * 450
        # clusters are estimated at n * min(n - 1, K): 100 requests of 3 atoms fit by edges
        with srv._cv:
            srv._queues["ff"].clear()
            for _ in range(100):
                srv._queues["ff"].append((_req(3), serving.Pending(srv._done_cv)))
            _, batch, est = srv._take_batch(0)
        assert len(batch) == 64 and est[0] == 64 * 3 * 2
    finally:
        srv.close()


def test_densities_rise_when_a_batch_exceeds_its_estimate(monkeypatch):
    monkeypatch.setattr(serving, "Calculator", _MemCalc)
    _MemCalc.edges_per_atom = 900  # denser than the starting estimate of 450
    try:
        srv = serving.Server({"ff": object()}, workers=1, max_batch_atoms=512, edges_per_atom=450)
        out, _ = serving.replay(srv, [_periodic(64) for _ in range(8)])
        srv.close()
        assert all(not isinstance(o, Exception) for o in out)
        assert srv.footprints["ff"].edges_per_atom >= 900
        assert srv.reallocations >= 1  # the first batch outgrew the reservation
        rep = srv.memory_report()
        assert rep["reallocations"] == srv.reallocations and rep["contexts"][0]["edges"] >= 64 * 900
        assert all(b.edges > 0 and b.est_edges > 0 for b in srv.batches)
    finally:
        _MemCalc.edges_per_atom = 100


def test_memory_budget_bounds_the_reservation(monkeypatch):
    from xreac_gb300 import Calculator

    monkeypatch.setattr(serving, "Calculator", _MemCalc)
    monkeypatch.setattr(_MemCalc, "footprint_bytes", staticmethod(Calculator.footprint_bytes), raising=False)
    budget = 4 * Calculator.footprint_bytes(2048, 512, 2048 * 450, 2048 * 30)
    srv = serving.Server({"ff": object(), "ff2": object()}, workers=2, max_batch_atoms=16384, memory_budget=budget)
    try:
        assert 1800 < srv.max_batch_atoms <= 2048
        assert Calculator.footprint_bytes(srv.max_batch_atoms, 512, srv.max_batch_atoms * 450,
                                          srv.max_batch_atoms * 30) <= budget / 4
    finally:
        srv.close()
    with pytest.raises(ValueError, match="too small"):
        serving.Server({"ff": object()}, workers=1, memory_budget=1000)
