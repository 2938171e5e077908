"""Continuous-batching evaluation server on one GPU.

Requests (one system each: symbols, positions, optional cell/pbc/total charge, a force-field name
and an optional session key) are admitted into per-force-field queues. Each worker owns a device
context (its own CUDA stream and buffers) and repeatedly takes every request waiting for one force
field, up to an atom budget, and evaluates them as one ragged batch (``Calculator.evaluate_many``,
C entry point ``xr_eval_batch``). With two or more workers a new batch is formed and launched while
the previous one is still on the GPU, so requests that arrive during a batch join the next one and
the batches' work overlaps on the device. The C library releases the Python GIL for the duration
of a batch.

Admission by device footprint: every worker context is reserved at start-up (atoms, systems,
directed edges, bond candidates), within ``memory_budget`` when one is given, so that no batch
allocates device memory while others run (a reallocation synchronises the device). A batch takes
requests, oldest first, while its estimated lists still fit the context: a request of n atoms is
estimated at n * min(n - 1, K) directed edges (n * K when periodic) and n * min((n - 1) / 2, K_b)
bond candidates, where K and K_b per force field start at ``edges_per_atom`` and
``bonds_per_atom`` and rise whenever a batch's lists turn out larger than estimated.

Sessions: requests that carry the same ``session`` key are successive steps of one system (a
relaxation or MD trajectory). The server keeps the last QEq charges of each session and starts the
next step's solve from them (a warm start); results meet the same tolerance either way.

xreac itself has no serving layer; every request's result is the ``Evaluation`` that
``Calculator.evaluate`` (src/xreac/calculator.py:76-165) would return for it alone.
"""

from __future__ import annotations

import collections
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from .calculator import Calculator


@dataclass
class Request:
    """One evaluation request."""

    symbols: list
    positions: np.ndarray
    force_field: str
    cell: np.ndarray | None = None
    pbc: object = None
    total_charge: float = 0.0
    session: object = None
    arrival: float = field(default=0.0)  # time.perf_counter() at admission (set by submit)

    @property
    def natoms(self):
        return len(self.symbols)


class Pending:
    """Handle of a submitted request. ``result()`` waits for its batch and returns the
    :class:`Served` (or raises the request's error); ``done()`` tells whether it has finished.

    One condition variable of the server wakes all waiters once per finished batch, rather than
    one synchronisation object per request."""

    __slots__ = ("_cv", "_value", "_error", "_done")

    def __init__(self, cv):
        self._cv = cv
        self._value = None
        self._error = None
        self._done = False

    def done(self):
        return self._done

    def result(self, timeout=None):
        if not self._done:
            with self._cv:
                if not self._cv.wait_for(self.done, timeout):
                    raise TimeoutError("request not finished")
        if self._error is not None:
            raise self._error
        return self._value

    def exception(self, timeout=None):
        try:
            self.result(timeout)
        except TimeoutError:
            raise
        except Exception as err:  # noqa: BLE001 - the request's own error
            return err
        return None


@dataclass(slots=True)
class Served:
    """Result of one request: the evaluation plus its timing."""

    evaluation: object
    arrival: float
    done: float
    batch_size: int
    start: float = 0.0  # when its batch was formed

    @property
    def queued(self):
        return self.start - self.arrival

    @property
    def latency(self):
        return self.done - self.arrival


@dataclass
class Batch:
    """Record of one evaluated batch."""

    force_field: str
    requests: int
    atoms: int
    seconds: float       # wall time of the batch call (host preparation, device work, results)
    launches: int        # kernels launched
    qeq_iterations: int  # conjugate-gradient iterations summed over its systems
    qeq_bytes: float     # algorithmic matrix-free bytes of those iterations
    h2d_bytes: int = 0   # host-to-device bytes of the batch call
    d2h_bytes: int = 0   # device-to-host bytes of the batch call
    est_edges: int = 0   # directed edges the admission estimated
    edges: int = 0       # directed edges of the batch's lists
    device_bytes: int = 0  # the worker context's device bytes after the batch


class Footprint:
    """Per-force-field density model of the admission: directed edges and bond candidates per atom
    (K, K_b), raised when a batch exceeds its estimate."""

    __slots__ = ("edges_per_atom", "bonds_per_atom")

    def __init__(self, edges_per_atom, bonds_per_atom):
        self.edges_per_atom = float(edges_per_atom)
        self.bonds_per_atom = float(bonds_per_atom)

    def estimate(self, natoms, periodic):
        """(directed edges, bond candidates) expected for one request."""
        if periodic:
            return natoms * self.edges_per_atom, natoms * self.bonds_per_atom
        return natoms * min(natoms - 1, self.edges_per_atom), natoms * min(0.5 * (natoms - 1), self.bonds_per_atom)

    def observe(self, est_edges, edges, est_bonds, bonds):
        """A batch's actual list sizes against their estimate: raise the densities (5 % above the
        observed ratio) where the estimate fell short."""
        if est_edges > 0 and edges > est_edges:
            self.edges_per_atom *= 1.05 * edges / est_edges
        if est_bonds > 0 and bonds > est_bonds:
            self.bonds_per_atom *= 1.05 * bonds / est_bonds


class Server:
    """Continuous-batching server.

    ``force_fields`` maps names to ``ForceField`` objects. ``workers`` device contexts run batches
    concurrently; ``max_batch_atoms`` and ``max_batch_requests`` bound one batch, and every context
    is sized for that bound at start-up (``reserve``), so admission never waits on a device
    allocation. ``memory_budget`` (bytes, optional) caps the device memory of all contexts together:
    the atom bound is lowered until every context's reservation fits its share. ``edges_per_atom``
    and ``bonds_per_atom`` are the admission's starting densities (see the module docstring).
    ``warm_start`` enables the per-session QEq warm start.
    """

    def __init__(self, force_fields, *, workers=4, max_batch_atoms=16384, max_batch_requests=512, device=0,
                 warm_start=True, max_expanded_atoms=512, reserve=True, memory_budget=None, edges_per_atom=450.0,
                 bonds_per_atom=30.0):
        if workers < 1:
            raise ValueError("workers must be at least 1")
        self.force_fields = dict(force_fields)
        self.max_batch_atoms = int(max_batch_atoms)
        self.max_batch_requests = int(max_batch_requests)
        self.warm_start = warm_start
        self.footprints = {name: Footprint(edges_per_atom, bonds_per_atom) for name in self.force_fields}
        self.reallocations = 0  # batches after which a context held more device memory than before
        if memory_budget is not None:
            share = float(memory_budget) / (workers * max(1, len(self.force_fields)))
            self.max_batch_atoms = self._atoms_within(share, edges_per_atom, bonds_per_atom)
        self._queues = {name: collections.deque() for name in self.force_fields}
        self._cv = threading.Condition()
        self._done_cv = threading.Condition()  # signalled once per finished batch
        self._closed = False
        self._charges = {}  # session -> its last evaluation (the next step starts from its charges)
        self._charges_lock = threading.Lock()
        self.batches = []  # (force field, requests, atoms, seconds) per batch, for reporting
        self._calcs = [
            {name: Calculator(ff, device=device, max_expanded_atoms=max_expanded_atoms)
             for name, ff in self.force_fields.items()}
            for _ in range(workers)
        ]
        self._reserved = bool(reserve)
        if reserve:
            # size every context for the largest admissible batch up front: a buffer growth during
            # serving would reallocate device memory and stall the other workers' batches
            for calcs in self._calcs:
                for calc in calcs.values():
                    calc.reserve(self.max_batch_atoms, self.max_batch_requests, edges_per_atom=edges_per_atom,
                                 bonds_per_atom=bonds_per_atom)
        # what each context holds without allocating: (atoms, systems, edges, bonds)
        self._caps = [{name: self._capacity(calc) for name, calc in calcs.items()} for calcs in self._calcs]
        self._threads = [threading.Thread(target=self._worker, args=(k,), daemon=True) for k in range(workers)]
        for t in self._threads:
            t.start()

    # ------------------------------------------------------------------ client side
    def submit(self, request, arrival=None):
        """Admit a request; returns a :class:`Pending` that resolves to a :class:`Served`."""
        if request.force_field not in self._queues:
            raise ValueError(f"Unknown force field {request.force_field!r}")
        fut = Pending(self._done_cv)
        request.arrival = time.perf_counter() if arrival is None else arrival
        with self._cv:
            if self._closed:
                raise RuntimeError("server is closed")
            self._queues[request.force_field].append((request, fut))
            self._cv.notify()
        return fut

    def submit_many(self, requests, arrival=None):
        """Admit several requests at once (one lock acquisition and one wake-up for all of them);
        returns their :class:`Pending` handles in order."""
        for request in requests:
            if request.force_field not in self._queues:
                raise ValueError(f"Unknown force field {request.force_field!r}")
        now = time.perf_counter() if arrival is None else arrival
        cv = self._done_cv
        futs = [Pending(cv) for _ in requests]
        queues = self._queues
        with self._cv:
            if self._closed:
                raise RuntimeError("server is closed")
            for request, fut in zip(requests, futs):
                request.arrival = now
                queues[request.force_field].append((request, fut))
            self._cv.notify_all()
        return futs

    def close(self):
        """Stop accepting requests, finish the queued ones and join the workers."""
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _atoms_within(self, share, edges_per_atom, bonds_per_atom):
        """The largest atom bound (at most max_batch_atoms) whose reservation fits ``share`` bytes."""
        def need(a):
            return Calculator.footprint_bytes(a, self.max_batch_requests, int(a * edges_per_atom),
                                              int(a * bonds_per_atom))

        if need(1) > share:
            raise ValueError("memory_budget is too small for a single-atom batch on every worker")
        lo, hi = 1, self.max_batch_atoms
        while lo < hi:
            mid = (lo + hi + 1) // 2
            if need(mid) <= share:
                lo = mid
            else:
                hi = mid - 1
        return lo

    def _capacity(self, calc):
        mem = getattr(calc, "memory", None)
        if mem is None or not self._reserved:
            # unreserved contexts grow on demand, and a calculator without memory reporting has only
            # the configured bounds
            return (self.max_batch_atoms, self.max_batch_requests, float("inf"), float("inf"))
        m = mem()
        return (min(m["atoms"], self.max_batch_atoms), min(m["systems"], self.max_batch_requests), m["edges"],
                m["bonds"])

    def memory_report(self):
        """Device memory of every worker context: bytes and capacities, the admission's densities per
        force field and the number of reallocations during serving."""
        contexts = []
        for k, calcs in enumerate(self._calcs):
            for name, calc in calcs.items():
                if hasattr(calc, "memory"):
                    contexts.append(dict(worker=k, force_field=name, **calc.memory()))
        densities = {name: (f.edges_per_atom, f.bonds_per_atom) for name, f in self.footprints.items()}
        return dict(contexts=contexts, densities=densities, reallocations=self.reallocations)

    # ------------------------------------------------------------------ instrumentation
    def set_profiling(self, enable=True):
        """Per-stage CUDA-event timing on every worker context (resets the accumulators)."""
        for calcs in self._calcs:
            for calc in calcs.values():
                calc.set_profiling(enable)

    def stage_times(self):
        """Summed per-stage device milliseconds over every context, and the number of batches."""
        total, calls = np.zeros(8), 0
        for calcs in self._calcs:
            for calc in calcs.values():
                ms, n = calc.stage_times()
                total += ms
                calls += n
        return total, calls

    # ------------------------------------------------------------------ worker side
    def _take_batch(self, k=0):
        """Oldest-first: the force field whose head request waited longest, then FIFO while the
        batch's estimated footprint fits worker k's context (the first request always goes)."""
        best = None
        for name, q in self._queues.items():
            if q and (best is None or q[0][0].arrival < self._queues[best][0][0].arrival):
                best = name
        if best is None:
            return None, [], (0, 0)
        q = self._queues[best]
        cap_atoms, cap_sys, cap_edges, cap_bonds = self._caps[k][best]
        fp = self.footprints[best]
        batch, atoms, edges, bonds = [], 0, 0.0, 0.0
        while q and len(batch) < cap_sys:
            req = q[0][0]
            n = req.natoms
            p = req.pbc
            e, b = fp.estimate(n, False if p is None or p is False else (True if p is True else bool(np.any(p))))
            if batch and (atoms + n > cap_atoms or edges + e > cap_edges or bonds + b > cap_bonds):
                break
            batch.append(q.popleft())
            atoms, edges, bonds = atoms + n, edges + e, bonds + b
        return best, batch, (edges, bonds)

    def _worker(self, k):
        calcs = self._calcs[k]
        while True:
            with self._cv:
                while not self._closed and not any(self._queues.values()):
                    self._cv.wait()
                name, batch, est = self._take_batch(k)
                if not batch:
                    if self._closed:
                        return
                    continue
            try:
                self._run(calcs[name], name, batch, est, k)
            except BaseException as err:  # noqa: BLE001 - an unexpected failure fails the batch, not the worker
                for _, fut in batch:
                    if not fut._done:
                        fut._error = err if isinstance(err, Exception) else RuntimeError(repr(err))
                        fut._done = True
                with self._done_cv:
                    self._done_cv.notify_all()

    def _run(self, calc, name, batch, est=(0, 0), k=0):
        charges = self._charges
        warm = self.warm_start
        items = []
        with self._charges_lock:
            for req, _ in batch:
                prev = charges.get(req.session) if warm and req.session is not None else None
                g = None if prev is None else prev.charges  # the session's last evaluation
                if g is not None and len(g) != len(req.symbols):
                    g = None
                items.append((req.symbols, req.positions, req.total_charge, req.cell, req.pbc, g))
        t0 = time.perf_counter()
        try:
            results = calc._evaluate_items(items)
        except Exception:
            # isolate the failing request(s): evaluate one by one
            results = []
            for it in items:
                try:
                    results.append(calc._evaluate_items([it])[0])
                except Exception as err:  # noqa: BLE001 - reported through the future
                    results.append(err)
        done = time.perf_counter()
        its, qbytes = calc.qeq_work()
        h2d, d2h = calc.transfer_bytes()
        edges, dev_bytes = 0, 0
        if hasattr(calc, "memory"):
            sizes = calc.list_sizes()
            edges = sizes[0]
            before = self._caps[k][name]
            cap = self._capacity(calc)
            dev_bytes = calc.memory()["device_bytes"]
            # no server lock: the densities only rise (a lost update between two workers is re-learned
            # on a later batch), and worker k alone reads and writes its contexts' capacities
            self.footprints[name].observe(est[0], sizes[0], est[1], sizes[2])
            if cap != before:
                self.reallocations += 1
                self._caps[k][name] = cap
        self.batches.append(Batch(name, len(batch), sum(len(it[0]) for it in items), done - t0, calc.last_launches,
                                  its, qbytes, h2d, d2h, int(est[0]), edges, dev_bytes))
        nb = len(batch)
        with self._charges_lock:
            for (req, fut), res in zip(batch, results):
                if isinstance(res, Exception):
                    fut._error = res
                else:
                    if req.session is not None:
                        charges[req.session] = res  # its charges are read when the session's next step comes
                    fut._value = Served(res, req.arrival, done, nb, t0)
                fut._done = True
        with self._done_cv:
            self._done_cv.notify_all()


def replay(server, requests, arrivals=None, speedup=1.0):
    """Submit ``requests`` at their ``arrivals`` (seconds from the start; None = all at once) and
    wait for all results. Returns (list of Served or exceptions in request order, wall seconds)."""
    t_start = time.perf_counter()
    if arrivals is None:
        futures = server.submit_many(requests, arrival=t_start)
    else:
        futures = []
        for k, req in enumerate(requests):
            target = t_start + arrivals[k] / speedup
            delay = target - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            futures.append(server.submit(req, arrival=max(target, t_start)))
    out = []
    for f in futures:
        try:
            out.append(f.result())
        except Exception as err:  # noqa: BLE001
            out.append(err)
    return out, time.perf_counter() - t_start
