#!/usr/bin/env python
"""Benchmark: served vs plain atoms*evals/s of E+F+QEq requests on one GB300, with p50/p99 latency.

Workload (the serving stream): 4,096 seeded E+F+QEq requests, sizes log-uniform on 3-512 atoms,
clusters of H2O (ffield.reax.HO.2015) or CH4/O2/H2O/CO2 (ffield.reax.CHO.2008) 50/50, 10 % periodic
cubic cells of 20-30 A, 1 % net charge +-1, Poisson arrivals at 2,000 req/s, 25 % repeat
evaluations of an earlier system with 0.01 A jitter (warm-started QEq). FP64 throughout.

One step = one pass of the whole stream through the continuous-batching server
(``xreac_gb300.serving.Server``, two worker contexts), all requests admitted at once (saturated).

- ``value``: atoms ÷ device time of the served batches (CUDA events on each worker's stream from
  the first kernel to the last of every batch; inputs and outputs cross the bus outside it).
- ``e2e``: atoms ÷ wall time of the same passes through ``Server.submit`` with host numpy arrays
  (requests in, ``Evaluation`` results out); ``plain``: the same stream through one
  ``Calculator.evaluate`` call per request; ``served_over_plain`` = e2e / plain.
- ``latency_ms``: p50/p99 of completion minus arrival when the stream is replayed in real time at its
  Poisson arrival times.
- ``roofline``: the dominant stage of the served batches (the QEq solve): matrix-free algorithmic
  bytes (iterations x (8 B per pair + 16 B per atom)) ÷ its CUDA-event time.
- ``water_box``: the 4,608-atom periodic water box (1,536 H2O, 35.8 A) evaluated alone with
  device-resident positions, L2 flushed before every step: per-stage times and the roofline of its
  dominant kernel (k_qeq_grid).
- ``differentiation``: 256 perturbed copies of the TiO2/water slab: reference E+F, then the E+F
  squared-error loss and its force-field parameter gradient (device adjoint) per copy.
- ``cpu_baseline``: the unmodified reference (xreac v0.10.0 installed in ``baseline/_ref``, run through
  the torch-backed autograd stand-in of ``tests/golden/shim``) on a sample of the stream; the CPU
  oracle (the reference's algorithm restated) only where that install is absent.

``--impl reference`` times the same reference, one ``xreac.Calculator.evaluate`` per request of the
same seeded stream (consecutive requests, each step a bounded sample), with every host thread, and
prints the same JSON line with ``"impl": "reference"`` and the same ``config``. That arm imports
nothing of the product package: the stream comes from ``xreac_gb300/workloads.py`` loaded from its
file (pure numpy), and force fields are parsed by the reference itself.
"""

from __future__ import annotations

import argparse
import dataclasses
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "atoms*evals/s (E+F+QEq, <=1e-8 rel E) served vs plain on 1 GB300; p50/p99 ms"
UNIT = "atoms*evals/s"
WORKLOAD = ("serving stream: 4096 E+F+QEq requests, 3-512 atoms log-uniform, HO.2015/CHO.2008 50/50, "
            "10% periodic 20-30 A cubes, 1% charged, 25% repeats with 0.01 A jitter, Poisson 2000 req/s")
BOX_WORKLOAD = "plain E+F+QEq, periodic liquid water, 1536 H2O = 4608 atoms, 35.8 A cubic cell, ffield.reax.HO.2015"
FORCE_FIELDS = ("ffield.reax.HO.2015", "ffield.reax.CHO.2008")


def peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


class NvmlClockSampler:
    """SM clock and clock-event reasons polled through NVML (ctypes) every few ms during the timed
    region; read-only queries. Falls back to ``nvidia-smi -lms 200`` when NVML cannot be loaded."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, device=0, period_s=0.002):
        self.device = device
        self.period = period_s
        self.sm, self.reasons, self.max_mhz = [], set(), None
        self.lib = self.handle = None
        self.stop = threading.Event()
        self.thread = None
        self.fallback = None

    def _open(self):
        import ctypes

        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        handle = ctypes.c_void_p()
        bus = None
        try:
            import torch

            pr = torch.cuda.get_device_properties(self.device)
            bus = f"{pr.pci_domain_id:08X}:{pr.pci_bus_id:02X}:{pr.pci_device_id:02X}.0"
        except Exception:
            bus = None
        ok = bus is not None and lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(handle)) == 0
        if not ok and lib.nvmlDeviceGetHandleByIndex_v2(self.device, ctypes.byref(handle)) != 0:
            raise OSError("no NVML handle")
        mx = ctypes.c_uint()
        if lib.nvmlDeviceGetMaxClockInfo(handle, 1, ctypes.byref(mx)) == 0:
            self.max_mhz = float(mx.value)
        self.lib, self.handle = lib, handle

    def _poll(self):
        import ctypes

        clk = ctypes.c_uint()
        rs = ctypes.c_ulonglong()
        get_reasons = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None)
        while not self.stop.is_set():
            if self.lib.nvmlDeviceGetClockInfo(self.handle, 1, ctypes.byref(clk)) == 0:
                self.sm.append(float(clk.value))
            if get_reasons is not None and get_reasons(self.handle, ctypes.byref(rs)) == 0:
                for bit, name in self.REASONS.items():
                    if rs.value & bit:
                        self.reasons.add(name)
            time.sleep(self.period)

    def __enter__(self):
        try:
            self._open()
        except Exception:
            self.fallback = SmiClockSampler(self.device).__enter__()
            return self
        self.thread = threading.Thread(target=self._poll, daemon=True)
        self.thread.start()
        return self

    def __exit__(self, *exc):
        if self.fallback is not None:
            return self.fallback.__exit__(*exc)
        self.stop.set()
        if self.thread is not None:
            self.thread.join(timeout=2)

    def summary(self):
        if self.fallback is not None:
            return self.fallback.summary()
        if not self.sm:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": sorted(self.reasons), "samples": 0,
                    "source": "nvml"}
        return {"sm_mhz": statistics.median(self.sm), "sm_max_mhz": self.max_mhz or max(self.sm),
                "reasons": sorted(self.reasons), "samples": len(self.sm), "source": "nvml"}


class SmiClockSampler:
    """nvidia-smi clock and throttle-reason samples during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return self

        def reader():
            for line in self.proc.stdout:
                self.rows.append([v.strip() for v in line.split(",")])

        self.thread = threading.Thread(target=reader, daemon=True)
        self.thread.start()
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0, "source": "nvidia-smi"}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm),
                "source": "nvidia-smi"}


def profiled_traffic(kernel):
    """DRAM bytes per launch of ``kernel`` recorded from an ``ncu`` capture in profiles/traffic.txt."""
    path = ROOT / "profiles" / "traffic.txt"
    try:
        for line in path.read_text().splitlines():
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kernel and not line.startswith("#"):
                return float(parts[1])
    except OSError:
        pass
    return None


def profiled_fp64(kernel):
    """FP64-pipe utilisation (% of peak, elapsed) of ``kernel`` from an ``ncu`` capture, recorded in
    profiles/fp64_pipe.txt."""
    path = ROOT / "profiles" / "fp64_pipe.txt"
    try:
        for line in path.read_text().splitlines():
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kernel and not line.startswith("#"):
                return float(parts[1])
    except OSError:
        pass
    return None


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


REFERENCE_DIR = ROOT / "baseline" / "_ref"
SHIM_DIR = ROOT / "tests" / "golden" / "shim"


def workloads_module():
    """The seeded input generator, ``xreac_gb300/workloads.py`` (numpy only), loaded from its file under
    its own name: the reference arm gets the same requests without importing the product package."""
    import importlib.util

    name = "xr_bench_workloads"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, ROOT / "xreac_gb300" / "workloads.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def reference_package():
    """``(xreac module, None)`` for the unmodified reference installed in baseline/_ref, or ``(None,
    reason)``. Every installed file must still match the SHA-256 recorded at install time, which in
    turn matched the reference checkout (baseline/install_reference.py). HIPS autograd is absent, so
    its torch-backed stand-in goes first on sys.path."""
    import hashlib

    record = REFERENCE_DIR / "XREAC_INSTALL.json"
    if not record.is_file():
        return None, "baseline/_ref is not installed (python baseline/install_reference.py <checkout>)"
    rec = json.loads(record.read_text())
    for rel, v in rec["files"].items():
        path = REFERENCE_DIR / "xreac" / rel
        if not path.is_file() or hashlib.sha256(path.read_bytes()).hexdigest() != v["sha256"] \
                or v["sha256"] != v["source_sha256"]:
            return None, f"baseline/_ref/xreac/{rel} differs from the reference checkout"
    for p in (str(REFERENCE_DIR), str(SHIM_DIR)):
        if p not in sys.path:
            sys.path.insert(0, p)
    import xreac

    if Path(xreac.__file__).resolve().parent != (REFERENCE_DIR / "xreac").resolve():
        return None, f"another xreac shadows baseline/_ref ({xreac.__file__})"
    return xreac, None


def stream_requests():
    """The serving stream as server requests (sessions mark repeat evaluations)."""
    from xreac_gb300.serving import Request

    stream = workloads_module().request_stream()
    reqs = [Request(r.system.symbols, r.system.positions, r.system.force_field, r.system.cell, r.system.pbc,
                    r.system.total_charge, session=r.index if r.repeat_of is None else r.repeat_of) for r in stream]
    arrivals = np.array([r.arrival for r in stream])
    return reqs, arrivals - arrivals[0]


def serialised_device(reqs, ffs, local, steps, warmup):
    """The stream's batches (the server's grouping: per force field in arrival order, up to
    SERVER_BATCH_ATOMS atoms each) evaluated one after another on one context per force field, with
    CUDA-event stage times: the device time of a pass when no two batches overlap. Returns the
    stage milliseconds per pass, the QEq algorithmic bytes per pass, kernel launches per pass and
    the number of batches per pass."""
    from xreac_gb300 import Calculator

    calcs = {name: Calculator(ff, device=local) for name, ff in ffs.items()}
    for c in calcs.values():
        c.reserve(SERVER_BATCH_ATOMS, 512)
    batches, cur, held = [], {n: [] for n in ffs}, {n: 0 for n in ffs}
    for r in reqs:
        n = r.force_field
        if cur[n] and held[n] + r.natoms > SERVER_BATCH_ATOMS:
            batches.append((n, cur[n]))
            cur[n], held[n] = [], 0
        cur[n].append((r.symbols, r.positions, r.total_charge, r.cell, r.pbc, None))
        held[n] += r.natoms
    batches += [(n, items) for n, items in cur.items() if items]
    for _ in range(max(warmup, 1)):
        for n, items in batches[:4]:
            calcs[n]._evaluate_items(items)
    for c in calcs.values():
        c.set_profiling(True)
    qbytes, launches = 0.0, 0
    for _ in range(steps):
        for n, items in batches:
            calcs[n]._evaluate_items(items)
            qbytes += calcs[n].qeq_work()[1]
            launches += calcs[n].last_launches
    total = np.zeros(len(STAGE_NAMES))
    for c in calcs.values():
        total += c.stage_times()[0]
        c.set_profiling(False)
    return total / steps, qbytes / steps, launches / steps, len(batches)


def stream_pass(reqs, tag, part=None):
    """A fresh copy of the stream (or of its first ``part`` requests) for one pass: session keys are
    tagged with the pass, so the only warm starts are the stream's own repeat evaluations (25 %,
    0.01 A jitter), never a request started from the charges of the identical request in an
    earlier pass."""
    return [dataclasses.replace(r, session=None if r.session is None else (tag, r.session))
            for r in (reqs if part is None else reqs[:part])]


class CpuArm:
    """The CPU implementation timed as the reference: the unmodified xreac from baseline/_ref
    (``kind`` "reference"), or, where it is absent, the CPU oracle ("port")."""

    def __init__(self):
        self.xreac, why = reference_package()
        self.kind = "reference" if self.xreac is not None else "port"
        self.why = why
        self.calcs = {}
        if self.xreac is None:
            import oracle

            self.oracle = oracle

    def describe(self):
        if self.kind == "reference":
            return ("unmodified xreac v0.10.0 (baseline/_ref), Calculator.evaluate per request; HIPS autograd "
                    "replaced by the torch-backed stand-in tests/golden/shim")
        return f"CPU oracle (the reference's algorithm restated; {self.why})"

    def evaluate(self, system):
        s = system
        if self.kind == "reference":
            calc = self.calcs.get(s.force_field)
            if calc is None:
                calc = self.calcs[s.force_field] = self.xreac.Calculator(self.xreac.ForceField.bundled(s.force_field))
            return calc.evaluate(s.symbols, s.positions, total_charge=s.total_charge, cell=s.cell, pbc=s.pbc)
        from xreac_gb300.forcefield import ForceField

        ff = self.calcs.get(s.force_field)
        if ff is None:
            ff = self.calcs[s.force_field] = ForceField.bundled(s.force_field)
        return self.oracle.evaluate(ff, s.symbols, s.positions, total_charge=s.total_charge, cell=s.cell, pbc=s.pbc,
                                    dense_bond_orders=False)

    def sample(self, stream, start, budget_s, min_requests=1):
        """Consecutive requests of the stream from ``start`` (wrapping) until ``budget_s`` is spent.
        Returns (atoms evaluated, seconds, requests evaluated)."""
        atoms, k, t0 = 0, start, time.perf_counter()
        while k - start < min_requests or time.perf_counter() - t0 < budget_s:
            r = stream[k % len(stream)]
            self.evaluate(r.system)
            atoms += r.system.n
            k += 1
        return atoms, time.perf_counter() - t0, k - start


def bench_config(atoms):
    """``config`` of both arms' lines: the workload, whatever implementation runs it."""
    return {"workload": WORKLOAD, "requests": 4096, "atoms_per_pass": atoms,
            "l2": "not flushed: every pass streams 4,096 distinct systems (inputs about 13 MB)"}


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    import torch

    cores = os.cpu_count() or 1
    torch.set_num_threads(cores)
    stream = workloads_module().request_stream()
    atoms_per_pass = sum(r.system.n for r in stream)
    arm = CpuArm()
    step_budget = float(os.environ.get("XR_REFERENCE_STEP_S", "5"))
    pos = 0
    for _ in range(max(args.warmup, 1)):
        _, _, n = arm.sample(stream, pos, 0.0)
        pos += n
    atoms, secs, nreq, first = 0, 0.0, 0, pos
    for _ in range(args.steps):
        a, t, n = arm.sample(stream, pos, step_budget)
        atoms, secs, nreq, pos = atoms + a, secs + t, nreq + n, pos + n
    value = atoms / secs
    sample = (f"requests {first}..{pos - 1} of the stream ({nreq} requests, {atoms} atoms) in arrival order, one "
              f"evaluation each; {args.steps} steps of about {step_budget:.0f} s, {cores} threads")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": max(args.warmup, 1),
        "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded request stream; molecules placed at random)",
        "config": bench_config(atoms_per_pass),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": arm.kind,
                         "sample": sample, "implementation": arm.describe()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def water_box_numbers(lib, nat, local, steps, warmup):
    """The 4,608-atom water box alone, device-resident positions: per-stage times and the roofline of
    the QEq kernel (the dominant one)."""
    import ctypes

    import torch
    from xreac_gb300 import Calculator, ForceField, workloads

    system = workloads.water_box()
    n = system.n
    ff = ForceField.bundled(system.force_field)
    calc = Calculator(ff, device=local)
    stream = torch.cuda.current_stream()
    ctx = nat.Context(local, stream.cuda_stream)
    types = np.ascontiguousarray(ff.type_indices(system.symbols))
    cell = np.ascontiguousarray(system.cell, dtype=np.float64)
    pos_dev = torch.tensor(system.positions, dtype=torch.float64, device="cuda")
    out = dict(forces=torch.zeros((n, 3), dtype=torch.float64, device="cuda"),
               charges=torch.zeros(n, dtype=torch.float64, device="cuda"),
               tbo=torch.zeros(n, dtype=torch.float64, device="cuda"),
               nlp=torch.zeros(n, dtype=torch.float64, device="cuda"),
               counts=torch.zeros(n, dtype=torch.int32, device="cuda"))
    energy = np.zeros(15)
    dipole = np.zeros(3)
    sysd = nat.System()
    sysd.natoms = n
    sysd.types = nat.addr(types)
    sysd.positions = pos_dev.data_ptr()
    sysd.cell = nat.addr(cell)
    for d in range(3):
        sysd.pbc[d] = 1
    res = nat.Result()
    res.energy = nat.addr(energy)
    res.forces = out["forces"].data_ptr()
    res.charges = out["charges"].data_ptr()
    res.total_bond_orders = out["tbo"].data_ptr()
    res.lone_pairs = out["nlp"].data_ptr()
    res.bond_counts = out["counts"].data_ptr()
    res.dipole = nat.addr(dipole)

    def step_device():
        code = lib.xr_eval(ctx.handle, calc._ff.handle, ctypes.byref(sysd), nat.XR_FLAG_DEVICE_IO, ctypes.byref(res))
        if code != nat.XR_OK:
            raise RuntimeError(f"xr_eval failed ({code}): {ctx.last_error()}")

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for k in range(max(warmup, 3)):
        flush.fill_(float(k))
        step_device()
    check = calc.evaluate(system.symbols, system.positions, cell=system.cell, pbc=system.pbc)
    assert abs(check.energy - energy[14]) <= 1e-8 * abs(check.energy), (check.energy, energy[14])
    lib.xr_ctx_set_profiling(ctx.handle, 1)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    torch.cuda.synchronize()
    launches = 0
    for k in range(steps):
        flush.fill_(float(k))
        starts[k].record(stream)
        step_device()
        ends[k].record(stream)
        launches += int(lib.xr_last_launches(ctx.handle))
    torch.cuda.synchronize()
    total_ms = sum(s_.elapsed_time(e_) for s_, e_ in zip(starts, ends))
    stage_ms = (ctypes.c_double * 8)()
    calls = ctypes.c_longlong()
    lib.xr_ctx_stage_times(ctx.handle, stage_ms, len(STAGE_NAMES), ctypes.byref(calls))
    sizes = (ctypes.c_longlong * 6)()
    lib.xr_last_list_sizes(ctx.handle, sizes, 6)
    stages = {nm: stage_ms[k] / max(calls.value, 1) for k, nm in enumerate(STAGE_NAMES)}
    its = ctypes.c_longlong()
    qbytes = ctypes.c_double()
    lib.xr_last_qeq_work(ctx.handle, ctypes.byref(its), ctypes.byref(qbytes))
    nb_count = ctypes.c_longlong()
    lib.xr_get_neighbors(ctx.handle, 0, None, None, None, 0, ctypes.byref(nb_count))
    pk = peaks()
    hbm_peak = float(pk.get("hbm_gbs", 6800.0))
    achieved = qbytes.value / (stages["qeq_cg"] / 1e3) / 1e9
    pair_bytes = 8.0 * (nb_count.value // 2) + 76.0 * n
    # bond orders: 8 B per candidate half-edge (r <= 5 A), 28 B per atom, 32 B per active bond
    bo_bytes = 8.0 * sizes[2] + 28.0 * n + 32.0 * sizes[4]
    bo_ms = stages["bond_orders"]
    return {
        "workload": BOX_WORKLOAD,
        "value": steps * n / (total_ms / 1e3),
        "unit": UNIT,
        "ms_per_step": total_ms / steps,
        "l2": "flushed before every step (256 MiB write, outside the timed events)",
        "directed_edges": int(nb_count.value),
        "qeq_cg_iterations": int(its.value),
        "stages_ms": stages,
        "gpu_launches_per_step": launches / steps,
        "roofline": {"bound": "hbm", "kernel": "k_qeq_grid", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": profiled_traffic("k_qeq_grid"),
                     "algorithmic_bytes_per_launch": qbytes.value,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in pk else "fallback 6800 GB/s"},
        # the pair kernel against both roofs: its algorithmic bytes (8 B per half pair + 76 B per atom)
        # over the pair stage's event time against HBM, and the FP64 pipe's busy share from ncu
        "pair_kernel": {"kernel": "k_pairs (stage: k_pairs + k_hval)", "bound": "fp64 pipe",
                        "algorithmic_bytes": pair_bytes,
                        "achieved_gbs": pair_bytes / (stages["pairs_vdw_shield"] / 1e3) / 1e9,
                        "hbm_frac": pair_bytes / (stages["pairs_vdw_shield"] / 1e3) / 1e9 / hbm_peak,
                        "fp64_pipe_busy_pct": profiled_fp64("k_pairs"),
                        "traffic": profiled_traffic("k_pairs")},
        "bond_order_kernel": {"kernel": "k_bo1 + k_deltap + k_bo2 (stage: bond_orders)", "bound": "fp64 pipe",
                              "bond_candidates": int(sizes[2]), "active_bonds": int(sizes[4]),
                              "algorithmic_bytes": bo_bytes, "ms": bo_ms,
                              "achieved_gbs": bo_bytes / (bo_ms / 1e3) / 1e9,
                              "hbm_frac": bo_bytes / (bo_ms / 1e3) / 1e9 / hbm_peak,
                              "fp64_pipe_busy_pct": {"k_bo1": profiled_fp64("k_bo1"), "k_bo2": profiled_fp64("k_bo2")},
                              "traffic": {"k_bo1": profiled_traffic("k_bo1"), "k_bo2": profiled_traffic("k_bo2")}},
    }


def differentiation_numbers(local, copies=256):
    """The differentiation workload: per perturbed copy, the E+F squared-error loss against the
    unperturbed force field's E, F and its parameter gradient (device adjoint). The copies' force
    fields are parameter sets of one device force field, so the workload is three batched device
    calls: the reference E, F of every copy, the copies at x with a gradient per system, and the
    copies at x +- h v (the force term's central difference)."""
    import torch
    from xreac_gb300 import Calculator, ForceField, workloads
    from xreac_gb300.differentiation import perturbed_copies_loss

    base = ForceField.bundled("ffield.reax.TiOH.Kim2013")
    pairs = list(workloads.perturbed_copies(n_copies=copies))
    calc = Calculator(base, device=local)
    perturbed_copies_loss(pairs, base, calculator=calc)  # warm-up: context, buffers, parameter sets
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = perturbed_copies_loss(pairs, base, calculator=calc)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    n = len(out.losses)
    return {"workload": f"{copies} perturbed copies of the anatase TiO2 4x4x1 slab + 32 H2O (288 atoms), "
                        "ffield.reax.TiOH.Kim2013, +-2% bond/angle/vdW parameters, 0.05 A displacements",
            "copies": n, "seconds": wall, "ms_per_copy": 1e3 * wall / n,
            "evaluations_per_copy": 4, "atoms_evals_per_s": 4 * 288 * n / wall,
            "mean_loss": float(np.mean(out.losses)), "parameters": len(out.vector),
            "note": "each copy's force field is a parameter set of one device force field; three batched calls: "
                    "reference E+F of all copies, the copies at x with per-system parameter gradients, the copies "
                    "at x +- h v (force term's central difference) with per-system gradients"}


# Server shape: six worker contexts keep enough batches in flight to fill the GPU (measured on one GB300:
# 3.5 M atoms*evals/s with two workers, 4.7 M with four, 5.0 M with six and 8,192-atom batches, after which
# the host's Python work per request bounds it). A batch's QEq lasts about as long as its largest
# systems' cluster solves, so batches of 16,384 atoms spread that time over twice the atoms: the
# serialised device time of a pass fell from 77 to 52 ms (QEq 35 to 20 ms), with the wall-clock
# throughput and the latencies unchanged.
SERVER_WORKERS = 6
SERVER_BATCH_ATOMS = 16384

STAGE_NAMES = ["neighbour_count_scan", "neighbour_fill_reverse", "pairs_vdw_shield", "qeq_cg", "charge_response",
               "bond_orders", "bonded_terms_and_adjoint", "coulomb_forces_reduce_pack"]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", choices=("serving", "water"),
                    help="only run W + K passes of one workload (for an ncu launch list or capture) and print a "
                         "short summary: 'serving' streams the requests through the server, 'water' evaluates the "
                         "4,608-atom water box")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from xreac_gb300 import Calculator, ForceField
    from xreac_gb300 import _native as nat
    from xreac_gb300.build import build
    from xreac_gb300.serving import Server, replay

    build()
    lib = nat.load()
    reqs, arrivals = stream_requests()
    atoms = sum(r.natoms for r in reqs)
    ffs = {name: ForceField.bundled(name) for name in FORCE_FIELDS}
    if args.profile == "water":
        d = water_box_numbers(lib, nat, local, max(args.steps, 1), args.warmup)
        print(json.dumps({"profile": "water", "ms_per_step": d["ms_per_step"], "stages_ms": d["stages_ms"]}), flush=True)
        return 0
    if args.profile == "serving":
        with Server(ffs, workers=SERVER_WORKERS, max_batch_atoms=SERVER_BATCH_ATOMS, device=local) as srv:
            for k in range(args.warmup):
                replay(srv, stream_pass(reqs, ("warmup", k), 512))
            for k in range(args.steps):
                out, _ = replay(srv, stream_pass(reqs, ("timed", k)))
            nb = len(srv.batches)
        print(json.dumps({"profile": "serving", "passes": args.steps, "batches": nb,
                          "errors": sum(isinstance(o, Exception) for o in out)}), flush=True)
        return 0

    # plain: one Calculator.evaluate per request, in arrival order
    plain = {name: Calculator(ff, device=local) for name, ff in ffs.items()}
    for r in reqs[:64]:
        plain[r.force_field].evaluate(r.symbols, r.positions, cell=r.cell, pbc=r.pbc, total_charge=r.total_charge)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in reqs:
        plain[r.force_field].evaluate(r.symbols, r.positions, cell=r.cell, pbc=r.pbc, total_charge=r.total_charge)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    plain_value = world * atoms / plain_s

    # served: whole-stream passes through the continuous-batching server
    warm_passes = [stream_pass(reqs, ("warmup", k), 512) for k in range(max(args.warmup, 3))]
    timed_passes = [stream_pass(reqs, ("timed", k)) for k in range(args.steps)]
    latency_pass = stream_pass(reqs, "latency")
    with Server(ffs, workers=SERVER_WORKERS, max_batch_atoms=SERVER_BATCH_ATOMS, device=local) as srv:
        for wp in warm_passes:
            replay(srv, wp)
        # The long-lived objects made so far (the stream's copies, force fields, contexts) go to the
        # collector's permanent generation, as a serving process does after start-up: otherwise every
        # full collection during the timed passes walks them again.
        gc.collect()
        gc.freeze()
        srv.batches.clear()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        wall = []
        with NvmlClockSampler(local) as clocks:
            for tp in timed_passes:
                t0 = time.perf_counter()
                out, _ = replay(srv, tp)
                torch.cuda.synchronize()
                wall.append(time.perf_counter() - t0)
        if dist is not None:
            dist.barrier()
        errors = sum(isinstance(o, Exception) for o in out)
        timed_passes.clear()
        batches = list(srv.batches)
        # latency: the stream replayed at its arrival times, with the throughput passes' results
        # released first
        del out
        gc.collect()
        gc.freeze()
        srv.batches.clear()
        timed, _ = replay(srv, latency_pass, arrivals=arrivals)
        lat = np.array([o.latency for o in timed if not isinstance(o, Exception)]) * 1e3
        qwait = np.array([o.queued for o in timed if not isinstance(o, Exception)]) * 1e3
        replay_batches = len(srv.batches)
    # device time of a pass with the batches run one after another (no overlap between batches)
    stage_ms, qeq_bytes, serial_launches, serial_batches = serialised_device(reqs, ffs, local, args.steps,
                                                                             args.warmup)
    device_ms = float(stage_ms.sum())
    wall_s = float(sum(wall))
    if dist is not None:
        t = torch.tensor([device_ms, wall_s], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        device_ms, wall_s = float(t[0]), float(t[1])
    value = world * atoms / (device_ms / 1e3)
    e2e_value = world * atoms * args.steps / wall_s
    stages = {nm: float(stage_ms[k]) for k, nm in enumerate(STAGE_NAMES)}
    dominant = max(stages, key=stages.get)
    qeq_achieved = qeq_bytes / (stages["qeq_cg"] / 1e3) / 1e9
    pk = peaks()
    hbm_peak = float(pk.get("hbm_gbs", 6800.0))
    # bytes crossing the bus per pass, counted by the library per batch
    h2d = sum(b.h2d_bytes for b in batches) // args.steps
    d2h = sum(b.d2h_bytes for b in batches) // args.steps
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": max(args.warmup, 3),
        "ms_per_step": device_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded request stream; molecules placed at random)",
        "config": bench_config(atoms),
        "server": {"workers": SERVER_WORKERS, "max_batch_atoms": SERVER_BATCH_ATOMS,
                   "parallelism": "replicas" if world > 1 else "single"},
        "plain": {"value": plain_value, "unit": UNIT, "ms_per_request": 1e3 * plain_s / len(reqs),
                  "api": "one xreac_gb300.Calculator.evaluate per request"},
        "served_over_plain": e2e_value / plain_value,
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "max": float(lat.max()), "queue_p50": float(np.percentile(qwait, 50)),
                       "queue_p99": float(np.percentile(qwait, 99)), "arrival_rate_per_s": 2000,
                       "batches": replay_batches, "requests": int(len(lat)), "max_atoms_per_request": 512},
        "roofline": {"bound": "hbm", "kernel": "k_qeq_cluster (QEq solve of the served batches)",
                     "achieved": qeq_achieved, "peak": hbm_peak, "unit": "GB/s", "frac": qeq_achieved / hbm_peak,
                     "traffic": profiled_traffic("k_qeq_cluster"),
                     "algorithmic_bytes_per_launch": qeq_bytes / max(serial_batches, 1), "dominant_stage": dominant,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in pk else "fallback 6800 GB/s",
                     "note": "achieved = matrix-free algorithmic bytes / QEq event time, averaged over the launches "
                             "(one per batch); traffic = DRAM bytes of one served batch's launch from an ncu "
                             "capture. The solve keeps its matrix rows on chip and is bound by the cluster "
                             "exchanges and shared-memory gathers, not HBM"},
        "stages_ms_per_pass": stages,
        "device_time": "value, ms_per_step and stages: the stream's batches (16,384 atoms at most, per force field) "
                       "evaluated one after another on one context, CUDA events per stage, no overlap between batches; "
                       "e2e: the server's workers run batches concurrently",
        "batches_per_pass": len(batches) / args.steps,
        "errors": errors,
        "clocks": clocks.summary(),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "pass_ms": [round(1e3 * t, 2) for t in wall],
                "api": "xreac_gb300.serving.Server.submit_many (the whole pass at once) with host numpy arrays, "
                       "results as Evaluation objects"},
        "gpu_launches": int(sum(b.launches for b in batches)),
    }
    line["water_box"] = water_box_numbers(lib, nat, local, max(3, min(args.steps * 4, 20)), args.warmup)
    line["differentiation"] = differentiation_numbers(local)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        torch.set_num_threads(cores)
        arm = CpuArm()
        stream = workloads_module().request_stream()
        arm.sample(stream, 0, 0.0)  # imports and first-call costs
        a, secs, n = arm.sample(stream, 1, 10.0)
        line["cpu_baseline"] = {
            "value": a / secs,
            "unit": UNIT,
            "cores": cores,
            "kind": arm.kind,
            "sample": f"requests 1..{n} of the stream ({a} atoms) evaluated one by one, {cores} threads",
            "implementation": arm.describe(),
        }
    if dist is not None:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
