#!/usr/bin/env python
"""Benchmark: atoms*evals/s of full E+F+QEq evaluations of the 4,608-atom periodic water box.

Workload: 1,536 rigid H2O (O-H 0.97 A, H-O-H 104.5 deg) in a 35.8 A cubic cell (1.0 g/cm^3),
seeded placement with minimum-image O-O >= 2.5 A and 0.05 A Gaussian jitter on every atom,
ffield.reax.HO.2015, FP64. One step = one complete evaluation: neighbour list, bond orders,
QEq charges, the 14 energy components and fixed-charge forces.

- ``value``: device-resident positions (uploaded before timing), results left on the device;
  per-step CUDA events on the library's stream, L2 flushed (256 MiB write) before every step,
  the flush outside the events.
- ``e2e``: the public ``Calculator.evaluate`` with host numpy arrays: host->device copy of the
  inputs, device->host copy of energy, forces, charges and bond properties every step.
- ``roofline``: the dominant kernel's (QEq) algorithmic bytes / live CUDA-event time against the
  measured HBM copy bandwidth; ``cpu_baseline``: the CPU oracle on the host cores.

``--impl reference`` times the CPU oracle (the reference's algorithm restated for the CPU) on the
same workload, using every host thread, and prints the same JSON line with ``"impl": "reference"``.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "atoms*evals/s (E+F+QEq, <=1e-8 rel E)"
UNIT = "atoms*evals/s"
WORKLOAD = "plain E+F+QEq, periodic liquid water, 1536 H2O = 4608 atoms, 35.8 A cubic cell, ffield.reax.HO.2015"


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


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def oracle_eval_seconds(system, budget_s, min_runs=1, max_runs=1000):
    """Time full CPU-oracle evaluations of ``system`` until ``budget_s`` is spent."""
    import oracle
    from xreac_gb300.forcefield import ForceField

    ff = ForceField.bundled(system.force_field)
    times = []
    t_start = time.perf_counter()
    while len(times) < max_runs and (len(times) < min_runs or time.perf_counter() - t_start < budget_s):
        t0 = time.perf_counter()
        oracle.evaluate(ff, system.symbols, system.positions, cell=system.cell, pbc=system.pbc, dense_bond_orders=False)
        times.append(time.perf_counter() - t0)
    return times


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    import torch
    from xreac_gb300 import workloads

    cores = os.cpu_count() or 1
    torch.set_num_threads(cores)
    system = workloads.water_box()
    n = system.n
    warm = oracle_eval_seconds(system, 0.0, min_runs=max(1, min(args.warmup, 1)), max_runs=max(1, min(args.warmup, 1)))
    budget = float(os.environ.get("XR_REFERENCE_BUDGET_S", "150"))
    times = oracle_eval_seconds(system, budget, min_runs=1, max_runs=args.steps)
    steps = len(times)
    total = sum(times)
    value = n * steps / total
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": steps,
        "warmup": len(warm),
        "ms_per_step": 1e3 * total / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "atoms": n, "parallelism": "cpu"},
        "cpu_baseline": {
            "value": value,
            "unit": UNIT,
            "cores": cores,
            "kind": "port",
            "sample": f"{steps} full evaluations of the {n}-atom box by the CPU oracle (torch/numpy FP64, "
                      f"{cores} threads); steps capped by a {budget:.0f} s budget",
        },
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import ctypes

    import numpy as np
    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from xreac_gb300 import Calculator, ForceField, workloads
    from xreac_gb300 import _native as nat
    from xreac_gb300.build import build

    build()
    system = workloads.water_box()
    n = system.n
    ff = ForceField.bundled(system.force_field)
    calc = Calculator(ff, device=local)
    lib = nat.load()
    # The library's context runs on torch's current stream, so events recorded there time it.
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
    sysd.types = nat.ptr(types, nat.c_int)
    sysd.positions = ctypes.cast(pos_dev.data_ptr(), ctypes.POINTER(ctypes.c_double))
    sysd.cell = nat.ptr(cell, nat.c_double)
    for d in range(3):
        sysd.pbc[d] = 1
    sysd.total_charge = 0.0
    res = nat.Result()
    res.energy = nat.ptr(energy, nat.c_double)
    res.forces = ctypes.cast(out["forces"].data_ptr(), ctypes.POINTER(ctypes.c_double))
    res.charges = ctypes.cast(out["charges"].data_ptr(), ctypes.POINTER(ctypes.c_double))
    res.total_bond_orders = ctypes.cast(out["tbo"].data_ptr(), ctypes.POINTER(ctypes.c_double))
    res.lone_pairs = ctypes.cast(out["nlp"].data_ptr(), ctypes.POINTER(ctypes.c_double))
    res.bond_counts = ctypes.cast(out["counts"].data_ptr(), ctypes.POINTER(ctypes.c_int))
    res.dipole = nat.ptr(dipole, nat.c_double)

    def step_device():
        code = lib.xr_eval(ctx.handle, calc._ff.handle, ctypes.byref(sysd), nat.XR_FLAG_DEVICE_IO, ctypes.byref(res))
        if code != nat.XR_OK:
            raise RuntimeError(f"xr_eval failed ({code}): {ctx.last_error()}")

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for k in range(max(args.warmup, 3)):
        flush.fill_(float(k))
        step_device()
    # energy parity spot check of the timed configuration against the host API
    check = calc.evaluate(system.symbols, system.positions, cell=system.cell, pbc=system.pbc)
    assert abs(check.energy - energy[14]) <= 1e-8 * abs(check.energy), (check.energy, energy[14])

    lib.xr_ctx_set_profiling(ctx.handle, 1)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches = 0
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with NvmlClockSampler(local) as clocks:
        t_wall = time.perf_counter()
        for k in range(args.steps):
            flush.fill_(float(k))
            starts[k].record(stream)
            step_device()
            ends[k].record(stream)
            launches += int(lib.xr_last_launches(ctx.handle))
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    if dist is not None:
        dist.barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = sum(step_ms)
    if dist is not None:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * n * args.steps / (total_ms / 1e3)
    stage_ms = (ctypes.c_double * 8)()
    calls = ctypes.c_longlong()
    lib.xr_ctx_stage_times(ctx.handle, stage_ms, 7, ctypes.byref(calls))
    stage_names = ["neighbour_count_scan", "neighbour_fill_reverse", "pairs_vdw_shield", "qeq_cg", "coulomb",
                   "bonded_and_adjoint", "forces_reduce_pack"]
    stages = {nm: stage_ms[k] / max(calls.value, 1) for k, nm in enumerate(stage_names)}
    qeq_iterations = int(lib.xr_last_qeq_iterations(ctx.handle))

    # e2e: the public API with host arrays, every step copying inputs in and results out
    h2d = ctypes.c_longlong()
    d2h = ctypes.c_longlong()
    for _ in range(2):
        calc.evaluate(system.symbols, system.positions, cell=system.cell, pbc=system.pbc)
    e2e_steps = max(5, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        r = calc.evaluate(system.symbols, system.positions, cell=system.cell, pbc=system.pbc)
        _ = r.energy
    e2e_s = time.perf_counter() - t0
    lib.xr_last_transfer_bytes(calc._ctx.handle, ctypes.byref(h2d), ctypes.byref(d2h))
    e2e_value = world * n * e2e_steps / e2e_s

    # Roofline of the dominant kernel (the QEq solve, one k_qeq_grid launch per evaluation, timed
    # alone between the stage events on the library stream). Algorithmic bytes per launch: a
    # matrix-free mat-vec reads 8 B per unordered pair and 16 B per atom per CG iteration.
    pk = peaks()
    dominant = max(stages, key=stages.get)
    nb_count = ctypes.c_longlong()
    lib.xr_get_neighbors(ctx.handle, 0, None, None, None, 0, ctypes.byref(nb_count))
    m_half = nb_count.value // 2
    hbm_peak = float(pk.get("hbm_gbs", 6800.0))
    peak_source = "MEASURED_PEAKS.json hbm_gbs (burst copy)" if "hbm_gbs" in pk else "fallback 6800 GB/s"
    qeq_bytes = (8 * m_half + 16 * n) * max(qeq_iterations, 1)
    qeq_achieved = qeq_bytes / (stages["qeq_cg"] / 1e3) / 1e9
    roofline = {
        "bound": "hbm",
        "kernel": "k_qeq_grid",
        "achieved": qeq_achieved,
        "peak": hbm_peak,
        "unit": "GB/s",
        "frac": qeq_achieved / hbm_peak,
        "traffic": profiled_traffic("k_qeq_grid"),
        "algorithmic_bytes_per_launch": qeq_bytes,
        "peak_source": peak_source,
        "dominant_stage": dominant,
        "note": "latency/FP64-bound: CG iterations are separated by grid barriers; matrix rows stay on chip",
    }
    pair_bytes = 8 * m_half + 76 * n
    pair_achieved = pair_bytes / (stages["pairs_vdw_shield"] / 1e3) / 1e9
    roofline_pairs = {"bound": "hbm", "kernel": "k_pairs + k_hval", "achieved": pair_achieved, "peak": hbm_peak,
                      "unit": "GB/s", "frac": pair_achieved / hbm_peak, "traffic": profiled_traffic("k_pairs"),
                      "algorithmic_bytes_per_launch": pair_bytes}
    clk = clocks.summary()
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": max(args.warmup, 3),
        "ms_per_step": total_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded water box)",
        "config": {"workload": WORKLOAD, "atoms": n, "directed_edges": 2 * m_half, "qeq_cg_iterations": qeq_iterations,
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed before every step (256 MiB write, outside the timed events)"},
        "roofline": roofline,
        "roofline_pairs": roofline_pairs,
        "stages_ms": stages,
        "clocks": clk,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d.value),
                "d2h_bytes_per_step": int(d2h.value), "api": "xreac_gb300.Calculator.evaluate (host numpy arrays)"},
        "gpu_launches": launches,
        "wall_s_timed_region": t_wall,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import torch as _t

        cores = os.cpu_count() or 1
        _t.set_num_threads(cores)
        times = oracle_eval_seconds(system, 10.0, min_runs=1, max_runs=3)
        line["cpu_baseline"] = {
            "value": n * len(times) / sum(times),
            "unit": UNIT,
            "cores": cores,
            "kind": "port",
            "sample": f"{len(times)} full evaluation(s) of the {n}-atom box by the CPU oracle "
                      f"(torch/numpy FP64, {cores} threads)",
        }
    if dist is not None:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
