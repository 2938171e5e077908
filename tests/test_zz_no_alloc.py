"""Allocation-free neighbour counting (xr_count_neighbors_static) against xr_eval's neighbour list.

The static entry point runs the same count pass as xr_eval with its scratch in a static device
array. Its per-atom counts must equal the row lengths of the list that the allocating path
(Calculator.evaluate -> xr_eval -> xr_get_neighbors) builds for the same system, on consecutive
calls that reuse the shared scratch. This file is collected last so that it also runs after every
other GPU test in the same process.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system_struct(nat, x, cell, pbc):
    s = nat.System()
    s.natoms = len(x)
    s.types = None
    s.positions = nat.addr(x)
    s.cell = nat.addr(cell)
    for d in range(3):
        s.pbc[d] = int(pbc)
    s.total_charge = 0.0
    return s


def _static_counts(nat, lib, x, cell, pbc, cutoff):
    x = np.ascontiguousarray(x, dtype=np.float64)
    cellm = None if cell is None else np.ascontiguousarray(cell, dtype=np.float64)
    s = _system_struct(nat, x, cellm, pbc)
    counts = np.full(len(x), -1, dtype=np.int32)
    total = ctypes.c_longlong(-1)
    code = lib.xr_count_neighbors_static(ctypes.byref(s), float(cutoff), None, nat.ptr(counts, nat.c_int),
                                         ctypes.byref(total))
    assert code == nat.XR_OK, lib.xr_static_last_error().decode()
    return counts, total.value


def _evaluate_counts(system):
    from xreac_gb300 import Calculator, ForceField

    ff = ForceField.bundled(system.force_field)
    calc = Calculator(ff)
    calc.evaluate(system.symbols, system.positions, cell=system.cell, pbc=system.pbc)
    i, _, _ = calc.neighbor_list()
    return np.bincount(i, minlength=len(system.symbols)).astype(np.int32), float(ff.general[12])


def test_static_counts_equal_the_evaluate_rows_on_consecutive_calls():
    from xreac_gb300 import _native as nat
    from xreac_gb300.workloads import cho_mixture, water_box, water_cluster

    lib = nat.load()
    systems = [water_box(), cho_mixture(), water_cluster(jitter=0.05)]
    expected = [_evaluate_counts(s) for s in systems]
    for _ in range(2):
        for s, (want, cutoff) in zip(systems, expected):
            got, total = _static_counts(nat, lib, s.positions, s.cell, s.pbc, cutoff)
            np.testing.assert_array_equal(got, want)
            assert total == int(want.sum())


def test_static_counts_reject_systems_above_the_limit():
    from xreac_gb300 import _native as nat

    lib = nat.load()
    n = nat.XR_STATIC_MAX_ATOMS + 1
    x = np.zeros((n, 3))
    s = _system_struct(nat, x, None, False)
    counts = np.zeros(n, dtype=np.int32)
    code = lib.xr_count_neighbors_static(ctypes.byref(s), 10.0, None, nat.ptr(counts, nat.c_int), None)
    assert code == nat.XR_ECAPACITY
    assert "XR_STATIC_MAX_ATOMS" in lib.xr_static_last_error().decode()


def test_static_counts_of_a_small_cell_match_the_image_list():
    from xreac_gb300 import Calculator, ForceField
    from xreac_gb300 import _native as nat

    ff = ForceField.bundled("ffield.reax.HO.2015")
    calc = Calculator(ff)
    rng = np.random.default_rng(11)
    cell = np.array([[6.2, 0.0, 0.0], [0.7, 5.9, 0.0], [-0.4, 0.3, 6.4]])
    frac = rng.random((12, 3))
    x = frac @ cell
    # keep atoms apart so the evaluation is well defined
    while True:
        d = x[:, None, :] - x[None, :, :]
        r = np.sqrt((d ** 2).sum(-1)) + np.eye(len(x)) * 10
        if r.min() > 1.5:
            break
        x = rng.random((12, 3)) @ cell
    symbols = ["O", "H", "H"] * 4
    calc.evaluate(symbols, x, cell=cell, pbc=True)
    i, _, _ = calc.neighbor_list()
    want = np.bincount(i, minlength=len(x)).astype(np.int32)
    got, total = _static_counts(nat, nat.load(), x, cell, True, float(ff.general[12]))
    np.testing.assert_array_equal(got, want)
    assert total == len(i)


def test_static_counts_reject_a_left_handed_cell():
    from xreac_gb300 import _native as nat

    lib = nat.load()
    x = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
    cell = np.diag([-20.0, 20.0, 20.0])  # det < 0: xr_eval rejects it with the same message
    s = _system_struct(nat, x, cell, True)
    counts = np.zeros(2, dtype=np.int32)
    code = lib.xr_count_neighbors_static(ctypes.byref(s), 10.0, None, nat.ptr(counts, nat.c_int), None)
    assert code == nat.XR_EINPUT
    assert lib.xr_static_last_error().decode() == "Periodic cells must be nonsingular and right-handed"
