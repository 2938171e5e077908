"""The batch packing fast path (``Calculator._pack``: the host module, then the Python checks of cells
and initial charges) against the per-request general path (``Calculator._prepare`` and the initial
charges' checks), on CPU with the device layer stubbed out: every request gets the same types,
positions, periodicity, cell, repetitions, total charge and initial charges whichever path it takes."""

import ctypes
import importlib

import numpy as np
import pytest

import xreac_gb300.calculator as C
from xreac_gb300 import ForceField, workloads
from xreac_gb300 import _native as nat


class _Handle:
    handle = None


@pytest.fixture()
def calc(monkeypatch):
    from xreac_gb300.build import build_host

    if build_host() is None:
        pytest.skip("no Python headers for the host module")
    monkeypatch.setattr(C, "_host", importlib.import_module("xreac_gb300._lib._xr_host"))
    monkeypatch.setattr(nat, "ForceFieldHandle", lambda *a, **k: _Handle())
    monkeypatch.setattr(nat, "Context", lambda *a, **k: _Handle())
    monkeypatch.setattr(nat, "load", lambda: None)
    return C.Calculator(ForceField.bundled("ffield.reax.HO.2015"))


def items_to_pack():
    stream = [r.system for r in workloads.request_stream(n_requests=400) if r.system.force_field.endswith("HO.2015")]
    rng = np.random.default_rng(5)
    items = []
    for k, s in enumerate(stream[:120]):
        initial = None
        if k % 4 == 1:
            initial = np.full(s.n, s.total_charge / s.n)  # float64 array: taken in place
        elif k % 8 == 3:
            initial = [s.total_charge / s.n] * s.n  # a list: checked and converted in Python
        elif k % 8 == 7:
            initial = np.full(s.n, s.total_charge / s.n, dtype=np.float32)
        items.append((s.symbols, s.positions, s.total_charge, s.cell, s.pbc, initial))
    water = ["O", "H", "H"]
    xw = np.array([[0.0, 0.0, 0.0], [0.96, 0.0, 0.0], [-0.24, 0.93, 0.0]]) + 1.0
    items += [
        (np.array(water), xw, 0, None, None, None),                          # labels as an array
        (water, xw.tolist(), 0, None, None, None),                           # positions as a list
        (water, xw, 0, [12.0, 12.0, 30.0], [True, True, False], None),       # partly periodic
        (water, xw, 0, [25.0, 25.0, 25.0], None, None),                      # periodic through the cell
        (water, xw, 1, np.diag([8.0, 8.0, 8.0]), True, np.full(3, 1 / 3)),   # replicated small cell
        (water, xw + rng.normal(0, 0.01, (3, 3)), 0.0, None, False, None),
    ]
    return items


def test_packed_batch_matches_the_general_path(calc):
    items = items_to_pack()
    types, x, offsets, flags_l, cells, charges, guesses, reps = calc._pack(items, False)
    assert isinstance(guesses, C._GuessAddresses)
    for k, (symbols, positions, total_charge, cell, pbc, initial) in enumerate(items):
        _, xr, tr, fr, cr, rr = calc._prepare(symbols, positions, total_charge, cell, pbc, False)
        a0, a1 = int(offsets[k]), int(offsets[k + 1])
        np.testing.assert_array_equal(types[a0:a1], tr)
        np.testing.assert_array_equal(x[a0:a1], xr)
        np.testing.assert_array_equal(flags_l[k], fr)
        assert (cells[k] is None) == (cr is None)
        if cr is not None:
            np.testing.assert_array_equal(cells[k], cr)
        assert tuple(reps[k]) == tuple(rr)
        assert charges[k] == float(total_charge)
        g = C._guess(initial, a1 - a0)
        addr = int(guesses.addr[k])
        if g is None:
            assert addr == 0
        else:
            held = np.ctypeslib.as_array((ctypes.c_double * (a1 - a0)).from_address(addr))
            np.testing.assert_array_equal(held, g)


def test_bad_initial_charges_keep_their_message(calc):
    water = ["O", "H", "H"]
    xw = np.array([[0.0, 0.0, 0.0], [0.96, 0.0, 0.0], [-0.24, 0.93, 0.0]])
    for bad in (np.zeros(2), [0.0, np.nan, 0.0], np.zeros((3, 1))):
        with pytest.raises(ValueError, match="initial_charges must be a finite array"):
            calc._pack([(water, xw, 0, None, None, bad)], False)
