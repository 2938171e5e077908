"""Validation of caller-supplied neighbour lists, on the host (no GPU).

The cases and messages are those of xreac's own test of supplied lists
(tests/test_neighbors.py:317-342 of the reference, a ZnO dimer without a cell) and of its ordering
test with image shifts (tests/test_neighbors.py:137-154): the Python-side checks of
``supplied_arrays`` first, then the library's (``xr_neighbors_check``, the same code that
``xr_eval_neighbors`` runs before any device work).
"""

import ctypes

import numpy as np
import pytest

from xreac_gb300 import _native as nat
from xreac_gb300.neighbors import supplied_arrays


def check(neighbors, natoms, pbc):
    """Raise ValueError with the message of the first failed check, as Calculator.evaluate does."""
    i, j, s = supplied_arrays(neighbors, natoms)
    lib = nat.load()
    nb = nat.Neighbors(len(i), nat.addr(i), nat.addr(j), nat.addr(s))
    flags = (ctypes.c_int * 3)(*[int(bool(v)) for v in np.broadcast_to(pbc, (3,))])
    msg = ctypes.create_string_buffer(256)
    code = lib.xr_neighbors_check(natoms, flags, ctypes.byref(nb), msg, 256)
    if code != nat.XR_OK:
        raise ValueError(msg.value.decode())
    return code


@pytest.fixture(scope="module", autouse=True)
def built_library():
    from xreac_gb300.build import build

    build()


@pytest.mark.parametrize(
    "neighbors,message",
    [
        (([0], [1]), "tuple"),
        (([0], [1, 0], [[0, 0, 0]]), "shape"),
        (([0], [1], [[0, 0]]), "shape"),
        (([0.0, 1.0], [1, 0], [[0, 0, 0], [0, 0, 0]]), "integers"),
        (([0, 1], [1, 0], [[0.0, 0, 0], [0, 0, 0]]), "integers"),
        (([-1, 1], [1, 0], [[0, 0, 0], [0, 0, 0]]), "out of range"),
        (([0, 1], [2, 0], [[0, 0, 0], [0, 0, 0]]), "out of range"),
        (([0, 1], [1, 0], [[1, 0, 0], [-1, 0, 0]]), "nonperiodic"),
        (([0], [0], [[0, 0, 0]]), "self neighbors"),
        (([0, 0, 1], [1, 1, 0], [[0, 0, 0]] * 3), "Duplicate"),
        (([0], [1], [[0, 0, 0]]), "both directions"),
    ],
)
def test_supplied_neighbor_validation(neighbors, message):
    with pytest.raises(ValueError, match=message):
        check(neighbors, 2, False)


@pytest.mark.parametrize("index_dtype", [np.int64, np.uint64])
def test_image_shifts_in_any_order_pass_and_their_faults_are_found(index_dtype):
    i = np.array([1, 0, 0, 1, 0, 1], dtype=index_dtype)
    j = 1 - i
    shifts = np.array([[1, 0, 0], [0, 0, 0], [-1, 0, 0], [0, 0, 0], [-2, 0, 0], [2, 0, 0]])
    assert check((i, j, shifts), 2, True) == nat.XR_OK
    with pytest.raises(ValueError, match="both directions"):
        check((i[:-1], j[:-1], shifts[:-1]), 2, True)
    with pytest.raises(ValueError, match="Duplicate"):
        check((np.r_[i, i[:1]], np.r_[j, j[:1]], np.concatenate((shifts, shifts[:1]))), 2, True)
    # a shifted reverse is not a reverse
    bad = shifts.copy()
    bad[0] = [3, 0, 0]
    with pytest.raises(ValueError, match="both directions"):
        check((i, j, bad), 2, True)


def test_self_images_and_partial_pbc():
    # nonzero-shift self edges in a periodic direction are edges; a shift in a non-periodic one is not
    i = np.array([0, 0])
    s = np.array([[1, 0, 0], [-1, 0, 0]])
    assert check((i, i, s), 1, [True, False, False]) == nat.XR_OK
    with pytest.raises(ValueError, match="nonperiodic"):
        check((i, i, s[:, ::-1].copy()), 1, [True, False, False])


def test_shifts_beyond_the_device_range_are_a_capacity_error():
    i = np.array([0, 1])
    j = np.array([1, 0])
    s = np.array([[300, 0, 0], [-300, 0, 0]])
    with pytest.raises(ValueError, match="supported range"):
        check((i, j, s), 2, True)
    with pytest.raises(ValueError, match="supported range"):
        check((i, j, s * 2**40), 2, True)


def test_a_large_shuffled_list_of_a_periodic_box():
    """A full list with a skin, shuffled, is valid; removing one edge of any pair breaks it."""
    from oracle import neighbor_list
    from xreac_gb300 import workloads

    box = workloads.water_box(n_mol=64, box=12.42, seed=2)
    i, j, s = neighbor_list(box.positions, 11.0, box.cell, box.pbc)
    order = np.random.default_rng(3).permutation(len(i))
    i, j, s = i[order], j[order], s[order]
    assert check((i, j, s), box.n, box.pbc) == nat.XR_OK
    with pytest.raises(ValueError, match="both directions"):
        check((i[1:], j[1:], s[1:]), box.n, box.pbc)
