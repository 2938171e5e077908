"""The scalar fast path for fully periodic cells (``geometry.periodic_cell``) against the general path
(``boundary`` + ``cell_repetitions``, which follow src/xreac/geometry.py:15-79): whenever the fast path
answers, the general path accepts the same input and gives the same flags, cell matrix and
replication counts. CPU only."""

import numpy as np

from xreac_gb300.geometry import boundary, cell_repetitions, periodic_cell


def general(cell, pbc, cutoff, atoms, limit):
    try:
        flags, m = boundary(cell, pbc)
        return flags, m, cell_repetitions(cutoff, flags, m, atoms, limit)
    except ValueError as err:
        return err


def random_cells(rng, count):
    for k in range(count):
        kind = k % 5
        if kind == 0:  # three lengths, some below the cutoff (replicated cells)
            yield rng.uniform(2.0, 40.0, 3)
        elif kind == 1:  # upper-triangular, right-handed
            yield np.diag(rng.uniform(3.0, 40.0, 3)) + np.triu(rng.normal(0.0, 4.0, (3, 3)), 1)
        elif kind == 2:  # arbitrary matrices: left-handed or nearly singular ones included
            yield rng.normal(0.0, 15.0, (3, 3))
        elif kind == 3:  # lengths with a sign flipped
            yield rng.uniform(3.0, 40.0, 3) * rng.choice([1.0, -1.0], 3)
        else:  # a rotated orthorhombic box given as a matrix
            q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
            q *= np.sign(np.linalg.det(q))
            yield (np.diag(rng.uniform(4.0, 30.0, 3)) @ q).tolist()


def test_fast_path_agrees_with_the_general_path():
    rng = np.random.default_rng(11)
    answered = 0
    for cell in random_cells(rng, 2000):
        pbc = [True, None][int(rng.integers(0, 2))]
        atoms = int(rng.integers(1, 300))
        cutoff = 10.0
        fast = periodic_cell(cell, pbc, cutoff, atoms, 512)
        ref = general(cell, pbc, cutoff, atoms, 512)
        if fast is None:
            continue
        answered += 1
        assert not isinstance(ref, Exception), (cell, ref)
        np.testing.assert_array_equal(fast[0], ref[0])
        np.testing.assert_array_equal(fast[1], ref[1])
        assert fast[2] == ref[2]
    assert answered > 800  # the fast path takes most valid cells


def test_fast_path_declines_what_it_does_not_take():
    cutoff = 10.0
    # partial periodicity, no periodicity, bad shapes and values go to the general path
    assert periodic_cell(np.full(3, 20.0), [True, True, False], cutoff, 10, 512) is None
    assert periodic_cell(None, None, cutoff, 10, 512) is None
    assert periodic_cell(np.full(3, 20.0), False, cutoff, 10, 512) is None
    assert periodic_cell(np.full(2, 20.0), True, cutoff, 10, 512) is None
    assert periodic_cell([20.0, float("nan"), 20.0], True, cutoff, 10, 512) is None
    assert periodic_cell([20.0, -1.0, 20.0], True, cutoff, 10, 512) is None
    assert periodic_cell(np.diag([20.0, 20.0, -20.0]), True, cutoff, 10, 512) is None  # left-handed
    assert periodic_cell("abc", True, cutoff, 10, 512) is None
    # a face height exactly at the cutoff: the general path's rounding decides
    assert periodic_cell(np.full(3, 10.0), True, cutoff, 10, 512) is None
    # over the expansion limit: the general path raises xreac's error
    assert periodic_cell(np.full(3, 4.0), True, cutoff, 100, 512) is None
    assert isinstance(general(np.full(3, 4.0), True, cutoff, 100, 512), ValueError)
