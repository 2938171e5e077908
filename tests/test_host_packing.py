"""The host packing module (``_xr_host.fill``, xreac_gb300/csrc/xr_host.cpp): one C pass over a batch's
request tuples that maps labels to type indices and copies positions, and leaves every request it
cannot take as is to the Python path (which applies xreac's checks and messages). CPU only."""

import numpy as np
import pytest


@pytest.fixture(scope="module")
def host():
    from xreac_gb300.build import build_host

    if build_host() is None:
        pytest.skip("no Python headers for the host module")
    from xreac_gb300._lib import _xr_host

    return _xr_host


TYPES = {"C": 0, "H": 1, "O": 2}


def pack(host, items, type_map=TYPES):
    total = sum(len(it[0]) for it in items)
    types = np.full(total, -7, dtype=np.int32)
    x = np.full((total, 3), -7.0)
    slow = host.fill(items, type_map, types, x)
    return slow, types, x


def request(symbols, positions, total_charge=0, cell=None, pbc=None, initial=None):
    return (symbols, positions, total_charge, cell, pbc, initial)


def test_fill_packs_labels_and_positions(host):
    rng = np.random.default_rng(3)
    sym = [["O", "H", "H"], ("C", "O", "O"), ["H"] * 5 + ["C"]]
    pos = [rng.normal(size=(len(s), 3)) for s in sym]
    slow, types, x = pack(host, [request(s, p, q) for s, p, q in zip(sym, pos, (0, 1, -1.0))])
    assert slow == []
    assert types.tolist() == [TYPES[a] for s in sym for a in s]
    np.testing.assert_array_equal(x, np.concatenate(pos))


def test_fill_leaves_other_inputs_to_python(host):
    good = np.arange(6.0).reshape(2, 3)
    items = [
        request(["C", "H"], good),                                  # 0 taken
        request(["C", "Xx"], good),                                 # 1 label missing from the map
        request(["C", "H"], good.astype(np.float32)),               # 2 not float64
        request(["C", "H"], np.array([[0, 0, 0], [np.nan, 0, 0]])),  # 3 non-finite coordinate
        request(["C", "H"], np.asfortranarray(np.arange(6.0).reshape(2, 3))[:, :]),  # 4 see below
        request(["C", "H"], good, float("nan")),                    # 5 non-finite total charge
        request(["C", "H"], good, np.float64(0.0)),                 # 6 not a plain float or int
        request(["C", "H"], good, True),                            # 7 a bool is not a charge
        request(np.array(["C", "H"]), good),                        # 8 not a list or tuple
        request(("O", "O"), good + 1.0),                            # 9 taken
        request(["C", "H"], good.tolist()),                         # 10 no buffer
        (["C", "H"], good, 0, None, None),                          # 11 not the six fields
        request(["C", "H"], np.arange(12.0).reshape(4, 3)[1:3]),   # 12 a C-contiguous view at an offset: taken
    ]
    # a Fortran-ordered (2, 3) array is not C-contiguous
    assert not items[4][1].flags["C_CONTIGUOUS"]
    slow, types, x = pack(host, items)
    assert slow == [1, 2, 3, 4, 5, 6, 7, 8, 10, 11]
    # the requests it took sit at their offsets (the Python path fills the others' slots)
    assert types[0:2].tolist() == [0, 1] and x[0:2].tolist() == good.tolist()
    assert types[18:20].tolist() == [2, 2] and x[18:20].tolist() == (good + 1.0).tolist()
    assert types[24:26].tolist() == [0, 1] and x[24:26].tolist() == np.arange(3.0, 9.0).reshape(2, 3).tolist()


def test_fill_maps_more_labels_than_it_remembers(host):
    labels = [f"E{k}" for k in range(11)]
    type_map = {s: 10 + k for k, s in enumerate(labels)}
    sym = [labels[k % 11] for k in range(40)] + labels[::-1]
    slow, types, _ = pack(host, [request(sym, np.zeros((len(sym), 3)))], type_map)
    assert slow == []
    assert types.tolist() == [type_map[s] for s in sym]


def test_fill_checks_its_arguments(host):
    item = request(["C", "H"], np.zeros((2, 3)))
    types = np.zeros(2, dtype=np.int32)
    x = np.zeros((2, 3))
    with pytest.raises(TypeError):
        host.fill((item,), TYPES, types, x)  # items must be a list
    with pytest.raises(TypeError):
        host.fill([item], list(TYPES.items()), types, x)  # the map must be a dict
    with pytest.raises(ValueError):
        host.fill([item], TYPES, np.zeros(2, dtype=np.int64), x)
    with pytest.raises(ValueError):
        host.fill([item], TYPES, types, np.zeros((3, 3)))
    with pytest.raises(ValueError):
        host.fill([item, item], TYPES, types, x)  # more atoms than the outputs hold
    with pytest.raises(ValueError):
        host.fill([["C", "H"]], TYPES, types, x)  # a request is a tuple


def test_guesses_takes_float64_charges_in_place(host):
    sym = ["C", "H", "O"]
    q = np.array([0.1, -0.2, 0.1])
    wide = np.array([[0.1, -0.2, 0.1], [0.0, 0.0, 0.0]])
    items = [
        request(sym, np.zeros((3, 3))),                                  # 0 none: address 0
        request(sym, np.zeros((3, 3)), initial=q),                       # 1 taken in place
        request(sym, np.zeros((3, 3)), initial=q.astype(np.float32)),    # 2 not float64
        request(sym, np.zeros((3, 3)), initial=q[:2]),                   # 3 not one per atom
        request(sym, np.zeros((3, 3)), initial=np.array([0.1, np.inf, 0.0])),  # 4 non-finite
        request(sym, np.zeros((3, 3)), initial=q.tolist()),              # 5 no buffer
        request(sym, np.zeros((3, 3)), initial=wide[:, 0:3:1][0:1]),     # 6 two-dimensional
        request(sym, np.zeros((3, 3)), initial=np.arange(6.0)[::2]),     # 7 strided
        request(sym, np.zeros((3, 3)), initial=wide[1]),                 # 8 a C-contiguous row view: taken
        (sym, np.zeros((3, 3)), 0, None, None),                          # 9 not the six fields
        request(sym, np.zeros((3, 3)), initial=memoryview(q)),           # 10 a buffer, not an array
    ]
    addr = np.full(len(items), 99, dtype=np.uint64)
    slow = host.guesses(items, addr)
    assert slow == [2, 3, 4, 5, 6, 7, 9, 10]
    assert addr[0] == 0
    assert addr[1] == q.__array_interface__["data"][0]
    assert addr[8] == wide.__array_interface__["data"][0] + 24
    with pytest.raises(ValueError):
        host.guesses(items, np.zeros(len(items) - 1, dtype=np.uint64))
    with pytest.raises(TypeError):
        host.guesses(tuple(items), addr)
