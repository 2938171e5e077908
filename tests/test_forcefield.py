"""The parameter parser against the reference parser's dicts (tests/golden/forcefields.json)."""

import json

import numpy as np
import pytest

from conftest import GOLDEN
from xreac_gb300.forcefield import ForceField

REF = json.loads((GOLDEN / "forcefields.json").read_text())


def _same(a, b):
    np.testing.assert_array_equal(np.asarray(a, dtype=float), np.asarray(b, dtype=float))


@pytest.mark.parametrize("name", sorted(REF))
def test_parser_matches_reference(name):
    ff, ref = ForceField.bundled(name), REF[name]
    assert ff.checksum == ref["checksum"] and ff.citation == ref["citation"]
    assert list(ff.elements) == ref["elements"] and ff.vdw_type == ref["vdw_type"]
    _same(ff.general, ref["general"])
    assert set(ff.atoms) == set(ref["atoms"])
    for s, a in ff.atoms.items():
        assert a.keys() == ref["atoms"][s].keys()
        for k, v in a.items():
            _same(v, ref["atoms"][s][k])
    assert {f"{s}|{t}" for s, t in ff.pairs} == set(ref["pairs"])
    for (s, t), p in ff.pairs.items():
        r = ref["pairs"][f"{s}|{t}"]
        assert p.keys() == r.keys()
        for k, v in p.items():
            _same(v, r[k])
    for table in ("angles", "torsions", "hydrogen_bonds"):
        mine = getattr(ff, table)
        assert {"|".join(k) for k in mine} == set(ref[table])
        for k, v in mine.items():
            _same(np.asarray(v, dtype=float).ravel(), np.asarray(ref[table]["|".join(k)], dtype=float).ravel())


def test_known_parameter_values():
    """Values asserted by the reference (tests/test_calculator.py:207-216, tests/test_general.py:430-446)."""
    zn = ForceField.bundled("ffield.reax.ZnOH.2010")
    assert zn.checksum == "b5af5a65573ce60f32405a973e33f7cc89a90bc69e624a8ca89811eb67b1a07b"
    assert zn.atoms["O"]["eta"] == 2 * 8.3122
    assert zn.pairs["Zn", "O"]["r_vdW"] == 2 * 2.1414
    assert zn.pairs["Zn", "O"]["r_p"] == pytest.approx((1.0548 - 1.6836) / 2)
    ho = ForceField.bundled("ffield.reax.HO.2015")
    assert ho.elements == ("H", "O", "X")
    np.testing.assert_array_equal(ho.torsions["H", "O", "O", "H"], [2.5, -4.0, 0.9, -2.5, -1.0])
    np.testing.assert_array_equal(ho.torsions["X", "O", "O", "X"], [0.5511, 25.415, 1.133, -5.1903, -1.0])
    np.testing.assert_array_equal(ho.torsions["O", "H", "O", "H"], [0, 0.1, 0.02, -2.5415, 0])
    assert ho.pairs["X", "O"]["gamma"] > 0 and ho.pairs["X", "O"]["De_s"] == 0


def test_format_variants(tmp_path):
    """D exponents, an omitted hydrogen-bond block, empty and truncated files (tests/test_general.py:459-473)."""
    ff = ForceField.bundled("ffield.reax.HO.2015")
    text = ff.path.read_text().replace("50.0000", "5.00000D+1", 1)
    text = text[: text.index("  1    ! Nr of hydrogen bonds")]
    f = tmp_path / "without_hb.ff"
    f.write_text(text)
    parsed = ForceField.from_file(f)
    np.testing.assert_array_equal(parsed.general, ff.general)
    assert parsed.hydrogen_bonds == {}
    f.write_text("")
    with pytest.raises(ValueError, match="Empty"):
        ForceField.from_file(f)
    f.write_text(ff.path.read_text()[:500])
    with pytest.raises(ValueError):
        ForceField.from_file(f)
    with pytest.raises(ValueError, match="plain filename"):
        ForceField.bundled("../pyproject.toml")


def test_wildcard_precedence(tmp_path):
    """Explicit torsion rows win regardless of their position (tests/test_general.py:442-456)."""
    ff = ForceField.bundled("ffield.reax.HO.2015")
    lines = ff.path.read_text().splitlines()
    start = next(i for i, line in enumerate(lines) if "Nr of torsions" in line) + 1
    lines[start : start + 6] = lines[start + 3 : start + 6] + lines[start : start + 3]
    path = tmp_path / "reordered.ff"
    path.write_text("\n".join(lines) + "\n")
    reordered = ForceField.from_file(path)
    assert ff.torsions.keys() == reordered.torsions.keys()
    for key in ff.torsions:
        np.testing.assert_array_equal(ff.torsions[key], reordered.torsions[key])
