"""Shared test configuration: the ``gpu`` marker and golden-fixture loading."""

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


def golden_names():
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load_golden(name):
    """One reference fixture as a plain dict (see tests/golden/make_golden.py)."""
    z = np.load(GOLDEN / f"{name}.npz")
    d = {k: z[k] for k in z.files}
    d["ff"] = str(d["ff"])
    d["symbols"] = [str(s) for s in d["symbols"]]
    d["cell"] = None if d["cell"].size == 0 else d["cell"]
    d["total_charge"] = float(d["total_charge"])
    d["full_derivative"] = bool(d["full_derivative"])
    d["pbc"] = [bool(v) for v in d["pbc"]]
    return d


@pytest.fixture(scope="session")
def golden():
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = load_golden(name)
        return cache[name]

    return get
