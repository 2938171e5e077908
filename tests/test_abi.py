"""The C ABI library builds, loads without a GPU and exports every entry point of include/xreac_gb300.h."""

import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "xreac_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(xr_[a-z_]+)\s*\(", text)))


def test_header_declares_the_api():
    names = declared_functions()
    for name in ("xr_ff_create", "xr_ctx_create", "xr_eval", "xr_eval_batch", "xr_last_error"):
        assert name in names


def test_library_exports_every_declared_symbol():
    from xreac_gb300.build import build
    from xreac_gb300 import _native

    build()
    lib = _native.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(declared_functions()) == set(_native.EXPORTED)


def test_package_never_imports_the_oracle():
    for path in (ROOT / "xreac_gb300").rglob("*.py"):
        text = path.read_text()
        assert "import oracle" not in text and "from oracle" not in text, path


def test_integration_guide_lists_every_entry_point():
    doc = (ROOT / "INTEGRATION.md").read_text()
    missing = [n for n in declared_functions() if f"`{n}`" not in doc]
    assert not missing, missing
