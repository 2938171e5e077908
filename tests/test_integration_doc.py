"""The reference-side ctypes binding in INTEGRATION.md matches the C header and the package's own
binding: same structure fields, in the same order, with the same sizes (no GPU needed)."""

import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _doc_binding():
    text = (ROOT / "INTEGRATION.md").read_text()
    block = re.search(r"```python\n# src/xreac/_gb300.py.*?```", text, flags=re.S).group(0)
    code = block.split("\n", 1)[1].rsplit("```", 1)[0]
    code = code.replace('_lib = ctypes.CDLL("libxreac_gb300.so")', "_lib = None")
    code = re.sub(r"^_lib\.\w+\.\w+ = .*$", "", code, flags=re.M)
    ns = {}
    exec(compile(code, "INTEGRATION.md", "exec"), ns)  # noqa: S102 - the documented stub, library calls removed
    return ns


def _header_struct(name):
    text = (ROOT / "include" / "xreac_gb300.h").read_text()
    body = re.search(r"typedef struct \{([^}]*)\} " + name + ";", text).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if decl:
            fields.append(re.sub(r"\[\d+\]$", "", decl.split()[-1].lstrip("*")))
    return fields


def test_documented_structs_match_the_header_and_the_package():
    from xreac_gb300 import _native

    ns = _doc_binding()
    for doc, pkg, cname in ((ns["_System"], _native.System, "xr_system"), (ns["_Result"], _native.Result, "xr_result")):
        doc_fields = [f[0] for f in doc._fields_]
        assert doc_fields == [f[0] for f in pkg._fields_]
        assert doc_fields == _header_struct(cname)
        assert ctypes.sizeof(doc) == ctypes.sizeof(pkg)
        for (name, _), (_, _) in zip(doc._fields_, pkg._fields_):
            assert getattr(doc, name).offset == getattr(pkg, name).offset, name
