"""Install the unmodified xreac reference into ``baseline/_ref`` for ``bench.py --impl reference``.

Usage (in the build container, where the reference checkout exists):

    python baseline/install_reference.py <path of the xreac v0.10.0 checkout>

Step 1 is the offline pip install of the checkout (from a copy under /tmp, since the checkout is
read-only):

    python -m pip install --no-index --no-build-isolation [--no-deps] --find-links /opt/wheelhouse \
        --target baseline/_ref <copy>

xreac's pyproject.toml declares ``license`` as an SPDX expression, which needs setuptools >= 77;
where the installed setuptools is older and the wheelhouse has no newer one, that build fails while
preparing its metadata, before anything is installed. Step 2 then lays the package out exactly as
its wheel would, following the pyproject's ``package-dir`` and ``package-data`` tables
(``src/xreac`` -> ``xreac``, ``data`` -> ``xreac/data``), copying every file byte for byte. xreac
is pure Python, so nothing is compiled either way.

Either way the script writes ``baseline/_ref/XREAC_INSTALL.json``: the method used, the pip error (if
any) and the SHA-256 of every installed module and data file next to that of its source file, so
that a run on another machine can check that the installed reference is unmodified.

HIPS ``autograd`` (a dependency of xreac) is not installable offline here; the reference arm puts
the torch-backed stand-in ``tests/golden/shim`` first on ``sys.path``, as the fixture generator does.
"""

from __future__ import annotations

import fnmatch
import hashlib
import json
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
TARGET = HERE / "_ref"
DATA_PATTERNS = ("ffield.reax.*", "ffield.AgZnO", "*.md", "NOTICE", "LICENSES/*.txt")


def _sha(path):
    return hashlib.sha256(Path(path).read_bytes()).hexdigest()


def _pip(src_copy):
    base = [sys.executable, "-m", "pip", "install", "--no-index", "--no-build-isolation", "--find-links",
            "/opt/wheelhouse", "--target", str(TARGET)]
    errors = []
    for extra in ([], ["--no-deps"]):
        r = subprocess.run(base[:5] + extra + base[5:] + [str(src_copy)], capture_output=True, text=True)
        if r.returncode == 0:
            return True, errors
        lines = [ln.strip() for ln in (r.stdout + r.stderr).splitlines() if ln.strip()]
        key = [ln for ln in lines if "configuration error" in ln] or [ln for ln in lines if "error:" in ln.lower()]
        errors.append(" ".join(extra) + ": " + (key[0] if key else (lines[-1] if lines else "failed")))
    return False, errors


def _layout(reference):
    """The wheel's file layout, copied byte for byte."""
    pairs = []
    for f in sorted((reference / "src" / "xreac").glob("*.py")):
        pairs.append((f, TARGET / "xreac" / f.name))
    data = reference / "data"
    for f in sorted(p for p in data.rglob("*") if p.is_file()):
        rel = f.relative_to(data).as_posix()
        if any(fnmatch.fnmatch(rel, pat) for pat in DATA_PATTERNS):
            pairs.append((f, TARGET / "xreac" / "data" / rel))
    for src, dst in pairs:
        dst.parent.mkdir(parents=True, exist_ok=True)
        shutil.copyfile(src, dst)
    return pairs


def main(reference):
    reference = Path(reference).resolve()
    if not (reference / "src" / "xreac" / "calculator.py").is_file():
        sys.exit(f"{reference} is not an xreac checkout")
    if TARGET.exists():
        shutil.rmtree(TARGET)
    with tempfile.TemporaryDirectory() as tmp:
        copy = Path(tmp) / "xreac"
        shutil.copytree(reference, copy)
        ok, errors = _pip(copy)
    method = "pip install --target" if ok else "wheel layout copied byte for byte (pip install failed)"
    if not ok:
        if TARGET.exists():
            shutil.rmtree(TARGET)
        _layout(reference)
    installed = {}
    for f in sorted(p for p in (TARGET / "xreac").rglob("*") if p.is_file() and "__pycache__" not in p.parts):
        rel = f.relative_to(TARGET / "xreac").as_posix()
        src = reference / "src" / "xreac" / rel
        if rel.startswith("data/"):
            src = reference / "data" / rel[len("data/"):]
        installed[rel] = {"sha256": _sha(f), "source_sha256": _sha(src) if src.is_file() else None}
    mismatched = [k for k, v in installed.items() if v["sha256"] != v["source_sha256"]]
    version = next((ln.split("=", 1)[1].strip().strip('"') for ln in (reference / "pyproject.toml").read_text().splitlines()
                    if ln.startswith("version")), None)
    record = {"package": "xreac", "version": version, "method": method, "pip_errors": errors,
              "files": installed, "modified_files": mismatched}
    (TARGET / "XREAC_INSTALL.json").write_text(json.dumps(record, indent=1, sort_keys=True))
    print(f"{method}; {len(installed)} files, {len(mismatched)} differing from the checkout")
    if errors:
        print("pip:", *errors, sep="\n  ")
    return 0 if not mismatched else 1


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python baseline/install_reference.py <path of the xreac v0.10.0 checkout>")
    sys.exit(main(sys.argv[1]))
