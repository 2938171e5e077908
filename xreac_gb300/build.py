"""Build the CUDA library ``libxreac_gb300.so`` in-tree with nvcc (sm_103a only).

Each translation unit compiles in parallel to an object file under ``xreac_gb300/_build``;
the shared library is linked into ``xreac_gb300/_lib``. Rebuilds only what changed.

    python -m xreac_gb300.build [--force]
"""

from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libxreac_gb300.so"
SOURCES = ("xr_topology.cu", "xr_bonded.cu", "xr_nonbonded.cu", "xr_engine.cu", "xr_static.cu", "xr_lists.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (Path(cand).exists() or cand == "nvcc"):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [ROOT / "include" / "xreac_gb300.h"]


def _stale(target, deps):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
    """Compile every translation unit for sm_103a and link the shared library; returns its path."""
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    jobs = []
    for src in SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        if force or _stale(obj, [CSRC / src] + headers):
            cmd = [nvcc, *ARCH, *FLAGS, *extra_flags, "-I", str(ROOT / "include"), "-I", str(CSRC), "-c",
                   str(CSRC / src), "-o", str(obj)]
            jobs.append((src, cmd))

    def run(job):
        src, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, r

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as pool:
        for src, r in pool.map(run, jobs):
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr, file=sys.stderr)
    objs = [BUILD / (Path(s).stem + ".o") for s in SOURCES]
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_host(force, verbose)
    return LIB


def build_host(force=False, verbose=False):
    """The host-side batch packing module ``_lib/_xr_host.so`` (CPython C API, g++). Skipped, with the
    pure-Python packing path used instead, when the compiler or the Python headers are missing."""
    import sysconfig

    src = CSRC / "xr_host.cpp"
    out = LIBDIR / "_xr_host.so"
    include = sysconfig.get_paths().get("include")
    if not include or not (Path(include) / "Python.h").exists():
        return None
    if not force and not _stale(out, [src]):
        return out
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", include, str(src), "-o", str(out)]
    if verbose:
        print(" ".join(cmd), flush=True)
    try:
        r = subprocess.run(cmd, capture_output=True, text=True)
    except OSError:
        return None
    if r.returncode != 0:
        raise RuntimeError(f"host module build failed:\n{r.stdout}\n{r.stderr}")
    return out


if __name__ == "__main__":
    path = build(force="--force" in sys.argv, verbose=True,
                 extra_flags=("-Xptxas", "-v") if "--ptxas" in sys.argv else ())
    print(path)
