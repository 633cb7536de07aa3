"""Builds libqsv.so (the CUDA kernels plus the C ABI declared in include/qsv.h) in-tree.

Each ``csrc/*.cu`` file is compiled for sm_103a only (``-gencode
arch=compute_103a,code=sm_103a``), in parallel, then linked into
``qip_gb300/libqsv.so``.  A file is rebuilt when it, a header it includes, or this
script is newer than its object.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libqsv.so")
# Bounds-checked variant: every computed state index tested before the access, bad
# ones counted and skipped (see qsv_bounds_report); for tests, not for speed.
BUILD_CHECKED = os.path.join(PKG, "_build_checked")
LIB_CHECKED = os.path.join(PKG, "libqsv_checked.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand) and shutil.which(cand) is None:
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libqsv")
    return cand


def _deps_mtime() -> float:
    files = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def _compile(src: str, verbose: bool, checked: bool = False) -> str:
    obj = os.path.join(BUILD_CHECKED if checked else BUILD, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _deps_mtime()):
        return obj
    cmd = [_nvcc(), *ARCH, *FLAGS, *(["-DQSV_BOUNDS_CHECK"] if checked else []), "-c", src, "-o", obj + ".tmp"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        print(res.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False, checked: bool = False) -> str:
    """Compile every csrc/*.cu (in parallel) and link libqsv.so, or with ``checked`` the
    bounds-checked libqsv_checked.so; returns the library's path."""
    out_dir, lib = (BUILD_CHECKED, LIB_CHECKED) if checked else (BUILD, LIB)
    os.makedirs(out_dir, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with ThreadPoolExecutor(max_workers=max(1, min(len(sources), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, checked), sources))
    if not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", lib + ".tmp", *objs]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(lib + ".tmp", lib)
    return lib


if __name__ == "__main__":
    import sys

    print(build(verbose="-v" in sys.argv))
