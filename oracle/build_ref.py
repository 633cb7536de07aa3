"""Build recipe for the reference's own CPU kernels (test and baseline infrastructure only).

The reference (Renmusxd/QIP) implements its state-vector hot path as three Cython
modules: ``qip/ext/kronprod.pyx`` (gate kernel ``cdot_loop`` and the measurement
kernels), ``qip/ext/util.pyx`` (``entwine_bit``/``set_bit``/``get_bit``) and
``qip/ext/func_apply.pyx``.  This script compiles them from the sources where they
lie, without the reference's own ``setup.py``:

* stage 1 (needs the reference checkout and Cython): cythonize the three ``.pyx``
  files into C under ``oracle/_ref/src``.  Directives follow what Cython 3 needs to
  accept the 2018-era sources: ``language_level=3``, ``cpow=True`` (``2**n`` on C
  ints, ``func_apply.pyx:68``) and ``legacy_implicit_noexcept=True``.
* stage 2 (needs gcc, Python and numpy headers): compile each C file into an
  extension module under ``oracle/_ref/lib`` with the reference's flags from
  ``setup.py:36,42`` (``-O3 -ffast-math -fopenmp``) minus ``-march=native``, which is
  dropped so the same recipe builds on x86_64 and aarch64 hosts.

Stage 2 runs on its own when the generated C is present but the reference checkout is
not (a machine that only received ``oracle/_ref``).  Outputs go to ``oracle/_ref``
only; that folder is git-ignored.

Nothing in the product imports these modules: they are used by ``tests/golden``
(fixture generation) and by ``bench.py --impl reference`` (the CPU baseline arm).
"""
from __future__ import annotations

import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
LIB = os.path.join(OUT, "lib")
MODULES = ("util", "kronprod", "func_apply")


def reference_checkout():
    """The reference's source checkout: ``QIP_REFERENCE_ROOT`` when set, else a folder
    named ``reference`` beside this repository; None when neither holds ``qip/ext``."""
    for cand in (os.environ.get("QIP_REFERENCE_ROOT"), os.path.join(os.path.dirname(REPO), "reference")):
        if cand and os.path.isdir(os.path.join(cand, "qip", "ext")):
            return os.path.abspath(cand)
    return None


def _cythonize() -> bool:
    """Stage 1: .pyx -> .c (only where the reference checkout and Cython exist)."""
    checkout = reference_checkout()
    if checkout is None:
        return False
    ref_ext = os.path.join(checkout, "qip", "ext")
    try:
        from Cython.Compiler import Options  # noqa: F401
        from Cython.Compiler.Main import compile as cy_compile, CompilationOptions
    except ImportError:
        return False
    os.makedirs(SRC, exist_ok=True)
    for name in MODULES:
        pyx = os.path.join(ref_ext, name + ".pyx")
        out_c = os.path.join(SRC, name + ".c")
        if os.path.exists(out_c) and os.path.getmtime(out_c) >= os.path.getmtime(pyx):
            continue
        opts = CompilationOptions(
            output_file=out_c,
            include_path=[ref_ext],
            compiler_directives={
                "language_level": 3,
                "cpow": True,
                "legacy_implicit_noexcept": True,
            },
        )
        # Compile as a top-level module (the reference cimports ``util`` by its bare
        # name, ``kronprod.pyx:14``), so the runtime import is ``import util``.
        opts.module_name = name
        res = cy_compile(pyx, opts, full_module_name=name)
        if res.num_errors:
            raise RuntimeError(f"cythonize failed for {pyx}")
    return True


def _compile_one(name: str) -> str:
    import numpy

    c_file = os.path.join(SRC, name + ".c")
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    out = os.path.join(LIB, name + suffix)
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(c_file):
        return out
    cmd = [
        os.environ.get("CC", "gcc"), "-shared", "-fPIC", "-O3", "-ffast-math", "-fopenmp",
        "-fno-strict-aliasing", "-w",
        "-I" + sysconfig.get_paths()["include"], "-I" + numpy.get_include(),
        "-DNPY_NO_DEPRECATED_API=0",
        c_file, "-o", out + ".tmp", "-lm",
    ]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


def build(verbose: bool = False) -> bool:
    """Build the reference extension modules.  Returns True when ``oracle/_ref/lib``
    holds all three modules afterwards, False when neither the reference checkout nor
    previously generated C sources are available."""
    _cythonize()
    if not all(os.path.exists(os.path.join(SRC, m + ".c")) for m in MODULES):
        return False
    os.makedirs(LIB, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(MODULES)) as ex:
        outs = list(ex.map(_compile_one, MODULES))
    if verbose:
        for o in outs:
            print("built", o)
    return True


def load():
    """Import the built reference modules.  Returns ``(kronprod, func_apply)``.

    Applies the two runtime shims the 2018 sources need on current numpy/Python:
    ``numpy.int`` (used as a dtype at ``kronprod.pyx:139``) and
    ``collections.Iterable`` (used by ``qip/util.py:153`` when the pure-Python
    package is imported next to these modules)."""
    import collections
    import collections.abc
    import numpy

    if not hasattr(numpy, "int"):
        numpy.int = int  # type: ignore[attr-defined]
    if not hasattr(collections, "Iterable"):
        collections.Iterable = collections.abc.Iterable  # type: ignore[attr-defined]
    if LIB not in sys.path:
        sys.path.insert(0, LIB)
    import kronprod  # type: ignore
    import func_apply  # type: ignore

    return kronprod, func_apply


def available() -> bool:
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    return all(os.path.exists(os.path.join(LIB, m + suffix)) for m in MODULES)


if __name__ == "__main__":
    ok = build(verbose=True)
    print("reference kernels", "built" if ok else "unavailable (no sources)")
