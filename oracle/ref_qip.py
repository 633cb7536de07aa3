"""Import the reference QIP package (pure-Python layers plus the Cython kernels built by
``oracle/build_ref.py``).

Test infrastructure only: used by ``tests/golden/make_golden.py`` to generate golden
vectors from the reference itself, by the CPU tests that pin the oracle and this
package's host layer against the reference, and by the GPU test in which the
reference's own ``run()`` drives ``GpuBackend``.  The Python layers come from the
reference package installed into ``baseline/_ref`` (``oracle/install_ref.py``), which
travels with the repository, else from the reference checkout
(``build_ref.reference_checkout()``); the kernels from ``oracle/_ref``.
"""
from __future__ import annotations

import os
import sys
import types

HERE = os.path.dirname(os.path.abspath(__file__))
INSTALLED = os.path.join(os.path.dirname(HERE), "baseline", "_ref")
if HERE not in sys.path:
    sys.path.insert(0, HERE)
import build_ref  # noqa: E402


def package_root():
    """Folder holding the reference's ``qip`` package, or None."""
    if os.path.isfile(os.path.join(INSTALLED, "qip", "pipeline.py")):
        return INSTALLED
    return build_ref.reference_checkout()


def available() -> bool:
    """The package is present and its kernels are built or can be built here."""
    if package_root() is None:
        return False
    if build_ref.available():
        return True
    try:
        return build_ref.build()
    except Exception:
        return False


def import_reference():
    """Return the reference ``qip`` package with ``qip.ext.*`` bound to the modules
    compiled into ``oracle/_ref/lib``."""
    root = package_root()
    if root is None:
        raise RuntimeError("reference package not found")
    if not build_ref.available():
        if not build_ref.build():
            raise RuntimeError("reference kernels unavailable")
    kronprod, func_apply = build_ref.load()
    if root not in sys.path:
        sys.path.insert(0, root)
    # ``qip/ext/__init__.py`` is empty; bind the compiled kernels as its submodules.
    import qip  # noqa: F401
    ext = sys.modules.get("qip.ext")
    if ext is None:
        ext = types.ModuleType("qip.ext")
        ext.__path__ = [os.path.join(root, "qip", "ext")]
        sys.modules["qip.ext"] = ext
    sys.modules["qip.ext.kronprod"] = kronprod
    sys.modules["qip.ext.func_apply"] = func_apply
    ext.kronprod = kronprod
    ext.func_apply = func_apply
    import qip.backend  # noqa: F401
    import qip.operators  # noqa: F401
    import qip.pipeline  # noqa: F401
    import qip.qfft  # noqa: F401
    import qip.qip  # noqa: F401
    import qip.qubit_util  # noqa: F401
    import qip.util  # noqa: F401
    return sys.modules["qip"]
