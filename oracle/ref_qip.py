"""Import the reference QIP package (pure-Python layers plus the Cython kernels built by
``oracle/build_ref.py``) in the development container.

Test infrastructure only: used by ``tests/golden/make_golden.py`` to generate golden
vectors from the reference itself, and by the CPU tests that pin the oracle against
the reference when the checkout is present.  The reference checkout does not exist on
GPU machines, so nothing on a GPU code path imports this module.
"""
from __future__ import annotations

import os
import sys
import types

REF_ROOT = os.environ.get("QIP_REFERENCE_ROOT", "/root/reference")


def available() -> bool:
    return os.path.isdir(os.path.join(REF_ROOT, "qip"))


def import_reference():
    """Return the reference ``qip`` package with ``qip.ext.*`` bound to the modules
    compiled into ``oracle/_ref/lib``."""
    here = os.path.dirname(os.path.abspath(__file__))
    if here not in sys.path:
        sys.path.insert(0, here)
    import build_ref  # type: ignore

    if not build_ref.available():
        if not build_ref.build():
            raise RuntimeError("reference kernels unavailable")
    kronprod, func_apply = build_ref.load()
    if REF_ROOT not in sys.path:
        sys.path.insert(0, REF_ROOT)
    # ``qip/ext/__init__.py`` is empty; bind the compiled kernels as its submodules.
    import qip  # noqa: F401
    ext = sys.modules.get("qip.ext")
    if ext is None:
        ext = types.ModuleType("qip.ext")
        ext.__path__ = [os.path.join(REF_ROOT, "qip", "ext")]
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
