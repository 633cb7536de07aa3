"""Install recipe for the reference's pure-Python package (test and baseline
infrastructure only).

``python -m pip install --no-index --no-build-isolation --no-deps --target
baseline/_ref <copy of the reference checkout>`` puts the reference's ``qip`` package
(graph API, operators, executor, backend classes) into ``baseline/_ref`` (git-ignored).
The install runs from a temporary copy because the build writes into its source tree.
``--no-deps``: numpy is already present and there is no package index.  The
reference's ``setup.py`` builds its Cython extensions only from ``qip/ext/*.c`` files
(absent in the checkout) or with ``CYTHON`` set, so the install holds Python files only;
the compiled kernels come from ``oracle/build_ref.py`` (``oracle/_ref``), which
``oracle/ref_qip.py`` binds as ``qip.ext.*`` at import.  Both folders travel to GPU
machines with the repository, so the reference's own ``run()`` can drive the GPU
backend there (``tests/test_gpu_reference_dropin.py``).

The reference checkout is found through ``build_ref.reference_checkout()``
(``QIP_REFERENCE_ROOT``, else ``reference`` beside the repository).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
TARGET = os.path.join(ROOT, "baseline", "_ref")
if HERE not in sys.path:
    sys.path.insert(0, HERE)
import build_ref  # noqa: E402


def installed() -> bool:
    return os.path.isfile(os.path.join(TARGET, "qip", "pipeline.py"))


def install(force: bool = False) -> bool:
    """Install the reference package into baseline/_ref.  Returns True when it is there
    afterwards, False when there is no checkout to install from."""
    if installed() and not force:
        return True
    src = build_ref.reference_checkout()
    if src is None:
        return False
    with tempfile.TemporaryDirectory() as tmp:
        copy = os.path.join(tmp, "qip_src")
        shutil.copytree(src, copy, ignore=shutil.ignore_patterns(".git", "__pycache__", "build", "*.egg-info"))
        cmd = [sys.executable, "-m", "pip", "install", "--no-index", "--no-build-isolation", "--no-deps",
               "--upgrade", "--target", TARGET, copy]
        if os.path.isdir("/opt/wheelhouse"):
            cmd[5:5] = ["--find-links", "/opt/wheelhouse"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("reference install failed:\n" + res.stdout[-2000:] + res.stderr[-2000:])
    return installed()


if __name__ == "__main__":
    print("reference package", "installed in " + TARGET if install(force="--force" in sys.argv) else "unavailable")
