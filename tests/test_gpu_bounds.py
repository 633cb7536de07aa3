"""Bounds-checked build: every computed state index of every kernel is tested against the
state's size before the access (bad ones counted and skipped, nothing traps).  A
workload reaching every kernel family runs on that library in its own process; the
kernels must record no out-of-range index and the results must still match the
oracle.  This stands in for a memory checker where compute-sanitizer cannot be run."""
import os
import subprocess
import sys

import pytest

from qip_gb300 import build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_no_kernel_indexes_out_of_range():
    build.build(checked=True)
    env = dict(os.environ, QSV_BOUNDS_CHECK="1")
    res = subprocess.run([sys.executable, os.path.join(HERE, "bounds_workload.py")], env=env,
                         capture_output=True, text=True, timeout=900)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "out-of-range accesses: 0" in res.stdout, res.stdout
