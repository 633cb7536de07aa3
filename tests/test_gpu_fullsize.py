"""Parity at the benchmark's full sizes, through properties that do not need an FP64
state of that size on the host:

* brickwork n=28 depth 40 (the headline circuit), fed gate by gate through the
  backend: the fused complex64 state against the complex128 per-gate state (both on
  the device; the per-gate path is pinned to the reference and the oracle at smaller
  sizes), infidelity <= 1e-6 (the metric's bound) and the norm (5e-4: see below);
* the same brickwork followed by its inverse (every gate's adjoint, in reverse order)
  returns to |0...0>: a round trip that involves no other GPU path, at full size, for
  the fused complex64 path (fidelity 1 - 1e-6) and the complex128 per-gate path (1e-12);
* QFT + 8 Grover iterations (config 3's circuit) at n=32 complex64 (fused) and n=31
  complex128 (per-gate, 32 GiB each): the marked probability and every single-qubit
  marginal against Grover's closed form (relative 1e-4 for complex64, 1e-10 for
  complex128), and the norm.
"""
import ctypes

import numpy
import pytest

from qip_gb300 import GpuBackend, _native as nat, circuits

pytestmark = pytest.mark.gpu


def test_brickwork_n28_fused_matches_fp64_per_gate_path():
    n = 28
    gl = circuits.brickwork(n, 40, seed=1234)
    fused = GpuBackend.make_state(n, [], [], statetype=numpy.complex64, fusion=True)
    plain = GpuBackend.make_state(n, [], [], statetype=numpy.complex128, fusion=False)
    try:
        for g in gl:
            fused.kronselect_dot(g)
            plain.kronselect_dot(g)
        fused.flush()
        lib = nat.load()
        re_, im_ = ctypes.c_double(), ctypes.c_double()
        nat.check(lib.qsv_inner_product(fused.handle, plain.handle, ctypes.byref(re_), ctypes.byref(im_)),
                  fused.handle, "inner_product")
        n64, n128 = fused.total_prob(), plain.total_prob()
        infid = 1.0 - (re_.value ** 2 + im_.value ** 2) / (n64 * n128)
        assert abs(n128 - 1.0) < 1e-12
        # Fused blocks shrink the norm slightly (the FP32 accumulation rounds towards
        # zero; measured 1.4e-5 after the 67 blocks of this circuit); the direction of the
        # state, which the metric bounds, is far tighter.
        assert abs(n64 - 1.0) < 5e-4
        assert infid < 1e-6, infid
        assert fused.stats["blocks"] > 0
    finally:
        fused.close()
        plain.close()


def _inverse(gate):
    """The adjoint of one kron dictionary: every entry's conjugate transpose (CMat and
    SwapMat entries of this workload are real symmetric or permutations)."""
    out = {}
    for key, m in gate.items():
        out[key] = m if getattr(m, "_kron_struct", None) in (2, 3) else numpy.conj(numpy.asarray(m)).T
    return out


@pytest.mark.parametrize("statetype,tol", [(numpy.complex64, 1e-6), (numpy.complex128, 1e-12)])
def test_brickwork_n28_round_trip_returns_to_zero_state(statetype, tol):
    n = 28
    gl = circuits.brickwork(n, 40, seed=1234)
    for g in gl:  # the workload's CMat entries hold Z or SwapMat(1): self-inverse
        for m in g.values():
            if getattr(m, "_kron_struct", None) == 2:
                assert getattr(m.m, "_kron_struct", None) == 3 or numpy.allclose(m.m, numpy.diag([1, -1]))
    st = GpuBackend.make_state(n, [], [], statetype=statetype, fusion=statetype == numpy.complex64)
    try:
        for g in gl:
            st.kronselect_dot(g)
        for g in reversed(gl):
            st.kronselect_dot(_inverse(g))
        norm2 = st.total_prob()
        a0 = st.get_relative_range(0, 1)[0]
        probe = st.get_relative_range(1, 1 << 12)
    finally:
        st.close()
    fidelity = abs(a0) ** 2 / norm2
    assert 1.0 - fidelity < tol, 1.0 - fidelity
    assert numpy.max(numpy.abs(probe)) < (1e-4 if statetype == numpy.complex64 else 1e-7)


@pytest.mark.parametrize("n,statetype,rtol", [(32, numpy.complex64, 1e-4), (31, numpy.complex128, 1e-10)])
def test_grover_full_size_closed_form(n, statetype, rtol):
    iterations = 8
    gl, marked = circuits.grover_gates(n, iterations, seed=7)
    st = GpuBackend.make_state(n, [], [], statetype=statetype, fusion=statetype == numpy.complex64)
    try:
        for g in gl:
            st.kronselect_dot(g)
        marg, norm2 = st.qubit_marginals()
        amp = st.get_relative_range(marked, marked + 1)[0]
    finally:
        st.close()
    N = 2.0 ** n
    theta = numpy.arcsin(1 / numpy.sqrt(N))
    pm = numpy.sin((2 * iterations + 1) * theta) ** 2
    pu = (1 - pm) / (N - 1)
    bits = numpy.array([(marked >> (n - 1 - q)) & 1 for q in range(n)])
    want = pm * bits + pu * (N / 2 - bits)
    # complex64: fused blocks move the norm by ~1e-5 each (see the brickwork test).
    assert abs(norm2 - 1.0) < (5e-4 if statetype == numpy.complex64 else 1e-12)
    numpy.testing.assert_allclose(abs(amp) ** 2, pm, rtol=rtol)
    numpy.testing.assert_allclose(marg, want, rtol=rtol)
