"""Exhaustive small-register sweep (n=7): every qubit position, every ordered
target/control pair and every controlled-swap triple, for each gate kind, in both
precisions, against the FP64 oracle — the bounds and index coverage that a sanitizer
would otherwise give.  Also the host-side rejection of non-finite matrices."""
import itertools

import numpy
import pytest

import statevector as sv
from qip_gb300 import GpuBackend, circuits
from qip_gb300.operators import CMat, SwapMat

pytestmark = pytest.mark.gpu

N = 7
X = numpy.array([[0, 1], [1, 0]], dtype=complex)


def cases(rng):
    for q in range(N):
        yield {(q,): circuits.haar_2x2(rng)}
        yield {(q,): numpy.diag([1.0, numpy.exp(1.1j)])}
        yield {(q,): X}
    for c, t in itertools.permutations(range(N), 2):
        yield {(c, t): CMat(X)}
        yield {(c, t): CMat(circuits.haar_2x2(rng))}
    for a, b in itertools.combinations(range(N), 2):
        yield {(a, b): SwapMat(1)}
        yield {(a, b): numpy.diag([1, 1, 1, -1]).astype(complex)}
        u = numpy.linalg.qr(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)))[0]
        yield {(a, b): u}
    for c, a, b in itertools.permutations(range(N), 3):
        if a < b:
            yield {(c, a, b): CMat(SwapMat(1))}


@pytest.mark.parametrize("statetype,atol", [(numpy.complex128, 1e-12), (numpy.complex64, 2e-6)])
def test_every_position_and_control_pattern(statetype, atol):
    rng = numpy.random.default_rng(71)
    v = (rng.standard_normal(2 ** N) + 1j * rng.standard_normal(2 ** N)) / numpy.sqrt(2 ** (N + 1))
    count = 0
    for mats in cases(rng):
        st = GpuBackend.make_state(N, [list(range(N))], [v], statetype=statetype, fusion=False)
        st.kronselect_dot(mats)
        got = st.get_state()
        st.close()
        want = sv.kronselect_dot(mats, v.astype(statetype).astype(complex), N)
        numpy.testing.assert_allclose(got, want, rtol=0, atol=atol, err_msg=str(list(mats)))
        count += 1
    assert count == 273


def test_non_finite_matrices_are_rejected_before_launch():
    st = GpuBackend.make_state(5, [], [], statetype=numpy.complex64)
    bad = numpy.array([[1, numpy.nan], [0, 1]], dtype=complex)
    with pytest.raises(ValueError, match="non-finite"):
        st.kronselect_dot({(2,): bad})
    with pytest.raises(ValueError, match="non-finite"):
        st.kronselect_dot({(1, 3): CMat(numpy.array([[numpy.inf, 0], [0, 1]], dtype=complex))})
    out = st.get_state()
    assert out[0] == 1 and numpy.count_nonzero(out) == 1  # nothing was applied
    st.close()
