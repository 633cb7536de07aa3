"""Edge cases on the GPU against the oracle: the smallest states (n = 1, 2) in both
precisions through every StateType call the executor makes, empty dictionaries and
identity matrices (nothing to launch), fusion requested on states too small for a
tensor-core tile (the per-gate kernels take over), and out-of-range qubit indices
(rejected on the host before anything is queued)."""
import numpy
import pytest

import statevector as sv
from qip_gb300 import GpuBackend

pytestmark = pytest.mark.gpu

H = numpy.array([[1, 1], [1, -1]]) / numpy.sqrt(2)
X = numpy.array([[0, 1], [1, 0]])


@pytest.mark.parametrize("statetype,atol", [(numpy.complex128, 1e-12), (numpy.complex64, 1e-6)])
@pytest.mark.parametrize("n", [1, 2])
def test_smallest_states(n, statetype, atol):
    rng = numpy.random.default_rng(n)
    v = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    v /= numpy.linalg.norm(v)
    st = GpuBackend.make_state(n, [list(range(n))], [v], statetype=statetype)
    want = v.copy()
    for g in ({0: H}, {n - 1: X}, {0: numpy.diag([1, 1j])}):
        st.kronselect_dot(g)
        want = sv.kronselect_dot(g, want, n)
    numpy.testing.assert_allclose(st.get_state(), want, atol=atol)
    assert st.get_state_size() == 2 ** n
    assert st.total_prob() == pytest.approx(1.0, abs=10 * atol)
    numpy.testing.assert_allclose(st.measure_probabilities(list(range(n))),
                                  sv.measure_probabilities(list(range(n)), n, want), atol=atol)
    p0 = float(numpy.sum(numpy.abs(want.reshape(2, -1)[0]) ** 2))
    m, p = st.measure([0], measured=0, measured_prob=p0)
    assert m == 0 and p == pytest.approx(p0, abs=atol)
    got = st.get_state()
    assert numpy.all(got.reshape(2, -1)[1] == 0)
    assert numpy.linalg.norm(got) == pytest.approx(1.0, abs=10 * atol)
    st.close()


def test_empty_dictionaries_and_identities_launch_nothing():
    st = GpuBackend.make_state(10, [], [], statetype=numpy.complex128)
    before = st.stats["launch_calls"]
    st.kronselect_dot({})
    st.kronselect_dot({3: numpy.eye(2)})
    st.kronselect_dot({(2, 5): numpy.eye(4)})
    assert st.stats["launch_calls"] == before
    want = numpy.zeros(2 ** 10, dtype=complex)
    want[0] = 1
    numpy.testing.assert_array_equal(st.get_state(), want)
    st.close()


@pytest.mark.parametrize("n", [3, 8, 12])
def test_fusion_on_states_too_small_for_tensor_core_tiles(n):
    rng = numpy.random.default_rng(n)
    gl = []
    for _ in range(4):
        for q in range(n):
            u = numpy.linalg.qr(rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2)))[0]
            gl.append({q: u})
        for q in range(0, n - 1, 2):
            gl.append({(q, q + 1): numpy.diag([1, 1, 1, -1]).astype(complex)})
    st = GpuBackend.make_state(n, [], [], statetype=numpy.complex64, fusion=True)
    want = numpy.zeros(2 ** n, dtype=complex)
    want[0] = 1
    for g in gl:
        st.kronselect_dot(g)
        want = sv.kronselect_dot(g, want, n)
    numpy.testing.assert_allclose(st.get_state(), want, atol=2e-6)
    st.close()


@pytest.mark.parametrize("fusion", [False, True])
def test_out_of_range_qubits_are_rejected_before_queueing(fusion):
    st = GpuBackend.make_state(6, [], [], statetype=numpy.complex64, fusion=fusion)
    st.kronselect_dot({0: H})
    with pytest.raises(ValueError):
        st.kronselect_dot({6: H})
    with pytest.raises(ValueError):
        st.kronselect_dot({(1, 7): numpy.eye(4)[::-1]})
    want = numpy.zeros(64, dtype=complex)
    want[0] = want[32] = 1 / numpy.sqrt(2)
    numpy.testing.assert_allclose(st.get_state(), want, atol=1e-6)
    st.close()
