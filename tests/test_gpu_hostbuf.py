"""Page-locked readback arrays: correct values, never reused while an array still
refers to them, reused once released, and the opt-out."""
import numpy
import pytest

import statevector as sv
from qip_gb300 import GpuBackend, hostbuf

pytestmark = pytest.mark.gpu


def addr(a):
    return a.__array_interface__["data"][0]


def test_readback_arrays_are_owned_by_the_caller(monkeypatch):
    n = 20
    rng = numpy.random.default_rng(6)
    v = (rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)).astype(numpy.complex64)
    st = GpuBackend.make_state(n, [list(range(n))], [v], statetype=numpy.complex64, fusion=False)
    a = st.get_state()
    assert isinstance(a.base, hostbuf._PinnedOwner)
    assert numpy.array_equal(a, v)
    h = numpy.array([[1, 1], [1, -1]]) / numpy.sqrt(2)
    st.kronselect_dot({3: h})
    b = st.get_state()
    assert addr(a) != addr(b)             # a is still alive: b got another buffer
    assert numpy.array_equal(a, v)        # ... and a was not overwritten
    numpy.testing.assert_allclose(b, sv.kronselect_dot({3: h}, v.astype(complex), n), atol=1e-6)
    old = addr(a)
    del a
    c = st.get_state()                    # the released buffer comes back from the pool
    assert addr(c) == old
    assert numpy.array_equal(c, b)
    monkeypatch.setenv("QSV_PINNED_READBACK", "0")
    d = st.get_state()
    assert not isinstance(d.base, hostbuf._PinnedOwner)
    assert numpy.array_equal(d, b)
    st.close()


def test_parked_state_buffers_start_clean():
    """A closed state's buffers are reused by the next state: the new state still starts
    as |0...0> and computes correctly, for the same size, another size, and after the
    parked buffers were released."""
    n = 20
    rng = numpy.random.default_rng(8)
    v = (rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)).astype(numpy.complex64)
    h = numpy.array([[1, 1], [1, -1]]) / numpy.sqrt(2)
    st = GpuBackend.make_state(n, [list(range(n))], [v], statetype=numpy.complex64, fusion=True)
    for q in range(n):
        st.kronselect_dot({q: h})
    st.get_state()
    st.close()
    e0 = numpy.zeros(2 ** n, dtype=numpy.complex64)
    e0[0] = 1
    for size in (n, n + 1, n):
        st = GpuBackend.make_state(size, [], [], statetype=numpy.complex64, fusion=True)
        want = numpy.zeros(2 ** size, dtype=numpy.complex64)
        want[0] = 1
        assert numpy.array_equal(st.get_state(), want)
        st.kronselect_dot({0: h})
        got = st.get_state()
        st.close()
        numpy.testing.assert_allclose(got, sv.kronselect_dot({0: h}, want.astype(complex), size), atol=1e-6)
    GpuBackend.release_parked_buffers()
    st = GpuBackend.make_state(n, [], [], statetype=numpy.complex128)
    assert numpy.array_equal(st.get_state(), e0.astype(numpy.complex128))
    st.close()


@pytest.mark.parametrize("statetype", [numpy.complex64, numpy.complex128])
def test_device_state_is_a_view_of_the_state(statetype):
    """device_state(): a torch tensor over the device buffer with queued gates applied;
    it reads what get_state reads and writes through to the state."""
    import torch

    n = 16
    h = numpy.array([[1, 1], [1, -1]]) / numpy.sqrt(2)
    st = GpuBackend.make_state(n, [], [], statetype=statetype, fusion=statetype == numpy.complex64)
    for q in range(n):
        st.kronselect_dot({q: h})
    t = st.device_state()
    assert t.is_cuda and t.dtype == (torch.complex64 if statetype == numpy.complex64 else torch.complex128)
    assert t.shape == (2 ** n,) and t.data_ptr() == st.device_ptr()
    numpy.testing.assert_allclose(t.cpu().numpy(), st.get_state(), atol=1e-7)
    t.mul_(2.0)
    torch.cuda.synchronize()
    assert st.total_prob() == pytest.approx(4.0, rel=1e-5)
    del t
    st.close()
