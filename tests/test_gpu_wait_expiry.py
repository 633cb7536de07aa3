"""Failure detection on the GPU without a fault: a bounded device wait is made to run out.

``qsv_inject_block_stall`` arms the next fused-block launch so that each CTA's first
wait for its tensor-core products is on an mbarrier nothing arrives on, with a short
limit.  The kernel gives up, drains the products it has in flight (bounded), frees its
tensor memory and sets the handle's status word; nothing traps, nothing hangs.  The
test checks the error status, that the status word clears, that the aborted launch left
the state as it was (every CTA's first wait precedes its first store), and that the
same handle then applies the block correctly.
"""
import numpy
import pytest

import statevector as sv
from qip_gb300 import GpuBackend, _native as nat
from qip_gb300.fusion import Block

pytestmark = pytest.mark.gpu


def _unitary(k, seed):
    rng = numpy.random.default_rng(seed)
    z = rng.standard_normal((2 ** k, 2 ** k)) + 1j * rng.standard_normal((2 ** k, 2 ** k))
    return numpy.linalg.qr(z)[0]


@pytest.mark.parametrize("targets", [(0, 1, 2, 3, 4, 5), (2, 3, 4, 5, 14, 16)])
def test_block_wait_expiry_reports_timeout_and_the_handle_recovers(targets):
    n = 17
    rng = numpy.random.default_rng(3)
    x = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    x /= numpy.linalg.norm(x)
    st = GpuBackend.make_state(n, [list(range(n))], [x], statetype=numpy.complex64, fusion=True)
    lib = nat.load()
    try:
        before = st.get_state().copy()
        u = _unitary(len(targets), 11)
        block = Block(tuple(targets), u, 1, 1.0)
        assert lib.qsv_inject_block_stall(st.handle, 10) == nat.QSV_ERR_INVALID  # below 1 us
        assert lib.qsv_inject_block_stall(st.handle, 200_000) == nat.QSV_OK  # 200 us
        st.apply_blocks([block])
        assert lib.qsv_synchronize(st.handle) == nat.QSV_ERR_TIMEOUT
        assert b"bounded device wait" in lib.qsv_last_error(st.handle)
        assert lib.qsv_synchronize(st.handle) == nat.QSV_OK  # the status word was cleared
        assert numpy.array_equal(st.get_state(), before)  # the aborted launch stored nothing
        st.apply_blocks([block])  # not armed any more: a normal launch
        assert lib.qsv_synchronize(st.handle) == nat.QSV_OK
        got = st.get_state()
    finally:
        st.close()
    want = sv.apply_on(before.astype(numpy.complex128), n, list(targets), u)
    assert numpy.max(numpy.abs(got - want)) < 2e-5
