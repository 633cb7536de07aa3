"""qsv_probabilities_static: the allocation-free marginal-probability entry point, for
callers that cannot allocate device memory when they read a distribution (their HBM is
owned by another allocator, or allocating is not allowed where they call from).  Called
through the C ABI with a caller-owned state and output buffer, and compared with the
allocating entry point (qsv_probabilities) on two calls in a row.

Collected last on purpose: it shares one device array across calls, so any failure
here must not hide the results of the other tests."""
import ctypes

import numpy
import pytest

pytestmark = pytest.mark.gpu


def _static_probs(lib, st, qubits, d_out):
    q = (ctypes.c_int * max(1, len(qubits)))(*qubits)
    dtype = 0 if st.statetype == numpy.complex64 else 1
    return lib.qsv_probabilities_static(ctypes.c_void_p(st.device_ptr()), st.n, dtype, len(qubits), q,
                                        ctypes.c_void_p(d_out.data_ptr()), None)


@pytest.mark.parametrize("statetype,atol", [(numpy.complex128, 1e-12), (numpy.complex64, 1e-6)])
def test_static_scratch_probabilities_match_allocating_entry_point(statetype, atol):
    import torch

    from qip_gb300 import GpuBackend, _native

    lib = _native.load()
    rng = numpy.random.default_rng(11)
    n = 20
    v = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    v /= numpy.linalg.norm(v)
    st = GpuBackend.make_state(n, [list(range(n))], [v], statetype=statetype)
    try:
        cases = [[0, 1, 2, 3], [19], [5, 17, 2], [], list(range(n - 16, n)), [12, 0, 19, 7, 3]]
        for call in range(2):  # two calls in a row share (and reuse) the static array
            for qubits in cases:
                want = st.measure_probabilities(qubits)  # allocating path
                st.synchronize()
                d_out = torch.full((2 ** len(qubits),), -1.0, dtype=torch.float64, device="cuda")
                torch.cuda.synchronize()
                rc = _static_probs(lib, st, qubits, d_out)
                assert rc == 0, lib.qsv_last_error(None).decode()
                torch.cuda.synchronize()
                got = d_out.cpu().numpy()
                numpy.testing.assert_allclose(got, want, rtol=0, atol=atol, err_msg=f"call {call} {qubits}")
        # Sizes beyond the static array are rejected with a clear error.
        d_out = torch.empty(2 ** 17, dtype=torch.float64, device="cuda")
        rc = _static_probs(lib, st, list(range(17)), d_out)
        assert rc == _native.QSV_ERR_INVALID
        assert b"at most 16" in lib.qsv_last_error(None)
        # An output buffer that is not device memory of the current GPU is rejected
        # before any launch (here: host memory).
        host_out = numpy.zeros(16)
        q = (ctypes.c_int * 4)(0, 1, 2, 3)
        dtype = 0 if st.statetype == numpy.complex64 else 1
        rc = lib.qsv_probabilities_static(ctypes.c_void_p(st.device_ptr()), st.n, dtype, 4, q,
                                          host_out.ctypes.data_as(ctypes.c_void_p), None)
        assert rc == _native.QSV_ERR_INVALID
        assert b"not device memory" in lib.qsv_last_error(None) or b"not a CUDA pointer" in lib.qsv_last_error(None)
        assert numpy.all(host_out == 0)
    finally:
        st.close()
