"""The drop-in on the GPU: the reference's own graph executor and operator objects drive
``GpuBackend``.

``run(*outputs, feed=..., backend_constructor=GpuBackend.make_state, statetype=...)`` of
the reference (``qip/pipeline.py:71-135``) builds the state through this package's
``make_state`` and hands every gate to ``GpuBackend.kronselect_dot`` as the reference's
own ``{indices: numpy | CMat | SwapMat}`` dictionaries (``qip/operators.py:195-268``);
measurements arrive as its ``measure`` / ``measure_probabilities`` calls
(``qip/qip.py:148-155,177-182``).  Results are compared with the goldens the
reference's own ``CythonBackend`` produced for the same scenarios
(``tests/golden/make_golden.py``).

The reference package comes from ``baseline/_ref`` (``oracle/install_ref.py``) and its
Cython kernels from ``oracle/_ref`` (``oracle/build_ref.py``); without them the test is
skipped.
"""
import types

import numpy
import pytest

import ref_qip
from conftest import load_npz
from qip_gb300 import GpuBackend

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_qip.available(), reason="reference package or kernels not present")]

C64, C128 = numpy.complex64, numpy.complex128


def reference_api():
    qip = ref_qip.import_reference()
    ns = types.SimpleNamespace()
    for mod in (qip.qip, qip.operators, qip.pipeline, qip.qfft, qip.qubit_util):
        for k in dir(mod):
            if not k.startswith("_"):
                setattr(ns, k, getattr(mod, k))
    return ns


@pytest.mark.parametrize("statetype,fusion,atol,patol", [(C128, False, 1e-12, 1e-12), (C64, True, 2e-5, 1e-6),
                                                          (C64, False, 1e-5, 1e-6)])
def test_reference_run_drives_gpu_backend(statetype, fusion, atol, patol):
    from scenarios import SCENARIOS

    d, meta = load_npz("scenarios.npz")
    api = reference_api()

    def ctor(n, groups, feeds, statetype=statetype):
        return GpuBackend.make_state(n, groups, feeds, statetype=statetype, fusion=fusion)

    checked = 0
    for name, fn in SCENARIOS.items():
        for r, (outs, feed, measured) in enumerate(fn(api)):
            o, classic = api.run(*outs, feed=feed, backend_constructor=ctor, statetype=statetype)
            assert isinstance(o, numpy.ndarray) and o.dtype == numpy.dtype(statetype)
            numpy.testing.assert_allclose(o, d[f"{name}_{r}_state"], rtol=0, atol=atol, err_msg=f"{name}[{r}]")
            for j, node in enumerate(measured):
                val = classic[node]
                if meta[name][r]["measured"][j] == "topk":
                    numpy.testing.assert_allclose(val[1], d[f"{name}_{r}_m{j}_p"], atol=patol)
                else:
                    numpy.testing.assert_allclose(val, d[f"{name}_{r}_m{j}_p"], atol=patol)
            checked += 1
    assert checked >= 20


def test_reference_qfft_on_gpu_is_the_inverse_dft():
    """The reference's own ``QFFT`` graph (``qip/qfft.py:8-43``) at n=16, as config 1
    runs it, through ``GpuBackend`` in complex128: the inverse DFT of the input, and the
    top-4-qubit distribution of a ``StochasticMeasure``."""
    api = reference_api()
    n = 16
    rng = numpy.random.default_rng(2024)
    x = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    x /= numpy.linalg.norm(x)
    q = api.Qubit(n=n)
    out = api.QFFT(q)
    top = out.split([4])
    sm = api.StochasticMeasure(top[0])
    o, classic = api.run(sm, top[1], feed={q: x}, backend_constructor=GpuBackend.make_state)
    want = numpy.fft.ifft(x, norm="ortho")
    numpy.testing.assert_allclose(o, want, rtol=0, atol=1e-12)
    i = numpy.arange(2 ** n)
    outcome = sum(((i >> (n - 1 - j)) & 1) << j for j in range(4))
    numpy.testing.assert_allclose(classic[sm], numpy.bincount(outcome, weights=numpy.abs(want) ** 2, minlength=16),
                                  rtol=0, atol=1e-12)
