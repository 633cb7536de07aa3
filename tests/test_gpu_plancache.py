"""Replay of kept whole-circuit plans on the device: a second stream of the same circuit
structure runs the kept plan's blocks, and streams that leave the structure stay exact
(complex64 fused blocks against the complex128 per-gate kernels)."""
import numpy
import pytest

from qip_gb300 import backend as backend_mod
from qip_gb300 import circuits
from qip_gb300.backend import GpuBackend
from qip_gb300.plancache import PlanCache

pytestmark = pytest.mark.gpu

C64 = numpy.complex64


def _new_matrices(gl, seed):
    rng = numpy.random.default_rng(seed)
    return [{k: circuits.haar_2x2(rng) if isinstance(m, numpy.ndarray) else m for k, m in g.items()} for g in gl]


def _fused(n, gl, v):
    st = GpuBackend.make_state(n, [list(range(n))], [v], statetype=C64, fusion=True, autotune=False)
    for g in gl:
        st.kronselect_dot(g)
    out = st.get_state().copy()
    stats = dict(st.stats)
    st.close()
    return out, stats


def _exact(n, gl, v):
    st = GpuBackend.make_state(n, [list(range(n))], [v], statetype=numpy.complex128, fusion=False)
    for g in gl:
        st.kronselect_dot(g)
    out = st.get_state().copy()
    st.close()
    return out


def _infidelity(a, b):
    a = numpy.asarray(a, dtype=numpy.complex128)
    b = numpy.asarray(b, dtype=numpy.complex128)
    return 1.0 - abs(numpy.vdot(a, b)) ** 2 / (numpy.vdot(a, a).real * numpy.vdot(b, b).real)


def test_replayed_plan_matches_the_per_gate_path(monkeypatch):
    n = 20
    cache = PlanCache()
    monkeypatch.setattr(backend_mod, "default_cache", lambda: cache)
    rng = numpy.random.default_rng(11)
    v = (rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n))
    v /= numpy.linalg.norm(v)
    base = circuits.brickwork(n, 24, seed=3)
    got, first = _fused(n, base, v)
    assert first["replayed_steps"] == 0
    assert _infidelity(got, _exact(n, base, v)) < 1e-6
    cache.wait()
    assert len(cache._entries) == 1
    kept = len(cache._entries[0].steps)
    gl = _new_matrices(base, 4)
    got, second = _fused(n, gl, v)
    assert second["replayed_steps"] == kept
    assert second["blocks"] <= first["blocks"]
    assert _infidelity(got, _exact(n, gl, v)) < 1e-6


@pytest.mark.parametrize("cut", [150, 400])
def test_streams_leaving_a_kept_structure_match_the_per_gate_path(monkeypatch, cut):
    n = 18
    cache = PlanCache()
    monkeypatch.setattr(backend_mod, "default_cache", lambda: cache)
    rng = numpy.random.default_rng(12)
    v = (rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n))
    v /= numpy.linalg.norm(v)
    base = circuits.brickwork(n, 24, seed=5)
    _fused(n, base, v)
    cache.wait()
    other = circuits.brickwork(n, 24, seed=8)
    shifted = [{tuple((q + 3) % n for q in k): m for k, m in g.items()} for g in other]
    for gl in (base[:cut], base[:cut] + shifted[cut:]):
        got, stats = _fused(n, gl, v)
        assert stats["replayed_steps"] > 0
        assert _infidelity(got, _exact(n, gl, v)) < 1e-6
