"""Host tests of the structure-keyed plan cache and of the backend's replay of kept plans.

The replay logic runs here on a stand-in backend whose ``run_plan`` applies the emitted
steps to a numpy state with the oracle, so every emitted order is checked against the
gate list applied one gate at a time."""
import numpy
import pytest

import statevector as sv
from qip_gb300 import backend as backend_mod
from qip_gb300 import circuits, fusion, gates
from qip_gb300.backend import GpuBackend
from qip_gb300.plancache import Entry, PlanCache, step_hash


def _new_matrices(gl, seed):
    """The same circuit structure with new single-qubit matrices."""
    rng = numpy.random.default_rng(seed)
    return [{k: circuits.haar_2x2(rng) if isinstance(m, numpy.ndarray) else m for k, m in g.items()} for g in gl]


def _structure(gl):
    ops = [op for g in gl for op in gates.decompose(g)]
    return ops, [op.qmask for op in ops], [op.amp_update_weight() for op in ops]


def test_prefix_hashes_and_lookup():
    ops, masks, weights = _structure(circuits.brickwork(8, 12, seed=3))
    h = 0
    for m, w in zip(masks[:40], weights[:40]):
        h = step_hash(h, m, w)
    e = Entry(6, masks, weights, [[i] for i in range(len(masks))])
    assert e.prefix[40] == h and e.length == len(masks)
    cache = PlanCache(capacity=2)
    cache.add(e)
    assert cache.find(6, 40, h) is e
    assert cache.find(5, 40, h) is None  # another fusion width
    assert cache.find(6, 41, h) is None
    assert cache.has(6, len(masks), e.prefix[-1]) and not cache.has(6, 40, h)
    # A weight is part of the structure: the same masks with a control differ.
    assert step_hash(0, 3, 1.0) != step_hash(0, 3, 0.5)
    # Masks above 64 qubits are hashed too.
    assert step_hash(0, 1 << 70, 1.0) != step_hash(0, 1 << 71, 1.0)
    for k in range(2):
        cache.add(Entry(6, masks[:10 + k], weights[:10 + k], [[i] for i in range(10 + k)]))
    assert cache.find(6, 40, h) is None  # the oldest was dropped


def test_background_plan_is_the_whole_circuit_plan():
    ops, masks, weights = _structure(circuits.brickwork(10, 16, seed=5))
    cache = PlanCache()
    h = Entry(6, masks, weights, [[0]]).prefix[-1]
    cache.plan_in_background(6, masks, weights, h)
    cache.wait()
    e = cache.find(6, len(masks), h)
    assert e is not None and cache.has(6, len(masks), h)
    assert sorted(i for s in e.steps for i in s) == list(range(len(masks)))
    want, _ = fusion.plan_indices(masks, weights, kmax=6, beam=fusion.BEAM_WIDE)
    assert e.steps == want
    cache.plan_in_background(6, masks[:20], weights[:20], 1)  # too short to keep
    cache.wait()
    assert cache.find(6, 20, 1) is None


class _OracleBackend(GpuBackend):
    """The backend's host logic with the device replaced by the oracle."""

    def __init__(self, n, v, keep_plans=True):
        GpuBackend.__init__(self, n, None, numpy.complex64, fusion=True, autotune=False, keep_plans=keep_plans)
        self.v = v.copy()

    def run_plan(self, steps):
        for st in steps:
            if isinstance(st, fusion.Block):
                self.v = sv.apply_on(self.v, self.n, st.qubits, st.matrix)
                self.stats["blocks"] += 1
            else:
                order, m = st.matrix()
                self.v = sv.apply_on(self.v, self.n, order, m)
                self.stats["ops"] += 1


def _run(n, gl, cache, monkeypatch, v, keep_plans=True):
    monkeypatch.setattr(backend_mod, "default_cache", lambda: cache)
    b = _OracleBackend(n, v, keep_plans)
    for g in gl:
        b.kronselect_dot(g)
    b.flush()
    want = v
    for g in gl:
        want = sv.kronselect_dot(g, want, n)
    numpy.testing.assert_allclose(b.v, want, atol=1e-10)
    return b


def test_second_stream_of_a_structure_replays_the_whole_circuit_plan(monkeypatch):
    n = 12
    cache = PlanCache()
    v = numpy.random.default_rng(1).standard_normal(2 ** n) + 0j
    first = _run(n, circuits.brickwork(n, 24, seed=1), cache, monkeypatch, v)
    assert first.stats["replayed_steps"] == 0
    cache.wait()
    # New matrices, same structure: every step comes from the kept plan.
    gl = _new_matrices(circuits.brickwork(n, 24, seed=1), 2)
    ops, masks, weights = _structure(gl)
    e = cache.find(first._kmax(), len(masks), Entry(6, masks, weights, [[0]]).prefix[-1])
    assert e is not None
    second = _run(n, gl, cache, monkeypatch, v)
    assert second.stats["replayed_steps"] == len(e.steps)
    assert second.stats["blocks"] + second.stats["ops"] == len(e.steps)
    assert len(e.steps) <= first.stats["blocks"] + first.stats["ops"]
    cache.wait()
    assert len(cache._entries) == 1  # a replayed circuit is not planned again


@pytest.mark.parametrize("cut", [130, 200, 300])
def test_streams_that_leave_the_kept_structure_stay_exact(monkeypatch, cut):
    """Same first ``cut`` gates as a kept circuit, then another tail (or none): the
    replay stops where the structure departs and the rest is planned as usual."""
    n = 12
    cache = PlanCache()
    v = numpy.random.default_rng(4).standard_normal(2 ** n) + 0j
    base = circuits.brickwork(n, 24, seed=1)
    _run(n, base, cache, monkeypatch, v)
    cache.wait()
    other = circuits.brickwork(n, 24, seed=7)
    shifted = [{tuple((q + 1) % n for q in k): m for k, m in g.items()} for g in other]
    for gl in (base[:cut], base[:cut] + shifted[cut:], base[:cut] + shifted[:5]):
        b = _run(n, gl, cache, monkeypatch, v)
        assert b.stats["replayed_steps"] > 0


def test_long_streams_are_not_kept(monkeypatch):
    n = 10
    cache = PlanCache()
    monkeypatch.setattr(GpuBackend, "TRACE_MAX", 200)
    v = numpy.random.default_rng(6).standard_normal(2 ** n) + 0j
    _run(n, circuits.brickwork(n, 40, seed=1), cache, monkeypatch, v)
    cache.wait()
    assert cache._entries == []


def test_disabled_cache_keeps_nothing():
    cache = PlanCache(capacity=0)
    ops, masks, weights = _structure(circuits.brickwork(10, 16, seed=5))
    cache.plan_in_background(6, masks, weights, 7)
    cache.wait()
    assert cache.find(6, len(masks), 7) is None and cache._busy == {}


def test_states_that_keep_no_plans_neither_replay_nor_keep(monkeypatch):
    n = 12
    cache = PlanCache()
    v = numpy.random.default_rng(8).standard_normal(2 ** n) + 0j
    gl = circuits.brickwork(n, 24, seed=1)
    _run(n, gl, cache, monkeypatch, v, keep_plans=False)
    cache.wait()
    assert cache._entries == []
    _run(n, gl, cache, monkeypatch, v)
    cache.wait()
    b = _run(n, _new_matrices(gl, 5), cache, monkeypatch, v, keep_plans=False)
    assert b.stats["replayed_steps"] == 0 and len(cache._entries) == 1
