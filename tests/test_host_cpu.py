"""Host logic on CPU: the graph API mirror, the kron-dictionary decomposition and the
fusion planner, each checked with the oracle as the state executor.  No GPU."""
import types

import numpy
import pytest

import qip_gb300 as api_mod
import statevector as sv
from conftest import load_npz
from make_golden import decode
from qip_gb300 import circuits, fusion, gates
from qip_gb300.operators import CMat, SwapMat
from scenarios import SCENARIOS


def api_ns():
    return types.SimpleNamespace(**{k: getattr(api_mod, k) for k in api_mod.__all__})


def run_scenarios(backend_constructor, statetype=numpy.complex128, names=None, atol=1e-12):
    d, meta = load_npz("scenarios.npz")
    api = api_ns()
    checked = 0
    for name, fn in SCENARIOS.items():
        if names and name not in names:
            continue
        runs = fn(api)
        assert len(runs) == len(meta[name])
        for r, (outs, feed, measured) in enumerate(runs):
            o, classic = api.run(*outs, feed=feed, backend_constructor=backend_constructor, statetype=statetype)
            numpy.testing.assert_allclose(o, d[f"{name}_{r}_state"], rtol=0, atol=atol, err_msg=f"{name}[{r}]")
            for j, node in enumerate(measured):
                kind = meta[name][r]["measured"][j]
                val = classic[node]
                if kind == "topk":
                    numpy.testing.assert_allclose(val[1], d[f"{name}_{r}_m{j}_p"], atol=atol)
                    refp = d[f"{name}_{r}_m{j}_p"]
                    refm = d[f"{name}_{r}_m{j}_idx"]
                    for k in range(len(refm)):
                        if numpy.sum(numpy.abs(refp - refp[k]) < 1e-12) == 1:
                            assert int(val[0][k]) == int(refm[k]), f"{name}[{r}] top-k index {k}"
                else:
                    numpy.testing.assert_allclose(val, d[f"{name}_{r}_m{j}_p"], atol=atol)
            checked += 1
    return checked


def test_graph_api_mirror_matches_reference_runs():
    assert run_scenarios(sv.OracleBackend.make_state) >= 40


def test_replayed_walks_match_fresh_walks():
    """run() records a graph's walk and replays it on later runs of the same graph: every
    scenario run twice (first walk, replay) gives the goldens both times, and a graph
    with a node that overrides ``feed`` is walked afresh every time."""
    from qip_gb300 import pipeline

    pipeline.clear_compiled_walks()
    d, meta = load_npz("scenarios.npz")
    api = api_ns()
    for name, fn in SCENARIOS.items():
        for r, (outs, feed, measured) in enumerate(fn(api)):
            for rep in range(2):
                o, classic = api.run(*outs, feed=feed, backend_constructor=sv.OracleBackend.make_state)
                numpy.testing.assert_allclose(o, d[f"{name}_{r}_state"], rtol=0, atol=1e-12,
                                              err_msg=f"{name}[{r}] run {rep}")
                for j, node in enumerate(measured):
                    val = classic[node]
                    want = d[f"{name}_{r}_m{j}_p"]
                    got = val[1] if meta[name][r]["measured"][j] == "topk" else val
                    numpy.testing.assert_allclose(got, want, atol=1e-12)
    assert len(pipeline._WALKS) > 0

    class Tracing(api_mod.Qubit):
        seen = 0

        def feed(self, state, qbitindex, n):
            Tracing.seen += 1
            return super().feed(state, qbitindex, n)

    q = api_mod.Qubit(n=2)
    h = api_mod.H(q)
    t = Tracing(h)
    for _ in range(3):
        o, _ = api_mod.run(t, feed={q: [0, 1, 0, 0]}, backend_constructor=sv.OracleBackend.make_state)
    assert Tracing.seen == 3
    numpy.testing.assert_allclose(o, [0.5, -0.5, 0.5, -0.5], atol=1e-15)


def test_qft_negate_keyword_is_dropped_like_reference():
    # QubitOpWrapper forwards only construction-time kwargs, so QFFT's negate=True has
    # no effect and the circuit is the inverse DFT (matches the reference output).
    n = 5
    rng = numpy.random.default_rng(0)
    x = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    x /= numpy.linalg.norm(x)
    q = api_mod.Qubit(n=n)
    o, _ = api_mod.run(api_mod.QFFT(q), feed={q: x}, backend_constructor=sv.OracleBackend.make_state)
    numpy.testing.assert_allclose(o, numpy.fft.ifft(x, norm="ortho"), atol=1e-13)


def test_no_cloning_and_argument_errors():
    q = api_mod.Qubit(n=1)
    api_mod.Qubit(q)
    with pytest.raises(Exception):
        api_mod.Qubit(q)
    with pytest.raises(ValueError):
        api_mod.Qubit(n=2, default=[1, 0, 0])
    a, b = api_mod.Qubit(n=1), api_mod.Qubit(n=2)
    with pytest.raises(Exception):
        api_mod.SwapOp(a, b)
    with pytest.raises(ValueError):
        api_mod.C(api_mod.H)(api_mod.Qubit(n=2), api_mod.Qubit(n=1))
    with pytest.raises(ValueError):
        r = api_mod.Qubit(n=1)
        api_mod.run(api_mod.H(r), strict=True, backend_constructor=sv.OracleBackend.make_state)


def test_decompose_equals_reference_semantics():
    """Every kron dictionary of the golden set: the structured ops, applied one by one,
    give the reference output."""
    d, cases = load_npz("kron_cases.npz")
    for c in cases:
        mats = decode(c["mats"], d, CMat, SwapMat)
        ops = gates.decompose(mats)
        v = d[f"k{c['id']}_in"].astype(complex)
        for op in ops:
            order, m = op.matrix()
            v = sv.apply_on(v, c["n"], order, m)
        numpy.testing.assert_allclose(v, d[f"k{c['id']}_out"], atol=1e-12, err_msg=str(c))


def test_decompose_mixed_dictionaries_against_oracle():
    # Dictionaries the reference cannot pack (mixed key lengths / kinds) follow the
    # entry-product semantics of the oracle.
    rng = numpy.random.default_rng(4)
    n = 6
    for _ in range(20):
        a, b, c, e = (int(x) for x in rng.choice(n, 4, replace=False))
        u2 = numpy.linalg.qr(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)))[0]
        u1 = numpy.linalg.qr(rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2)))[0]
        for mats in ({(a, b): u2, (c,): u1}, {(a, b): CMat(u1), (c, e): SwapMat(1)},
                     {(a, b, c): CMat(CMat(u1)), (e,): u1}, {(a, b): u2, (b, c): u2}):
            v = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
            want = sv.kronselect_dot(mats, v, n)
            got = v.copy()
            for op in gates.decompose(mats):
                order, m = op.matrix()
                got = sv.apply_on(got, n, order, m)
            numpy.testing.assert_allclose(got, want, atol=1e-12)


def test_decompose_errors_match_reference():
    with pytest.raises(Exception, match="Type of indices"):
        gates.decompose({"a": numpy.eye(2)})
    with pytest.raises(Exception, match="Shape of square submatrix"):
        gates.decompose({(0, 1): numpy.eye(2)})
    with pytest.raises(ValueError, match="Cannot pass matrices"):
        gates.decompose({(0,): types.SimpleNamespace(shape=(2, 2))})


def test_decompose_classifies_structure():
    h = numpy.array([[1, 1], [1, -1]]) / numpy.sqrt(2)
    assert gates.decompose({0: h})[0].kind == "dense"
    assert gates.decompose({0: numpy.diag([1, 1j])})[0].kind == "diag"
    assert gates.decompose({0: numpy.array([[0, 1], [1, 0]])})[0].kind == "mono"
    assert gates.decompose({0: numpy.eye(2)}) == []
    op = gates.decompose({(3, 1, 2): CMat(CMat(numpy.diag([1, -1])))})[0]
    assert op.kind == "diag" and op.controls == (3, 1) and op.targets == (2,)
    op = gates.decompose({(0, 1, 2): CMat(SwapMat(1))})[0]
    assert op.kind == "swap" and op.controls == (0,) and op.targets == (1,) and op.swap_b == (2,)


@pytest.mark.parametrize("kmax", [3, 4, 5, 6])
def test_fusion_plan_preserves_the_circuit(kmax):
    n = 9
    gl = circuits.brickwork(n, 6, seed=2) + circuits.grover_gates(n, 1, seed=1)[0]
    ops = [op for g in gl for op in gates.decompose(g)]
    steps = fusion.plan(ops, kmax=kmax)
    v0 = numpy.zeros(2 ** n, dtype=complex)
    v0[0] = 1
    want = v0
    for g in gl:
        want = sv.kronselect_dot(g, want, n)
    got = v0
    nblocks = 0
    for st in steps:
        if isinstance(st, fusion.Block):
            assert len(st.qubits) <= kmax
            got = sv.apply_on(got, n, st.qubits, st.matrix)
            nblocks += 1
        else:
            order, m = st.matrix()
            got = sv.apply_on(got, n, order, m)
    numpy.testing.assert_allclose(got, want, atol=1e-11)
    assert len(steps) < len(ops)
    assert sum(st.ngates if isinstance(st, fusion.Block) else 1 for st in steps) == len(ops)


@pytest.mark.parametrize("low_bits", [(3, 2, 1, 0), (4, 3, 2, 1, 0), (4, 3, 2, 1), (12, 7, 5, 3), (12, 10, 9, 1)])
def test_small_blocks_are_widened_to_six_qubits(low_bits):
    """A tensor-core block of fewer than 6 qubits gets identity qubits on the highest
    free bits (also between its own qubits); the circuit is unchanged, other steps are
    untouched."""
    n = 13
    low_qubits = tuple(sorted(n - 1 - b for b in low_bits))
    rng = numpy.random.default_rng(11)
    gl = []
    for _ in range(6):
        for q in low_qubits:
            gl.append({q: circuits.haar_2x2(rng)})
        for a, b in zip(low_qubits[:-1], low_qubits[1:]):
            gl.append({(a, b): numpy.diag([1, 1, 1, -1]).astype(complex)})
    ops = [op for g in gl for op in gates.decompose(g)]
    steps = fusion.plan(ops, kmax=6) + gates.decompose({(0, 1): numpy.diag([1, 1, 1, -1]).astype(complex)})
    wide = fusion.widen_blocks(steps, n)
    assert fusion.widen_blocks(wide, n) == wide           # idempotent
    blocks = [s for s in wide if isinstance(s, fusion.Block)]
    extra = [q for q in range(n) if q not in low_qubits][:6 - len(low_qubits)]
    assert blocks and blocks[0].qubits == tuple(sorted(tuple(low_qubits) + tuple(extra)))
    assert len(wide) == len(steps) and wide[-1] is steps[-1]
    v = numpy.random.default_rng(3).standard_normal(2 ** n) + 0j
    want = got = v
    for a, b in zip(steps, wide):
        for x, st in ((0, a), (1, b)):
            if isinstance(st, fusion.Block):
                r = sv.apply_on(want if x == 0 else got, n, st.qubits, st.matrix)
            else:
                order, m = st.matrix()
                r = sv.apply_on(want if x == 0 else got, n, order, m)
            if x == 0:
                want = r
            else:
                got = r
    numpy.testing.assert_allclose(got, want, atol=1e-12)


def test_fusion_keeps_wide_gates_standalone():
    n = 12
    ops = [op for g in circuits.grover_gates(n, 1, seed=5)[0] for op in gates.decompose(g)]
    steps = fusion.plan(ops, kmax=6)
    wide = [s for s in steps if not isinstance(s, fusion.Block) and s.width > 6]
    assert len(wide) == 2  # the two (n-1)-controlled Z gates


def test_incremental_plan_equals_full_plan():
    n = 14
    gl = circuits.brickwork(n, 10, seed=4) + circuits.grover_gates(n, 1, seed=2)[0] + circuits.brickwork(n, 3, seed=5)
    ops = [op for g in gl for op in gates.decompose(g)]
    full = fusion.plan(ops, kmax=6, beam=(1, 1))
    got, pending = [], []
    for i, op in enumerate(ops):
        pending.append(op)
        if len(pending) >= 50 and i % 7 == 0:
            steps, pending = fusion.plan_prefix(pending, kmax=6, nqubits=n, beam=(1, 1))
            got.extend(steps)
    got.extend(fusion.plan(pending, kmax=6, beam=(1, 1)))
    assert len(got) == len(full)
    for a, b in zip(got, full):
        assert type(a) is type(b)
        if isinstance(a, fusion.Block):
            assert a.qubits == b.qubits and a.ngates == b.ngates
            numpy.testing.assert_allclose(a.matrix, b.matrix, atol=1e-13)
        else:
            assert a is b


def _synthetic_tuner(cost):
    from qip_gb300.autotune import MODES, Autotuner

    t = Autotuner()
    for k in (4, 5, 6):
        for low in range(128):
            if bin(low).count("1") <= k:
                ms = cost(k, low)
                t._ms[(20, k, low)] = ([ms, ms * 1.5] + [-1.0] * (len(MODES) - 2), 0)
    return t


def test_autotuner_prices_plans_and_picks_the_cheapest_width():
    from qip_gb300.autotune import placement_class

    n = 20
    assert placement_class((19, 18, 0), n) == (3, 0b11)
    assert placement_class((0, 1, 2, 3), n) == (4, 0)
    ops = [op for g in circuits.brickwork(n, 8, seed=3) for op in gates.decompose(g)]
    # Every pass costs the same: the widest blocks (fewest passes) win.
    t = _synthetic_tuner(lambda k, low: 1.0)
    w, steps, report = t.choose_width(None, n, ops)
    assert w == 6 and set(report) == {4, 5, 6} and report[6] == min(report.values())
    assert report[6] == pytest.approx(sum(1.0 if isinstance(s, fusion.Block) else s.amp_update_weight()
                                          for s in steps))
    # Wide blocks made expensive: a narrower width wins and is remembered for n.
    t = _synthetic_tuner(lambda k, low: 1.0 if k == 4 else 50.0)
    w, _, report = t.choose_width(None, n, ops)
    assert w == 4 and t.width_for(n) == 4
    # Times measured on 26 qubits scale to larger states.
    t._ms[(26, 6, 0)] = ([2.0, 3.0, -1.0], 0)
    assert t.block_ms(30, 6, 0) == pytest.approx(32.0)


def test_autotuner_cache_round_trip(tmp_path):
    from qip_gb300.autotune import Autotuner

    path = str(tmp_path / "tune.json")
    n = 20
    ops = [op for g in circuits.brickwork(n, 6, seed=4) for op in gates.decompose(g)]
    t = _synthetic_tuner(lambda k, low: 1.0 + 0.1 * bin(low).count("1"))
    t.cache_path = path
    w, steps, report = t.choose_width(None, n, ops)
    t2 = Autotuner(cache_path=path)
    assert t2.width_for(n) == w and t2._ms == t._ms
    assert sorted(t2._unpinned) == sorted((k, low, best) for (_, k, low), (_, best) in t._ms.items())
    # A loaded decision is reused without pricing the other widths again.
    t2._unpinned = []
    w2, steps2, report2 = t2.choose_width(None, n, ops)
    assert w2 == w and report2 == report and len(steps2) == len(steps)


def _same_steps(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert type(x) is type(y)
        if isinstance(x, fusion.Block):
            assert x.qubits == y.qubits and x.ngates == y.ngates
            numpy.testing.assert_allclose(x.matrix, y.matrix, atol=1e-12)
        else:
            assert x is y


@pytest.mark.parametrize("kmax", [3, 4, 6])
def test_native_planner_matches_python_reference(kmax):
    """qsv_fusion_plan / qsv_block_matrices (the library, loadable without a GPU) give
    the Python planner's steps and matrices: whole lists and both prefix modes."""
    rng = numpy.random.default_rng(kmax)
    n = 12
    lists = [circuits.brickwork(n, 8, seed=7) + circuits.grover_gates(n, 1, seed=3)[0],
             circuits.random_circuit(rng, n, 200), circuits.qft_gates(n)]
    for gl in lists:
        ops = [op for g in gl for op in gates.decompose(g)]
        for beam in ((1, 1), (4, 4), fusion.BEAM):   # rounds only, streaming beam, full beam
            _same_steps(fusion.plan(ops, kmax=kmax, beam=beam), fusion.plan_py(ops, kmax=kmax, beam=beam))
            for cut in (40, 120):
                for strict, keep in ((True, 0), (False, 0), (False, 30)):
                    s1, r1 = fusion.plan_prefix(ops[:cut], kmax=kmax, nqubits=n, strict=strict, min_pending=keep,
                                                beam=beam)
                    s2, r2 = fusion.plan_prefix_py(ops[:cut], kmax=kmax, nqubits=n, strict=strict,
                                                   min_pending=keep, beam=beam)
                    _same_steps(s1, s2)
                    assert all(x is y for x, y in zip(r1, r2)) and len(r1) == len(r2)


def test_beam_plan_preserves_the_circuit_and_saves_blocks():
    """The beam plan is a valid reordering (same state as the gate list) and never
    uses more steps than rounds alone on the brickwork benchmark family."""
    n = 14
    gl = circuits.brickwork(n, 16, seed=9)
    ops = [op for g in gl for op in gates.decompose(g)]
    beam = fusion.plan(ops, kmax=6)
    rounds = fusion.plan(ops, kmax=6, beam=(1, 1))
    assert len(beam) <= len(rounds)
    v = numpy.random.default_rng(2).standard_normal(2 ** n) + 0j
    want = v
    for g in gl:
        want = sv.kronselect_dot(g, want, n)
    got = v
    for st in beam:
        if isinstance(st, fusion.Block):
            got = sv.apply_on(got, n, st.qubits, st.matrix)
        else:
            order, m = st.matrix()
            got = sv.apply_on(got, n, order, m)
    numpy.testing.assert_allclose(got, want, atol=1e-11)


def test_injected_allocation_failure_raises_memory_error(monkeypatch):
    """Host-side fault injection: the state allocation fails before any device call (so
    this runs without a GPU) and surfaces as the reference's MemoryError."""
    from qip_gb300 import GpuBackend

    monkeypatch.setenv("QSV_INJECT_ALLOC_FAILURE", "1")
    with pytest.raises(MemoryError, match="injected"):
        GpuBackend.make_state(12, [], [], statetype=numpy.complex64)


def test_trace_ranges_are_callable_without_a_profiler():
    from qip_gb300 import _native as nat

    lib = nat.load()
    assert lib.qsv_trace_push(b"node") == 0 and lib.qsv_trace_pop() == 0


def test_decompose_cache_follows_matrix_content():
    """Decompositions are cached by content: a matrix edited in place after a call is
    decomposed again, the cached ops never alias the caller's arrays, and every call
    returns its own op objects."""
    u = numpy.array([[0.6, 0.8], [0.8, -0.6]], dtype=numpy.complex128)
    a = gates.decompose({3: u})
    b = gates.decompose({3: u})
    assert a[0] is not b[0] and a[0].kind == b[0].kind == "dense"
    assert not numpy.shares_memory(a[0].mat, u)
    u[:] = numpy.diag([1.0, -1.0])
    c = gates.decompose({3: u})
    assert c[0].kind == "diag"
    numpy.testing.assert_array_equal(a[0].mat, [[0.6, 0.8], [0.8, -0.6]])
    d = gates.decompose({(0, 1): CMat(numpy.array([[0, 1], [1, 0]]))})
    assert d[0].kind == "mono" and d[0].controls == (0,) and d[0].targets == (1,)


def test_autotuner_widens_small_blocks_only_where_measured_faster():
    """Autotuner.place: a 4- or 5-qubit block becomes its 6-qubit form (identity on the
    added qubits) when the 6-qubit class measured no slower than its own, else it stays;
    other steps pass through untouched."""
    n = 20
    rng = numpy.random.default_rng(12)
    u4 = numpy.linalg.qr(rng.standard_normal((16, 16)) + 1j * rng.standard_normal((16, 16)))[0]
    small = fusion.Block((3, 7, 9, 12), u4, 5, 5.0)
    op = gates.decompose({(1,): numpy.array([[0, 1], [1, 0]])})[0]
    fast6 = _synthetic_tuner(lambda k, low: 1.0 if k == 6 else 2.0)
    out = fast6.place(None, n, [small, op])
    assert len(out[0].qubits) == 6 and set(small.qubits) <= set(out[0].qubits) and out[1] is op
    v = rng.standard_normal(2 ** n) + 0j
    numpy.testing.assert_allclose(sv.apply_on(v, n, out[0].qubits, out[0].matrix),
                                  sv.apply_on(v, n, small.qubits, small.matrix), atol=1e-12)
    slow6 = _synthetic_tuner(lambda k, low: 3.0 if k == 6 else 1.0)
    out = slow6.place(None, n, [small, op])
    assert out[0] is small and out[1] is op


def test_native_block_matrices_match_numpy_for_every_gate_kind():
    """qsv_block_matrices (diagonal and one-qubit fast paths, general gather loop) against
    numpy products of the same gates, for blocks of 2..7 qubits."""
    rng = numpy.random.default_rng(17)
    n = 9

    def unitary(k):
        z = rng.standard_normal((2 ** k, 2 ** k)) + 1j * rng.standard_normal((2 ** k, 2 ** k))
        return numpy.linalg.qr(z)[0]

    def rand_gate():
        kind = rng.integers(6)
        qs = [int(x) for x in rng.choice(n, size=3, replace=False)]
        if kind == 0:
            return {(qs[0],): unitary(1)}
        if kind == 1:
            return {(qs[0],): numpy.diag(numpy.exp(1j * rng.uniform(0, 6, 2)))}
        if kind == 2:
            return {(qs[0], qs[1]): CMat(numpy.diag([1, -1.0]))}
        if kind == 3:
            return {tuple(qs[:2]): unitary(2)}
        if kind == 4:
            return {tuple(qs): CMat(SwapMat(1))}
        return {tuple(qs): unitary(3)}

    ops = [op for _ in range(400) for op in gates.decompose(rand_gate())]
    groups, cur, cur_q = [], [], set()
    for op in ops:
        kmax = int(rng.integers(2, 8))
        if cur and len(cur_q | set(op.qubits)) > kmax:
            groups.append(cur)
            cur, cur_q = [], set()
        cur.append(op)
        cur_q |= set(op.qubits)
    groups.append(cur)
    groups = [g for g in groups if len(g) > 1]
    assert len(groups) > 50
    steps = fusion.emit_native(groups)
    for grp, st in zip(groups, steps):
        qs, want = fusion.block_matrix(grp)
        assert st.qubits == qs
        numpy.testing.assert_allclose(st.matrix, want, rtol=0, atol=1e-13)
