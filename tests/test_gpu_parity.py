"""GPU parity: libqsv through its C ABI (via GpuBackend) against the reference's own
outputs (golden vectors) and the FP64 oracle.

Tolerances: complex128 1e-12 absolute (amplitudes and probabilities), complex64
per-gate 1e-6, complex64 fused tensor-core blocks 2e-5 on amplitudes / 1e-6 on
probabilities at these sizes; permutations (SwapMat, X, CNOT, func_apply) bit-exact.
"""
import types

import numpy
import pytest

import qip_gb300 as api_mod
import statevector as sv
from conftest import load_npz
from make_golden import decode
from qip_gb300 import GpuBackend, circuits, gates
from qip_gb300.operators import CMat, SwapMat
from scenarios import SCENARIOS

pytestmark = pytest.mark.gpu

C128, C64 = numpy.complex128, numpy.complex64


def fresh(n, vec=None, statetype=C128, fusion=None):
    if vec is None:
        return GpuBackend.make_state(n, [], [], statetype=statetype, fusion=fusion)
    return GpuBackend.make_state(n, [list(range(n))], [vec], statetype=statetype, fusion=fusion)


def is_permutation(mats):
    for m in mats.values():
        while getattr(m, "_kron_struct", None) == 2:
            m = m.m
        if getattr(m, "_kron_struct", None) == 3:
            continue
        a = numpy.asarray(m)
        if not (numpy.all((a == 0) | (a == 1)) and numpy.all((a != 0).sum(0) == 1)):
            return False
    return True


@pytest.mark.parametrize("statetype,atol", [(C128, 1e-12), (C64, 1e-6)])
def test_kron_cases_match_reference(statetype, atol):
    d, cases = load_npz("kron_cases.npz")
    for c in cases:
        mats = decode(c["mats"], d, CMat, SwapMat)
        st = fresh(c["n"], d[f"k{c['id']}_in"], statetype=statetype, fusion=False)
        st.kronselect_dot(mats)
        got = st.get_state()
        st.close()
        want = d[f"k{c['id']}_out"]
        if is_permutation(mats):
            inp = d[f"k{c['id']}_in"].astype(statetype)
            assert numpy.array_equal(got, want.astype(statetype)), c
            assert sorted(got.tolist(), key=lambda z: (z.real, z.imag)) == \
                sorted(inp.tolist(), key=lambda z: (z.real, z.imag))
        else:
            numpy.testing.assert_allclose(got, want, rtol=0, atol=atol, err_msg=str(c))


def test_kron_mixed_dictionaries_match_oracle():
    rng = numpy.random.default_rng(8)
    n = 7
    for _ in range(10):
        a, b, c, e = (int(x) for x in rng.choice(n, 4, replace=False))
        u2 = numpy.linalg.qr(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)))[0]
        u1 = numpy.linalg.qr(rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2)))[0]
        for mats in ({(a, b): u2, (c,): u1}, {(a, b): CMat(u1), (c, e): SwapMat(1)},
                     {(a, b): u2, (b, c): u2}):
            v = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
            st = fresh(n, v)
            st.kronselect_dot(mats)
            numpy.testing.assert_allclose(st.get_state(), sv.kronselect_dot(mats, v, n), atol=1e-12)
            st.close()


@pytest.mark.parametrize("statetype,atol", [(C128, 1e-12), (C64, 1e-6)])
def test_measurement_matches_reference(statetype, atol):
    d, cases = load_npz("measure_cases.npz")
    for c in cases:
        n, idx, m, p = c["n"], c["idx"], c["m"], c["p"]
        vec = d[f"c{c['id']}_vec"]
        st = fresh(n, vec, statetype=statetype)
        numpy.testing.assert_allclose(st.measure_probabilities(numpy.array(idx, dtype=numpy.int32)),
                                      d[f"c{c['id']}_probs"], atol=atol)
        tm, tp = st.measure_probabilities(idx, top_k=2 ** len(idx))
        numpy.testing.assert_allclose(tp, d[f"c{c['id']}_topp"], atol=atol)
        refp, refm = d[f"c{c['id']}_topp"], d[f"c{c['id']}_topm"]
        for j in range(len(tm)):
            if numpy.sum(numpy.abs(refp - refp[j]) < 1e-5) == 1:
                assert int(tm[j]) == int(refm[j])
        sm, sp = st.soft_measure(idx, measured=m)
        assert sm == c["soft"][0] and abs(sp - c["soft"][1]) < atol
        assert abs(st.total_prob() - float(numpy.sum(numpy.abs(vec) ** 2))) < atol
        mm, pp = st.measure(idx, measured=m, measured_prob=p)
        assert (mm, pp) == (m, p)
        numpy.testing.assert_allclose(st.get_state(), d[f"c{c['id']}_collapse"], atol=atol * 10)
        st.close()
        st = fresh(n, vec, statetype=statetype)
        st.reduce_measure(idx, measured=m, measured_prob=p)
        assert st.n == n - len(idx)
        numpy.testing.assert_allclose(st.get_state(), d[f"c{c['id']}_reduce"], atol=atol * 10)
        st.close()


def test_measure_samples_and_collapses_consistently():
    rng = numpy.random.default_rng(1)
    n = 9
    for _ in range(20):
        v = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
        v /= numpy.linalg.norm(v)
        idx = [int(x) for x in rng.choice(n, 3, replace=False)]
        st = fresh(n, v)
        m, p = st.measure(idx)
        pm = sv.probs_msb(idx, n, v)
        assert abs(p - pm[m]) < 1e-12 and p > 0
        numpy.testing.assert_allclose(st.get_state(), sv.collapse(idx, n, v, m, p), atol=1e-12)
        assert abs(st.total_prob() - 1.0) < 1e-12
        st.close()


def test_measure_argument_errors():
    st = fresh(3)
    with pytest.raises(ValueError):
        st.measure([0, 1], measured=4)
    with pytest.raises(ValueError):
        st.measure([0], measured=0, measured_prob=0.0)
    with pytest.raises(ValueError):
        st.kronselect_dot({(5,): numpy.eye(2) * 1j})
    with pytest.raises(ValueError):
        st.kronselect_dot({(0, 0): numpy.eye(4) * 1j})
    st.close()


def test_func_apply_matches_reference_bit_exact():
    d, cases = load_npz("func_cases.npz")
    for c in cases:
        t = c["table"]
        for statetype in (C128, C64):
            st = fresh(c["n"], d[f"f{c['id']}_vec"], statetype=statetype)
            st.func_apply(c["reg1"], c["reg2"], lambda x: t[x])
            assert numpy.array_equal(st.get_state(), d[f"f{c['id']}_out"].astype(statetype))
            st.close()
    # A third register that is left alone (every value of it is permuted).
    rng = numpy.random.default_rng(2)
    n = 8
    v = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    st = fresh(n, v)
    st.func_apply([6, 1], [3, 0, 5], lambda x: 5 * x + 3)
    assert numpy.array_equal(st.get_state(), sv.func_apply([6, 1], [3, 0, 5], lambda x: 5 * x + 3, v, n))
    st.close()


def api_ns():
    return types.SimpleNamespace(**{k: getattr(api_mod, k) for k in api_mod.__all__})


@pytest.mark.parametrize("statetype,fusion,atol", [(C128, False, 1e-12), (C64, False, 1e-6), (C64, True, 2e-5)])
def test_scenarios_match_reference_runs(statetype, fusion, atol):
    d, meta = load_npz("scenarios.npz")
    api = api_ns()

    def ctor(n, groups, feeds, statetype=statetype):
        return GpuBackend.make_state(n, groups, feeds, statetype=statetype, fusion=fusion)

    for name, fn in SCENARIOS.items():
        for r, (outs, feed, measured) in enumerate(fn(api)):
            o, classic = api.run(*outs, feed=feed, backend_constructor=ctor, statetype=statetype)
            numpy.testing.assert_allclose(o, d[f"{name}_{r}_state"], rtol=0, atol=atol, err_msg=f"{name}[{r}]")
            for j, node in enumerate(measured):
                val = classic[node]
                pa = 1e-12 if statetype == C128 else 1e-6
                if meta[name][r]["measured"][j] == "topk":
                    numpy.testing.assert_allclose(val[1], d[f"{name}_{r}_m{j}_p"], atol=pa)
                else:
                    numpy.testing.assert_allclose(val, d[f"{name}_{r}_m{j}_p"], atol=pa)


def test_config1_qft_swaps_bit_exact():
    """The Swap steps of the n=16 QFT are pure permutations: applying them alone to the
    state before the swaps reproduces the reference bit for bit."""
    n = 16
    rng = numpy.random.default_rng(2024)
    x = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    x /= numpy.linalg.norm(x)
    gl = circuits.qft_gates(n)
    pre, swaps = gl[:-(n // 2)], gl[-(n // 2):]
    st = fresh(n, x)
    for g in pre:
        st.kronselect_dot(g)
    before = st.get_state()
    for g in swaps:
        st.kronselect_dot(g)
    after = st.get_state()
    st.close()
    want = before.copy()
    for g in swaps:
        want = sv.kronselect_dot(g, want, n)
    assert numpy.array_equal(after, want)


def _gpu_run(gl, n, statetype=C128, fusion=None, feeds=None):
    if feeds is None:
        st = GpuBackend.make_state(n, [], [], statetype=statetype, fusion=fusion)
    else:
        st = GpuBackend.make_state(n, [[q] for q in range(n)], feeds, statetype=statetype, fusion=fusion)
    for g in gl:
        st.kronselect_dot(g)
    out = st.get_state()
    st.close()
    return out


def test_workloads_match_reference():
    d = load_npz("workloads.npz")[0]
    for statetype, fusion, atol in ((C128, False, 1e-12), (C64, False, 1e-5), (C64, True, 2e-5)):
        numpy.testing.assert_allclose(_gpu_run(circuits.brickwork(10, 12, seed=11), 10, statetype, fusion),
                                      d["brickwork_n10"], atol=atol)
        gates_, marked = circuits.grover_gates(8, iterations=2, seed=3)
        numpy.testing.assert_allclose(_gpu_run(gates_, 8, statetype, fusion), d["grover_n8"], atol=atol)
        wrng = numpy.random.default_rng(99)
        for i in range(6):
            nn, depth = int(wrng.integers(4, 11)), int(wrng.integers(20, 61))
            gl = circuits.random_circuit(wrng, nn, depth)
            feeds = circuits.random_product_feed(wrng, nn)
            numpy.testing.assert_allclose(_gpu_run(gl, nn, statetype, fusion, feeds), d[f"random_{i}_state"],
                                          atol=atol)
        numpy.testing.assert_allclose(_gpu_run(circuits.ansatz_layers(6, 3, d["ansatz_n6_thetas"]), 6, statetype,
                                               fusion), d["ansatz_n6"], atol=atol)


def infidelity(a, b):
    a = numpy.asarray(a, dtype=numpy.complex128)
    b = numpy.asarray(b, dtype=numpy.complex128)
    return 1.0 - abs(numpy.vdot(a, b)) ** 2 / (numpy.vdot(a, a).real * numpy.vdot(b, b).real)


@pytest.mark.parametrize("k", [4, 5, 6])
def test_tensor_core_block_matches_oracle(k):
    """One fused block on every kind of target placement (low bits, high bits, mixed,
    unsorted) against the FP64 oracle."""
    rng = numpy.random.default_rng(k)
    n = 14
    placements = [list(range(k)), list(range(n - k, n)), [int(x) for x in rng.choice(n, k, replace=False)],
                  [int(x) for x in rng.choice(n, k, replace=False)][::-1]]
    for tg in placements:
        u = numpy.linalg.qr(rng.standard_normal((2 ** k, 2 ** k)) + 1j * rng.standard_normal((2 ** k, 2 ** k)))[0]
        v = (rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)) / numpy.sqrt(2 ** (n + 1))
        st = fresh(n, v, statetype=C64)
        from qip_gb300.fusion import Block

        st.apply_blocks([Block(tuple(tg), u, 1, 1.0)])
        got = st.get_state()
        st.close()
        want = sv.apply_on(v, n, tg, u)
        err = numpy.max(numpy.abs(got - want)) / numpy.max(numpy.abs(want))
        assert err < 5e-5, (tg, err)
        assert infidelity(got, want) < 1e-8


BLOCK_PLACEMENTS = [  # target bit positions below bit 7 (the rest sit at the top bits)
    (6, ()), (6, (5, 6)), (6, (0,)), (6, (0, 1)),  # direct
    (6, (0, 1, 2, 3, 4, 5)), (6, (0, 1, 2, 3)),  # prefix (transposed products; a prefix of 4 or more)
    (6, (4,)), (6, (3, 4)), (6, (1, 2)), (6, (0, 2)), (6, (4, 5, 6)), (6, (1, 2, 3, 4)),  # shuffle
    (6, (0, 1, 4, 5, 6)), (6, (2, 3, 4, 5, 6)), (5, (1, 3)), (5, (0, 2, 3, 4)), (4, (2, 3, 4)),
    (4, (1, 2, 3, 4)), (4, (0, 2, 3, 4)),  # staged (all four targets below bit 5, not a prefix)
]


@pytest.mark.parametrize("k,low", BLOCK_PLACEMENTS)
def test_tensor_core_block_modes_match_oracle(k, low):
    """Each access mode of the tensor-core block kernel (direct, shuffle, staged, prefix), with
    the block's qubits in ascending, descending and shuffled matrix order."""
    n = 15
    rng = numpy.random.default_rng(100 * k + len(low))
    bits = list(low) + [n - 1 - i for i in range(k - len(low))]
    from qip_gb300.fusion import Block

    for order in ("asc", "desc", "shuffled"):
        qubits = [n - 1 - b for b in bits]
        if order == "asc":
            qubits.sort()
        elif order == "desc":
            qubits.sort(reverse=True)
        else:
            rng.shuffle(qubits)
        u = numpy.linalg.qr(rng.standard_normal((2 ** k, 2 ** k)) + 1j * rng.standard_normal((2 ** k, 2 ** k)))[0]
        v = (rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)) / numpy.sqrt(2 ** (n + 1))
        st = fresh(n, v, statetype=C64)
        st.apply_blocks([Block(tuple(qubits), u, 1, 1.0)])
        got = st.get_state()
        st.close()
        want = sv.apply_on(v, n, qubits, u)
        err = numpy.max(numpy.abs(got - want)) / numpy.max(numpy.abs(want))
        assert err < 5e-5, (qubits, err)
        assert infidelity(got, want) < 1e-8


@pytest.mark.parametrize("statetype,atol", [(C64, 2e-6), (C128, 1e-12)])
def test_per_gate_low_bit_targets_match_oracle(statetype, atol):
    """Dense gates whose targets include address bits 0/1 (vector accesses for
    complex64) in every target order, with and without controls, and single-qubit and
    register swaps, against the oracle."""
    from qip_gb300.gates import GateOp

    n = 10
    rng = numpy.random.default_rng(31)
    q = lambda bit: n - 1 - bit  # noqa: E731
    cases = []
    for bits in ([0], [1], [0, 1], [1, 0], [0, 5], [5, 0], [1, 0, 4], [0, 4, 1], [4, 1, 0], [0, 2], [2, 1, 0]):
        for ctrl in ([], [7], [3, 8]):
            k = len(bits)
            u = numpy.linalg.qr(rng.standard_normal((2 ** k, 2 ** k)) + 1j * rng.standard_normal((2 ** k, 2 ** k)))[0]
            cases.append(GateOp("dense", tuple(q(b) for b in bits), tuple(q(c) for c in ctrl), u))
    for a, b, ctrl in ((0, 1, []), (1, 0, []), (0, 6, [2]), (7, 3, [0, 9]), (9, 0, [])):
        cases.append(GateOp("swap", (q(a),), tuple(q(c) for c in ctrl), swap_b=(q(b),)))
    cases.append(GateOp("swap", (q(0), q(3)), (q(6),), swap_b=(q(1), q(8))))
    for bits, ctrl in (([0], []), ([1, 0], [5]), ([4], [0, 1])):
        d = numpy.exp(1j * rng.uniform(0, 6.28, 2 ** len(bits)))
        d[0] = 1.0
        cases.append(GateOp("diag", tuple(q(b) for b in bits), tuple(q(c) for c in ctrl), d))
    for op in cases:
        v = (rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)) / numpy.sqrt(2 ** (n + 1))
        st = fresh(n, v, statetype=statetype, fusion=False)
        st.apply_op(op)
        got = st.get_state()
        st.close()
        order, m = op.matrix()
        want = sv.apply_on(v.astype(statetype).astype(complex), n, order, m)
        if op.kind == "swap":
            assert numpy.array_equal(got, want.astype(statetype)), op
        else:
            numpy.testing.assert_allclose(got, want, rtol=0, atol=atol, err_msg=str(op))


def test_fused_brickwork_infidelity_n20():
    n, depth = 20, 12
    gl = circuits.brickwork(n, depth, seed=3)
    ref = _gpu_run(gl, n, C128, False)
    fused = _gpu_run(gl, n, C64, True)
    plain = _gpu_run(gl, n, C64, False)
    assert infidelity(fused, ref) < 1e-6
    assert infidelity(plain, ref) < 1e-6
    # The FP64 path against the oracle (independent check of the plain kernels).
    v = numpy.zeros(2 ** n, dtype=complex)
    v[0] = 1
    for g in gl[: 3 * n]:
        v = sv.kronselect_dot(g, v, n)
    part = _gpu_run(gl[: 3 * n], n, C128, False)
    numpy.testing.assert_allclose(part, v, atol=1e-12)


def test_qubit_marginals_match_oracle():
    rng = numpy.random.default_rng(6)
    for n in (9, 16, 20):
        v = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
        v /= numpy.linalg.norm(v)
        for statetype, atol in ((C128, 1e-12), (C64, 1e-6)):
            st = fresh(n, v, statetype=statetype)
            marg, nrm = st.qubit_marginals()
            want = numpy.array([sv.measure_probabilities([q], n, v)[1] for q in range(n)])
            numpy.testing.assert_allclose(marg, want, atol=atol)
            assert abs(nrm - 1.0) < atol
            st.close()


def test_product_state_feeds():
    rng = numpy.random.default_rng(4)
    n = 10
    groups = [[3, 0], [7], [9, 5, 1]]
    feeds = [rng.standard_normal(4) + 1j * rng.standard_normal(4), [0.6, 0.8],
             rng.standard_normal(8)]
    st = GpuBackend.make_state(n, groups, feeds)
    numpy.testing.assert_allclose(st.get_state(), sv.make_state(n, groups, feeds), atol=1e-15)
    st.close()
    st = GpuBackend.make_state(4, [[0, 1, 2, 3]], [5])  # basis-index feed
    want = numpy.zeros(16)
    want[5] = 1
    assert numpy.array_equal(st.get_state(), want)
    st.close()


def test_ranges_and_reset():
    n = 6
    v = numpy.arange(2 ** n) + 1j
    st = fresh(n, v)
    numpy.testing.assert_array_equal(st.get_relative_range(8, 20), v[8:20])
    st.overwrite_relative_range(0, 4, [9, 9, 9, 9])
    st.addto_relative_range(4, 8, [1, 1, 1, 1])
    want = v.copy()
    want[0:4] = 9
    want[4:8] += 1
    numpy.testing.assert_array_equal(st.get_state(), want)
    assert st.get_state_size() == 2 ** n
    st.close()


def test_make_circuit_mat_is_the_unitary():
    q = api_mod.Qubit(n=3)
    out = api_mod.QFFT(q)
    m = api_mod.make_circuit_mat(out)
    x = numpy.eye(8)
    want = numpy.stack([numpy.fft.ifft(x[:, i], norm="ortho") for i in range(8)], axis=1)
    numpy.testing.assert_allclose(m, want, atol=1e-12)


@pytest.mark.parametrize("low_bits", [(4, 3, 2, 1), (4, 3, 2, 1, 0)])
def test_widened_low_blocks_through_the_backend(low_bits):
    """Gates on address bits 0..4 only: the fused backend widens their block by one
    identity qubit (shuffle access instead of staged); the state matches the oracle."""
    n = 16
    qs = [n - 1 - b for b in low_bits]
    rng = numpy.random.default_rng(len(low_bits))
    gl = []
    for _ in range(5):
        gl += [{q: circuits.haar_2x2(rng)} for q in qs]
        gl += [{(a, b): numpy.diag([1, 1, 1, -1]).astype(complex)} for a, b in zip(qs[:-1], qs[1:])]
    v = (rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)) / numpy.sqrt(2 ** (n + 1))
    st = fresh(n, v, statetype=C64, fusion=True)
    for g in gl:
        st.kronselect_dot(g)
    got = st.get_state()
    assert st.stats["blocks"] == 1 and st.stats["ops"] == 0
    st.close()
    want = v.astype(complex)
    for g in gl:
        want = sv.kronselect_dot(g, want, n)
    err = numpy.max(numpy.abs(got - want)) / numpy.max(numpy.abs(want))
    assert err < 5e-5, err
    assert infidelity(got, want) < 1e-8
