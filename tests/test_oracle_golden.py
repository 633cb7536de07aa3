"""The oracle pinned against golden vectors produced by the reference's own kernels
(tests/golden/make_golden.py) and against the reference unit tests' known answers."""
import numpy
import pytest

import statevector as sv
from conftest import load_npz
from make_golden import decode
from qip_gb300 import circuits
from qip_gb300.operators import CMat, SwapMat


def test_oracle_kron_matches_reference_cdot_loop():
    d, cases = load_npz("kron_cases.npz")
    assert len(cases) > 100
    for c in cases:
        mats = decode(c["mats"], d, CMat, SwapMat)
        got = sv.kronselect_dot(mats, d[f"k{c['id']}_in"], c["n"])
        numpy.testing.assert_allclose(got, d[f"k{c['id']}_out"], rtol=0, atol=1e-12, err_msg=str(c))


def test_oracle_kron_reference_unit_test_answers():
    # tests/utiltest.py:9-66 of the reference: kron against numpy.kron, per basis column.
    i2 = numpy.eye(2)
    for a, b in ((numpy.array([[1, 1], [1, -1]]), numpy.array([[1, 1], [1, -1]])),
                 (numpy.array([[1, 2], [3, 4]]), numpy.array([[5, 6], [7, 8]]))):
        ref = numpy.kron(a, numpy.kron(i2, b))
        for col in range(8):
            v = numpy.zeros(8, dtype=complex)
            v[col] = 1
            for mats in ({0: a, 2: b}, {(0, 2): numpy.kron(a, b)}, {(2, 0): numpy.kron(b, a)}):
                assert numpy.array_equal(sv.kronselect_dot(mats, v, 3), ref[:, col])


def test_oracle_kron_windows():
    # Output/input offset windows (tests/utiltest.py:68-125).
    h = numpy.array([[1, 1], [1, -1]])
    ref = numpy.kron(h, numpy.kron(numpy.eye(2), h))
    for col in range(8):
        v = numpy.zeros(8, dtype=complex)
        v[col] = 1
        for off in range(4):
            out = sv.kronselect_dot_window({0: h, 2: h}, v, 3, 4, output_offset=off)
            assert numpy.array_equal(out, ref[off:off + 4, col])
        acc = numpy.zeros(8, dtype=complex)
        for off in range(0, 8, 2):
            acc = acc + sv.kronselect_dot_window({(0, 2): numpy.kron(h, h)}, v[off:off + 2], 3, 8, input_offset=off)
        assert numpy.array_equal(acc, ref[:, col])


def test_oracle_measurement_matches_reference():
    d, cases = load_npz("measure_cases.npz")
    for c in cases:
        n, idx, m, p = c["n"], c["idx"], c["m"], c["p"]
        vec = d[f"c{c['id']}_vec"]
        numpy.testing.assert_allclose(sv.measure_probabilities(idx, n, vec), d[f"c{c['id']}_probs"], atol=1e-14)
        tm, tp = sv.measure_top_probabilities(idx, n, 2 ** len(idx), vec)
        numpy.testing.assert_allclose(tp, d[f"c{c['id']}_topp"], atol=1e-14)
        # Outcome indices agree wherever probabilities are distinct.
        refm = d[f"c{c['id']}_topm"]
        refp = d[f"c{c['id']}_topp"]
        for j in range(len(tm)):
            if numpy.sum(numpy.abs(refp - refp[j]) < 1e-15) == 1:
                assert tm[j] == refm[j]
        sm, sp = sv.soft_measure(idx, n, vec, measured=m, r=0.3)
        assert sm == c["soft"][0]
        assert abs(sp - c["soft"][1]) < 1e-14
        numpy.testing.assert_allclose(sv.collapse(idx, n, vec, m, p), d[f"c{c['id']}_collapse"], atol=1e-14)
        numpy.testing.assert_allclose(sv.reduce_measure(idx, n, vec, m, p), d[f"c{c['id']}_reduce"], atol=1e-14)


def test_oracle_known_measure_answers():
    # tests/qiptest.py:296-315 and a known-answer state [.1, .2, .3, sqrt(.86)].
    v = numpy.array([0.1, 0.2, 0.3, numpy.sqrt(0.86)])
    numpy.testing.assert_allclose(sv.measure_probabilities([0, 1], 2, v), [0.01, 0.09, 0.04, 0.86])
    m, p = sv.measure_top_probabilities([0, 1], 2, 4, v)
    assert m == [3, 2, 1, 0]
    numpy.testing.assert_allclose(p, [0.86, 0.09, 0.04, 0.01])


def test_oracle_func_apply_matches_reference():
    d, cases = load_npz("func_cases.npz")
    for c in cases:
        t = c["table"]
        got = sv.func_apply(c["reg1"], c["reg2"], lambda x: t[x], d[f"f{c['id']}_vec"], c["n"])
        numpy.testing.assert_array_equal(got, d[f"f{c['id']}_out"])


def test_oracle_func_apply_reference_unit_test():
    # tests/utiltest.py:127-153.
    state = numpy.zeros(16, dtype=complex)
    state[0], state[8], state[4], state[12] = 1, 2, 3, 4
    out = sv.func_apply([0, 1], [2, 3], lambda x: (x + 1) % 4, state, 4)
    assert out[1] == 1 and out[11] == 2 and out[6] == 3 and out[12] == 4


def _run_gates(gates, n, vec):
    for g in gates:
        vec = sv.kronselect_dot(g, vec, n)
    return vec


def test_oracle_workloads_match_reference():
    d = load_npz("workloads.npz")[0]
    v0 = numpy.zeros(2 ** 10, dtype=complex)
    v0[0] = 1
    numpy.testing.assert_allclose(_run_gates(circuits.brickwork(10, 12, seed=11), 10, v0), d["brickwork_n10"],
                                  atol=1e-12)
    gates, marked = circuits.grover_gates(8, iterations=2, seed=3)
    assert marked == int(d["grover_n8_marked"])
    v0 = numpy.zeros(2 ** 8, dtype=complex)
    v0[0] = 1
    numpy.testing.assert_allclose(_run_gates(gates, 8, v0), d["grover_n8"], atol=1e-12)
    wrng = numpy.random.default_rng(99)
    for i in range(6):
        nn, depth = int(wrng.integers(4, 11)), int(wrng.integers(20, 61))
        assert [nn, depth] == list(d[f"random_{i}_shape"])
        gl = circuits.random_circuit(wrng, nn, depth)
        feeds = circuits.random_product_feed(wrng, nn)
        st = sv.make_state(nn, [[q] for q in range(nn)], feeds)
        numpy.testing.assert_allclose(_run_gates(gl, nn, st), d[f"random_{i}_state"], atol=1e-12)
    v0 = numpy.zeros(2 ** 6, dtype=complex)
    v0[0] = 1
    numpy.testing.assert_allclose(_run_gates(circuits.ansatz_layers(6, 3, d["ansatz_n6_thetas"]), 6, v0),
                                  d["ansatz_n6"], atol=1e-12)


def test_oracle_qft_is_inverse_dft():
    # Known answer: QFFT(rev=True) of the reference equals numpy.fft.ifft(x, norm="ortho").
    rng = numpy.random.default_rng(3)
    n = 7
    x = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    x /= numpy.linalg.norm(x)
    numpy.testing.assert_allclose(_run_gates(circuits.qft_gates(n), n, x), numpy.fft.ifft(x, norm="ortho"),
                                  atol=1e-13)


def test_entwine_bit_is_ordered_deposit():
    for n in range(1, 7):
        for mask in range(2 ** n):
            k = bin(mask).count("1")
            for m in range(2 ** k):
                for j in range(0, 2 ** (n - k), max(1, 2 ** (n - k) // 4)):
                    e = sv.entwine_bit(k, n - k, m, j, mask)
                    mpos = [p for p in range(n) if (mask >> p) & 1]
                    npos = [p for p in range(n) if not (mask >> p) & 1]
                    want = 0
                    for b, p in enumerate(mpos):
                        want |= ((m >> b) & 1) << p
                    for b, p in enumerate(npos):
                        want |= ((j >> b) & 1) << p
                    assert e == want
