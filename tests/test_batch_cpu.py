"""Batched-circuit host encoding on CPU: the gate records, interpreted with numpy,
reproduce the oracle's result for random circuits (checks the record semantics the
persistent kernel implements)."""
import numpy

import statevector as sv
from qip_gb300 import batch, circuits


def interpret(recs, n, state):
    v = state.astype(numpy.complex128).copy()
    for r in recs:
        m = r["m"][0::2].astype(numpy.float64) + 1j * r["m"][1::2].astype(numpy.float64)
        k = int(r["kind"])
        if k == batch.DENSE1:
            v = sv.apply_on(v, n, [int(r["q0"])], m.reshape(2, 2))
        elif k == batch.PHASE1:
            v = sv.apply_on(v, n, [int(r["q0"])], numpy.diag([1, m[0]]))
        elif k == batch.X:
            v = sv.apply_on(v, n, [int(r["q0"])], numpy.array([[0, 1], [1, 0]]))
        elif k == batch.CX:
            cx = numpy.eye(4)[[0, 1, 3, 2]]
            v = sv.apply_on(v, n, [int(r["q1"]), int(r["q0"])], cx)
        elif k == batch.CSWAP:
            cs = numpy.eye(8)[[0, 1, 2, 3, 4, 6, 5, 7]]
            v = sv.apply_on(v, n, [int(r["q0"]), int(r["q1"]), int(r["q2"])], cs)
    return v


def test_gate_records_reproduce_the_circuit():
    circs, feeds, sizes = batch.random_batch(12, seed=3, nmin=3, nmax=9, dmin=10, dmax=40)
    for gl, f, n in zip(circs, feeds, sizes):
        st = sv.make_state(n, [[q] for q in range(n)], f)
        want = st
        for g in gl:
            want = sv.kronselect_dot(g, want, n)
        got = interpret(batch.encode_gates(gl), n, st)
        numpy.testing.assert_allclose(got, want, atol=1e-6)


def test_record_layouts_match_the_c_header():
    assert batch.GATE_DTYPE.itemsize == 48
    assert batch.CIRC_DTYPE.itemsize == 32
    assert [batch.CIRC_DTYPE.fields[k][1] for k in ("n", "ngates", "gate_offset", "state_offset", "feed_offset")] == \
        [0, 4, 8, 16, 24]
