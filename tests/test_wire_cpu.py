"""The wire format (``qip_gb300.wire``) against messages written by the reference's own
protobuf code (``tests/golden/wire_cases.npz``, made by ``make_wire_golden.py``): byte
for byte re-encoding, decoded operations applied with the oracle against the reference
backend's states, and the worker's replies."""
import numpy
import pytest

import statevector as sv
from conftest import load_npz
from qip_gb300 import wire
from qip_gb300.operators import CMat, SwapMat

SIZES = (4, 6, 8)


def _msgs(d, key):
    blob, off = bytes(d[key]), d[key + "_off"]
    return [blob[off[i]:off[i + 1]] for i in range(len(off) - 1)]


@pytest.fixture(scope="module")
def cases():
    return load_npz("wire_cases.npz")


@pytest.mark.parametrize("n", SIZES)
def test_reference_messages_reencode_byte_for_byte(cases, n):
    d, meta = cases
    p = "n{}_".format(n)
    setup = bytes(d[p + "setup"])
    assert wire.StateSetup.FromString(setup).SerializeToString() == setup
    for kind, cls in (("ops", wire.WorkerOperation), ("mops", wire.WorkerOperation), ("replies", wire.WorkerConfirm)):
        for raw in _msgs(d, p + kind):
            assert cls.FromString(raw).SerializeToString() == raw


@pytest.mark.parametrize("n", SIZES)
def test_decoded_operations_give_the_reference_state(cases, n):
    d, meta = cases
    p = "n{}_".format(n)
    setup = wire.StateSetup.FromString(bytes(d[p + "setup"]))
    assert setup.n == n
    groups = [wire.pbindices_to_indices(s.indices) for s in setup.states]
    feeds = []
    for g, s in zip(groups, setup.states):
        v = wire.get_state_value(s)
        feeds.append(v if isinstance(v, numpy.ndarray) else numpy.eye(2 ** len(g))[v])
    state = sv.make_state(n, groups, feeds)
    ops = _msgs(d, p + "ops")
    assert len(ops) == meta[str(n)]["ops"]
    kinds = set()
    for raw in ops:
        op = wire.WorkerOperation.FromString(raw)
        assert op.WhichOneof() == "kronprod" and op.job_id == meta[str(n)]["job"]
        mats = {}
        for matop in op.kronprod.matrices:
            indices, mat = wire.pbmatop_to_matop(matop)
            mats[indices] = mat
            kinds.add(type(mat).__name__)
        state = sv.kronselect_dot(mats, state, n)
    assert kinds == {"ndarray", "CMat", "SwapMat"}
    numpy.testing.assert_allclose(state, d[p + "final"], atol=1e-12)


@pytest.mark.parametrize("n", SIZES)
def test_worker_replies_encode_as_the_reference_worker_does(cases, n):
    d, meta = cases
    p = "n{}_".format(n)
    m = meta[str(n)]
    top_raw, meas_raw = _msgs(d, p + "replies")
    top = wire.WorkerConfirm(job_id=m["job"], measure_result=wire.MeasureResult(
        top_k_indices=wire.indices_to_pbindices(m["top_k"][0])))
    top.measure_result.top_k_probs = numpy.array(m["top_k"][1])
    assert top.SerializeToString() == top_raw
    meas = wire.WorkerConfirm(job_id=m["job"], measure_result=wire.MeasureResult(
        measured_bits=m["measured"][0], measured_prob=m["measured"][1]))
    assert meas.SerializeToString() == meas_raw
    # The measurement requests decode to what the worker dispatches on.
    top_op, meas_op = (wire.WorkerOperation.FromString(x) for x in _msgs(d, p + "mops"))
    assert top_op.measure.top_k == 4 and top_op.measure.indices.index == [n - 1, 0]
    assert meas_op.measure.reduce is False and meas_op.measure.measure_result.measured_bits == m["measured"][0]


def test_conversions_round_trip():
    rng = numpy.random.default_rng(3)
    u = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
    for key, mat in (((0, 1), u), ((2, 0, 1), CMat(u)), ((3, 4, 0, 1, 2), CMat(CMat(CMat(numpy.diag([1, 1j]))))),
                     ((0, 1, 2, 3), SwapMat(2)), ((5, 0, 1), CMat(SwapMat(1)))):
        pb = wire.MatrixOp.FromString(wire.matop_to_pbmatop(key, mat).SerializeToString())
        idx, back = wire.pbmatop_to_matop(pb)
        assert idx == key
        a, b, depth = mat, back, 0
        while getattr(a, "_kron_struct", None) == 2:
            assert getattr(b, "_kron_struct", None) == 2
            a, b, depth = a.m, b.m, depth + 1
        if getattr(a, "_kron_struct", None) == 3:
            assert getattr(b, "_kron_struct", None) == 3 and b.n == a.n
        else:
            numpy.testing.assert_array_equal(b, numpy.asarray(a, dtype=complex))
    v = rng.standard_normal(8) + 1j * rng.standard_normal(8)
    numpy.testing.assert_array_equal(wire.pbvec_to_vec(wire.vec_to_pbvec(v)), v)
    assert wire.pbstatetype_to_statetype(wire.WorkerSetup.COMPLEX128) is numpy.complex128
    with pytest.raises(ValueError):
        wire.pbstatetype_to_statetype(3)


def test_reader_edges():
    # Packed encoding of a normally unpacked repeated int32, negative values, unknown fields.
    idx = wire.Indices.FromString(bytes([0x0A, 0x03, 0x01, 0x02, 0x03]))
    assert idx.index == [1, 2, 3]
    neg = wire.Indices(index=[-1, 5])
    raw = neg.SerializeToString()
    assert len(raw) == 1 + 10 + 2 and wire.Indices.FromString(raw).index == [-1, 5]
    extra = raw + bytes([0x98, 0x06, 0x07])  # field 99, varint 7
    assert wire.Indices.FromString(extra).index == [-1, 5]
    # Explicit False and empty sub-messages are written; unset fields are not.
    m = wire.Measure(reduce=False, indices=wire.Indices())
    assert m.SerializeToString() == bytes([0x0A, 0x00, 0x20, 0x00])
    assert wire.Measure().SerializeToString() == b""
    # A oneof keeps its last member.
    op = wire.WorkerOperation(total_prob=True)
    op.close = True
    assert op.WhichOneof() == "close" and op.total_prob is None
    # Malformed input.
    for bad in (bytes([0x0A, 0x05, 0x01]), bytes([0x08]), bytes([0x0B]), bytes([0x80] * 11)):
        with pytest.raises(ValueError):
            wire.Indices.FromString(bad)
    with pytest.raises(ValueError):
        wire.ComplexVector.FromString(bytes([0x0A, 0x03, 0, 0, 0]))
    with pytest.raises(ValueError):
        wire.pbvec_to_vec(wire.ComplexVector(real=numpy.zeros(2), imag=numpy.zeros(3)))
    with pytest.raises(ValueError):
        wire.pbmatop_to_matop(wire.MatrixOp(indices=wire.Indices(index=[0])))


def test_worker_refuses_a_slice_of_a_distributed_state():
    setup = wire.WorkerSetup(n=10, state_index_start=0, state_index_end=512, state_handle="s")
    with pytest.raises(ValueError, match="whole state"):
        wire.WireWorker(setup)
    with pytest.raises(ValueError, match="basis-state feed"):
        wire.WireWorker(wire.StateSetup(n=4, states=[wire.State(indices=wire.Indices(index=[0]), index=2)]))


@pytest.mark.parametrize("n", SIZES)
def test_worker_session_dispatch_on_the_oracle(cases, n):
    """Every branch of the worker's dispatch (the GPU runs the same session in
    test_gpu_wire.py), driven by the reference's messages with the oracle as backend."""
    d, meta = cases
    p = "n{}_".format(n)
    m = meta[str(n)]
    w = wire.WireWorker(bytes(d[p + "setup"]), job_id=m["job"], backend_constructor=sv.OracleBackend.make_state)
    done = wire.WorkerConfirm(job_id=m["job"]).SerializeToString()
    for raw in _msgs(d, p + "ops"):
        assert w.handle_bytes(raw) == done
    numpy.testing.assert_allclose(w.state.get_state(), d[p + "final"], atol=1e-12)
    top_op, meas_op = _msgs(d, p + "mops")
    top = wire.WorkerConfirm.FromString(w.handle_bytes(top_op))
    numpy.testing.assert_allclose(top.measure_result.top_k_probs, m["top_k"][1], atol=1e-12)
    assert top.measure_result.top_k_indices.index == m["top_k"][0]
    meas = wire.WorkerConfirm.FromString(w.handle_bytes(meas_op))
    assert meas.measure_result.measured_bits == m["measured"][0]
    assert abs(meas.measure_result.measured_prob - m["measured"][1]) < 1e-12
    numpy.testing.assert_allclose(w.state.get_state(), d[p + "after_measure"], atol=1e-12)

    # Soft measurement of a given outcome: its marginal, state unchanged.
    before = numpy.array(w.state.get_state())
    want = sv.measure_probabilities([1], n, before)[1]
    soft = wire.WorkerOperation(job_id="q", measure=wire.Measure(indices=wire.indices_to_pbindices([1]), soft=True,
                                                                 measure_result=wire.MeasureResult(measured_bits=1)))
    r = wire.WorkerConfirm.FromString(w.handle_bytes(soft.SerializeToString()))
    assert r.job_id == "q" and r.measure_result.measured_bits == 1
    assert abs(r.measure_result.measured_prob - want) < 1e-12
    numpy.testing.assert_array_equal(w.state.get_state(), before)
    # Reduce with a given outcome and probability: the state loses that qubit.
    p0 = sv.measure_probabilities([1], n, before)[0]
    red = wire.WorkerOperation(job_id="r", measure=wire.Measure(
        indices=wire.indices_to_pbindices([1]), reduce=True,
        measure_result=wire.MeasureResult(measured_bits=0, measured_prob=float(p0))))
    r = wire.WorkerConfirm.FromString(w.handle_bytes(red.SerializeToString()))
    assert r.measure_result.measured_bits == 0 and abs(r.measure_result.measured_prob - p0) < 1e-15
    assert w.state.get_state_size() == 2 ** (n - 1)
    numpy.testing.assert_allclose(w.state.get_state(), sv.reduce_measure([1], n, before, 0, p0), atol=1e-12)
    tp = wire.WorkerConfirm.FromString(w.handle_bytes(wire.WorkerOperation(job_id="t", total_prob=True)
                                                      .SerializeToString()))
    assert abs(tp.measure_result.measured_prob - 1.0) < 1e-12
    assert w.handle_bytes(wire.WorkerOperation(job_id="s", sync=wire.Sync(set_up_to=4)).SerializeToString()) == \
        wire.WorkerConfirm(job_id="s").SerializeToString()
    with pytest.raises(ValueError, match="unknown operation"):
        w.handle(wire.WorkerOperation(job_id="x"))
    assert w.handle_bytes(wire.WorkerOperation(close=True).SerializeToString()) == b""
    with pytest.raises(ValueError, match="closed"):
        w.handle(wire.WorkerOperation(total_prob=True))
