"""Reference wire-format messages (``tests/golden/wire_cases.npz``) driving a GPU state
through ``wire.WireWorker``: the state after the operations, the replies to a top-k and
an explicit-outcome measurement, and the collapsed state, against what the reference
backend computed from the same messages."""
import numpy
import pytest

from conftest import load_npz
from qip_gb300 import wire

pytestmark = pytest.mark.gpu

SIZES = (4, 6, 8)


def _msgs(d, key):
    blob, off = bytes(d[key]), d[key + "_off"]
    return [blob[off[i]:off[i + 1]] for i in range(len(off) - 1)]


@pytest.mark.parametrize("statetype,atol", [(numpy.complex128, 1e-12), (numpy.complex64, 5e-6)])
@pytest.mark.parametrize("n", SIZES)
def test_worker_session_matches_the_reference(n, statetype, atol):
    d, meta = load_npz("wire_cases.npz")
    p = "n{}_".format(n)
    m = meta[str(n)]
    w = wire.WireWorker(bytes(d[p + "setup"]), job_id=m["job"], statetype=statetype)
    done = wire.WorkerConfirm(job_id=m["job"]).SerializeToString()
    for raw in _msgs(d, p + "ops"):
        assert w.handle_bytes(raw) == done
    numpy.testing.assert_allclose(w.state.get_state(), d[p + "final"], atol=atol)

    top_op, meas_op = _msgs(d, p + "mops")
    top = wire.WorkerConfirm.FromString(w.handle_bytes(top_op))
    assert top.job_id == m["job"]
    want_idx, want_p = m["top_k"]
    numpy.testing.assert_allclose(top.measure_result.top_k_probs, want_p, atol=10 * atol)
    # Outcomes of equal probability may come in either order; distinct ones must agree.
    got = dict(zip(top.measure_result.top_k_indices.index, top.measure_result.top_k_probs))
    for i, pr in zip(want_idx, want_p):
        assert abs(got[i] - pr) < 10 * atol

    meas = wire.WorkerConfirm.FromString(w.handle_bytes(meas_op))
    assert meas.measure_result.measured_bits == m["measured"][0]
    assert abs(meas.measure_result.measured_prob - m["measured"][1]) < 10 * atol
    numpy.testing.assert_allclose(w.state.get_state(), d[p + "after_measure"], atol=10 * atol)

    tp = wire.WorkerConfirm.FromString(w.handle_bytes(wire.WorkerOperation(job_id="t", total_prob=True)
                                                      .SerializeToString()))
    assert tp.job_id == "t" and abs(tp.measure_result.measured_prob - 1.0) < 1e-5
    assert w.handle_bytes(wire.WorkerOperation(job_id="s", sync=wire.Sync()).SerializeToString()) == \
        wire.WorkerConfirm(job_id="s").SerializeToString()
    assert w.handle_bytes(wire.WorkerOperation(close=True).SerializeToString()) == b""
    with pytest.raises(ValueError):
        w.handle(wire.WorkerOperation(total_prob=True))
