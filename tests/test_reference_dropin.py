"""The reference's own graph executor (Renmusxd/QIP, imported from its checkout when it is
present in the development container) driving this package's host layer: the
reference's CMat/SwapMat objects and call pattern go through qip_gb300.gates.decompose
and the backend's measurement helpers; the oracle executes the resulting ops (no GPU).
This pins the backend_constructor boundary against the reference's side of it."""
import types

import numpy
import pytest

import ref_qip
import statevector as sv
from qip_gb300 import backend as gb
from qip_gb300 import gates

pytestmark = pytest.mark.skipif(not ref_qip.available(), reason="reference checkout not present")


class HostLayerState:
    """StateType built from GpuBackend's host logic, executing ops with the oracle."""

    def __init__(self, n, vec):
        self.n = n
        self.vec = vec

    @staticmethod
    def make_state(n, index_groups, feed_list, statetype=numpy.complex128, **_):
        feeds = [gb._feed_vector(f, 2 ** len(g)) for g, f in zip(index_groups, feed_list)]
        return HostLayerState(n, sv.make_state(n, index_groups, feeds))

    def get_state(self):
        return self.vec

    def kronselect_dot(self, mats, input_offset=0, output_offset=0):
        for op in gates.decompose(mats):
            order, m = op.matrix()
            self.vec = sv.apply_on(self.vec, self.n, order, m)

    def measure_probabilities(self, indices, top_k=0):
        if top_k:
            return gb.top_k_outcomes(sv.probs_msb(indices, self.n, self.vec), top_k)
        return sv.measure_probabilities(indices, self.n, self.vec)

    def measure(self, indices, measured=None, measured_prob=None, input_offset=0, output_offset=0):
        gb.check_measured(len(indices), measured, measured_prob)
        pm = sv.probs_msb(indices, self.n, self.vec)
        m, p = gb.sample_outcome(pm, measured, 0.25 * float(pm.sum()))
        self.vec = sv.collapse(indices, self.n, self.vec, m, p)
        return m, p

    def func_apply(self, reg1, reg2, func, input_offset=0, output_offset=0):
        self.vec = sv.func_apply(reg1, reg2, func, self.vec, self.n)


def reference_api():
    qip = ref_qip.import_reference()
    ns = types.SimpleNamespace()
    for mod in (qip.qip, qip.operators, qip.pipeline, qip.qfft, qip.qubit_util):
        for k in dir(mod):
            if not k.startswith("_"):
                setattr(ns, k, getattr(mod, k))
    return ns


def test_reference_graph_drives_the_host_layer():
    from scenarios import SCENARIOS

    api = reference_api()
    for name, fn in SCENARIOS.items():
        if name == "qft_config1":
            continue
        for outs, feed, measured in fn(api):
            got, gc = api.run(*outs, feed=feed, backend_constructor=HostLayerState.make_state)
            ref, rc = api.run(*outs, feed=feed)
            numpy.testing.assert_allclose(got, ref, atol=1e-12, err_msg=name)
            for node in measured:
                if isinstance(rc[node], tuple):
                    numpy.testing.assert_allclose(gc[node][1], rc[node][1], atol=1e-12)
                else:
                    numpy.testing.assert_allclose(gc[node], rc[node], atol=1e-12)
