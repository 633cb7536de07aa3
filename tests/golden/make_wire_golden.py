"""Generate ``wire_cases.npz``: QIP wire-format messages written by the reference's own
protobuf code, with what the reference computes from them.

Runs only where the reference checkout exists (``oracle/ref_qip.py``), with the pure-Python
protobuf runtime (the reference's generated ``messages_pb2.py`` predates the current C
runtime).  For n = 4, 6, 8:

* ``setup``: a ``StateSetup`` built as ``qip/distributed/backend.py:31-54`` builds it
  (a vector feed on two qubits, an index feed on one, the rest unfed);
* ``ops``: one ``WorkerOperation`` per kron dictionary of ``make_golden.kron_dicts``,
  built as ``qip/distributed/backend.py:56-63`` builds it;
* ``final``: the reference ``CythonBackend`` state (the index feed given to it as the
  basis vector that ``State.index`` stands for) after applying the dictionaries
  decoded from those messages with ``conversion.pbmatop_to_matop``, as the worker does
  (``qip/distributed/worker/worker.py:68-73``);
* ``mops`` / ``replies``: a top-k and an explicit-outcome measurement, and the
  ``WorkerConfirm`` the reference worker sends for each
  (``qip/distributed/worker/worker_backends.py:44-59``), from the reference backend's
  results on the final state.

Usage: ``python tests/golden/make_wire_golden.py`` from the repository root.
"""
from __future__ import annotations

import json
import os
import sys

os.environ["PROTOCOL_BUFFERS_PYTHON_IMPLEMENTATION"] = "python"

import numpy  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import make_golden as mg  # noqa: E402


def _blob(parts):
    """Concatenated messages and their offsets."""
    offs = numpy.cumsum([0] + [len(p) for p in parts]).astype(numpy.int64)
    return numpy.frombuffer(b"".join(parts), dtype=numpy.uint8).copy(), offs


def main():
    import collections
    import collections.abc

    collections.Iterable = collections.abc.Iterable  # the reference's util.py predates 3.10
    if not hasattr(numpy, "complex_"):
        numpy.complex_ = numpy.complex128  # named in conversion.py's annotations
    qip, api = mg.reference_api()
    from qip.backend import CythonBackend
    from qip.distributed.proto import conversion as cv
    from qip.distributed.proto import messages_pb2 as pb
    from qip.operators import CMat, SwapMat

    rng = numpy.random.default_rng(2024)
    arrays, meta = {}, {}
    for n in (4, 6, 8):
        job = "job-{}".format(n)
        groups = [[1, 0], [2]]
        feeds = [mg.rand_state(rng, 2) * 1.5, 1]  # unnormalised vector feed, index feed
        setup = pb.StateSetup()
        setup.n = n
        for grp, feed in zip(groups, feeds):
            st = setup.states.add()
            st.indices.CopyFrom(cv.indices_to_pbindices(grp))
            if type(feed) == int:
                st.index = feed
            else:
                st.vector.CopyFrom(cv.vec_to_pbvec(feed))
        setup_bytes = setup.SerializeToString()

        # The index feed as messages.proto defines it (all zeros but that index): the
        # reference's make_state takes vectors only (its pipeline expands index feeds
        # before they reach a backend), so it gets the expanded vector here.
        expanded = [f if type(f) != int else numpy.eye(2 ** len(g))[f] for g, f in zip(groups, feeds)]
        state = CythonBackend.make_state(n, groups, expanded, statetype=numpy.complex128)
        ops, skipped = [], 0
        for d in mg.kron_dicts(rng, n, CMat, SwapMat):
            w = pb.WorkerOperation()
            for indices, mat in d.items():
                key = indices if isinstance(indices, tuple) else (indices,)
                cv.matop_to_pbmatop(key, mat, w.kronprod.matrices.add())
            w.job_id = job
            raw = w.SerializeToString()
            # What the worker does with the message (worker.py:68-73).
            mats = {}
            for matop in pb.WorkerOperation.FromString(raw).kronprod.matrices:
                indices, mat = cv.pbmatop_to_matop(matop)
                mats[indices] = mat
            try:
                state.kronselect_dot(mats)
            except ValueError:
                # Mixed key lengths in one dictionary: the reference cannot pack them on
                # current numpy (qip/util.py:62-64), before touching the state.
                skipped += 1
                continue
            ops.append(raw)
        final = numpy.array(state.get_state(), dtype=numpy.complex128)

        # Measurements on the final state: top-k over two qubits, then an explicit outcome.
        midx = [n - 1, 0]
        top = pb.WorkerOperation()
        top.job_id = job
        top.measure.top_k = 4
        cv.indices_to_pbindices(midx, top.measure.indices)
        tk_idx, tk_p = state.measure_probabilities(numpy.array(midx, dtype=numpy.int32), top_k=4)
        rep_top = pb.WorkerConfirm()
        rep_top.job_id = job
        rep_top.measure_result.top_k_indices.index.extend(tk_idx)
        rep_top.measure_result.top_k_probs.extend(tk_p)

        outcome = int(tk_idx[0])
        meas = pb.WorkerOperation()
        meas.job_id = job
        meas.measure.reduce = False
        cv.indices_to_pbindices(midx, meas.measure.indices)
        meas.measure.measure_result.measured_bits = outcome
        m, p = state.measure(numpy.array(midx, dtype=numpy.int32), measured=outcome)
        rep_meas = pb.WorkerConfirm()
        rep_meas.job_id = job
        rep_meas.measure_result.measured_bits = m
        rep_meas.measure_result.measured_prob = p
        after = numpy.array(state.get_state(), dtype=numpy.complex128)

        p_ = "n{}_".format(n)
        arrays[p_ + "setup"] = numpy.frombuffer(setup_bytes, dtype=numpy.uint8).copy()
        arrays[p_ + "ops"], arrays[p_ + "ops_off"] = _blob(ops)
        arrays[p_ + "mops"], arrays[p_ + "mops_off"] = _blob([top.SerializeToString(), meas.SerializeToString()])
        arrays[p_ + "replies"], arrays[p_ + "replies_off"] = _blob([rep_top.SerializeToString(), rep_meas.SerializeToString()])
        arrays[p_ + "final"] = final
        arrays[p_ + "after_measure"] = after
        meta[str(n)] = {"job": job, "ops": len(ops), "skipped": skipped, "top_k": [list(map(int, tk_idx)), list(map(float, tk_p))],
                        "measured": [int(m), float(p)]}
    arrays["meta"] = numpy.array(json.dumps(meta))
    numpy.savez_compressed(os.path.join(HERE, "wire_cases.npz"), **arrays)
    print("wrote wire_cases.npz:", {k: v["ops"] for k, v in meta.items()})


if __name__ == "__main__":
    main()
