"""Batched persistent launch on the GPU against the oracle (per circuit), including
circuits above the shared-memory size, graph replays and latency records."""
import numpy
import pytest

import statevector as sv
from qip_gb300 import batch

pytestmark = pytest.mark.gpu


def test_batched_circuits_match_oracle():
    import torch

    circs, feeds, sizes = batch.random_batch(40, seed=9, nmin=3, nmax=16, dmin=20, dmax=60)
    b = batch.CircuitBatch(circs, feeds, sizes)
    stream = torch.cuda.Stream()
    try:
        for _ in range(2):  # the captured graph replays
            b.run(stream.cuda_stream)
            stream.synchronize()
        for i, (gl, f, n) in enumerate(zip(circs, feeds, sizes)):
            want = sv.make_state(n, [[q] for q in range(n)], f)
            for g in gl:
                want = sv.kronselect_dot(g, want, n)
            got = b.state(i)
            err = numpy.max(numpy.abs(got - want))
            assert err < 2e-5, (i, n, err)
        lat = b.latencies_ns()
        assert numpy.all(lat > 0)
    finally:
        b.close()


def test_streamed_circuits_many_segments_match_oracle():
    """Circuits of 17..20 qubits (streamed through shared memory in segments of 14
    local bits, up to 64 chunks per segment), one without gates, mixed with small ones."""
    import torch

    from qip_gb300.circuits import random_circuit, random_product_feed

    rng = numpy.random.default_rng(77)
    circs, feeds, sizes = [], [], []
    for n, depth in ((20, 100), (19, 80), (17, 60), (18, 0), (9, 40), (14, 50)):
        circs.append(random_circuit(rng, n, depth))
        feeds.append(random_product_feed(rng, n))
        sizes.append(n)
    b = batch.CircuitBatch(circs, feeds, sizes)
    stream = torch.cuda.Stream()
    try:
        b.run(stream.cuda_stream)
        stream.synchronize()
        for i, (gl, f, n) in enumerate(zip(circs, feeds, sizes)):
            want = sv.make_state(n, [[q] for q in range(n)], f)
            for g in gl:
                want = sv.kronselect_dot(g, want, n)
            err = numpy.max(numpy.abs(b.state(i) - want))
            assert err < 2e-5, (i, n, err)
    finally:
        b.close()


def test_config4_list_seeded_subset_matches_oracle():
    """The benchmark's own list (4096 circuits, n ~ U[8,20], depth ~ U[20,100], seed 4096)
    in one launch; a seeded subset of 24 circuits, covering every n from 8 to 20
    (n > 14 streamed), against the oracle."""
    import torch

    circs, feeds, sizes = batch.random_batch(4096, seed=4096)
    b = batch.CircuitBatch(circs, feeds, sizes)
    stream = torch.cuda.Stream()
    rng = numpy.random.default_rng(404)
    pick = []
    for n in range(8, 21):
        cands = [i for i, s in enumerate(sizes) if s == n]
        pick.append(int(rng.choice(cands)))
    pick += [int(i) for i in rng.choice(len(sizes), 11, replace=False)]
    try:
        b.run(stream.cuda_stream)
        stream.synchronize()
        for i in pick:
            n = sizes[i]
            want = sv.make_state(n, [[q] for q in range(n)], feeds[i])
            for g in circs[i]:
                want = sv.kronselect_dot(g, want, n)
            err = numpy.max(numpy.abs(b.state(i) - want))
            assert err < 2e-5, (i, n, err)
        lat = b.latencies_ns()
        assert lat.shape == (4096,) and numpy.all(lat > 0)
    finally:
        b.close()


@pytest.mark.parametrize("cluster", ["1", "2", "4", "8"])
def test_cluster_sizes_match_oracle(cluster, monkeypatch):
    """Every cluster size (QSV_CIRCUIT_CLUSTER, read when the batch is created) gives the
    oracle's states: large streamed circuits shared by a cluster's CTAs (n=20 down to the
    size's threshold, one of them without gates), smaller streamed ones and shared-memory
    ones one CTA each."""
    import torch

    from qip_gb300.circuits import random_circuit, random_product_feed

    monkeypatch.setenv("QSV_CIRCUIT_CLUSTER", cluster)
    rng = numpy.random.default_rng(int(cluster) + 100)
    circs, feeds, sizes = [], [], []
    for n, depth in ((20, 40), (19, 0), (18, 30), (17, 25), (16, 20), (15, 20), (12, 30), (8, 10)):
        circs.append(random_circuit(rng, n, depth))
        feeds.append(random_product_feed(rng, n))
        sizes.append(n)
    b = batch.CircuitBatch(circs, feeds, sizes)
    stream = torch.cuda.Stream()
    try:
        for _ in range(2):
            b.run(stream.cuda_stream)
        stream.synchronize()
        for i, (gl, f, n) in enumerate(zip(circs, feeds, sizes)):
            want = sv.make_state(n, [[q] for q in range(n)], f)
            for g in gl:
                want = sv.kronselect_dot(g, want, n)
            err = numpy.max(numpy.abs(b.state(i) - want))
            assert err < 2e-5, (cluster, i, n, err)
        assert numpy.all(b.latencies_ns() > 0)
    finally:
        b.close()
