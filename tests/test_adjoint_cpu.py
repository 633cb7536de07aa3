"""Adjoint-gradient host logic on CPU: the oracle's finite-difference gradient is pinned
to the reference's parameter-shift gradient (tests/golden), and the ansatz gate list /
per-gate matrices agree with the circuit generator."""
import numpy
import torch

import statevector as sv
from conftest import load_npz
from qip_gb300 import adjoint, circuits


def oracle_energy(th, n, layers):
    v = numpy.zeros(2 ** n, dtype=complex)
    v[0] = 1
    for g in circuits.ansatz_layers(n, layers, th):
        v = sv.kronselect_dot(g, v, n)
    w = n - 2 * numpy.array([bin(i).count("1") for i in range(2 ** n)])
    return float(numpy.sum(w * numpy.abs(v) ** 2))


def test_oracle_gradients_match_reference_parameter_shift():
    d = load_npz("workloads.npz")[0]
    n, layers = (int(x) for x in d["ansatz_ps_shape"])
    for th, e, g in zip(d["ansatz_ps_thetas"], d["ansatz_ps_energies"], d["ansatz_ps_grads"]):
        assert abs(oracle_energy(th, n, layers) - e) < 1e-12
        h = 1e-3
        fd = []
        for j in range(th.size):
            tp, tm = th.copy(), th.copy()
            tp[j] += h
            tm[j] -= h
            fd.append((oracle_energy(tp, n, layers) - oracle_energy(tm, n, layers)) / (2 * h))
        numpy.testing.assert_allclose(fd, g, atol=1e-5)


def test_ansatz_gate_list_matches_circuit_generator():
    """Kinds, qubits and parameter indices of Ansatz.gates() are those of the circuit
    generator's dictionaries (the matrices are checked on the GPU, where
    qsv_batch_rotation_matrices builds them)."""
    n, layers = 5, 2
    a = adjoint.Ansatz(n, layers)
    th = numpy.random.default_rng(0).uniform(0, 6, a.nparams)
    dicts = circuits.ansatz_layers(n, layers, th)
    assert len(dicts) == len(a.gates())
    for g, (kind, tgt, ctl, pi) in enumerate(a.gates()):
        (key, m), = dicts[g].items()
        if kind == adjoint.CNOT:
            assert key == (ctl, tgt) and pi == -1
            numpy.testing.assert_array_equal(m.m, circuits.X_MAT)
        else:
            assert key == (tgt,)
            want = circuits.ry_mat(th[pi]) if kind == adjoint.RY else circuits.rz_mat(th[pi])
            numpy.testing.assert_allclose(m, want, atol=1e-15)


def test_segment_plan_is_the_same_circuit():
    """Segments (gates reordered only past gates on other qubits) reproduce the circuit;
    every segment's gates act on its local bits, which include address bits 0..4."""
    n, layers = 10, 3
    a = adjoint.Ansatz(n, layers)
    rng = numpy.random.default_rng(3)
    th = rng.uniform(0, 2 * numpy.pi, a.nparams)
    mats = circuits.ansatz_layers(n, layers, th)
    # ansatz_layers gives one dictionary per gate in ansatz.gates() order.
    assert len(mats) == len(a.gates())
    v0 = (rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n))
    want = v0.copy()
    for g in mats:
        want = sv.kronselect_dot(g, want, n)
    for lb in (7, 8, 10):
        segs = adjoint.plan_segments(a, lb)
        assert sorted(gi for _, gl in segs for gi in gl) == list(range(len(mats)))
        got = v0.copy()
        for lpos, gl in segs:
            assert len(lpos) == min(lb, n) and set(range(5)) <= set(lpos)
            for gi in gl:
                kind, t, c, _ = a.gates()[gi]
                assert n - 1 - t in lpos and (c < 0 or n - 1 - c in lpos)
                got = sv.kronselect_dot(mats[gi], got, n)
        numpy.testing.assert_allclose(got, want, atol=1e-12)
        if lb < n:
            assert len(segs) > 1


def test_segment_device_tables_decode_to_the_circuit():
    """The group / gate records the kernels read (decoded back to global qubits through
    each segment's local bits and each group's bits) replay the circuit exactly."""
    n, layers = 10, 3
    a = adjoint.Ansatz(n, layers)
    rng = numpy.random.default_rng(8)
    th = rng.uniform(0, 2 * numpy.pi, a.nparams)
    mats = circuits.ansatz_layers(n, layers, th)
    v0 = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    want = v0.copy()
    for g in mats:
        want = sv.kronselect_dot(g, want, n)
    for lb in (7, 9):
        got = v0.copy()
        seen = []
        for lpos, nl, ngr, gtab, ng, tab in adjoint.segment_tables(a, lb, "cpu"):
            lpos = list(lpos)
            for nb, packed, first, count in gtab.tolist():
                gbits = [(packed >> (8 * j)) & 0xFF for j in range(nb)]
                assert 1 <= nb <= 3 and gbits == sorted(gbits) and count <= adjoint.GROUP_GATES
                for tb, cb, gi, gp in tab[first:first + count].tolist():
                    kind, t, c, pi = a.gates()[gi]
                    assert n - 1 - lpos[gbits[tb]] == t
                    assert (cb < 0 and c < 0) or n - 1 - lpos[gbits[cb]] == c
                    assert (gp >> 24) & 3 == {adjoint.RY: 1, adjoint.RZ: 2}.get(kind, 0)
                    assert (gp >> 24) & 3 == 0 or (gp & 0xFFFFFF) == pi
                    seen.append(gi)
                    got = sv.kronselect_dot(mats[gi], got, n)
        assert sorted(seen) == list(range(len(mats)))
        numpy.testing.assert_allclose(got, want, atol=1e-12)


def test_tensor_core_block_partition_is_a_valid_order():
    """The six-qubit blocks of the tensor-core adjoint cover every gate once, and their
    concatenated gate order applied by the oracle gives the circuit's state (the blocks
    only move gates past gates on other qubits)."""
    from qip_gb300 import adjoint

    n, layers = 8, 3
    a = adjoint.Ansatz(n, layers)
    blocks = adjoint.block_partition(a)
    order = [i for _, step in blocks for i in step]
    assert sorted(order) == list(range(len(a.gates())))
    gates = a.gates()
    for qs, step in blocks:
        assert len(qs) == 6 and list(qs) == sorted(set(qs))
        for i in step:
            _, t, c, _ = gates[i]
            assert t in qs and (c < 0 or c in qs)
    rng = numpy.random.default_rng(3)
    th = rng.uniform(0, 2 * numpy.pi, a.nparams)
    mats = circuits.ansatz_layers(n, layers, th)
    want = numpy.zeros(2 ** n, complex)
    want[0] = 1
    got = want.copy()
    for g in mats:
        want = sv.kronselect_dot(g, want, n)
    for i in order:
        got = sv.kronselect_dot(mats[i], got, n)
    numpy.testing.assert_allclose(got, want, atol=1e-12)
