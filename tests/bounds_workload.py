"""Workload for the bounds-checked library (run by tests/test_gpu_bounds.py in a process
with QSV_BOUNDS_CHECK=1): reaches every kernel family — per-gate kernels of both
precisions with controls, every access mode of the tensor-core block kernel over many
tiles, streamed fusion, measurement, collapse, reduction, the function oracle, the
batched persistent launch with streamed segments, and both adjoint sweeps — checks a
result of each against the oracle, and prints the out-of-range count the kernels
recorded.  Exits non-zero on any mismatch."""
import ctypes
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

import numpy  # noqa: E402

import statevector as sv  # noqa: E402
from qip_gb300 import GpuBackend, _native as nat, batch, circuits  # noqa: E402
from qip_gb300.fusion import Block  # noqa: E402


def close(got, want, atol, what):
    err = float(numpy.max(numpy.abs(numpy.asarray(got) - numpy.asarray(want))))
    if not err < atol:
        raise SystemExit(f"{what}: max error {err:.3e} > {atol}")


def per_gate(rng):
    n = 12
    for statetype, atol in ((numpy.complex128, 1e-12), (numpy.complex64, 2e-5)):
        gl = circuits.random_circuit(rng, n, 150)
        v = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
        v /= numpy.linalg.norm(v)
        st = GpuBackend.make_state(n, [list(range(n))], [v], statetype=statetype, fusion=False)
        want = v.copy()
        for g in gl:
            st.kronselect_dot(g)
            want = sv.kronselect_dot(g, want, n)
        close(st.get_state(), want, atol, f"per-gate {statetype.__name__}")
        idx = [0, 5, 11]
        close(st.measure_probabilities(idx), sv.measure_probabilities(idx, n, want), atol, "probabilities")
        marg, _ = st.qubit_marginals()
        close(marg, [sv.measure_probabilities([q], n, want)[1] for q in range(n)], atol, "marginals")
        p0 = float(sv.measure_probabilities([3], n, want)[0])
        st.measure([3], measured=0, measured_prob=p0)
        st.reduce_measure([7], measured=None)
        st.func_apply([1, 2], [4, 6], lambda x: (3 * x + 1) & 3)
        st.close()


def block_modes(rng):
    n = 22
    lib = nat.load()
    for k, low, mode in ((6, 0b0000000, 0), (6, 0b0000001, 0), (6, 0b0000011, 0), (6, 0b0011000, 2),
                         (6, 0b0111111, 2), (6, 0b0111111, 3), (6, 0b0000111, 3), (6, 0b1111110, 4),
                         (6, 0b1111100, 5), (6, 0b0011000, 1),
                         (5, 0b0011110, 1), (4, 0b0000000, 0)):
        bits = [b for b in range(7) if (low >> b) & 1]
        bits += [n - 1 - i for i in range(k - len(bits))]
        qubits = [n - 1 - b for b in bits]
        rng.shuffle(qubits)
        u = numpy.linalg.qr(rng.standard_normal((2 ** k, 2 ** k)) + 1j * rng.standard_normal((2 ** k, 2 ** k)))[0]
        v = (rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)) / numpy.sqrt(2 ** (n + 1))
        st = GpuBackend.make_state(n, [list(range(n))], [v], statetype=numpy.complex64, fusion=True, autotune=False)
        nat.check(lib.qsv_set_block_mode(st.handle, k, low, mode), st.handle, "set_block_mode")
        st.apply_blocks([Block(tuple(qubits), u, 1, 1.0)])
        got = st.get_state()
        lib.qsv_set_block_mode(st.handle, k, low, -1)
        st.close()
        want = sv.apply_on(v, n, qubits, u)
        close(got / numpy.max(numpy.abs(want)), want / numpy.max(numpy.abs(want)), 5e-5, f"block k={k} mode={mode}")


def streamed_fusion():
    n = 18
    gl = circuits.brickwork(n, 12, seed=4)
    st = GpuBackend.make_state(n, [], [], statetype=numpy.complex64, fusion=True)
    want = numpy.zeros(2 ** n, dtype=complex)
    want[0] = 1
    for g in gl:
        st.kronselect_dot(g)
        want = sv.kronselect_dot(g, want, n)
    close(st.get_state(), want, 2e-5, "streamed fusion")
    st.close()


def batched(rng):
    import torch

    circs, feeds, sizes = batch.random_batch(24, seed=3, nmin=4, nmax=17, dmin=10, dmax=40)
    b = batch.CircuitBatch(circs, feeds, sizes)
    s = torch.cuda.Stream()
    b.run(s.cuda_stream)
    s.synchronize()
    for i in (0, len(circs) - 1):
        n = sizes[i]
        want = sv.make_state(n, [[q] for q in range(n)], feeds[i])
        for g in circs[i]:
            want = sv.kronselect_dot(g, want, n)
        close(b.state(i), want, 2e-5, f"batched circuit {i}")
    b.close()


def adjoint_sweeps():
    import torch

    from qip_gb300 import adjoint

    a = adjoint.Ansatz(14, 3)
    th = torch.tensor(numpy.random.default_rng(1).uniform(0, 6, (2, a.nparams)), device="cuda")
    for statetype in (torch.complex64, torch.complex128):
        e1, g1 = adjoint.energy_and_grad(th, a, statetype, segmented=True)
        e0, g0 = adjoint.energy_and_grad(th, a, statetype, segmented=False)
        close(e1.cpu().numpy(), e0.cpu().numpy(), 1e-3, "adjoint energy")
        close(g1.cpu().numpy(), g0.cpu().numpy(), 1e-3, "adjoint gradient")


def main():
    rng = numpy.random.default_rng(2026)
    lib = nat.load()
    per_gate(rng)
    block_modes(rng)
    streamed_fusion()
    batched(rng)
    adjoint_sweeps()
    count, first = ctypes.c_ulonglong(), ctypes.c_ulonglong()
    nat.check(lib.qsv_bounds_report(ctypes.byref(count), ctypes.byref(first)), None, "bounds_report")
    print(f"out-of-range accesses: {count.value} (first index {first.value})")
    return 0 if count.value == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
