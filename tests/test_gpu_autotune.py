"""Autotuned fused-block path on the GPU: every access mode of the block kernel on every
placement class against the FP64 oracle (modes pinned through the C ABI), the tuner's
recorded choice, and circuits run with the measured fusion width."""
import ctypes

import numpy
import pytest

import statevector as sv
from qip_gb300 import GpuBackend, _native as nat, circuits, gates
from qip_gb300.autotune import MODES, Autotuner, placement_class
from qip_gb300.fusion import Block

pytestmark = pytest.mark.gpu

C64 = numpy.complex64

CLASSES = [(6, 0b0000000), (6, 0b1100000), (6, 0b0000011), (6, 0b0011000), (6, 0b0000110), (6, 0b1110000),
           (6, 0b0011110), (6, 0b0111111), (6, 0b0001111), (6, 0b0000111), (6, 0b1011111), (6, 0b1111110),
           (6, 0b0111100), (6, 0b1111100), (6, 0b1011110), (5, 0b0001010),
           (5, 0b0011101), (5, 0b0000111), (4, 0b0011100), (4, 0b0011110)]


def applicable(k, low):
    j = bin(low & 0x1F).count("1")
    return ([0, 1] + ([2] if 1 <= j <= k - 1 else []) + ([3] if k == 6 and low & 7 == 7 else [])
            + ([4] if k == 6 and low & 3 == 2 else []) + ([5] if k == 6 and low & 7 == 4 else []))


def block_qubits(n, k, low):
    bits = [b for b in range(7) if (low >> b) & 1]
    bits += [n - 1 - i for i in range(k - len(bits))]
    return [n - 1 - b for b in bits]


def infidelity(a, b):
    a = numpy.asarray(a, dtype=numpy.complex128)
    b = numpy.asarray(b, dtype=numpy.complex128)
    return 1.0 - abs(numpy.vdot(a, b)) ** 2 / (numpy.vdot(a, a).real * numpy.vdot(b, b).real)


@pytest.mark.parametrize("k,low", CLASSES)
def test_every_access_mode_matches_oracle(k, low):
    """Two blocks of the class in a row: consecutive launches on a state visit the tiles
    in opposite orders, so both orders are checked in every mode."""
    n = 15
    rng = numpy.random.default_rng(k * 1000 + low)
    lib = nat.load()
    for mode in applicable(k, low):
        qubits = block_qubits(n, k, low)
        rng.shuffle(qubits)
        u = numpy.linalg.qr(rng.standard_normal((2 ** k, 2 ** k)) + 1j * rng.standard_normal((2 ** k, 2 ** k)))[0]
        u2 = numpy.linalg.qr(rng.standard_normal((2 ** k, 2 ** k)) + 1j * rng.standard_normal((2 ** k, 2 ** k)))[0]
        v = (rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)) / numpy.sqrt(2 ** (n + 1))
        st = GpuBackend.make_state(n, [list(range(n))], [v], statetype=C64, fusion=True, autotune=False)
        try:
            nat.check(lib.qsv_set_block_mode(st.handle, k, low, mode), st.handle, "set_block_mode")
            st.apply_blocks([Block(tuple(qubits), u, 1, 1.0)])
            st.apply_blocks([Block(tuple(qubits), u2, 1, 1.0)])
            got = st.get_state()
        finally:
            lib.qsv_set_block_mode(st.handle, k, low, -1)
            st.close()
        want = sv.apply_on(sv.apply_on(v, n, qubits, u), n, qubits, u2)
        err = numpy.max(numpy.abs(got - want)) / numpy.max(numpy.abs(want))
        assert err < 5e-5, (k, low, mode, err)
        assert infidelity(got, want) < 1e-8


def test_block_mode_arguments_are_checked():
    st = GpuBackend.make_state(12, [], [], statetype=C64, fusion=True, autotune=False)
    lib = nat.load()
    with pytest.raises(ValueError):
        nat.check(lib.qsv_set_block_mode(st.handle, 6, 0, 2), st.handle, "set_block_mode")  # no low target
    with pytest.raises(ValueError):
        nat.check(lib.qsv_set_block_mode(st.handle, 3, 0, 0), st.handle, "set_block_mode")
    with pytest.raises(ValueError):
        nat.check(lib.qsv_set_block_mode(st.handle, 6, 0, 5), st.handle, "set_block_mode")
    with pytest.raises(ValueError):
        nat.check(lib.qsv_set_block_mode(st.handle, 6, 0b0000011, 3), st.handle, "set_block_mode")  # bit 2 free
    with pytest.raises(ValueError):
        nat.check(lib.qsv_set_block_mode(st.handle, 5, 0b0000111, 3), st.handle, "set_block_mode")  # k = 5
    with pytest.raises(ValueError):
        nat.check(lib.qsv_set_block_mode(st.handle, 6, 0b0011111, 4), st.handle, "set_block_mode")  # bit 0 a target
    with pytest.raises(ValueError):
        nat.check(lib.qsv_set_block_mode(st.handle, 6, 0b0011110, 5), st.handle, "set_block_mode")  # bit 1 a target
    st.close()


def test_tuner_records_the_fastest_mode_and_state_is_untouched():
    n = 20
    rng = numpy.random.default_rng(4)
    v = (rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)).astype(C64)
    st = GpuBackend.make_state(n, [list(range(n))], [v], statetype=C64, fusion=True, autotune=False)
    tuner = Autotuner(reps=2)
    tuner.tune(st.handle, n, CLASSES)
    assert numpy.array_equal(st.get_state(), v)
    for k, low in CLASSES:
        times, best = tuner.measured(n, k, low)
        ok = [m for m in range(len(MODES)) if times[m] >= 0]
        assert sorted(ok) == applicable(k, low)
        assert best == min(ok, key=lambda m: times[m])
        assert tuner.block_ms(n, k, low) == times[best]
    # The recorded modes drive the next launches; results stay exact to FP32 level.
    k, low = 6, 0b0011000
    qubits = block_qubits(n, k, low)
    u = numpy.linalg.qr(rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64)))[0]
    st.apply_blocks([Block(tuple(qubits), u, 1, 1.0)])
    assert infidelity(st.get_state(), sv.apply_on(v.astype(complex), n, qubits, u)) < 1e-8
    lib = nat.load()
    for k, low in CLASSES:
        lib.qsv_set_block_mode(st.handle, k, low, -1)
    st.close()


def test_measured_width_runs_the_circuit():
    n, depth = 18, 10
    gl = circuits.brickwork(n, depth, seed=9)
    ops = [op for g in gl for op in gates.decompose(g)]
    st = GpuBackend.make_state(n, [], [], statetype=C64, fusion=True, autotune=False)
    tuner = Autotuner(reps=2)
    w, steps, report = tuner.choose_width(st.handle, n, ops)
    assert w in (4, 5, 6) and set(report) == {4, 5, 6} and all(x > 0 for x in report.values())
    assert report[w] == min(report.values())
    st.run_plan(steps)
    got = st.get_state()
    st.close()
    ref = GpuBackend.make_state(n, [], [], statetype=numpy.complex128, fusion=False)
    for g in gl:
        ref.kronselect_dot(g)
    want = ref.get_state()
    ref.close()
    assert infidelity(got, want) < 1e-6


def test_autotuned_backend_streams_a_circuit():
    """The default backend path: width measured on the first queued gates, classes
    tuned before their first launch."""
    n, depth = 16, 12
    gl = circuits.brickwork(n, depth, seed=10)
    st = GpuBackend.make_state(n, [], [], statetype=C64)
    for g in gl:
        st.kronselect_dot(g)
    got = st.get_state()
    st.close()
    v = numpy.zeros(2 ** n, dtype=complex)
    v[0] = 1
    for g in gl:
        v = sv.kronselect_dot(g, v, n)
    assert infidelity(got, v) < 1e-6
