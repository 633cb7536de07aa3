"""Seeded synthetic workloads, expressed as lists of ``kronselect_dot`` dictionaries
(the unit the reference's backend consumes, ``qip/backend.py:112-116``).  The same
lists drive this package's GPU backend, the reference's Cython kernel and the oracle.

* ``brickwork``: Haar-random 2x2 on every qubit, then CZ on even/odd neighbour pairs,
  plus a C(Swap) on 3 seeded qubits every 10 layers; input |0...0>.
* ``qft_gates``: the gate sequence ``qip.qfft.QFFT`` builds (H, controlled phases from
  every later qubit, reversing Swaps).  Note the reference's op wrapper drops the
  ``negate=True`` keyword, so the phases are positive (the result is the inverse DFT).
* ``grover_gates``: QFT followed by amplitude-amplification iterations with an
  (n-1)-controlled Z oracle on a seeded marked index and an H/X diffusion step.
* ``random_circuit``: random gates from {H, X, Rm(1..8), CNOT, C(Swap), Haar 2x2}.
* ``ansatz_layers``: RY / RZ layers and a CNOT ring (adjoint-gradient workload).
"""
from __future__ import annotations

from typing import Dict, List, Sequence, Tuple

import numpy

from .operators import CMat, SwapMat

Mats = Dict[Tuple[int, ...], object]

H_MAT = (1 / numpy.sqrt(2)) * numpy.array([[1, 1], [1, -1]], dtype=numpy.complex128)
X_MAT = numpy.array([[0, 1], [1, 0]], dtype=numpy.complex128)
Z_MAT = numpy.array([[1, 0], [0, -1]], dtype=numpy.complex128)


def haar_2x2(rng: numpy.random.Generator) -> numpy.ndarray:
    """Haar-random U(2): QR of a complex Gaussian matrix with the phase of R's diagonal
    moved into Q."""
    z = (rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))) / numpy.sqrt(2.0)
    q, r = numpy.linalg.qr(z)
    d = numpy.diag(r)
    return q * (d / numpy.abs(d))[None, :]


def rm_mat(m: int, negate: bool = False) -> numpy.ndarray:
    phi = (-2 if negate else 2) * numpy.pi / pow(2.0, m)
    return numpy.array([[1, 0], [0, numpy.exp(1.0j * phi)]], dtype=numpy.complex128)


def brickwork(n: int, depth: int, seed: int = 1234, cswap_every: int = 10) -> List[Mats]:
    rng = numpy.random.default_rng(seed)
    gates: List[Mats] = []
    for layer in range(depth):
        for q in range(n):
            gates.append({(q,): haar_2x2(rng)})
        start = layer % 2
        for a in range(start, n - 1, 2):
            gates.append({(a, a + 1): CMat(Z_MAT)})
        if cswap_every and (layer + 1) % cswap_every == 0 and n >= 3:
            c, a, b = (int(x) for x in rng.choice(n, size=3, replace=False))
            gates.append({(c, a, b): CMat(SwapMat(1))})
    return gates


def gate_amp_updates(gates: Sequence[Mats], n: int) -> float:
    """Amplitude updates of a gate list: a dense k-qubit gate rewrites 2^n amplitudes,
    one with c controls 2^(n-c)."""
    total = 0.0
    for g in gates:
        for key, m in g.items():
            c = 0
            while getattr(m, "_kron_struct", None) == 2:
                c += 1
                m = m.m
            total += 2.0 ** (n - c)
    return total


def qft_schedule(n: int, rev: bool = True):
    """The QFT's steps over wire positions 0..n-1, in the order QIP's ``QFFT`` graph
    executes them (``qip/qfft.py:8-43``): ``("h", t)``; ``("cphase", c, t, m)``, an Rm(m)
    on t controlled by c, for every later wire c with m = 1 + c - t; then with ``rev``
    ``("swap", a, n-1-a)`` for the first n//2 wires.  Both ``qft_gates`` and the graph
    op ``qip_gb300.qfft.QFFT`` are built from this list."""
    for t in range(n):
        yield ("h", t)
        for c in range(t + 1, n):
            yield ("cphase", c, t, 1 + c - t)
    if rev:
        for a in range(n // 2):
            yield ("swap", a, n - 1 - a)


def qft_gates(n: int, first: int = 0, rev: bool = True) -> List[Mats]:
    """``QFFT`` on qubits first..first+n-1 as kron dictionaries, in execution order."""
    gates: List[Mats] = []
    for step in qft_schedule(n, rev):
        wires = tuple(first + w for w in step[1:3])
        if step[0] == "h":
            gates.append({wires[:1]: H_MAT})
        elif step[0] == "cphase":
            gates.append({wires: CMat(rm_mat(step[3]))})
        else:
            gates.append({wires: SwapMat(1)})
    return gates


def multi_controlled_z(qubits: Sequence[int]) -> Mats:
    """C^(k-1)(Z) on ``qubits`` (last = target) as nested CMats, as ``C(C(...(Z)))``
    builds it."""
    m: object = Z_MAT
    for _ in range(len(qubits) - 1):
        m = CMat(m)
    return {tuple(qubits): m}


def grover_gates(n: int, iterations: int = 8, seed: int = 7) -> Tuple[List[Mats], int]:
    rng = numpy.random.default_rng(seed)
    marked = int(rng.integers(0, 2 ** n))
    gates = qft_gates(n)
    allq = list(range(n))
    zero_bits = [q for q in allq if not (marked >> (n - 1 - q)) & 1]
    for _ in range(iterations):
        for q in zero_bits:
            gates.append({(q,): X_MAT})
        gates.append(multi_controlled_z(allq))
        for q in zero_bits:
            gates.append({(q,): X_MAT})
        for q in allq:
            gates.append({(q,): H_MAT})
        for q in allq:
            gates.append({(q,): X_MAT})
        gates.append(multi_controlled_z(allq))
        for q in allq:
            gates.append({(q,): X_MAT})
        for q in allq:
            gates.append({(q,): H_MAT})
    return gates, marked


def random_circuit(rng: numpy.random.Generator, n: int, depth: int) -> List[Mats]:
    """``depth`` gates drawn uniformly from H, X, Rm(1..8), CNOT, C(Swap), Haar 2x2."""
    gates: List[Mats] = []
    for _ in range(depth):
        kind = int(rng.integers(0, 6))
        if kind == 0:
            gates.append({(int(rng.integers(0, n)),): H_MAT})
        elif kind == 1:
            gates.append({(int(rng.integers(0, n)),): X_MAT})
        elif kind == 2:
            gates.append({(int(rng.integers(0, n)),): rm_mat(int(rng.integers(1, 9)))})
        elif kind == 3:
            c, t = (int(x) for x in rng.choice(n, size=2, replace=False))
            gates.append({(c, t): CMat(X_MAT)})
        elif kind == 4:
            c, a, b = (int(x) for x in rng.choice(n, size=3, replace=False))
            gates.append({(c, a, b): CMat(SwapMat(1))})
        else:
            gates.append({(int(rng.integers(0, n)),): haar_2x2(rng)})
    return gates


def random_product_feed(rng: numpy.random.Generator, n: int) -> List[numpy.ndarray]:
    """One Haar-random single-qubit state per qubit."""
    return [haar_2x2(rng)[:, 0].copy() for _ in range(n)]


def ry_mat(theta: float) -> numpy.ndarray:
    c, s = numpy.cos(theta / 2), numpy.sin(theta / 2)
    return numpy.array([[c, -s], [s, c]], dtype=numpy.complex128)


def rz_mat(phi: float) -> numpy.ndarray:
    e = numpy.exp(-0.5j * phi)
    return numpy.array([[e, 0], [0, numpy.conj(e)]], dtype=numpy.complex128)


def ansatz_layers(n: int, layers: int, thetas: numpy.ndarray) -> List[Mats]:
    """``layers`` x (RY(theta) on every qubit, RZ(phi) on every qubit, CNOT ring
    (i, i+1 mod n)); thetas has 2*n*layers angles, layer-major (RY block then RZ)."""
    thetas = numpy.asarray(thetas, dtype=numpy.float64).reshape(layers, 2, n)
    gates: List[Mats] = []
    for l in range(layers):
        for q in range(n):
            gates.append({(q,): ry_mat(thetas[l, 0, q])})
        for q in range(n):
            gates.append({(q,): rz_mat(thetas[l, 1, q])})
        for q in range(n):
            gates.append({(q, (q + 1) % n): CMat(X_MAT)})
    return gates
