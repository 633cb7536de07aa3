"""FP64 CPU oracle for the QIP state-vector hot path — TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use this
module, and only as the checker.  The product (``qip_gb300``) never imports it.

A clean-room numpy restatement of the reference's semantics (Renmusxd/QIP), each
function citing the reference lines it follows.  Pinned against the reference itself
through the golden vectors in ``tests/golden`` (generated by running the reference's
own Cython kernels, see ``tests/golden/make_golden.py``) and against the known answers
in the reference's unit tests.

Conventions (reference): qubit q is state-index bit (n-1-q) (``kronprod.pyx:168``); in a
gate's index tuple the first index is the MSB of the sub-matrix index
(``kronprod.pyx:184-189``).
"""
from __future__ import annotations

from typing import Any, Callable, Dict, List, Mapping, Optional, Sequence, Tuple

import numpy

KRON_CMAT = 2
KRON_SWAP = 3


# ---- bit helpers (qip/ext/util.pyx) -------------------------------------------------------

def entwine_bit(n_indices: int, n_non_indices: int, v_indices: int, v_non_indices: int, mask: int) -> int:
    """Interleave: walking positions from n-1 down to 0, masked positions take the next
    bit of v_indices (from its MSB), the others the next bit of v_non_indices
    (``qip/ext/util.pyx:2-23``)."""
    n = n_indices + n_non_indices
    out = 0
    ki, kn = n_indices, n_non_indices
    for pos in range(n - 1, -1, -1):
        out <<= 1
        if (mask >> pos) & 1:
            ki -= 1
            out |= (v_indices >> ki) & 1
        else:
            kn -= 1
            out |= (v_non_indices >> kn) & 1
    return out


def row_mask(indices: Sequence[int], n: int) -> int:
    m = 0
    for q in indices:
        m |= 1 << (n - 1 - int(q))
    return m


# ---- matrix entry rules (kronprod.pyx:203-235) ----------------------------------------------

def entry(mat: Any, i: int, j: int) -> complex:
    tag = getattr(mat, "_kron_struct", None)
    if tag == KRON_CMAT:
        half = mat.shape[0] >> 1
        if i < half and j < half:
            return 1.0 if i == j else 0.0
        if i >= half and j >= half:
            return entry(mat.m, i - half, j - half)
        return 0.0
    if tag == KRON_SWAP:
        k = mat.n
        low = (1 << k) - 1
        return 1.0 if (i & low) == (j >> k) and (j & low) == (i >> k) else 0.0
    return complex(numpy.asarray(mat)[i, j])


def dense_of(mat: Any) -> numpy.ndarray:
    d = mat.shape[0]
    if getattr(mat, "_kron_struct", None) is None:
        return numpy.asarray(mat, dtype=numpy.complex128)
    out = numpy.empty((d, d), dtype=numpy.complex128)
    for i in range(d):
        for j in range(d):
            out[i, j] = entry(mat, i, j)
    return out


def normalize(mats: Mapping[Any, Any]) -> Dict[Tuple[int, ...], Any]:
    """``qip/util.py:35-58``: int keys -> 1-tuples, lists -> arrays, shape check."""
    out = {}
    for key, m in mats.items():
        if type(key) == int:  # noqa: E721
            key = (key,)
        elif type(key) != tuple:  # noqa: E721
            raise Exception("Type of indices must be tuple: {}".format(key))
        if type(m) == list:  # noqa: E721
            m = numpy.array(m)
        if 2 ** len(key) != m.shape[0] or 2 ** len(key) != m.shape[1]:
            raise Exception("Shape of square submatrix must equal 2**(number of indices)")
        out[key] = m
    return out


def union_operator(mats: Mapping[Any, Any]) -> Tuple[List[int], numpy.ndarray]:
    """The operator cdot_loop applies, restricted to the sorted union of the indices:
    M[r, c] = prod_g M_g[r|g, c|g] (``kronprod.pyx:164-196``)."""
    mats = normalize(mats)
    flat = sorted({q for key in mats for q in key})
    u = len(flat)
    where = {q: u - 1 - i for i, q in enumerate(flat)}
    dim = 1 << u
    rows = numpy.arange(dim)
    out = numpy.ones((dim, dim), dtype=numpy.complex128)
    for key, m in mats.items():
        L = len(key)
        sub = numpy.zeros(dim, dtype=numpy.int64)
        for p, q in enumerate(key):
            sub |= ((rows >> where[q]) & 1) << (L - 1 - p)
        out *= dense_of(m)[sub[:, None], sub[None, :]]
    return flat, out


def apply_on(vec: numpy.ndarray, n: int, qubits: Sequence[int], mat: numpy.ndarray) -> numpy.ndarray:
    """out = (mat on ``qubits``, first qubit = MSB) applied to vec, by tensor reshape."""
    k = len(qubits)
    psi = numpy.asarray(vec, dtype=numpy.complex128).reshape((2,) * n)
    g = numpy.asarray(mat, dtype=numpy.complex128).reshape((2,) * (2 * k))
    out = numpy.tensordot(g, psi, axes=(list(range(k, 2 * k)), list(qubits)))
    out = numpy.moveaxis(out, list(range(k)), list(qubits))
    return numpy.ascontiguousarray(out).reshape(-1)


def kronselect_dot(mats: Mapping[Any, Any], vec: numpy.ndarray, n: int) -> numpy.ndarray:
    """Full-state ``cdot_loop`` semantics (``kronprod.pyx:41-200``) without offsets."""
    flat, op = union_operator(mats)
    return apply_on(vec, n, flat, op)


def kronselect_dot_window(mats, vec, n, output_len, input_offset=0, output_offset=0):
    """Windowed form (``kronprod.pyx:158,170-172``): vec holds amplitudes
    [input_offset, input_offset+len(vec)) and the result rows
    [output_offset, output_offset+output_len).  Small n only."""
    full = numpy.zeros(2 ** n, dtype=numpy.complex128)
    full[input_offset:input_offset + len(vec)] = vec
    res = kronselect_dot(mats, full, n)
    return res[output_offset:output_offset + output_len]


# ---- state preparation (qip/backend.py:73-104, qip/util.py:108-124) ------------------------

def make_state(n: int, index_groups: Sequence[Sequence[int]], feeds: Sequence[Any]) -> numpy.ndarray:
    state = numpy.zeros(2 ** n, dtype=numpy.complex128)
    if len(feeds) == 0:
        state[0] = 1.0
        return state
    qubits = [int(q) for g in index_groups for q in g]
    unfed = [q for q in range(n) if q not in qubits]
    vecs = []
    for g, f in zip(index_groups, feeds):
        if isinstance(f, (int, numpy.integer)) and not isinstance(f, bool):
            v = numpy.zeros(2 ** len(g), dtype=numpy.complex128)
            v[int(f)] = 1.0
        else:
            v = numpy.asarray(f, dtype=numpy.complex128).reshape(-1)
        vecs.append(v)
    # Tensor of the fed registers in feed order, then unfed qubits fixed at |0>.
    t = numpy.ones(1, dtype=numpy.complex128)
    for v in vecs:
        t = numpy.kron(t, v)
    order = qubits + unfed
    zero = numpy.zeros(2 ** len(unfed), dtype=numpy.complex128)
    zero[0] = 1.0
    t = numpy.kron(t, zero).reshape((2,) * n)
    # Axis a of t is qubit order[a]; permute to qubit order.
    perm = [order.index(q) for q in range(n)]
    return numpy.ascontiguousarray(numpy.transpose(t, perm)).reshape(-1)


# ---- measurement (qip/ext/kronprod.pyx:238-490) --------------------------------------------

def measure_probabilities(indices: Sequence[int], n: int, vec: numpy.ndarray) -> numpy.ndarray:
    """Marginal over ``indices``; outcome bit j <-> indices[j] (``kronprod.pyx:240-261``)."""
    p = numpy.abs(numpy.asarray(vec)) ** 2
    i = numpy.arange(2 ** n, dtype=numpy.int64)
    idx = numpy.zeros(2 ** n, dtype=numpy.int64)
    for j, q in enumerate(indices):
        idx |= ((i >> (n - 1 - int(q))) & 1) << j
    return numpy.bincount(idx, weights=p, minlength=2 ** len(indices)).astype(numpy.float64)


def probs_msb(indices: Sequence[int], n: int, vec: numpy.ndarray) -> numpy.ndarray:
    """Outcome probabilities in entwine order: outcome MSB = smallest qubit index
    (``kronprod.pyx:287-295, 371-376``)."""
    return measure_probabilities(sorted((int(q) for q in indices), reverse=True), n, vec)


def measure_top_probabilities(indices, n, top_k, vec) -> Tuple[List[int], List[float]]:
    """Top-k outcomes (descending, ties: lower outcome first) in entwine order."""
    pm = probs_msb(indices, n, vec)
    k = min(int(top_k), len(pm))
    order = numpy.lexsort((numpy.arange(len(pm)), -pm))[:k]
    return [int(i) for i in order], [float(pm[i]) for i in order]


def prob_magnitude(vec) -> float:
    """Squared norm (the intent of ``kronprod.pyx:318-326``, whose accumulator is
    uninitialised in the reference)."""
    v = numpy.asarray(vec)
    return float(numpy.sum(v.real ** 2 + v.imag ** 2))


def soft_measure(indices, n, vec, measured=None, r: float = 0.5) -> Tuple[int, float]:
    """Outcome walk of ``kronprod.pyx:362-383`` with the draw r in [0, 1) given."""
    pm = probs_msb(indices, n, vec)
    r = r * float(pm.sum())
    lo, hi = (0, len(pm)) if measured is None else (int(measured), int(measured) + 1)
    m, p = lo, 0.0
    for m in range(lo, hi):
        p = float(pm[m])
        r -= p
        if r <= 0:
            break
    return m, p


def collapse(indices, n, vec, m: int, p: float) -> numpy.ndarray:
    """``kronprod.pyx:428-444``: keep amplitudes whose measured bits equal the
    entwined outcome m, scaled by sqrt(1/p)."""
    mask = row_mask(indices, n)
    want = entwine_bit(len(indices), n - len(indices), int(m), 0, mask)
    i = numpy.arange(2 ** n, dtype=numpy.int64)
    keep = (i & mask) == want
    out = numpy.zeros(2 ** n, dtype=numpy.complex128)
    out[keep] = numpy.asarray(vec, dtype=numpy.complex128)[keep] * numpy.sqrt(1.0 / p)
    return out


def reduce_measure(indices, n, vec, m: int, p: float) -> numpy.ndarray:
    """Intent of ``kronprod.pyx:449-490``: out[j] = vec[entwine(m, j)] * sqrt(1/p),
    a 2^(n-len(indices)) state of the remaining qubits in order."""
    mask = row_mask(indices, n)
    k = len(indices)
    v = numpy.asarray(vec, dtype=numpy.complex128)
    out = numpy.empty(2 ** (n - k), dtype=numpy.complex128)
    for j in range(2 ** (n - k)):
        out[j] = v[entwine_bit(k, n - k, int(m), j, mask)] * numpy.sqrt(1.0 / p)
    return out


def func_apply(reg1, reg2, func: Callable[[int], int], vec, n) -> numpy.ndarray:
    """|x>|q>|r> -> |x>|f(x) xor q>|r> over every r (intent of
    ``qip/ext/func_apply.pyx:54-155``; f keeps its low len(reg2) bits)."""
    reg1 = [int(q) for q in reg1]
    reg2 = [int(q) for q in reg2]
    n1, n2 = len(reg1), len(reg2)
    table = numpy.array([int(func(x)) & ((1 << n2) - 1) for x in range(2 ** n1)], dtype=numpy.int64)
    i = numpy.arange(2 ** n, dtype=numpy.int64)
    x = numpy.zeros_like(i)
    for j, q in enumerate(reg1):
        x |= ((i >> (n - 1 - q)) & 1) << (n1 - 1 - j)
    f = table[x]
    flip = numpy.zeros_like(i)
    for j, q in enumerate(reg2):
        flip |= ((f >> (n2 - 1 - j)) & 1) << (n - 1 - q)
    v = numpy.asarray(vec, dtype=numpy.complex128)
    return v[i ^ flip]


# ---- a StateType for running circuits on the CPU --------------------------------------------

class OracleBackend:
    """CPU state with the backend interface of ``qip/backend.py:14-65`` (test harness)."""

    def __init__(self, n: int, state: numpy.ndarray):
        self.n = n
        self.state = state
        self.draws = []

    @staticmethod
    def make_state(n, index_groups, feed_list, statetype=numpy.complex128, **_):
        return OracleBackend(n, make_state(n, index_groups, feed_list))

    def get_state(self):
        return self.state

    def kronselect_dot(self, mats, input_offset=0, output_offset=0):
        self.state = kronselect_dot(mats, self.state, self.n)

    def func_apply(self, reg1, reg2, func, input_offset=0, output_offset=0):
        self.state = func_apply(reg1, reg2, func, self.state, self.n)

    def total_prob(self):
        return prob_magnitude(self.state)

    def measure_probabilities(self, indices, top_k=0):
        if top_k:
            return measure_top_probabilities(indices, self.n, top_k, self.state)
        return measure_probabilities(indices, self.n, self.state)

    def soft_measure(self, indices, measured=None, input_offset=0, r=None):
        import random

        r = random.random() if r is None else r
        self.draws.append(r)
        return soft_measure(indices, self.n, self.state, measured, r)

    def measure(self, indices, measured=None, measured_prob=None, input_offset=0, output_offset=0):
        if measured is not None and not (0 <= measured < 2 ** len(indices)):
            raise ValueError("Measured value must be less than 2**len(indices)")
        if measured_prob is not None and not 0.0 < measured_prob <= 1.0:
            raise ValueError("measured_prob must be 0 < p <= 1")
        if measured is None or measured_prob is None:
            m, p = self.soft_measure(indices, measured)
        else:
            m, p = measured, measured_prob
        self.state = collapse(indices, self.n, self.state, m, p)
        return m, p

    def reduce_measure(self, indices, measured=None, measured_prob=None, input_offset=0, output_offset=0):
        if measured is None or measured_prob is None:
            m, p = self.soft_measure(indices, measured)
        else:
            m, p = measured, measured_prob
        self.state = reduce_measure(indices, self.n, self.state, m, p)
        self.n -= len(indices)
        return m, p

    def get_state_size(self):
        return len(self.state)

    def get_relative_range(self, start, end):
        return self.state[start:end]

    def overwrite_relative_range(self, start, end, data):
        self.state[start:end] = data

    def addto_relative_range(self, start, end, data):
        self.state[start:end] += data

    def close(self):
        pass
