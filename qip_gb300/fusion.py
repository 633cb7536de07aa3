"""Gate fusion: merge runs of gates into dense 2^k x 2^k blocks (k <= 6).

Each round grows candidate blocks and keeps the one that absorbs the most work.  A
candidate starts at one of the first ``lookahead`` pending gates: the gates before the
start are left out, then the scan continues in program order and a gate joins when its
qubits fit in the block (at most ``kmax`` qubits in total) and none of its qubits is
"blocked" — touched by an earlier gate that was left out.  A gate left out blocks its
qubits for the rest of the scan, so every gate moved into the block commutes with
every gate it jumps over (they act on disjoint qubits).  Starting past the first gate
lets a round take the block that fits the circuit's light cone instead of whatever the
front gate implies (brickwork n=28, depth 40: 75 steps instead of 120 with a start at
the front only).  Gates wider than ``kmax`` are never fused; they run on the per-gate
kernels when they reach the front of the queue.

A block of 4..6 qubits runs on the tensor cores (one HBM pass for all its gates); a
block of 1..3 qubits becomes one dense (or diagonal) per-gate pass; a block holding
a single gate keeps that gate's own structured kernel.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Sequence, Tuple, Union

import numpy

from .gates import GateOp

TC_MIN = 4


@dataclass
class Block:
    qubits: Tuple[int, ...]  # ascending; qubits[0] is the matrix MSB
    matrix: numpy.ndarray    # 2^k x 2^k complex128
    ngates: int
    amp_weight: float        # sum of the member gates' amp-update fractions


Step = Union[Block, GateOp]


def _embed(U: numpy.ndarray, axis_of: dict, s: int, qubits: Sequence[int], G: numpy.ndarray) -> numpy.ndarray:
    """U <- G_on_qubits @ U for a block matrix U on s qubits."""
    q = len(qubits)
    T = U.reshape((2,) * s + (-1,))
    Gt = G.reshape((2,) * (2 * q))
    axes = [axis_of[x] for x in qubits]
    T = numpy.tensordot(Gt, T, axes=(list(range(q, 2 * q)), axes))
    T = numpy.moveaxis(T, list(range(q)), axes)
    return T.reshape(1 << s, 1 << s)


def block_matrix(gates: Sequence[GateOp]) -> Tuple[Tuple[int, ...], numpy.ndarray]:
    qs = tuple(sorted(set().union(*[g.qubits for g in gates])))
    s = len(qs)
    axis_of = {q: i for i, q in enumerate(qs)}
    U = numpy.eye(1 << s, dtype=numpy.complex128)
    for g in gates:
        order, G = g.matrix()
        U = _embed(U, axis_of, s, order, G)
    return qs, U


def _emit(chosen: List[GateOp]) -> Step:
    if len(chosen) == 1:
        return chosen[0]
    qs, U = block_matrix(chosen)
    return Block(qs, U, len(chosen), sum(g.amp_update_weight() for g in chosen))


LOOKAHEAD = 16


def plan(gates: Sequence[GateOp], kmax: int = 6, lookahead: int = LOOKAHEAD) -> List[Step]:
    """Group ``gates`` (program order) into fused blocks and standalone gates."""
    steps, rest = plan_prefix(gates, kmax, nqubits=None, lookahead=lookahead)
    assert not rest
    return steps


def _grow(remaining: Sequence[GateOp], start: int, kmax: int, full_at: int):
    """Candidate block starting at remaining[start].  Returns (chosen positions, qubit
    mask, blocked mask, final): the scan stops early once the block is final (full_at
    qubits and every one of them blocked: no later gate can join)."""
    S = 0
    nS = 0
    blocked = 0
    chosen: List[int] = []
    for i, g in enumerate(remaining):
        q = g.qmask
        if i < start or (q & blocked) or g.width > kmax:
            blocked |= q
            if nS >= full_at and (S & ~blocked) == 0:
                return chosen, S, blocked, True
            continue
        merged = S | q
        nm = bin(merged).count("1")
        if nm <= kmax:
            S, nS = merged, nm
            chosen.append(i)
        else:
            blocked |= q
            if nS >= full_at and (S & ~blocked) == 0:
                return chosen, S, blocked, True
    return chosen, S, blocked, nS >= full_at and (S & ~blocked) == 0


def plan_prefix(gates: Sequence[GateOp], kmax: int = 6, nqubits=None,
                lookahead: int = LOOKAHEAD) -> Tuple[List[Step], List[GateOp]]:
    """Plan of ``gates``.  With ``nqubits`` given, stop at the first round whose choice
    later gates could still change and return (steps so far, gates not yet planned): a
    candidate block is final once it is full (kmax qubits, or every qubit of the
    register) and each of its qubits is blocked by a gate left out of it, and a round is
    decided once all its candidates are final (the candidates and their blocks then no
    longer depend on later gates).  The steps returned are exactly the first steps of
    ``plan`` over any extension of ``gates``, so a caller can launch them while gates
    keep arriving.  With ``nqubits=None`` plans everything."""
    remaining = list(gates)
    steps: List[Step] = []
    while remaining:
        first = remaining[0]
        if first.width > kmax:
            steps.append(first)
            remaining = remaining[1:]
            continue
        best = None
        full_at = kmax if nqubits is None else min(kmax, nqubits)
        for start in range(min(lookahead, len(remaining))):
            if remaining[start].width > kmax:
                continue
            chosen, S, blocked, final = _grow(remaining, start, kmax, full_at)
            if nqubits is not None and not final:
                return steps, remaining
            work = sum(remaining[i].amp_update_weight() for i in chosen)
            if best is None or work > best[0]:
                best = (work, chosen)
        picked = set(best[1])
        steps.append(_emit([remaining[i] for i in best[1]]))
        remaining = [g for i, g in enumerate(remaining) if i not in picked]
    return steps, []
