"""Gate fusion: merge runs of gates into dense 2^k x 2^k blocks (k <= 6).

Greedy planner.  Each round scans the pending gates in program order and grows one
block: a gate joins when its qubits fit in the block (at most ``kmax`` qubits in
total) and none of its qubits is "blocked" — touched by an earlier gate that was
left out of this block.  A gate left out blocks its qubits for the rest of the scan,
so every gate moved into the block commutes with every gate it jumps over (they act
on disjoint qubits).  Gates wider than ``kmax`` are never fused; they run on the
per-gate kernels when they reach the front of the queue.

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


def plan(gates: Sequence[GateOp], kmax: int = 6) -> List[Step]:
    """Group ``gates`` (program order) into fused blocks and standalone gates."""
    steps, rest = plan_prefix(gates, kmax, nqubits=None)
    assert not rest
    return steps


def plan_prefix(gates: Sequence[GateOp], kmax: int = 6, nqubits=None) -> Tuple[List[Step], List[GateOp]]:
    """Greedy plan of ``gates``.  With ``nqubits`` given, stop at the first block that
    later gates could still join and return (steps so far, gates not yet planned): a
    block is final once it is full (kmax qubits, or every qubit of the register) and
    each of its qubits is blocked by a gate left out of it.  The steps returned are
    exactly the first steps of ``plan`` over any extension of ``gates``, so a caller
    can launch them while gates keep arriving.  With ``nqubits=None`` plans
    everything."""
    remaining = list(gates)
    steps: List[Step] = []
    while remaining:
        first = remaining[0]
        if first.width > kmax:
            steps.append(first)
            remaining = remaining[1:]
            continue
        S: set = set()
        chosen: List[GateOp] = []
        blocked: set = set()
        rest: List[GateOp] = []
        for g in remaining:
            q = g.qubits
            if (q & blocked) or g.width > kmax:
                blocked |= q
                rest.append(g)
                continue
            merged = S | q
            if len(merged) <= kmax:
                S = merged
                chosen.append(g)
            else:
                blocked |= q
                rest.append(g)
        if nqubits is not None:
            full = len(S) == kmax or len(S) == nqubits
            if not (full and S <= blocked):
                return steps, remaining
        remaining = rest
        steps.append(_emit(chosen))
    return steps, []
