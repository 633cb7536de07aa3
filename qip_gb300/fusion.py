"""Gate fusion: merge runs of gates into dense 2^k x 2^k blocks (k <= 6).

Each round grows candidate blocks and keeps the best: the one that, together with the
largest block that could follow it, absorbs the most work.  A candidate starts at one
of the first ``lookahead`` pending gates: the gates before the
start are left out, then the scan continues in program order and a gate joins when its
qubits fit in the block (at most ``kmax`` qubits in total) and none of its qubits is
"blocked" — touched by an earlier gate that was left out.  A gate left out blocks its
qubits for the rest of the scan, so every gate moved into the block commutes with
every gate it jumps over (they act on disjoint qubits).  Starting past the first gate
lets a round take the block that fits the circuit's light cone instead of whatever the
front gate implies (brickwork n=28, depth 40: 69 steps instead of 120 with a start at
the front only and no second-level score).  A beam search over rounds (``BEAM``: 16
states kept per level, 8 candidates offered per state) plans whole lists: 64 steps for
that circuit (62 with ``BEAM_WIDE``, 64 states, used where a circuit is planned once
ahead of its runs, and for the whole-circuit plans that ``qip_gb300.plancache`` keeps
by circuit structure).  Streams (gates planned while more keep arriving) use the rounds:
each call re-plans a window of pending gates, and there a beam gains nothing; a stream
whose structure has a kept plan replays that plan instead.  Gates wider than
``kmax`` are never fused; they run on the per-gate kernels when they reach the front
of the queue.

A block of 4..6 qubits runs on the tensor cores (one HBM pass for all its gates); a
block of 1..3 qubits becomes one dense (or diagonal) per-gate pass; a block holding
a single gate keeps that gate's own structured kernel.
"""
from __future__ import annotations

import ctypes
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


LOOKAHEAD = 16   # first-level candidates per round
LOOKAHEAD2 = 8   # next-round candidates scored after each of them (rounds without beam search)
BEAM = (16, 8)   # beam search: states kept per level, candidates offered per state
BEAM_WIDE = (64, 8)  # for a circuit planned once ahead of its runs (the measured width's plan)


def plan(gates: Sequence[GateOp], kmax: int = 6, lookahead: int = LOOKAHEAD,
         lookahead2: int = LOOKAHEAD2, beam: Tuple[int, int] = BEAM) -> List[Step]:
    """Group ``gates`` (program order) into fused blocks and standalone gates (native
    planner and block matrices, ``qsv_fusion_plan`` / ``qsv_block_matrices``)."""
    steps, rest = plan_prefix(gates, kmax, None, lookahead, lookahead2=lookahead2, beam=beam)
    assert not rest
    return steps


def plan_indices(qmasks: Sequence[int], weights: Sequence[float], kmax: int = 6, nqubits=None,
                 lookahead: int = LOOKAHEAD, strict: bool = True, min_pending: int = 0,
                 lookahead2: int = LOOKAHEAD2, beam: Tuple[int, int] = BEAM) -> Tuple[List[List[int]], int]:
    """The native planner on the gates' structure alone (qubit masks and amp-update
    weights, no matrices): (steps as lists of gate indices, number of gates planned)."""
    from . import _native as nat

    ng = len(qmasks)
    if ng == 0:
        return [], 0
    qm = numpy.array([int(m) for m in qmasks], dtype=numpy.uint64)
    w = numpy.ascontiguousarray(weights, dtype=numpy.float64)
    order = numpy.empty(ng, dtype=numpy.int32)
    starts = numpy.empty(ng + 1, dtype=numpy.int32)
    nsteps, nplanned = ctypes.c_int(), ctypes.c_int()
    nat.check(nat.load().qsv_fusion_plan(ng, qm.ctypes.data_as(ctypes.c_void_p), nat.dp(w), int(kmax),
                                         int(lookahead), int(lookahead2), int(beam[0]), int(beam[1]),
                                         -1 if nqubits is None else int(nqubits), int(bool(strict)),
                                         int(min_pending), nat.ip(order), nat.ip(starts), ctypes.byref(nsteps),
                                         ctypes.byref(nplanned)), None, "fusion_plan")
    return [order[starts[k]:starts[k + 1]].tolist() for k in range(nsteps.value)], nplanned.value


def plan_prefix(gates: Sequence[GateOp], kmax: int = 6, nqubits=None, lookahead: int = LOOKAHEAD,
                strict: bool = True, min_pending: int = 0,
                lookahead2: int = LOOKAHEAD2, beam: Tuple[int, int] = BEAM) -> Tuple[List[Step], List[GateOp]]:
    """``plan_prefix_py`` in native code: same steps, same matrices (to rounding)."""
    if not gates:
        return [], []
    idx, nplanned = plan_indices([g.qmask for g in gates], [g.amp_update_weight() for g in gates], kmax, nqubits,
                                 lookahead, strict, min_pending, lookahead2, beam)
    groups = [[gates[i] for i in step] for step in idx]
    planned = {i for step in idx for i in step}
    rest = [g for i, g in enumerate(gates) if i not in planned]
    return emit_native(groups), rest


def emit_native(groups: Sequence[Sequence[GateOp]]) -> List[Step]:
    """Steps for planned groups: one gate stays itself, several become a Block whose
    matrix comes from one ``qsv_block_matrices`` call for all of them."""
    from . import _native as nat

    multi = [grp for grp in groups if len(grp) > 1]
    mats = {}
    if multi:
        bk, bq, bn, gnq, gq, gm, qsets = [], [], [], [], [], [], []
        for grp in multi:
            qs = tuple(sorted(set().union(*[g.qubits for g in grp])))
            qsets.append(qs)
            bk.append(len(qs))
            bq.extend(qs)
            bn.append(len(grp))
            for g in grp:
                order, m = g.matrix()
                gnq.append(len(order))
                gq.extend(int(x) for x in order)
                gm.append(numpy.ascontiguousarray(m, dtype=numpy.complex128).reshape(-1))
        gmat = numpy.ascontiguousarray(numpy.concatenate(gm)).view(numpy.float64)
        out = numpy.empty(sum(4 ** k for k in bk), dtype=numpy.complex128)
        nat.check(nat.load().qsv_block_matrices(len(multi), nat.int_array(bk).ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                                nat.ip(nat.int_array(bq)), nat.ip(nat.int_array(bn)),
                                                nat.ip(nat.int_array(gnq)), nat.ip(nat.int_array(gq)), nat.dp(gmat),
                                                nat.dp(out.view(numpy.float64))), None, "block_matrices")
        off = 0
        for grp, qs in zip(multi, qsets):
            d = 1 << len(qs)
            mats[id(grp)] = (qs, out[off:off + d * d].reshape(d, d))
            off += d * d
    steps: List[Step] = []
    for grp in groups:
        if len(grp) == 1:
            steps.append(grp[0])
        else:
            qs, U = mats[id(grp)]
            steps.append(Block(qs, U, len(grp), sum(g.amp_update_weight() for g in grp)))
    return steps


KERNEL_MAX = 6   # widest tensor-core block


def widen_blocks(steps: Sequence[Step], n: int) -> List[Step]:
    """Place a plan on an n-qubit state: every tensor-core block of k < 6 qubits gets
    6 - k more qubits on the highest free address bits (qubit q <-> bit n-1-q), with the
    identity there.  The pass costs the same HBM traffic at any k, and the 6-qubit
    kernel runs it faster: its tiles are twice or four times larger, so the per-tile
    overhead is paid less often (n=26, targets on high bits: 0.19 ms at k=6 against
    0.23 ms at k=5 and 0.32 ms at k=4).  It also moves blocks whose qubits all sit on
    address bits 0..4 (staged access only: n=28, 4 qubits on bits 1..4, 1.40 ms) to the
    shuffle access.  Other steps are returned unchanged."""
    out: List[Step] = []
    for s in steps:
        if isinstance(s, Block):
            k = len(s.qubits)
            if TC_MIN <= k < KERNEL_MAX and n - KERNEL_MAX >= 7:
                extra = [q for q in range(n) if q not in s.qubits][:KERNEL_MAX - k]
                qs = tuple(sorted(tuple(s.qubits) + tuple(extra)))
                axis_of = {q: i for i, q in enumerate(qs)}
                U = _embed(numpy.eye(1 << KERNEL_MAX, dtype=numpy.complex128), axis_of, KERNEL_MAX,
                           tuple(s.qubits), numpy.asarray(s.matrix, numpy.complex128))
                out.append(Block(qs, U, s.ngates, s.amp_weight))
                continue
        out.append(s)
    return out


def plan_py(gates: Sequence[GateOp], kmax: int = 6, lookahead: int = LOOKAHEAD,
            lookahead2: int = LOOKAHEAD2, beam: Tuple[int, int] = BEAM) -> List[Step]:
    """Reference (pure Python) implementation of ``plan``."""
    steps, rest = plan_prefix_py(gates, kmax, None, lookahead, lookahead2=lookahead2, beam=beam)
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


def _round(remaining: List[GateOp], kmax: int, lookahead: int, nqubits, strict: bool, min_pending: int = 0,
           lookahead2: int = LOOKAHEAD2):
    """One planning round: (step, remaining after it), or (None, remaining) when
    ``nqubits`` is given and the round cannot be decided on these gates yet (a round is
    decided anyway while more than ``min_pending`` > 0 gates are pending).  A candidate
    scores its work plus the most work one of the next round's first ``lookahead2``
    candidates would take after it."""
    forced = min_pending > 0 and len(remaining) > min_pending
    prefix = nqubits is not None and not forced
    first = remaining[0]
    if first.width > kmax:
        return first, remaining[1:]
    best = None
    full_at = kmax if nqubits is None else min(kmax, nqubits)
    for start in range(min(lookahead, len(remaining))):
        if remaining[start].width > kmax:
            continue
        chosen, S, blocked, final = _grow(remaining, start, kmax, full_at)
        if prefix and strict and not final:
            return None, remaining
        work = sum(remaining[i].amp_update_weight() for i in chosen)
        score = work
        if lookahead2 > 0:
            picked = set(chosen)
            rest = [g for i, g in enumerate(remaining) if i not in picked]
            w2 = 0.0
            for s2 in range(min(lookahead2, len(rest))):
                if rest[s2].width > kmax:
                    continue
                c2, _, _, f2 = _grow(rest, s2, kmax, full_at)
                if prefix and strict and not f2:
                    return None, remaining
                w2 = max(w2, sum(rest[i].amp_update_weight() for i in c2))
            score += w2
        if best is None or score > best[0]:
            best = (score, chosen, final)
    if prefix and not best[2]:
        return None, remaining
    picked = set(best[1])
    return _emit([remaining[i] for i in best[1]]), [g for i, g in enumerate(remaining) if i not in picked]


_MASK64 = (1 << 64) - 1


def _gate_hash(g: int) -> int:
    """splitmix64 finaliser of g (the native planner's merge key of a planned gate)."""
    z = (g + 0x9E3779B97F4A7C15) & _MASK64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK64
    return z ^ (z >> 31)


def _beam_plan(gates: Sequence[GateOp], kmax: int, lookahead: int, width: int, branch: int) -> List[List[GateOp]]:
    """Beam search over planning rounds (the reference of the native one).  A state is
    the list of gates not yet planned; it offers its ``branch`` best distinct candidate
    blocks (most work first, ties to the earlier start; a gate wider than kmax at the
    front is a step of its own).  Children that planned the same gate set are merged
    (first kept) and the ``width`` with the least work left (ties: earlier child) form
    the next level.  Returns the steps (gate lists) of the first complete plan."""
    index = {id(g): i for i, g in enumerate(gates)}
    frontier = [(list(gates), sum(g.amp_update_weight() for g in gates), 0, [])]
    while True:
        for rem, _, _, path in frontier:
            if not rem:
                return path
        kids = []
        for si, (rem, _, _, _) in enumerate(frontier):
            if rem[0].width > kmax:
                opts = [(rem[0].amp_update_weight(), [0])]
            else:
                opts = []
                for s in range(min(lookahead, len(rem))):
                    if rem[s].width > kmax:
                        continue
                    chosen, _, _, _ = _grow(rem, s, kmax, kmax)
                    work = 0.0
                    for i in chosen:
                        work += rem[i].amp_update_weight()
                    opts.append((work, chosen))
                opts.sort(key=lambda o: -o[0])
            taken = 0
            for i, (work, chosen) in enumerate(opts):
                if taken >= branch:
                    break
                if any(opts[j][1] == chosen for j in range(i)):
                    continue
                kids.append((si, chosen, work))
                taken += 1
        keys, merged = set(), []
        for si, chosen, work in kids:
            rem, remw, key, path = frontier[si]
            for i in chosen:
                key = (key + _gate_hash(index[id(rem[i])])) & _MASK64
            if key in keys:
                continue
            keys.add(key)
            merged.append((remw - work, key, si, chosen))
        merged.sort(key=lambda m: m[0])
        nxt = []
        for remw, key, si, chosen in merged[:width]:
            rem, _, _, path = frontier[si]
            picked = set(chosen)
            nxt.append(([g for i, g in enumerate(rem) if i not in picked], remw, key,
                        path + [[rem[i] for i in chosen]]))
        frontier = nxt


def plan_prefix_py(gates: Sequence[GateOp], kmax: int = 6, nqubits=None, lookahead: int = LOOKAHEAD,
                   strict: bool = True, min_pending: int = 0,
                   lookahead2: int = LOOKAHEAD2, beam: Tuple[int, int] = BEAM) -> Tuple[List[Step], List[GateOp]]:
    """Reference (pure Python) plan of ``gates``.  With ``nqubits`` given, stop at the first round that later
    gates could still change and return (steps so far, gates not yet planned): a
    candidate block is final once it is full (kmax qubits, or every qubit of the
    register) and each of its qubits is blocked by a gate left out of it.  ``strict``:
    a round is decided once all its candidates are final (the candidates and their
    blocks then no longer depend on later gates), so the steps returned are exactly the
    first steps of ``plan(beam=(1, 1))`` (rounds only) over any extension of ``gates``.  Otherwise a round is
    decided once its best candidate on these gates is final — the block is just as valid
    (it only holds gates that commute with everything it jumps over) but a candidate
    that later gates would have grown may lose.  ``min_pending`` > 0: while more gates
    than that are pending a round is decided on them regardless.  With ``nqubits=None``
    plans everything.  ``beam`` = (width, branch) with either > 1: a beam search
    (``_beam_plan``) plans everything, or in prefix mode the steps taken while more than
    ``min_pending`` gates are pending; rounds plan the rest."""
    remaining = list(gates)
    steps: List[Step] = []
    if (beam[0] > 1 or beam[1] > 1) and remaining and (
            nqubits is None or (min_pending > 0 and len(remaining) > min_pending)):
        groups = _beam_plan(remaining, kmax, lookahead, beam[0], beam[1])
        left = len(remaining)
        done = set()
        for grp in groups:
            if nqubits is not None and left <= min_pending:
                break
            steps.append(_emit(grp))
            done.update(id(g) for g in grp)
            left -= len(grp)
        remaining = [g for g in remaining if id(g) not in done]
    while remaining:
        step, remaining = _round(remaining, kmax, lookahead, nqubits, strict, min_pending, lookahead2)
        if step is None:
            return steps, remaining
        steps.append(step)
    return steps, []
