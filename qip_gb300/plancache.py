"""Whole-circuit plans kept by circuit structure, replayed while a circuit of the same
structure streams in.

A fused plan depends only on the gates' qubits and amp-update weights, not on their
matrices.  A stream (gates submitted one by one) is otherwise planned window by window,
each window without the gates after it (brickwork n=28 depth 40: 67 blocks, against 62
for the whole circuit).  A program that submits circuits of one structure again and
again — a benchmark loop, a variational loop with new angles — gets the whole-circuit
plan from the second circuit on: after a circuit's final flush its structure is planned
once in a background thread (``fusion.plan_indices`` with the wide beam) and kept here;
a later stream whose structure so far matches a kept one emits that plan's steps as
soon as all their gates have arrived.

Validity does not rest on the cache being right about the future.  A step is emitted
only when every one of its gates has arrived and the whole structure so far (every
gate's qubit mask and weight, in order) equals the kept prefix, checked with a 64-bit
rolling hash per position and, for the gates of each emitted step, mask by mask.  Each
emitted step moves its gates only past earlier gates on other qubits, so if the stream
later departs from the kept structure, the gates not yet emitted go on in program order
through the ordinary stream planning and the result is the same operator.
"""
from __future__ import annotations

import os
import struct
import threading
from typing import Dict, List, Optional, Sequence, Tuple

_MASK64 = (1 << 64) - 1
_PRIME = 0x100000001B3


_WEIGHT_BITS: Dict[float, int] = {}


def step_hash(h: int, qmask: int, weight: float) -> int:
    """Rolling hash of a structure extended by one gate (FNV-1a style over the mask and
    the weight's bits)."""
    w = _WEIGHT_BITS.get(weight)
    if w is None:
        w = _WEIGHT_BITS.setdefault(weight, struct.unpack("<Q", struct.pack("<d", float(weight)))[0])
    h = ((h ^ (qmask & _MASK64)) * _PRIME) & _MASK64
    if qmask >> 64:
        h = ((h ^ (qmask >> 64)) * _PRIME) & _MASK64
    return ((h ^ w) * _PRIME) & _MASK64


class Entry:
    """One kept structure: masks, prefix hashes (prefix[i] = hash of the first i gates),
    the plan's steps (gate indices) and, per step, its largest gate index and the union
    of its gates' qubit masks."""

    def __init__(self, kmax: int, masks: Sequence[int], weights: Sequence[float], steps: List[List[int]]):
        self.kmax = kmax
        self.masks = list(masks)
        self.prefix = [0]
        for m, w in zip(masks, weights):
            self.prefix.append(step_hash(self.prefix[-1], m, w))
        self.steps = steps
        self.last = [max(s) for s in steps]
        self.step_mask = []
        for s in steps:
            m = 0
            for i in s:
                m |= self.masks[i]
            self.step_mask.append(m)
        self.all_qubits = 0
        for m in self.masks:
            self.all_qubits |= m

    @property
    def length(self) -> int:
        return len(self.masks)


class PlanCache:
    """Kept plans, at most ``capacity`` (the oldest is dropped)."""

    MIN_GATES = 64  # shorter circuits are not worth a background plan

    def __init__(self, capacity: int = 8):
        self.capacity = capacity
        self._lock = threading.Lock()
        self._entries: List[Entry] = []
        self._busy: Dict[Tuple[int, int, int], threading.Thread] = {}

    def find(self, kmax: int, length: int, h: int) -> Optional[Entry]:
        """A kept structure whose first ``length`` gates hash to ``h``."""
        with self._lock:
            for e in reversed(self._entries):
                if e.kmax == kmax and e.length >= length and e.prefix[length] == h:
                    return e
        return None

    def has(self, kmax: int, length: int, h: int) -> bool:
        e = self.find(kmax, length, h)
        return e is not None and e.length == length

    def add(self, entry: Entry) -> None:
        with self._lock:
            self._entries.append(entry)
            if len(self._entries) > self.capacity:
                self._entries.pop(0)

    def plan_in_background(self, kmax: int, masks: Sequence[int], weights: Sequence[float], h: int) -> None:
        """Plan a finished circuit's structure off the caller's thread and keep it."""
        from .fusion import BEAM_WIDE, plan_indices

        key = (kmax, len(masks), h)
        if self.capacity <= 0 or len(masks) < self.MIN_GATES or self.has(kmax, len(masks), h):
            return
        masks, weights = list(masks), list(weights)

        def work():
            try:
                steps, planned = plan_indices(masks, weights, kmax=kmax, beam=BEAM_WIDE)
                if planned == len(masks):
                    self.add(Entry(kmax, masks, weights, steps))
            finally:
                with self._lock:
                    self._busy.pop(key, None)

        t = threading.Thread(target=work, daemon=True)
        with self._lock:  # one planner per structure: the check and the claim are one step
            if key in self._busy:
                return
            self._busy[key] = t
        t.start()

    def wait(self, timeout: float = 60.0) -> None:
        """Wait for the background plans in flight (tests, benchmarks)."""
        with self._lock:
            threads = list(self._busy.values())
        for t in threads:
            t.join(timeout)

    def clear(self) -> None:
        self.wait()
        with self._lock:
            self._entries = []


_DEFAULT: Optional[PlanCache] = None


def default_cache() -> PlanCache:
    """The process's plan cache; ``QSV_PLAN_CACHE=0`` in the environment keeps no plans
    (every circuit is planned window by window, no background thread)."""
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = PlanCache(capacity=0 if os.environ.get("QSV_PLAN_CACHE", "1") == "0" else 8)
    return _DEFAULT
