"""Measured choices for the fused-block path: fusion width and tile access mode.

The tensor-core block kernel reads and writes a tile in one of six access modes
(direct, staged through shared memory, warp shuffles, and three with transposed products
for targets on or just above the lowest address bits; ``include/qsv.h``).  Which one
is fastest depends on where the block's targets sit among the low address bits, so it
is measured: ``qsv_tune_blocks`` times every applicable mode on a scratch state for
each placement class a plan uses, and the library keeps the fastest per device.

The fusion width (largest block, 4..6 qubits) is chosen per gate list: the planner runs
at each candidate width and each plan is priced from the measured times.  A tensor-core
block costs its class's tuned time; any other step costs one per-gate pass weighted by
the share of amplitudes it rewrites, where one pass is the tuned time of the k=4 block
with every target on a high bit (one HBM pass with the least arithmetic).  Times are
measured on min(n, 26) qubits and scaled by 2^(n - that) for an n-qubit state (every
pass is HBM-bound at those sizes).  The cheapest width wins and is remembered per n.

The caches assume one device per process, the library's own table is per device.
Decisions can be kept in a JSON file (``Autotuner(cache_path=...)``, or the
``QSV_TUNE_CACHE`` environment variable for the process-wide tuner): a tuner that loads
one pins the stored modes in the library before its first launch and reuses the stored
widths, so later processes run exactly the same kernels without measuring again (also
under a profiler, whose per-launch overhead would distort new measurements).  A cache
file belongs to one GPU model.
"""
from __future__ import annotations

import ctypes
import json
import os
import threading
from typing import Dict, Iterable, List, Optional, Sequence, Tuple

import numpy

from . import _native as nat
from .fusion import BEAM_WIDE, Block, plan, widen_blocks
from .gates import GateOp

SCRATCH_QUBITS = 26  # the library tunes on min(n, 26) qubits
BATCH_BITS = 7       # a tile's group bits: targets below this change the access pattern
MODES = ("direct", "staged", "shuffle", "prefix", "pair1", "pair2")


def placement_class(qubits: Sequence[int], n: int) -> Tuple[int, int]:
    """(k, low_mask) of a block on ``qubits`` (qubit q <-> address bit n-1-q)."""
    low = 0
    for q in qubits:
        b = n - 1 - q
        if b < BATCH_BITS:
            low |= 1 << b
    return len(qubits), low


def tensor_core_block(step, n: int) -> bool:
    return isinstance(step, Block) and len(step.qubits) >= 4 and n - len(step.qubits) >= BATCH_BITS


class Autotuner:
    def __init__(self, reps: int = 3, cache_path: Optional[str] = None):
        self.reps = int(reps)
        self.cache_path = cache_path
        self._lock = threading.RLock()
        self._ms: Dict[Tuple[int, int, int], Tuple[List[float], int]] = {}  # (nt, k, low) -> (ms per mode, best)
        self._width: Dict[int, int] = {}
        self._reports: Dict[int, Dict[int, float]] = {}
        self._unpinned: List[Tuple[int, int, int]] = []  # loaded (k, low, mode) not yet set in the library
        if cache_path and os.path.exists(cache_path):
            self._load(cache_path)

    # ---- persistence -----------------------------------------------------------------
    def _load(self, path: str) -> None:
        with open(path) as f:
            d = json.load(f)
        for row in d.get("classes", []):
            nt, k, low, times, best = row[0], row[1], row[2], row[3:-1], row[-1]
            times = [float(x) for x in times] + [-1.0] * (len(MODES) - len(times))
            self._ms[(int(nt), int(k), int(low))] = (times, int(best))
            self._unpinned.append((int(k), int(low), int(best)))
        self._width = {int(n): int(w) for n, w in d.get("widths", {}).items()}
        self._reports = {int(n): {int(w): float(ms) for w, ms in r.items()} for n, r in d.get("reports", {}).items()}

    def _save(self) -> None:
        if not self.cache_path:
            return
        d = {"classes": [[nt, k, low] + times + [best] for (nt, k, low), (times, best) in sorted(self._ms.items())],
             "widths": {str(n): w for n, w in self._width.items()},
             "reports": {str(n): {str(w): ms for w, ms in r.items()} for n, r in self._reports.items()}}
        tmp = self.cache_path + ".tmp"
        os.makedirs(os.path.dirname(os.path.abspath(self.cache_path)), exist_ok=True)
        with open(tmp, "w") as f:
            json.dump(d, f)
        os.replace(tmp, self.cache_path)

    def _pin_loaded(self, handle) -> None:
        """Set the modes read from the cache in the library (once)."""
        if not self._unpinned:
            return
        lib = nat.load()
        for k, low, mode in self._unpinned:
            nat.check(lib.qsv_set_block_mode(handle, k, low, mode), handle, "set_block_mode")
        self._unpinned = []

    # ---- access modes ----------------------------------------------------------------
    def tune(self, handle, n: int, classes: Iterable[Tuple[int, int]]) -> None:
        """Measure every class not measured yet (one library call for all of them)."""
        nt = min(n, SCRATCH_QUBITS)
        with self._lock:
            self._pin_loaded(handle)
            todo = sorted({c for c in classes if (nt,) + tuple(c) not in self._ms})
            if not todo:
                return
            lib = nat.load()
            ks = nat.int_array([k for k, _ in todo])
            lows = nat.int_array([low for _, low in todo])
            nm = len(MODES)
            ms = numpy.zeros(nm * len(todo), dtype=numpy.float64)
            best = numpy.zeros(len(todo), dtype=numpy.int32)
            nat.check(lib.qsv_tune_blocks(handle, len(todo), nat.ip(ks), nat.ip(lows), self.reps, nat.dp(ms),
                                          best.ctypes.data_as(ctypes.POINTER(ctypes.c_int))),
                      handle, "tune_blocks")
            for i, c in enumerate(todo):
                self._ms[(nt,) + tuple(c)] = ([float(x) for x in ms[nm * i:nm * i + nm]], int(best[i]))
            self._save()

    def measured(self, n: int, k: int, low: int) -> Optional[Tuple[List[float], int]]:
        return self._ms.get((min(n, SCRATCH_QUBITS), k, low))

    def block_ms(self, n: int, k: int, low: int) -> float:
        """Tuned time of one block of this class on an n-qubit state (ms)."""
        times, best = self._ms[(min(n, SCRATCH_QUBITS), k, low)]
        return times[best] * 2.0 ** (n - min(n, SCRATCH_QUBITS))

    def place(self, handle, n: int, steps) -> list:
        """``widen_blocks`` where it measured faster: each tensor-core block of fewer
        than 6 qubits becomes its 6-qubit form (identity on the added qubits) when that
        class's tuned time is not above its own."""
        wide = widen_blocks(steps, n)
        classes = {placement_class(s.qubits, n) for s in list(steps) + wide if tensor_core_block(s, n)}
        if classes:
            self.tune(handle, n, classes)
        out = []
        for a, b in zip(steps, wide):
            if a is not b and tensor_core_block(a, n) and tensor_core_block(b, n) and \
                    self.block_ms(n, *placement_class(b.qubits, n)) > self.block_ms(n, *placement_class(a.qubits, n)):
                b = a
            out.append(b)
        return out

    def ensure_plan(self, handle, n: int, steps) -> None:
        """Tune the placement classes of the tensor-core blocks of a plan."""
        classes = {placement_class(s.qubits, n) for s in steps if tensor_core_block(s, n)}
        if classes:
            self.tune(handle, n, classes)

    # ---- fusion width ----------------------------------------------------------------
    def predict_ms(self, handle, n: int, steps) -> float:
        """Predicted device time of a plan from the measured classes."""
        self.ensure_plan(handle, n, steps)
        self.tune(handle, n, [(4, 0)])
        one_pass = self.block_ms(n, 4, 0)
        total = 0.0
        for s in steps:
            if tensor_core_block(s, n):
                total += self.block_ms(n, *placement_class(s.qubits, n))
            elif isinstance(s, Block):
                total += one_pass
            else:
                total += one_pass * s.amp_update_weight()
        return total

    def candidate_widths(self, n: int, max_block: int = 6) -> List[int]:
        return [w for w in (4, 5, 6) if w <= max_block and n - w >= BATCH_BITS]

    def choose_width(self, handle, n: int, ops: Sequence[GateOp], max_block: int = 6):
        """Plan ``ops`` at every candidate width; returns (width, steps, {width: predicted ms}).
        The choice is remembered for n."""
        widths = self.candidate_widths(n, max_block)
        if not widths:
            return 3, plan(ops, kmax=3), {}
        if self._width.get(n) in widths and n in self._reports:
            # Decided before (this process or a loaded cache): reuse it.
            w = self._width[n]
            steps = self.place(handle, n, plan(ops, kmax=w, beam=BEAM_WIDE))
            return w, steps, dict(self._reports[n])
        best = None
        report = {}
        for w in widths:
            steps = self.place(handle, n, plan(ops, kmax=w, beam=BEAM_WIDE))
            ms = self.predict_ms(handle, n, steps)
            report[w] = ms
            if best is None or ms < best[0]:
                best = (ms, w, steps)
        with self._lock:
            self._width[n] = best[1]
            self._reports[n] = dict(report)
            self._save()
        return best[1], best[2], report

    def width_for(self, n: int) -> Optional[int]:
        return self._width.get(n)


_DEFAULT: Optional[Autotuner] = None


def default_tuner() -> Autotuner:
    """The process-wide tuner used by ``GpuBackend``."""
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = Autotuner(cache_path=os.environ.get("QSV_TUNE_CACHE") or None)
    return _DEFAULT
