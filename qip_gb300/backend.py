"""State backends: the ``StateType`` interface and the GB300 implementation.

``StateType`` restates the reference's backend interface (``qip/backend.py:14-65``):
the graph executor only ever talks to a state through these methods, so a backend
whose ``make_state`` is passed as ``run(..., backend_constructor=...)`` runs any
circuit unchanged (``qip/pipeline.py:95-96,133``).

``GpuBackend`` keeps the state resident in HBM in one buffer (no arena: every kernel is
in place) and drives it through libqsv's C ABI.  Calls are queued on a CUDA stream; the
host waits only where a value comes back (state readout, probabilities, norms,
measurement outcomes).  For complex64 states, gates are queued and fused into dense
blocks on the tensor cores when the state is next observed.
"""
from __future__ import annotations

import ctypes
import random
import time
from typing import Callable, List, Mapping, Optional, Sequence, Tuple, Union

import numpy

from . import _native as nat
from . import hostbuf
from .autotune import default_tuner
from .fusion import Block, emit_native, plan, plan_prefix, widen_blocks
from .gates import GateOp, classify_matrix, decompose
from .plancache import PlanCache, default_cache, step_hash
from .util import InitialState, IndexType, MatrixType


class StateType(object):
    """Backend interface of the graph executor (``qip/backend.py:14-65``)."""

    def __init__(self, n: int, state: object):
        self.n = n
        self.state = state

    def get_state(self) -> object:
        return self.state

    def kronselect_dot(self, mats: Mapping[IndexType, MatrixType],
                       input_offset: int = 0, output_offset: int = 0) -> None:
        raise NotImplementedError("kronselect_dot not implemented by base class")

    def func_apply(self, reg1_indices: Sequence[int], reg2_indices: Sequence[int],
                   func: Callable[[int], int], input_offset: int = 0, output_offset: int = 0) -> None:
        raise NotImplementedError("func_apply not implemented by base class")

    def total_prob(self) -> float:
        raise NotImplementedError("total_prob not implemented by base class")

    def measure(self, indices: Sequence[int], measured: Optional[int] = None,
                measured_prob: Optional[float] = None,
                input_offset: int = 0, output_offset: int = 0) -> Tuple[int, float]:
        raise NotImplementedError("measure not implemented by base class")

    def reduce_measure(self, indices: Sequence[int], measured: Optional[int] = None,
                       measured_prob: Optional[float] = None,
                       input_offset: int = 0, output_offset: int = 0) -> Tuple[int, float]:
        raise NotImplementedError("reduce_measure not implemented by base class")

    def soft_measure(self, indices: Sequence[int], measured: Optional[int] = None,
                     input_offset: int = 0) -> Tuple[int, float]:
        raise NotImplementedError("soft_measure not implemented by base class")

    def measure_probabilities(self, indices: Sequence[int], top_k: int = 0
                              ) -> Union[Sequence[float], Tuple[Sequence[int], Sequence[float]]]:
        """If top_k is 0, all outcome probabilities; else (indices, probs) of the top k."""
        raise NotImplementedError("measure_probabilities not implemented by base class")

    def get_state_size(self) -> int:
        raise NotImplementedError("get_state_size not implemented by base class")

    def get_relative_range(self, start: int, end: int) -> Sequence[complex]:
        raise NotImplementedError("get_relative_range not implemented by base class")

    def overwrite_relative_range(self, start: int, end: int, data: Sequence[complex]):
        raise NotImplementedError("overwrite_relative_range not implemented by base class")

    def addto_relative_range(self, start: int, end: int, data: Sequence[complex]):
        raise NotImplementedError("addto_relative_range not implemented by base class")

    def close(self):
        pass


# ---- helpers shared with the measurement semantics ------------------------------------

def check_measured(nindices: int, measured: Optional[int], measured_prob: Optional[float]) -> None:
    """Argument checks of ``measure``/``reduce_measure`` (``qip/ext/kronprod.pyx:402-407``)."""
    if measured is not None:
        if not (0 <= measured < 2 ** nindices):
            raise ValueError("Measured value must be less than 2**len(indices)")
    if measured_prob is not None:
        if not 0.0 < measured_prob <= 1.0:
            raise ValueError("measured_prob must be 0 < p <= 1")


def sample_outcome(probs_msb: numpy.ndarray, measured: Optional[int], r: float) -> Tuple[int, float]:
    """Walk outcomes in order subtracting their probability from r until r <= 0
    (``qip/ext/kronprod.pyx:371-383``).  ``probs_msb[m]`` is the probability of outcome
    m, whose most significant bit is the smallest measured qubit index.  When
    ``measured`` is given only that outcome is visited.  If the walk runs off the end
    the last outcome is returned, as the reference does."""
    lo, hi = (0, len(probs_msb)) if measured is None else (int(measured), int(measured) + 1)
    p = 0.0
    m = lo
    for m in range(lo, hi):
        p = float(probs_msb[m])
        r -= p
        if r <= 0:
            break
    return m, p


def top_k_outcomes(probs_msb: numpy.ndarray, top_k: int) -> Tuple[List[int], List[float]]:
    """The ``top_k`` most probable outcomes, descending; ties keep the lower outcome
    first.  (The reference's bounded heap, ``kronprod.pyx:287-315``, writes one slot
    past its end once more than top_k outcomes exist; this is the well-defined intent.)"""
    top_k = min(int(top_k), len(probs_msb))
    order = numpy.lexsort((numpy.arange(len(probs_msb)), -probs_msb))[:top_k]
    return [numpy.int64(i) for i in order], [numpy.float64(probs_msb[i]) for i in order]


def _feed_vector(feed, size: int) -> numpy.ndarray:
    if isinstance(feed, (int, numpy.integer)) and not isinstance(feed, bool):
        if not 0 <= int(feed) < size:
            raise ValueError("basis-state feed {} outside [0, {})".format(feed, size))
        v = numpy.zeros(size, dtype=numpy.complex128)
        v[int(feed)] = 1.0
        return v
    v = numpy.asarray(feed, dtype=numpy.complex128).reshape(-1)
    if v.shape[0] != size:
        raise ValueError("Feed of length {} for a register of {} states".format(v.shape[0], size))
    return v


_DTYPES = {numpy.dtype(numpy.complex64): nat.QSV_C64, numpy.dtype(numpy.complex128): nat.QSV_C128}


class _DeviceView:
    """``__cuda_array_interface__`` of a state's device buffer; holds the state."""

    def __init__(self, state: "GpuBackend"):
        self.state = state
        typestr = "<c8" if state.statetype == numpy.complex64 else "<c16"
        self.__cuda_array_interface__ = {"shape": (2 ** state.n,), "typestr": typestr,
                                         "data": (state.device_ptr(), False), "version": 2}


class GpuBackend(StateType):
    """GB300 state vector behind the ``StateType`` interface.

    Register it as ``run(..., backend_constructor=GpuBackend.make_state)``.  ``statetype``
    picks the precision: ``numpy.complex128`` runs every gate on FP64 per-gate kernels;
    ``numpy.complex64`` queues gates and applies them as fused tensor-core blocks
    (``fusion=False`` keeps the per-gate FP32 kernels).
    """

    FLUSH_LIMIT = 8192
    # Queued gates are planned incrementally and launched while the executor keeps feeding
    # gates: rounds whose best block no later gate can join, and any round while more than
    # a window of gates is queued.  The first window is small so the GPU starts early;
    # later ones are wider (better blocks) yet small enough that the last flush never
    # leaves the GPU waiting (brickwork n=28: 67 blocks instead of 69, first launch after
    # 170 gates instead of 384).
    PARTIAL_FLUSH_FIRST = 128
    PARTIAL_FLUSH = 512

    # Gates needed before the fusion width is measured on them (fewer: the static rule).
    AUTOTUNE_MIN_GATES = 64

    def __init__(self, n: int, handle: ctypes.c_void_p, statetype, fusion: bool, max_block: int = 6,
                 autotune: bool = True, keep_plans: bool = True):
        super().__init__(n, None)
        self._h = handle
        self._lib = nat.load()
        self.statetype = numpy.dtype(statetype)
        self.fusion = bool(fusion)
        self.max_block = int(max_block)
        self.autotune = bool(autotune)
        self.keep_plans = bool(keep_plans)
        self._pending: List[GateOp] = []
        self._window = self.PARTIAL_FLUSH_FIRST
        self._next_partial = self._window
        # This circuit's fused gates since the last full flush and the rolling hash of
        # their structure; a kept whole-circuit plan being replayed (qip_gb300.plancache).
        self._trace: List[GateOp] = []
        self._trace_hash = 0
        self._replay = None
        self._replay_next = 0
        self._replay_done: set = set()
        self._replay_emitted: List[bool] = []
        self._replay_tried = False
        self.stats = {"ops": 0, "blocks": 0, "block_gates": 0, "launch_calls": 0, "replayed_steps": 0}

    # ---- construction ---------------------------------------------------------------
    @staticmethod
    def make_state(n: int, index_groups: Sequence[Sequence[int]], feed_list: Sequence[InitialState],
                   inputstartindex: Optional[int] = None, inputendindex: Optional[int] = None,
                   outputstartindex: Optional[int] = None, outputendindex: Optional[int] = None,
                   statetype: type = numpy.complex128, fusion: Optional[bool] = None,
                   max_block: int = 6, autotune: bool = True, keep_plans: bool = True) -> "GpuBackend":
        """Same contract as ``CythonBackend.make_state`` (``qip/backend.py:73-104``): the
        product of the fed register vectors at their global indices, unfed qubits |0>,
        |0...0> without feeds, no normalisation.  ``autotune`` (fusion only): measure the
        fusion width and the block kernel's access modes (``qip_gb300.autotune``).
        ``keep_plans`` (fusion only): replay whole-circuit plans kept from earlier
        circuits of the same structure, and keep this one's (``qip_gb300.plancache``)."""
        full = 2 ** n
        for lo, hi in ((inputstartindex, inputendindex), (outputstartindex, outputendindex)):
            if (lo not in (None, 0)) or (hi not in (None, full)):
                raise ValueError("GpuBackend holds the whole state: index windows are not supported")
        dt = numpy.dtype(statetype)
        if dt not in _DTYPES:
            raise ValueError("statetype must be numpy.complex64 or numpy.complex128, not {}".format(statetype))
        # Feeds are checked on the host before any device memory is taken.
        product = GpuBackend._product_args(index_groups, feed_list) if len(feed_list) > 0 else None
        lib = nat.load()
        h = ctypes.c_void_p()
        nat.check(lib.qsv_create(int(n), _DTYPES[dt], ctypes.byref(h)), None, "qsv_create")
        if fusion is None:
            fusion = dt == numpy.dtype(numpy.complex64)
        st = GpuBackend(n, h, dt, fusion, max_block, autotune, keep_plans)
        if product is not None:
            st._set_product(*product)
        return st

    @staticmethod
    def _product_args(index_groups, feed_list):
        sizes, qubits, vecs = [], [], []
        for group, feed in zip(index_groups, feed_list):
            g = [int(q) for q in group]
            sizes.append(len(g))
            qubits.extend(g)
            vecs.append(_feed_vector(feed, 2 ** len(g)))
        return sizes, qubits, vecs

    def _set_product(self, sizes, qubits, vecs) -> None:
        sz = nat.int_array(sizes)
        qb = nat.int_array(qubits)
        feeds = numpy.ascontiguousarray(numpy.concatenate(vecs)).view(numpy.float64)
        self._check(self._lib.qsv_set_product_state(self._h, len(sizes), nat.ip(sz), nat.ip(qb), nat.dp(feeds)),
                    "make_state")

    # ---- plumbing ---------------------------------------------------------------------
    def _check(self, status: int, what: str) -> None:
        nat.check(status, self._h, what)

    @property
    def handle(self):
        return self._h

    def device_ptr(self) -> int:
        return int(self._lib.qsv_device_ptr(self._h))

    def device_state(self):
        """The state as a torch tensor over its device buffer (no copy), with every queued
        gate applied: for callers that keep working on the GPU, this skips the host
        readback of ``get_state``.  Writes through it change the state.  The view keeps
        this object alive; it is invalid after ``close()`` or a call that resizes the
        state (``reduce_measure``).  Use it after this call returns (the state's stream is
        synchronised) or order work with ``set_stream``."""
        import torch

        self.flush()
        self._check(self._lib.qsv_synchronize(self._h), "synchronize")
        return torch.as_tensor(_DeviceView(self), device="cuda")

    def set_stream(self, stream_ptr: int) -> None:
        self.flush()
        self._check(self._lib.qsv_set_stream(self._h, ctypes.c_void_p(stream_ptr)), "set_stream")

    def synchronize(self) -> None:
        self.flush()
        self._check(self._lib.qsv_synchronize(self._h), "synchronize")

    # ---- gates --------------------------------------------------------------------------
    def kronselect_dot(self, mats: Mapping[IndexType, MatrixType],
                       input_offset: int = 0, output_offset: int = 0) -> None:
        """Apply a ``{indices: matrix}`` Kronecker dictionary in place (replaces
        ``CythonBackend.kronselect_dot``, ``qip/backend.py:112-116``)."""
        if input_offset or output_offset:
            raise ValueError("GpuBackend holds the whole state: offsets must be 0")
        ops = decompose(mats, copy=False)  # read-only from here on
        for op in ops:
            if op.qmask >> self.n:  # (a negative index already failed building the mask)
                bad = [q for q in sorted(op.qubits) if not 0 <= q < self.n]
                raise ValueError("qubit index {} out of range for n={}".format(bad[0], self.n))
            # Checked on the host before anything is queued or launched: a NaN or an
            # infinity would silently spread over the whole state.
            finite = getattr(op, "finite", None)
            if finite is None:
                finite = op.mat is None or bool(numpy.all(numpy.isfinite(op.mat)))
            if not finite:
                raise ValueError("matrix on qubits {} has non-finite entries".format(sorted(op.qubits)))
        if self.fusion:
            self._queue(ops)
        else:
            for op in ops:
                self.apply_op(op)

    REPLAY_CHECK = 16  # gates between looks for replayable steps
    TRACE_MAX = 16384  # longer circuits are streamed without keeping their structure

    def _queue(self, ops: Sequence[GateOp]) -> None:
        """Queue gates of the fused path: while the circuit's structure matches a kept
        whole-circuit plan, emit its steps as their gates arrive; otherwise plan the
        stream window by window."""
        if not ops:
            return
        if self._trace_hash is not None and len(self._trace) + len(ops) <= self.TRACE_MAX:
            for op in ops:
                self._trace.append(op)
                self._trace_hash = step_hash(self._trace_hash, op.qmask, op.amp_update_weight())
        elif self._trace_hash is not None:
            # Too long to keep: streamed as usual from here on, no plan kept.
            if self._replay is not None:
                self._replay_abandon()
            self._trace_hash = None
        if self._replay is not None:
            if len(self._trace) % self.REPLAY_CHECK < len(ops) or len(self._trace) >= self._replay.length:
                self._replay_step()
            return
        self._pending.extend(ops)
        if len(self._pending) >= self.FLUSH_LIMIT:
            self._flush_pending()
        elif len(self._pending) >= self._next_partial:
            if (self.keep_plans and not self._replay_tried and self._trace_hash is not None
                    and len(self._pending) == len(self._trace)):
                # First decision of this circuit: replay a kept plan of its structure.
                self._replay_tried = True
                self._tune_width()
                entry = default_cache().find(self._kmax(), len(self._trace), self._trace_hash)
                if entry is not None:
                    self._replay, self._replay_next, self._pending = entry, 0, []
                    self._replay_emitted = [False] * len(entry.steps)
                    self._replay_step()
                    return
            self._partial_flush()

    def _replay_step(self, final: bool = False) -> None:
        """Emit the kept plan's steps whose gates have all arrived (``final``: the circuit
        is complete), or leave the replay when the structure no longer matches.

        A ready step goes ahead of earlier steps still waiting for gates when it shares no
        qubit with any of them: the steps it passes commute with it, and every gate
        before one of its gates on a shared qubit is already emitted (the plan's order is
        a dependency order), so the emitted gates stay closed under dependencies."""
        e, n = self._replay, len(self._trace)
        if n > e.length or e.prefix[n] != self._trace_hash or (final and n != e.length):
            self._replay_abandon()
            return
        groups, blocked, mismatch = [], 0, False
        emitted = self._replay_emitted
        k = self._replay_next
        while k < len(e.steps) and blocked != e.all_qubits:
            if not emitted[k]:
                if e.last[k] < n and not e.step_mask[k] & blocked:
                    idx = e.steps[k]
                    if any(self._trace[i].qmask != e.masks[i] for i in idx):
                        mismatch = True
                        break
                    groups.append([self._trace[i] for i in idx])
                    self._replay_done.update(idx)
                    emitted[k] = True
                else:
                    blocked |= e.step_mask[k]
            k += 1
        while self._replay_next < len(e.steps) and emitted[self._replay_next]:
            self._replay_next += 1
        if groups:
            self.stats["replayed_steps"] += len(groups)
            self.run_plan(emit_native(groups))
        if mismatch:
            self._replay_abandon()

    def _replay_abandon(self) -> None:
        """The stream left the kept structure: the gates not emitted yet go on, in program
        order, through the ordinary stream planning."""
        self._pending = [op for i, op in enumerate(self._trace) if i not in self._replay_done]
        self._replay = None
        self._window = self.PARTIAL_FLUSH
        self._next_partial = len(self._pending) + self._window // 3

    def _end_circuit(self, replayed: bool) -> None:
        """After a full flush: keep a plan of this circuit's structure for later streams
        (planned in the background) unless it was replayed from one, and start a new
        trace."""
        if (self.keep_plans and not replayed and self._trace_hash is not None
                and len(self._trace) >= PlanCache.MIN_GATES):
            default_cache().plan_in_background(self._kmax(), [op.qmask for op in self._trace],
                                               [op.amp_update_weight() for op in self._trace], self._trace_hash)
        self._trace, self._trace_hash = [], 0
        self._replay, self._replay_next, self._replay_done, self._replay_tried = None, 0, set(), False

    def _kmax(self) -> int:
        if self.autotune:
            w = default_tuner().width_for(self.n)
            if w is not None:
                return min(w, self.max_block)
        return min(self.max_block, max(1, self.n - 7)) if self.n >= 11 else 3

    def _tune_width(self) -> Optional[Tuple[int, list]]:
        """Measure the fusion width on the queued gates once per n; returns (width, plan
        of every queued gate at that width) when it measured now."""
        tuner = default_tuner()
        if (not self.autotune or tuner.width_for(self.n) is not None or len(self._pending) < self.AUTOTUNE_MIN_GATES
                or not tuner.candidate_widths(self.n, self.max_block)):
            return None
        w, steps, _ = tuner.choose_width(self._h, self.n, self._pending, self.max_block)
        return w, steps

    def _partial_flush(self) -> None:
        self._tune_width()
        steps, rest = plan_prefix(self._pending, kmax=self._kmax(), nqubits=self.n, strict=False,
                                  min_pending=self._window, beam=(1, 1))
        if steps:
            self._pending = rest
            self.run_plan(steps)
            self._window = self.PARTIAL_FLUSH
        # Retry once a further chunk of gates has arrived (keeps planning linear).
        self._next_partial = len(self._pending) + self._window // 3

    def apply_ops(self, ops: Sequence[GateOp]) -> None:
        """Queue (fusion) or launch (per-gate) pre-decomposed operations."""
        if self.fusion:
            self._queue(ops)
        else:
            for op in ops:
                self.apply_op(op)

    @staticmethod
    def _op_args(op: GateOp):
        """The C-ABI arguments of an op, built once and kept with it (copies of a cached
        decomposition share them through the template's ``shared`` dict)."""
        shared = getattr(op, "shared", None)
        args = shared.get("ffi") if shared is not None else getattr(op, "ffi", None)
        if args is None:
            t = nat.int_array(op.targets)
            c = nat.int_array(op.controls)
            keep = [t, c]
            if op.kind in ("dense", "diag"):
                m = nat.c128(op.mat)
                keep.append(m)
                args = (len(t), nat.ip(t), len(c), nat.ip(c), nat.dp(m))
            elif op.kind == "mono":
                p = nat.int_array(op.perm)
                ph = nat.c128(op.mat)
                keep += [p, ph]
                args = (len(t), nat.ip(t), len(c), nat.ip(c), nat.ip(p), nat.dp(ph))
            elif op.kind == "swap":
                b = nat.int_array(op.swap_b)
                keep.append(b)
                args = (len(t), nat.ip(t), nat.ip(b), len(c), nat.ip(c))
            else:
                raise ValueError(op.kind)
            args = (args, keep)
            if shared is not None:
                shared["ffi"] = args
            else:
                op.ffi = args
        return args[0]

    def apply_op(self, op: GateOp) -> None:
        lib, h = self._lib, self._h
        args = self._op_args(op)
        self.stats["ops"] += 1
        self.stats["launch_calls"] += 1
        kind = op.kind
        if kind == "dense":
            self._check(lib.qsv_apply_matrix(h, *args), "apply_matrix")
        elif kind == "diag":
            self._check(lib.qsv_apply_diagonal(h, *args), "apply_diagonal")
        elif kind == "mono":
            self._check(lib.qsv_apply_monomial(h, *args), "apply_monomial")
        else:
            self._check(lib.qsv_apply_swap(h, *args), "apply_swap")

    def apply_blocks(self, blocks: Sequence[Block]) -> None:
        """Apply fused blocks of 4..6 qubits on the tensor cores (complex64 only)."""
        if not blocks:
            return
        ks = nat.int_array([len(b.qubits) for b in blocks])
        tg = nat.int_array([q for b in blocks for q in b.qubits])
        mats = numpy.ascontiguousarray(numpy.concatenate([numpy.asarray(b.matrix, numpy.complex128).reshape(-1)
                                                          for b in blocks])).view(numpy.float64)
        self.stats["blocks"] += len(blocks)
        self.stats["block_gates"] += sum(b.ngates for b in blocks)
        self.stats["launch_calls"] += 1
        self._check(self._lib.qsv_apply_blocks(self._h, len(blocks), nat.ip(ks), nat.ip(tg), nat.dp(mats)),
                    "apply_blocks")

    def run_plan(self, steps) -> None:
        """Execute a fusion plan: runs of tensor-core blocks go in one call."""
        if self.autotune:
            steps = default_tuner().place(self._h, self.n, steps)
        else:
            steps = widen_blocks(steps, self.n)
        batch: List[Block] = []
        for st in steps:
            if isinstance(st, Block) and len(st.qubits) >= 4 and self.n - len(st.qubits) >= 7:
                batch.append(st)
                continue
            self.apply_blocks(batch)
            batch = []
            if isinstance(st, Block):
                # Narrow block: one structured per-gate pass (diagonal / monomial / dense).
                for op in classify_matrix(st.qubits, (), st.matrix):
                    self.apply_op(op)
            else:
                self.apply_op(st)
        self.apply_blocks(batch)

    def flush(self) -> None:
        """Fuse and launch every queued gate; the circuit so far ends here."""
        replayed = self._replay is not None
        if replayed:
            self._replay_step(final=True)
            replayed = self._replay is not None
            self._replay = None
        self._flush_pending()
        self._end_circuit(replayed)

    def _flush_pending(self) -> None:
        if not self._pending:
            return
        tuned = self._tune_width()
        pending, self._pending = self._pending, []
        self._window = self.PARTIAL_FLUSH_FIRST
        self._next_partial = self._window
        self.run_plan(tuned[1] if tuned else plan(pending, kmax=self._kmax()))

    # ---- readout -------------------------------------------------------------------------
    def get_state(self) -> numpy.ndarray:
        """The state in host memory: a page-locked array from a reuse pool (one DMA, no
        page faults; ``qip_gb300.hostbuf``), owned by the caller like the reference's
        returned state array."""
        self.flush()
        t0 = time.perf_counter()
        out = hostbuf.empty(2 ** self.n, self.statetype)
        t1 = time.perf_counter()
        self._check(self._lib.qsv_read_range(self._h, out.ctypes.data_as(ctypes.c_void_p), 0, out.shape[0]),
                    "get_state")
        self.stats["readback_buffer_ms"] = (t1 - t0) * 1e3
        self.stats["readback_copy_ms"] = (time.perf_counter() - t1) * 1e3
        self.stats["readback_page_locked"] = hostbuf.is_pooled(out)
        return out

    def get_state_size(self) -> int:
        return 2 ** self.n

    def get_relative_range(self, start: int, end: int) -> numpy.ndarray:
        self.flush()
        start, end = int(start), int(end)
        out = numpy.empty(max(0, end - start), dtype=self.statetype)
        self._check(self._lib.qsv_read_range(self._h, out.ctypes.data_as(ctypes.c_void_p), start, out.shape[0]),
                    "get_relative_range")
        return out

    def overwrite_relative_range(self, start: int, end: int, data: Sequence[complex]):
        self.flush()
        d = numpy.ascontiguousarray(numpy.asarray(data, dtype=self.statetype).reshape(-1))
        if d.shape[0] != int(end) - int(start):
            raise ValueError("data length does not match the range")
        self._check(self._lib.qsv_write_range(self._h, d.ctypes.data_as(ctypes.c_void_p), int(start), d.shape[0]),
                    "overwrite_relative_range")
        self._check(self._lib.qsv_synchronize(self._h), "overwrite_relative_range")

    def addto_relative_range(self, start: int, end: int, data: Sequence[complex]):
        self.flush()
        d = numpy.ascontiguousarray(numpy.asarray(data, dtype=self.statetype).reshape(-1))
        if d.shape[0] != int(end) - int(start):
            raise ValueError("data length does not match the range")
        self._check(self._lib.qsv_add_range(self._h, d.ctypes.data_as(ctypes.c_void_p), int(start), d.shape[0]),
                    "addto_relative_range")
        self._check(self._lib.qsv_synchronize(self._h), "addto_relative_range")

    # ---- probabilities and measurement ----------------------------------------------------
    def _probs(self, qubits: Sequence[int]) -> numpy.ndarray:
        """out[v], bit j of v <-> qubits[j] (LSB first)."""
        self.flush()
        q = nat.int_array(qubits)
        out = numpy.zeros(2 ** len(q), dtype=numpy.float64)
        self._check(self._lib.qsv_probabilities(self._h, len(q), nat.ip(q), nat.dp(out)), "probabilities")
        return out

    def _probs_msb(self, indices: Sequence[int]) -> numpy.ndarray:
        """Outcome order of soft_measure / top-k: MSB = smallest measured qubit index
        (``entwine_bit``, ``qip/ext/util.pyx:2-23``)."""
        return self._probs(sorted((int(i) for i in indices), reverse=True))

    def total_prob(self) -> float:
        self.flush()
        out = numpy.zeros(1, dtype=numpy.float64)
        self._check(self._lib.qsv_norm2(self._h, nat.dp(out)), "total_prob")
        return float(out[0])

    def qubit_marginals(self) -> Tuple[numpy.ndarray, float]:
        """P(qubit q = 1) for every qubit in one pass, plus the squared norm."""
        self.flush()
        out = numpy.zeros(self.n, dtype=numpy.float64)
        nrm = numpy.zeros(1, dtype=numpy.float64)
        self._check(self._lib.qsv_qubit_marginals(self._h, nat.dp(out), nat.dp(nrm)), "qubit_marginals")
        return out, float(nrm[0])

    def measure_probabilities(self, indices: Sequence[int], top_k: int = 0):
        """Replaces ``CythonBackend.measure_probabilities`` (``qip/backend.py:158-163``):
        all outcome probabilities with bit j <-> indices[j] (``kronprod.pyx:259``), or the
        top_k outcomes in the MSB-first outcome order of ``kronprod.pyx:294``."""
        if top_k:
            return top_k_outcomes(self._probs_msb(indices), top_k)
        return self._probs([int(i) for i in indices])

    def soft_measure(self, indices: Sequence[int], measured: Optional[int] = None,
                     input_offset: int = 0) -> Tuple[int, float]:
        """Sample an outcome without changing the state (``kronprod.pyx:329-383``).  The
        draw is ``random.random()`` scaled by the state's squared norm."""
        if input_offset:
            raise ValueError("GpuBackend holds the whole state: offsets must be 0")
        probs = self._probs_msb(indices)
        r = random.random() * float(probs.sum())
        return sample_outcome(probs, measured, r)

    def _outcome_pattern(self, indices: Sequence[int], m: int) -> Tuple[List[int], int]:
        """Qubits listed LSB first and the outcome value in that order, for outcome m in
        the MSB-first encoding."""
        qs = sorted((int(i) for i in indices), reverse=True)
        return qs, int(m)

    def measure(self, indices: Sequence[int], measured: Optional[int] = None,
                measured_prob: Optional[float] = None,
                input_offset: int = 0, output_offset: int = 0) -> Tuple[int, float]:
        """Measure and collapse (``kronprod.pyx:386-446``): amplitudes disagreeing with
        the outcome become 0, the rest are scaled by sqrt(1/p) in FP64."""
        if input_offset or output_offset:
            raise ValueError("GpuBackend holds the whole state: offsets must be 0")
        indices = [int(i) for i in indices]
        check_measured(len(indices), measured, measured_prob)
        if measured is None or measured_prob is None:
            m, p = self.soft_measure(indices, measured=measured)
        else:
            m, p = int(measured), float(measured_prob)
        self.flush()
        qs, v = self._outcome_pattern(indices, m)
        q = nat.int_array(qs)
        scale = float(numpy.sqrt(1.0 / p))
        self._check(self._lib.qsv_collapse(self._h, len(q), nat.ip(q), v, scale), "measure")
        return m, p

    def reduce_measure(self, indices: Sequence[int], measured: Optional[int] = None,
                       measured_prob: Optional[float] = None,
                       input_offset: int = 0, output_offset: int = 0) -> Tuple[int, float]:
        """Measure and remove the measured qubits; the state shrinks to 2^(n-len) and
        the remaining qubits keep their order (intent of ``kronprod.pyx:449-490``)."""
        if input_offset or output_offset:
            raise ValueError("GpuBackend holds the whole state: offsets must be 0")
        indices = [int(i) for i in indices]
        check_measured(len(indices), measured, measured_prob)
        if measured is None or measured_prob is None:
            m, p = self.soft_measure(indices, measured=measured)
        else:
            m, p = int(measured), float(measured_prob)
        self.flush()
        qs, v = self._outcome_pattern(indices, m)
        q = nat.int_array(qs)
        scale = float(numpy.sqrt(1.0 / p))
        self._check(self._lib.qsv_reduce(self._h, len(q), nat.ip(q), v, scale), "reduce_measure")
        self.n -= len(indices)
        return m, p

    # ---- function oracle ------------------------------------------------------------------
    def func_apply(self, reg1_indices: Sequence[int], reg2_indices: Sequence[int],
                   func: Callable[[int], int], input_offset: int = 0, output_offset: int = 0) -> None:
        """|x>|q>|r> -> |x>|f(x) xor q>|r> (``qip/ext/func_apply.pyx:9-112``).  f is
        tabulated on the host over all 2^len(reg1) inputs, as the reference's
        ``pregen`` path does, keeping the low len(reg2) bits of each value."""
        self.flush()
        r1 = [int(i) for i in reg1_indices]
        r2 = [int(i) for i in reg2_indices]
        mask = (1 << len(r2)) - 1
        table = numpy.array([int(func(x)) & mask for x in range(2 ** len(r1))], dtype=numpy.int64)
        a1, a2 = nat.int_array(r1), nat.int_array(r2)
        self._check(self._lib.qsv_func_apply(self._h, len(a1), nat.ip(a1), len(a2), nat.ip(a2),
                                             table.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))),
                    "func_apply")

    # ---- lifetime -------------------------------------------------------------------------
    def close(self):
        """Release the state; its device buffers are parked for the next state of this
        process (``qsv_destroy``)."""
        h, self._h = getattr(self, "_h", None), None
        if h:
            self._pending, self._trace, self._replay = [], [], None
            self._lib.qsv_destroy(h)

    @staticmethod
    def release_parked_buffers() -> None:
        """Free the buffers closed states left parked for later states (``qsv_trim``)."""
        nat.check(nat.load().qsv_trim(), None, "trim")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
