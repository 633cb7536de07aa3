"""Adjoint-method gradients of parameterised circuits behind a torch.autograd.Function.

Workload: the hardware-efficient ansatz of ``circuits.ansatz_layers`` — per layer RY(theta)
on every qubit, RZ(phi) on every qubit, then a CNOT ring (i, i+1 mod n) — on |0...0>,
objective E = <psi| sum_i Z_i |psi>, for a batch of parameter sets at once.

Forward: the gates (each set with its own 2x2 matrix built on the device from its
angle) run in segments: runs of gates whose qubits fit, with address bits 0..4, in 13
local bits (12 for complex128), reordered only past gates on other qubits (the fusion
planner's blocked-qubit rule).  One launch per segment brings every 2^13-amplitude
chunk of every set into shared memory once and applies all the segment's gates there.
Then lambda = (sum Z) psi and E in FP64.  Backward (adjoint method, no checkpoints):
the segments in reverse, each chunk's psi and lambda in shared memory; for each gate
from last to first, at a rotation dE/dtheta = Im <lambda| P |psi> (P = Y or Z) is
accumulated per set, then psi and lambda are un-computed by U^+.  Inside a segment
gates are grouped by at most 3 local bits and applied in registers to 8-amplitude
items, one shared-memory pass per group.  Two state vectors
per set (psi, lambda).  ``segmented=False`` runs the same algorithm one launch per gate.

On the tensor cores (``method="tensor"``, the default for complex64 states of n >= 13):
the gates are split into blocks of six qubits by the fusion planner.  Forward: per block,
every set's 64x64 block matrix is built on the device from its angles and applied to all
sets in one split-bf16 tensor-core launch.  Backward: per block (in reverse), one
tensor-core GEMM correlates psi and lambda over the other qubits,
X = sum_g psi[g] lambda[g]^+ (64x64 per set), and every gradient of the block follows
from X by a walk through the block's gates in FP64 (dE/dtheta_j = Im Tr(P_j Q_j),
Q <- U_j^+ Q U_j); then psi and lambda are un-computed by U^+ with two more block
launches (``qsv_adjoint_forward`` / ``qsv_adjoint_backward``).

There is no reference counterpart (the reference has no gradients); results are checked
against central finite differences and the parameter-shift rule on the FP64 oracle and
on the reference's own kernel (tests/golden).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import List, Tuple

import numpy
import torch

from . import _native as nat

RY, RZ, CNOT = 0, 1, 2


@dataclass
class Ansatz:
    n: int
    layers: int

    @property
    def nparams(self) -> int:
        return 2 * self.n * self.layers

    def gates(self) -> List[Tuple[int, int, int, int]]:
        """(kind, target, control, param index or -1), in application order.  Parameter
        layout: layer-major, RY block then RZ block (as ``circuits.ansatz_layers``)."""
        out = []
        n = self.n
        for l in range(self.layers):
            for q in range(n):
                out.append((RY, q, -1, (2 * l) * n + q))
            for q in range(n):
                out.append((RZ, q, -1, (2 * l + 1) * n + q))
            for q in range(n):
                out.append((CNOT, (q + 1) % n, q, -1))
        return out


def _dtype(statetype):
    if statetype in (torch.complex64, numpy.complex64):
        return torch.complex64, nat.QSV_C64
    return torch.complex128, nat.QSV_C128


_KIND_TABLES = {}


def gate_matrices(ansatz: Ansatz, thetas: torch.Tensor, cdtype) -> Tuple[torch.Tensor, torch.Tensor]:
    """Per-gate, per-set 2x2 matrices U and U^+ as [G, B, 4] tensors on the device, built
    by ``qsv_batch_rotation_matrices`` from the angles."""
    B = thetas.shape[0]
    gates = ansatz.gates()
    G = len(gates)
    key = (ansatz.n, ansatz.layers, str(thetas.device))
    if key not in _KIND_TABLES:
        _KIND_TABLES[key] = torch.tensor([[k, max(p, 0)] for k, _, _, p in gates], dtype=torch.int32,
                                         device=thetas.device)
    kinds = _KIND_TABLES[key]
    th = thetas.detach().to(torch.float64).contiguous()
    U = torch.empty((G, B, 4), dtype=cdtype, device=thetas.device)
    Ud = torch.empty_like(U)
    _, qdtype = _dtype(cdtype)
    _check(nat.load().qsv_batch_rotation_matrices(ctypes.c_void_p(th.data_ptr()), B, th.shape[1], G,
                                                  ctypes.c_void_p(kinds.data_ptr()), qdtype,
                                                  ctypes.c_void_p(U.data_ptr()), ctypes.c_void_p(Ud.data_ptr()),
                                                  ctypes.c_void_p(_stream_ptr())), "batch_rotation_matrices")
    return U, Ud


def _stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


def _check(rc: int, what: str):
    if rc != 0:
        nat.check(rc, None, what)


def forward_states(ansatz: Ansatz, U: torch.Tensor, cdtype, qdtype) -> torch.Tensor:
    lib = nat.load()
    B = U.shape[1]
    n = ansatz.n
    psi = torch.empty((B, 2 ** n), dtype=cdtype, device=U.device)
    st = ctypes.c_void_p(_stream_ptr())
    _check(lib.qsv_batch_reset(ctypes.c_void_p(psi.data_ptr()), B, n, qdtype, st), "batch_reset")
    stride = U.stride(0) * U.element_size()
    base = U.data_ptr()
    for g, (kind, tgt, ctl, _) in enumerate(ansatz.gates()):
        _check(lib.qsv_batch_apply_1q(ctypes.c_void_p(psi.data_ptr()), B, n, qdtype, tgt, ctl,
                                      ctypes.c_void_p(base + g * stride), st), "batch_apply_1q")
    return psi


SEG_FIXED_BITS = 5        # address bits 0..4 are always local (coalesced chunk accesses)
SEG_MAX_GATES = 512
SEG_MAX_PARAMS = 256


def local_bits(statetype, backward: bool = False) -> int:
    """Local bits of a segment: 2^lb amplitudes per chunk in shared memory.  The reverse
    sweep holds psi and lambda chunks, so it uses one bit less (two CTAs per SM); any
    segmentation is an equivalent order of the same circuit, so the two may differ."""
    lb = 13 if statetype in (torch.complex64, numpy.complex64) else 12
    return lb - 1 if backward else lb


def plan_segments(ansatz: Ansatz, lb: int) -> List[Tuple[Tuple[int, ...], List[int]]]:
    """[(local bit positions ascending, gate indices in execution order)] covering every
    gate once.  A gate joins the segment when its bits fit in lb local bits and none of
    them is blocked by an earlier gate left out (so it commutes with every gate it
    passes); left-out gates block their bits."""
    gates = ansatz.gates()
    n = ansatz.n
    lb = min(lb, n)
    fixed = set(range(min(SEG_FIXED_BITS, lb)))
    remaining = list(range(len(gates)))
    segs = []
    while remaining:
        S = set(fixed)
        chosen, rest, blocked = [], [], set()
        nparams = 0
        for gi in remaining:
            kind, t, c, _ = gates[gi]
            bits = {n - 1 - t} | ({n - 1 - c} if c >= 0 else set())
            gen = 1 if kind in (RY, RZ) else 0
            merged = S | bits
            if not (bits & blocked) and len(merged) <= lb and len(chosen) < SEG_MAX_GATES and \
                    nparams + gen <= SEG_MAX_PARAMS:
                S = merged
                chosen.append(gi)
                nparams += gen
            else:
                blocked |= bits
                rest.append(gi)
        p = 0
        while len(S) < lb:
            S.add(p) if p not in S else None
            p += 1
        segs.append((tuple(sorted(S)), chosen))
        remaining = rest
    return segs


GROUP_BITS = 3    # local bits of a register group (2^3 amplitudes per item)
GROUP_GATES = 8   # gates per group


def plan_groups(bits_of: List[Tuple[int, ...]], max_bits: int = GROUP_BITS,
                max_gates: int = GROUP_GATES) -> List[Tuple[Tuple[int, ...], List[int]]]:
    """Split a segment's gate sequence (bits_of[i] = local bits of gate i) into groups of
    at most max_bits bits and max_gates gates, with the blocked-bit rule (a gate moves
    ahead only past gates on other bits).  Returns [(bits ascending, gate positions)]."""
    remaining = list(range(len(bits_of)))
    groups = []
    while remaining:
        B, chosen, blocked, rest = set(), [], set(), []
        for i in remaining:
            bits = set(bits_of[i])
            if not (bits & blocked) and len(chosen) < max_gates and len(B | bits) <= max_bits:
                B |= bits
                chosen.append(i)
            else:
                blocked |= bits
                rest.append(i)
        groups.append((tuple(sorted(B)), chosen))
        remaining = rest
    return groups


_SEG_CACHE = {}


def segment_tables(ansatz: Ansatz, lb: int, device):
    """Planned segments with their device tables, cached: per segment (local bits,
    lb, groups int32 [ngroups, 4], gates int32 [ngates, 4]); gates are stored in group
    order, targets/controls as indices among their group's bits."""
    key = (ansatz.n, ansatz.layers, min(lb, ansatz.n), str(device))
    if key not in _SEG_CACHE:
        gates = ansatz.gates()
        n = ansatz.n
        out = []
        for lpos, gl in plan_segments(ansatz, lb):
            local = {b: i for i, b in enumerate(lpos)}
            lbits = []
            for gi in gl:
                kind, t, c, _ = gates[gi]
                lbits.append((local[n - 1 - t],) + ((local[n - 1 - c],) if c >= 0 else ()))
            grows, rows = [], []
            for gbits, members in plan_groups(lbits):
                idx = {b: j for j, b in enumerate(gbits)}
                packed = sum(b << (8 * j) for j, b in enumerate(gbits))
                grows.append([len(gbits), packed, len(rows), len(members)])
                for m in members:
                    kind, t, c, pi = gates[gl[m]]
                    gen = {RY: 1, RZ: 2}.get(kind, 0)
                    rows.append([idx[local[n - 1 - t]], idx[local[n - 1 - c]] if c >= 0 else -1, gl[m],
                                 (gen << 24) | (pi if gen else 0)])
            gtab = torch.tensor(grows, dtype=torch.int32, device=device)
            tab = torch.tensor(rows, dtype=torch.int32, device=device)
            out.append((nat.int_array(lpos), len(lpos), len(grows), gtab, len(rows), tab))
        _SEG_CACHE[key] = out
    return _SEG_CACHE[key]


def forward_states_segmented(ansatz: Ansatz, U: torch.Tensor, cdtype, qdtype, lb: int) -> torch.Tensor:
    lib = nat.load()
    B = U.shape[1]
    n = ansatz.n
    psi = torch.empty((B, 2 ** n), dtype=cdtype, device=U.device)
    st = ctypes.c_void_p(_stream_ptr())
    _check(lib.qsv_batch_reset(ctypes.c_void_p(psi.data_ptr()), B, n, qdtype, st), "batch_reset")
    for lpos, nl, ngr, gtab, ng, tab in segment_tables(ansatz, lb, U.device):
        _check(lib.qsv_batch_segment_forward(ctypes.c_void_p(psi.data_ptr()), B, n, qdtype, nl, nat.ip(lpos), ngr,
                                             ctypes.c_void_p(gtab.data_ptr()), ng, ctypes.c_void_p(tab.data_ptr()),
                                             ctypes.c_void_p(U.data_ptr()), st),
               "segment_forward")
    return psi


def adjoint_sweep_segmented(ansatz: Ansatz, psi, lam, Ud, qdtype, lb: int) -> torch.Tensor:
    """Reverse sweep by segments; consumes psi and lambda.  Returns dE/dtheta [B, P]."""
    lib = nat.load()
    B = psi.shape[0]
    P = ansatz.nparams
    grads = torch.zeros((B, P), dtype=torch.float64, device=psi.device)
    st = ctypes.c_void_p(_stream_ptr())
    for lpos, nl, ngr, gtab, ng, tab in reversed(segment_tables(ansatz, lb, psi.device)):
        _check(lib.qsv_batch_segment_adjoint(ctypes.c_void_p(psi.data_ptr()), ctypes.c_void_p(lam.data_ptr()), B,
                                             ansatz.n, qdtype, nl, nat.ip(lpos), ngr, ctypes.c_void_p(gtab.data_ptr()),
                                             ng, ctypes.c_void_p(tab.data_ptr()), ctypes.c_void_p(Ud.data_ptr()),
                                             ctypes.c_void_p(grads.data_ptr()), P, st),
               "segment_adjoint")
    return grads


def _scratch(B: int, device) -> torch.Tensor:
    return torch.empty(B * 4096, dtype=torch.float64, device=device)


TC_MIN_QUBITS = 13  # a six-qubit block needs seven more qubits for a tensor-core tile


class TensorCorePlan:
    """The ansatz split into blocks of six qubits (the fusion planner's steps, each a run
    of gates in a valid execution order; a step on fewer qubits gets identity qubits, the
    lowest-index ones not in it) and the native plan built from it (``qsv_adjoint_*``)."""

    def __init__(self, ansatz: Ansatz):
        gates = ansatz.gates()
        self.blocks = block_partition(ansatz)
        qubits_flat, ngates, recs = [], [], []
        for qs, step in self.blocks:
            qubits_flat.extend(qs)
            ngates.append(len(step))
            for i in step:
                kind, t, c, pi = gates[i]
                recs.extend([kind, t, c, pi])
        n = ansatz.n
        lib = nat.load()
        h = ctypes.c_void_p()
        qb, ng, gr = nat.int_array(qubits_flat), nat.int_array(ngates), nat.int_array(recs)
        _check(lib.qsv_adjoint_plan_create(n, len(self.blocks), nat.ip(qb), nat.ip(ng), nat.ip(gr), ctypes.byref(h)),
               "adjoint_plan_create")
        self.handle = h
        self.nparams = ansatz.nparams
        fused = ctypes.c_int()
        _check(lib.qsv_adjoint_plan_fused_blocks(h, ctypes.byref(fused)), "adjoint_plan_fused_blocks")
        # Blocks whose backward is one pass (correlation and both un-computes together).
        self.fused_blocks = fused.value

    def scratch(self, nsets: int, device) -> torch.Tensor:
        nbytes = int(nat.load().qsv_adjoint_scratch_bytes(self.handle, nsets))
        return torch.empty(nbytes, dtype=torch.uint8, device=device)

    def __del__(self):
        try:
            if self.handle:
                nat.load().qsv_adjoint_plan_destroy(self.handle)
        except Exception:
            pass


def block_partition(ansatz: Ansatz) -> List[Tuple[Tuple[int, ...], List[int]]]:
    """[(six qubits ascending, gate indices in execution order)] covering every gate of
    the ansatz once: the fusion planner's steps at width 6 (whole list, wide beam), each
    widened to six qubits by the lowest-index qubits it does not touch."""
    from .fusion import BEAM_WIDE, LOOKAHEAD, LOOKAHEAD2, plan_indices

    gates = ansatz.gates()
    qmasks = [(1 << t) | ((1 << c) if c >= 0 else 0) for _, t, c, _ in gates]
    steps, planned = plan_indices(qmasks, [1.0] * len(gates), 6, None, LOOKAHEAD, True, 0, LOOKAHEAD2, BEAM_WIDE)
    if planned != len(gates):
        raise RuntimeError("fusion planner left gates unplanned")
    blocks = []
    for step in steps:
        qs = {q for i in step for q in (gates[i][1], gates[i][2]) if q >= 0}
        for q in range(ansatz.n):
            if len(qs) >= 6:
                break
            qs.add(q)
        blocks.append((tuple(sorted(qs)), list(step)))
    return blocks


_TC_PLANS = {}


def tensor_core_plan(ansatz: Ansatz) -> TensorCorePlan:
    key = (ansatz.n, ansatz.layers)
    if key not in _TC_PLANS:
        _TC_PLANS[key] = TensorCorePlan(ansatz)
    return _TC_PLANS[key]


def _method(segmented, ansatz: Ansatz, cdtype) -> str:
    """``segmented``: True / False (segment kernels / one launch per gate, CUDA cores),
    a method name, or None: the tensor cores where they apply, else segments."""
    if isinstance(segmented, str):
        if segmented not in ("tensor", "segmented", "per_gate"):
            raise ValueError("method must be 'tensor', 'segmented' or 'per_gate'")
        if segmented == "tensor" and (cdtype != torch.complex64 or ansatz.n < TC_MIN_QUBITS):
            raise ValueError("the tensor-core adjoint needs complex64 states of at least 13 qubits")
        return segmented
    if segmented is None:
        return "tensor" if cdtype == torch.complex64 and ansatz.n >= TC_MIN_QUBITS else "segmented"
    return "segmented" if segmented else "per_gate"


class SumZExpectation(torch.autograd.Function):
    """E[b] = <psi(thetas[b])| sum_i Z_i |psi(thetas[b])> with adjoint gradients."""

    @staticmethod
    def forward(ctx, thetas: torch.Tensor, ansatz: Ansatz, statetype=torch.complex64, segmented=None):
        if not thetas.is_cuda:
            raise ValueError("thetas must live on the CUDA device")
        cdtype, qdtype = _dtype(statetype)
        method = _method(segmented, ansatz, cdtype)
        B = thetas.shape[0]
        lib = nat.load()
        if method == "tensor":
            plan = tensor_core_plan(ansatz)
            th64 = thetas.detach().to(torch.float64).contiguous()
            psi = torch.empty((B, 2 ** ansatz.n), dtype=cdtype, device=thetas.device)
            tc_scratch = plan.scratch(B, thetas.device)
            st = ctypes.c_void_p(_stream_ptr())
            _check(lib.qsv_batch_reset(ctypes.c_void_p(psi.data_ptr()), B, ansatz.n, qdtype, st), "batch_reset")
            _check(lib.qsv_adjoint_forward(plan.handle, ctypes.c_void_p(psi.data_ptr()), B,
                                           ctypes.c_void_p(th64.data_ptr()), ansatz.nparams,
                                           ctypes.c_void_p(tc_scratch.data_ptr()), tc_scratch.numel(), st),
                   "adjoint_forward")
            Ud = (plan, th64, tc_scratch)
        else:
            U, Ud = gate_matrices(ansatz, thetas.detach(), cdtype)
            lb = local_bits(cdtype)
            psi = forward_states_segmented(ansatz, U, cdtype, qdtype, lb) if method == "segmented" else \
                forward_states(ansatz, U, cdtype, qdtype)
        lam = torch.empty_like(psi)
        energies = torch.empty(B, dtype=torch.float64, device=thetas.device)
        scratch = _scratch(B, thetas.device)
        _check(lib.qsv_batch_observable_sumz(ctypes.c_void_p(psi.data_ptr()), ctypes.c_void_p(lam.data_ptr()),
                                             B, ansatz.n, qdtype, ctypes.c_void_p(energies.data_ptr()),
                                             ctypes.c_void_p(scratch.data_ptr()), scratch.numel(),
                                             ctypes.c_void_p(_stream_ptr())), "observable")
        ctx.ansatz, ctx.qdtype = ansatz, qdtype
        ctx.buffers = (psi, lam, Ud, scratch)
        ctx.tdtype = thetas.dtype
        ctx.method, ctx.lb = method, local_bits(cdtype, backward=True)
        return energies.to(thetas.dtype)

    @staticmethod
    def backward(ctx, grad_e: torch.Tensor):
        psi, lam, Ud, scratch = ctx.buffers
        ctx.buffers = None
        if ctx.method == "tensor":
            grads = adjoint_sweep_tensor(ctx.ansatz, psi, lam, *Ud)
        elif ctx.method == "segmented":
            grads = adjoint_sweep_segmented(ctx.ansatz, psi, lam, Ud, ctx.qdtype, ctx.lb)
        else:
            grads = adjoint_sweep(ctx.ansatz, psi, lam, Ud, scratch, ctx.qdtype)
        return (grad_e.to(torch.float64)[:, None] * grads).to(ctx.tdtype), None, None, None


def adjoint_sweep_tensor(ansatz: Ansatz, psi, lam, plan: TensorCorePlan, th64, tc_scratch) -> torch.Tensor:
    """Reverse sweep on the tensor cores; consumes psi and lambda.  Returns dE/dtheta
    [B, P] float64 (waits for the device: the status of its bounded waits is checked)."""
    lib = nat.load()
    B, P = psi.shape[0], ansatz.nparams
    grads = torch.zeros((B, P), dtype=torch.float64, device=psi.device)
    _check(lib.qsv_adjoint_backward(plan.handle, ctypes.c_void_p(psi.data_ptr()), ctypes.c_void_p(lam.data_ptr()), B,
                                    ctypes.c_void_p(th64.data_ptr()), P, ctypes.c_void_p(grads.data_ptr()), P,
                                    ctypes.c_void_p(tc_scratch.data_ptr()), tc_scratch.numel(),
                                    ctypes.c_void_p(_stream_ptr())), "adjoint_backward")
    _check(lib.qsv_adjoint_status(plan.handle), "adjoint_status")
    return grads


def adjoint_sweep(ansatz: Ansatz, psi, lam, Ud, scratch, qdtype) -> torch.Tensor:
    """Reverse sweep; consumes psi and lambda.  Returns dE/dtheta as [B, P] float64."""
    lib = nat.load()
    B = psi.shape[0]
    P = ansatz.nparams
    grads = torch.zeros((B, P), dtype=torch.float64, device=psi.device)
    st = ctypes.c_void_p(_stream_ptr())
    stride = Ud.stride(0) * Ud.element_size()
    gates = ansatz.gates()
    gp = grads.data_ptr()
    for g in range(len(gates) - 1, -1, -1):
        kind, tgt, ctl, pi = gates[g]
        gen = {RY: 1, RZ: 2}.get(kind, 0)
        gptr = ctypes.c_void_p(gp + 8 * pi) if gen else None
        _check(lib.qsv_batch_adjoint_step(ctypes.c_void_p(psi.data_ptr()), ctypes.c_void_p(lam.data_ptr()), B,
                                          ansatz.n, qdtype, tgt, ctl, ctypes.c_void_p(Ud.data_ptr() + g * stride),
                                          gen, gptr, P, ctypes.c_void_p(scratch.data_ptr()), scratch.numel(), st),
               "adjoint_step")
    return grads


def energy_and_grad(thetas: torch.Tensor, ansatz: Ansatz, statetype=torch.complex64, segmented=None):
    """Convenience: (E [B], dE/dtheta [B, P]) through the autograd Function."""
    th = thetas.detach().clone().requires_grad_(True)
    e = SumZExpectation.apply(th, ansatz, statetype, segmented)
    e.sum().backward()
    return e.detach(), th.grad
