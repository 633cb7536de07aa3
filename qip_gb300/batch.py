"""Many independent circuits in one persistent GPU launch (complex64).

Each circuit is a list of ``kronselect_dot`` dictionaries on n qubits (3 <= n <= 24)
with a product-state input (one 2-vector per qubit).  The gates are encoded into the
fixed records of ``include/qsv.h`` (``qsv_gate_rec``): dense single-qubit matrices,
single-qubit phases, X, controlled X and controlled Swap — the gate set of the batched
workload (H, X, Rm, CNOT, C(Swap), Haar 2x2).  Circuits are ordered for the device work
queues (the largest streamed ones first, each on a whole cluster of CTAs; then the rest
longest first); results come back in the caller's order.
"""
from __future__ import annotations

import ctypes
from typing import List, Sequence

import numpy

from . import _native as nat
from .gates import decompose

GATE_DTYPE = numpy.dtype([("kind", "<i4"), ("q0", "<i4"), ("q1", "<i4"), ("q2", "<i4"), ("m", "<f4", (8,))])
CIRC_DTYPE = numpy.dtype([("n", "<i4"), ("ngates", "<i4"), ("gate_offset", "<i8"), ("state_offset", "<i8"),
                          ("feed_offset", "<i8")])
assert GATE_DTYPE.itemsize == 48 and CIRC_DTYPE.itemsize == 32

DENSE1, PHASE1, X, CX, CSWAP = 0, 1, 2, 3, 4
SMEM_QUBITS = 14  # circuits up to this size run whole in one CTA's shared memory


def encode_gates(mats_list: Sequence[dict]) -> numpy.ndarray:
    """Records of one circuit's gates; raises for gates outside the supported set."""
    recs = []
    for mats in mats_list:
        for op in decompose(mats):
            r = numpy.zeros((), dtype=GATE_DTYPE)
            if op.kind == "swap" and len(op.targets) == 1 and len(op.controls) == 1:
                r["kind"], r["q0"], r["q1"], r["q2"] = CSWAP, op.controls[0], op.targets[0], op.swap_b[0]
            elif op.kind == "swap" and len(op.targets) == 1 and not op.controls:
                # A swap is three CNOTs.
                a, b = op.targets[0], op.swap_b[0]
                for t, c in ((a, b), (b, a), (a, b)):
                    rr = numpy.zeros((), dtype=GATE_DTYPE)
                    rr["kind"], rr["q0"], rr["q1"] = CX, t, c
                    recs.append(rr)
                continue
            elif op.kind == "mono" and len(op.targets) == 1 and len(op.controls) <= 1 and \
                    list(op.perm) == [1, 0] and numpy.all(numpy.asarray(op.mat) == 1):
                if op.controls:
                    r["kind"], r["q0"], r["q1"] = CX, op.targets[0], op.controls[0]
                else:
                    r["kind"], r["q0"] = X, op.targets[0]
            elif op.kind == "diag" and len(op.targets) == 1 and not op.controls and op.mat[0] == 1:
                r["kind"], r["q0"] = PHASE1, op.targets[0]
                r["m"][0], r["m"][1] = op.mat[1].real, op.mat[1].imag
            elif len(op.targets) == 1 and not op.controls and op.kind in ("dense", "diag", "mono"):
                _, m = op.matrix()
                r["kind"], r["q0"] = DENSE1, op.targets[0]
                r["m"][:] = numpy.asarray(m, dtype=numpy.complex64).reshape(-1).view(numpy.float32)
            else:
                raise NotImplementedError(f"gate {op.kind} on {op.targets} with controls {op.controls}")
            recs.append(r)
    return numpy.array(recs, dtype=GATE_DTYPE) if recs else numpy.zeros(0, dtype=GATE_DTYPE)


class CircuitBatch:
    """Device-resident batch: tables uploaded once; ``run`` replays one graph launch."""

    def __init__(self, circuits: Sequence[Sequence[dict]], feeds: Sequence[Sequence[numpy.ndarray]],
                 sizes: Sequence[int]):
        self._lib = nat.load()
        count = len(circuits)
        encoded = [encode_gates(c) for c in circuits]
        cost = [float(2 ** sizes[i]) * max(1, len(encoded[i])) for i in range(count)]
        # Device slot -> caller index: streamed circuits (n > 14) first, largest n first
        # (the library runs the leading ones with n >= 14 + log2(2 * cluster size) on a
        # whole cluster each), then the rest longest first.
        self.order = sorted(range(count), key=lambda i: (0, -sizes[i], -cost[i]) if sizes[i] > SMEM_QUBITS
                            else (1, 0, -cost[i]))
        self.slot_of = {c: s for s, c in enumerate(self.order)}
        circs = numpy.zeros(count, dtype=CIRC_DTYPE)
        gate_chunks, feed_chunks = [], []
        goff = soff = foff = 0
        for s, i in enumerate(self.order):
            n = int(sizes[i])
            circs[s] = (n, len(encoded[i]), goff, soff, foff)
            gate_chunks.append(encoded[i])
            f = numpy.asarray(feeds[i], dtype=numpy.complex64).reshape(n, 2)
            feed_chunks.append(f.reshape(-1))
            goff += len(encoded[i])
            soff += 2 ** n
            foff += 2 * n
        self.gates = numpy.ascontiguousarray(numpy.concatenate(gate_chunks)) if goff else numpy.zeros(1, GATE_DTYPE)
        self.circs = circs
        self.feeds = numpy.ascontiguousarray(numpy.concatenate(feed_chunks))
        self.sizes = [int(x) for x in sizes]
        self.ngates = goff
        self.total_amps = soff
        h = ctypes.c_void_p()
        nat.check(self._lib.qsv_circuits_create(self.gates.ctypes.data_as(ctypes.c_void_p), goff,
                                                self.circs.ctypes.data_as(ctypes.c_void_p), count,
                                                self.feeds.ctypes.data_as(ctypes.c_void_p), self.feeds.shape[0],
                                                ctypes.byref(h)), None, "circuits_create")
        self._h = h

    def run(self, stream_ptr: int) -> None:
        nat.check(self._lib.qsv_circuits_run(self._h, ctypes.c_void_p(stream_ptr)), None, "circuits_run")

    def state(self, index: int) -> numpy.ndarray:
        out = numpy.empty(2 ** self.sizes[index], dtype=numpy.complex64)
        nat.check(self._lib.qsv_circuits_read(self._h, self.slot_of[index], out.ctypes.data_as(ctypes.c_void_p)),
                  None, "circuits_read")
        return out

    def latencies_ns(self) -> numpy.ndarray:
        """Per-circuit device time (end - start) in ns, in the caller's order."""
        t = numpy.empty(2 * len(self.order), dtype=numpy.uint64)
        nat.check(self._lib.qsv_circuits_times(self._h, t.ctypes.data_as(ctypes.c_void_p)), None, "circuits_times")
        t = t.reshape(-1, 2).astype(numpy.int64)
        lat = t[:, 1] - t[:, 0]
        out = numpy.empty_like(lat)
        for s, i in enumerate(self.order):
            out[i] = lat[s]
        return out

    def close(self):
        h, self._h = getattr(self, "_h", None), None
        if h:
            self._lib.qsv_circuits_destroy(h)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def random_batch(count: int, seed: int = 4096, nmin: int = 8, nmax: int = 20, dmin: int = 20, dmax: int = 100):
    """The batched workload: n ~ U[nmin, nmax], depth ~ U[dmin, dmax], random gates from
    {H, X, Rm, CNOT, C(Swap), Haar 2x2}, Haar-random single-qubit product feeds."""
    from .circuits import random_circuit, random_product_feed

    rng = numpy.random.default_rng(seed)
    circuits, feeds, sizes = [], [], []
    for _ in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        depth = int(rng.integers(dmin, dmax + 1))
        circuits.append(random_circuit(rng, n, depth))
        feeds.append(random_product_feed(rng, n))
        sizes.append(n)
    return circuits, feeds, sizes
