"""QIP's wire format for operations and states (``qip/distributed/proto/messages.proto``),
read and written without a protobuf runtime, and applied to a ``GpuBackend``.

The reference's distributed client (``qip/distributed/backend.py:31-135``) serialises
every ``StateType`` call as a ``WorkerOperation`` and a worker
(``qip/distributed/worker/worker.py:57-170``) decodes it and calls its backend.  This
module is that worker's decode-and-apply step for a GB300 state: a program that speaks
the reference's messages (from a socket, a file, a queue — the transport is the
caller's) gets the same replies, computed on the device.  Only the messages that carry
states, operations and results are here; the reference's cluster bookkeeping
(``HostInformation``, ``WorkerSetup`` partners, ``SyncAccept``/``SyncState``) belongs to
its multi-node control plane.

Encoding follows proto2: a field is written only when set (an explicitly set ``False``
or empty sub-message is written), fields in number order, ``repeated int32`` unpacked
and ``repeated double [packed = true]`` packed, as the reference's generated code
writes them; readers accept both packed and unpacked repeated scalars and skip unknown
fields.  Packed doubles move through numpy without a per-element loop.
"""
from __future__ import annotations

import struct
from typing import Any, Dict, List, Optional, Tuple

import numpy

# ---- varints and field headers ----------------------------------------------------------
_VARINT, _I64, _LEN, _I32 = 0, 1, 2, 5


def _put_varint(out: bytearray, v: int) -> None:
    v &= (1 << 64) - 1  # negative int32/int64 are written as 10-byte two's complement
    while v >= 0x80:
        out.append((v & 0x7F) | 0x80)
        v >>= 7
    out.append(v)


def _get_varint(buf: bytes, pos: int) -> Tuple[int, int]:
    v = shift = 0
    while True:
        if pos >= len(buf):
            raise ValueError("truncated varint")
        b = buf[pos]
        pos += 1
        v |= (b & 0x7F) << shift
        if not b & 0x80:
            return v, pos
        shift += 7
        if shift >= 70:
            raise ValueError("varint longer than 10 bytes")


def _signed(v: int, bits: int) -> int:
    v &= (1 << bits) - 1
    return v - (1 << bits) if v >> (bits - 1) else v


def _fields(buf: bytes):
    """(field number, wire type, value) of each field; value is an int (varint), bytes
    (length-delimited) or the raw 8 / 4 bytes of a fixed field."""
    pos, end = 0, len(buf)
    while pos < end:
        key, pos = _get_varint(buf, pos)
        num, wt = key >> 3, key & 7
        if num == 0:
            raise ValueError("field number 0")
        if wt == _VARINT:
            v, pos = _get_varint(buf, pos)
        elif wt == _I64:
            v, pos = buf[pos:pos + 8], pos + 8
        elif wt == _LEN:
            n, pos = _get_varint(buf, pos)
            v, pos = buf[pos:pos + n], pos + n
        elif wt == _I32:
            v, pos = buf[pos:pos + 4], pos + 4
        else:
            raise ValueError("unsupported wire type {}".format(wt))
        if pos > end:
            raise ValueError("truncated field {}".format(num))
        yield num, wt, v


# ---- schema-driven messages -----------------------------------------------------------
class Message:
    """Base of the messages below.  ``FIELDS`` maps a field number to (name, kind,
    repeated, packed); kind is a scalar type name or a Message subclass.  Unset optional
    fields are ``None``; repeated fields are lists (packed doubles: float64 arrays)."""

    FIELDS: Dict[int, Tuple[str, Any, bool, bool]] = {}
    ONEOFS: Tuple[Tuple[str, ...], ...] = ()

    def __init__(self, **kw):
        for num, (name, kind, rep, packed) in self.FIELDS.items():
            object.__setattr__(self, name, _empty(kind, packed) if rep else None)
        for k, v in kw.items():
            setattr(self, k, v)

    def __setattr__(self, name, value):
        for group in self.ONEOFS:  # setting one member of a oneof clears the others
            if name in group and value is not None:
                for other in group:
                    if other != name:
                        object.__setattr__(self, other, None)
        object.__setattr__(self, name, value)

    def HasField(self, name: str) -> bool:
        return getattr(self, name) is not None

    def WhichOneof(self, group: int = 0) -> Optional[str]:
        for name in self.ONEOFS[group]:
            if getattr(self, name) is not None:
                return name
        return None

    def __eq__(self, other):
        if type(other) is not type(self):
            return NotImplemented
        for name, kind, rep, packed in self.FIELDS.values():
            a, b = getattr(self, name), getattr(other, name)
            if isinstance(a, numpy.ndarray) or isinstance(b, numpy.ndarray):
                if not numpy.array_equal(numpy.asarray(a), numpy.asarray(b)):
                    return False
            elif a != b:
                return False
        return True

    def __repr__(self):
        parts = ["{}={!r}".format(n, getattr(self, n)) for n, *_ in self.FIELDS.values() if getattr(self, n) is not None]
        return "{}({})".format(type(self).__name__, ", ".join(parts))

    # -- writing
    def SerializeToString(self) -> bytes:
        out = bytearray()
        self._write(out)
        return bytes(out)

    def _write(self, out: bytearray) -> None:
        for num in sorted(self.FIELDS):
            name, kind, rep, packed = self.FIELDS[num]
            v = getattr(self, name)
            if v is None:
                continue
            if rep:
                if packed:
                    if len(v):
                        data = _pack(kind, v)
                        _put_varint(out, (num << 3) | _LEN)
                        _put_varint(out, len(data))
                        out += data
                else:
                    for item in v:
                        _write_one(out, num, kind, item)
            else:
                _write_one(out, num, kind, v)

    # -- reading
    @classmethod
    def FromString(cls, buf: bytes):
        msg = cls()
        msg._merge(bytes(buf))
        return msg

    def _merge(self, buf: bytes) -> None:
        for num, wt, v in _fields(buf):
            spec = self.FIELDS.get(num)
            if spec is None:
                continue  # unknown field: skipped, as protobuf readers do
            name, kind, rep, packed = spec
            if rep and wt == _LEN and kind in _SCALAR_WT and _SCALAR_WT[kind] != _LEN:
                vals = _unpack(kind, v)  # packed form (accepted for unpacked fields too)
                cur = getattr(self, name)
                setattr(self, name, numpy.concatenate([cur, vals]) if isinstance(cur, numpy.ndarray)
                        else cur + list(vals))
                continue
            item = _read_one(kind, wt, v, num)
            if rep:
                cur = getattr(self, name)
                if isinstance(cur, numpy.ndarray):
                    setattr(self, name, numpy.append(cur, item))
                else:
                    cur.append(item)
            elif isinstance(kind, type) and getattr(self, name) is not None:
                getattr(self, name)._merge(v)  # a sub-message given twice merges
            else:
                setattr(self, name, item)


_SCALAR_WT = {"int32": _VARINT, "int64": _VARINT, "bool": _VARINT, "enum": _VARINT, "double": _I64,
              "string": _LEN}


def _empty(kind, packed):
    return numpy.empty(0, dtype=numpy.float64) if kind == "double" and packed else []


def _pack(kind, values) -> bytes:
    if kind == "double":
        return numpy.ascontiguousarray(values, dtype="<f8").tobytes()
    out = bytearray()
    for x in values:
        _put_varint(out, int(x))
    return bytes(out)


def _unpack(kind, data: bytes):
    if kind == "double":
        if len(data) % 8:
            raise ValueError("packed doubles of {} bytes".format(len(data)))
        return numpy.frombuffer(data, dtype="<f8").astype(numpy.float64)
    vals, pos = [], 0
    while pos < len(data):
        v, pos = _get_varint(data, pos)
        vals.append(_scalar(kind, v))
    return vals


def _scalar(kind, v: int):
    if kind == "int32" or kind == "enum":
        return _signed(v, 32)
    if kind == "int64":
        return _signed(v, 64)
    if kind == "bool":
        return v != 0
    raise ValueError(kind)


def _write_one(out: bytearray, num: int, kind, v) -> None:
    if isinstance(kind, type):
        data = v.SerializeToString()
        _put_varint(out, (num << 3) | _LEN)
        _put_varint(out, len(data))
        out += data
    elif kind == "double":
        _put_varint(out, (num << 3) | _I64)
        out += struct.pack("<d", float(v))
    elif kind == "string":
        data = v.encode("utf-8")
        _put_varint(out, (num << 3) | _LEN)
        _put_varint(out, len(data))
        out += data
    else:
        _put_varint(out, (num << 3) | _VARINT)
        _put_varint(out, int(v))


def _read_one(kind, wt: int, v, num: int):
    if isinstance(kind, type):
        if wt != _LEN:
            raise ValueError("field {}: message with wire type {}".format(num, wt))
        return kind.FromString(v)
    want = _SCALAR_WT[kind]
    if wt != want:
        raise ValueError("field {}: {} with wire type {}".format(num, kind, wt))
    if kind == "double":
        return struct.unpack("<d", v)[0]
    if kind == "string":
        return v.decode("utf-8")
    return _scalar(kind, v)


def _define(cls, fields, oneofs=()):
    cls.FIELDS = fields
    cls.ONEOFS = oneofs
    return cls


class ComplexVector(Message):
    pass


class ComplexMatrix(Message):
    pass


class Indices(Message):
    pass


class State(Message):
    pass


class StateSetup(Message):
    pass


class StateHandle(Message):
    pass


class WorkerPartner(Message):
    pass


class WorkerSetup(Message):
    COMPLEX128 = 0  # enum StateType


class WorkerCommand(Message):
    pass


class MatrixOp(Message):
    pass


class KronProd(Message):
    pass


class MeasureResult(Message):
    pass


class Measure(Message):
    pass


class Sync(Message):
    pass


class WorkerOperation(Message):
    pass


class WorkerConfirm(Message):
    pass


# Field numbers and types as declared in messages.proto (the format is the contract).
_define(ComplexVector, {1: ("real", "double", True, True), 2: ("imag", "double", True, True)})
_define(ComplexMatrix, {1: ("shape", "int32", True, False), 3: ("data", ComplexVector, False, False)})
_define(Indices, {1: ("index", "int32", True, False)})
_define(State, {1: ("indices", Indices, False, False), 2: ("vector", ComplexVector, False, False),
                3: ("index", "int64", False, False)}, (("vector", "index"),))
_define(StateSetup, {1: ("n", "int32", False, False), 2: ("states", State, True, False)})
_define(StateHandle, {1: ("state_handle", "string", False, False), 2: ("error_message", "string", False, False)},
        (("state_handle", "error_message"),))
_define(WorkerPartner, {1: ("job_id", "string", False, False), 2: ("addr", "string", False, False),
                        3: ("port", "int32", False, False), 4: ("state_index_start", "int64", False, False),
                        5: ("state_index_end", "int64", False, False), 6: ("output_index_start", "int64", False, False),
                        7: ("output_index_end", "int64", False, False)})
_define(WorkerSetup, {1: ("n", "int32", False, False), 2: ("states", State, True, False),
                      3: ("state_index_start", "int64", False, False), 4: ("state_index_end", "int64", False, False),
                      5: ("output_index_start", "int64", False, False), 6: ("output_index_end", "int64", False, False),
                      7: ("state_handle", "string", False, False), 8: ("partners", WorkerPartner, True, False),
                      9: ("statetype", "enum", False, False)})
_define(WorkerCommand, {1: ("setup", WorkerSetup, False, False), 2: ("shutdown", "bool", False, False)},
        (("setup", "shutdown"),))
_define(MatrixOp, {1: ("indices", Indices, False, False), 2: ("matrix", ComplexMatrix, False, False),
                   3: ("controlled_op", MatrixOp, False, False), 4: ("swap", "bool", False, False)},
        (("matrix", "controlled_op", "swap"),))
_define(KronProd, {1: ("matrices", MatrixOp, True, False)})
_define(MeasureResult, {1: ("measured_bits", "int32", False, False), 2: ("measured_prob", "double", False, False),
                        3: ("top_k_indices", Indices, False, False), 4: ("top_k_probs", "double", True, True),
                        5: ("top_k_errors", "double", True, True)})
_define(Measure, {1: ("indices", Indices, False, False), 2: ("measure_result", MeasureResult, False, False),
                  3: ("soft", "bool", False, False), 4: ("reduce", "bool", False, False),
                  5: ("top_k", "int32", False, False)})
_define(Sync, {1: ("set_up_to", "int64", False, False), 2: ("diagonal_overwrite", "bool", False, False)})
_define(WorkerOperation, {1: ("job_id", "string", False, False), 3: ("kronprod", KronProd, False, False),
                          4: ("measure", Measure, False, False), 5: ("total_prob", "bool", False, False),
                          6: ("sync", Sync, False, False), 7: ("close", "bool", False, False)},
        (("kronprod", "measure", "total_prob", "sync", "close"),))
_define(WorkerConfirm, {1: ("job_id", "string", False, False), 2: ("error_message", "string", False, False),
                        3: ("measure_result", MeasureResult, False, False)}, (("job_id", "error_message"),))


# ---- conversions (names and meaning of qip/distributed/proto/conversion.py) ------------
def indices_to_pbindices(indices, pbindices: Optional[Indices] = None) -> Indices:
    """``conversion.py:7-12``: append the indices to a (new) ``Indices``."""
    if pbindices is None:
        pbindices = Indices()
    pbindices.index.extend(int(i) for i in indices)
    return pbindices


def pbindices_to_indices(indices: Indices) -> Tuple[int, ...]:
    """``conversion.py:15-16``."""
    return tuple(indices.index)


def vec_to_pbvec(vec, pbvec: Optional[ComplexVector] = None) -> ComplexVector:
    """``conversion.py:19-25``: real and imaginary parts appended (one array operation)."""
    if pbvec is None:
        pbvec = ComplexVector()
    v = numpy.asarray(vec, dtype=numpy.complex128).reshape(-1)
    pbvec.real = numpy.concatenate([pbvec.real, v.real])
    pbvec.imag = numpy.concatenate([pbvec.imag, v.imag])
    return pbvec


def pbvec_to_vec(vec: ComplexVector, dtype=numpy.complex128) -> numpy.ndarray:
    """``conversion.py:28-29``: real + 1j * imag (parts of different lengths are an
    error, as numpy's broadcast makes them there)."""
    re, im = numpy.asarray(vec.real), numpy.asarray(vec.imag)
    if re.shape != im.shape:
        raise ValueError("ComplexVector with {} real and {} imaginary parts".format(re.size, im.size))
    out = numpy.empty(re.size, dtype=dtype)
    out.real, out.imag = re, im
    return out


def mat_to_pbmat(mat) -> ComplexMatrix:
    """``conversion.py:32-40``."""
    m = numpy.asarray(mat, dtype=numpy.complex128)
    return ComplexMatrix(shape=list(m.shape), data=vec_to_pbvec(m.reshape(-1)))


def pbmat_to_mat(mat: ComplexMatrix, dtype=numpy.complex128) -> numpy.ndarray:
    """``conversion.py:43-44``."""
    data = mat.data if mat.data is not None else ComplexVector()
    return pbvec_to_vec(data, dtype=dtype).reshape(tuple(mat.shape))


def matop_to_pbmatop(indices, mat, matop: Optional[MatrixOp] = None) -> MatrixOp:
    """``conversion.py:47-59``: a swap becomes ``swap = true``; ``CMat(m)`` a
    ``controlled_op`` holding m on the indices after the first (the control); any other
    matrix a ``ComplexMatrix``."""
    if matop is None:
        matop = MatrixOp()
    indices = tuple(indices) if not isinstance(indices, int) else (indices,)
    matop.indices = indices_to_pbindices(indices)
    kind = getattr(mat, "_kron_struct", None)
    if kind == 3:
        matop.swap = True
    elif kind == 2:
        matop.controlled_op = matop_to_pbmatop(indices[1:], mat.m)
    else:
        matop.matrix = mat_to_pbmat(mat)
    return matop


def pbmatop_to_matop(pbmatop: MatrixOp):
    """``conversion.py:62-71``: (indices, matrix) with ``SwapMat`` / ``CMat`` rebuilt.  A
    ``MatrixOp`` without an operation is an error here (the reference returns None)."""
    from .operators import CMat, SwapMat

    indices = pbindices_to_indices(pbmatop.indices if pbmatop.indices is not None else Indices())
    if pbmatop.swap is not None:
        return indices, SwapMat(int(len(indices) / 2))
    if pbmatop.matrix is not None:
        return indices, pbmat_to_mat(pbmatop.matrix)
    if pbmatop.controlled_op is not None:
        return indices, CMat(pbmatop_to_matop(pbmatop.controlled_op)[1])
    raise ValueError("MatrixOp on {} carries no operation".format(indices))


def pbstatetype_to_statetype(pbstatetype: int):
    """``conversion.py:74-77``."""
    if pbstatetype == WorkerSetup.COMPLEX128:
        return numpy.complex128
    raise ValueError("Unknown enum value: {}".format(pbstatetype))


def get_state_value(state: State):
    """A feed: its vector, or its basis index (``worker.py:172-176``)."""
    if state.vector is not None:
        return pbvec_to_vec(state.vector)
    return state.index if state.index is not None else 0


# ---- the worker's decode-and-apply step ------------------------------------------------
class WireWorker:
    """One state held on the GPU, driven by serialised ``WorkerOperation`` messages with
    the replies of a reference worker (``qip/distributed/worker/worker.py:57-170``):

    * ``kronprod``: the ``MatrixOp`` entries form one ``{indices: matrix}`` dictionary
      applied with ``kronselect_dot``; reply ``WorkerConfirm(job_id)``.
    * ``measure``: ``soft`` → ``soft_measure``, ``reduce`` → ``reduce_measure``,
      ``top_k`` → ``measure_probabilities(top_k)``, else ``measure``; a given
      ``measure_result`` supplies ``measured`` / ``measured_prob``; reply with the
      outcome and probability (top-k: indices and probabilities, under the state's job
      id as the reference's ``report_top_probs`` does).
    * ``total_prob``: reply ``measured_prob``.
    * ``sync``: this worker holds the whole state, so there is nothing to exchange;
      reply ``WorkerConfirm(job_id)``.
    * ``close``: release the state; no reply (``handle`` returns None).

    ``setup`` is a ``StateSetup`` or a ``WorkerSetup`` (or its bytes) covering the whole
    state; a ``WorkerSetup`` that gives this worker a slice of a distributed state is
    refused with ``ValueError``, since the slice exchange is the reference's multi-node
    control plane.  ``backend_constructor`` builds the state, as ``run()``'s argument of
    that name does (default ``GpuBackend.make_state``); ``backend_kw`` goes to it
    (``statetype``, ``fusion``, ...)."""

    def __init__(self, setup, job_id: str = "", backend_constructor=None, **backend_kw):
        if backend_constructor is None:
            from .backend import GpuBackend

            backend_constructor = GpuBackend.make_state

        if isinstance(setup, (bytes, bytearray, memoryview)):
            setup = StateSetup.FromString(bytes(setup))
        if isinstance(setup, WorkerSetup):
            whole = 1 << (setup.n or 0)
            for start, end in ((setup.state_index_start, setup.state_index_end),
                               (setup.output_index_start, setup.output_index_end)):
                if (start or 0) != 0 or (end is not None and end != whole):
                    raise ValueError("WorkerSetup for amplitudes [{}, {}) of 2^{}: a GPU worker holds the whole state"
                                     .format(start, end, setup.n))
            if setup.statetype is not None and "statetype" not in backend_kw:
                backend_kw["statetype"] = pbstatetype_to_statetype(setup.statetype)
            job_id = setup.state_handle or job_id
        if setup.n is None:
            raise ValueError("setup without n")
        self.job_id = job_id
        groups = [pbindices_to_indices(s.indices if s.indices is not None else Indices()) for s in setup.states]
        # An index feed is the basis vector it names (messages.proto: "all zeros except
        # this index"), as GpuBackend.make_state reads an int feed; the reference's worker
        # hands the bare int to a backend that takes vectors only.
        feeds = [get_state_value(s) for s in setup.states]
        self.state = backend_constructor(setup.n, groups, feeds, **backend_kw)
        self.closed = False

    def handle(self, operation) -> Optional[WorkerConfirm]:
        if isinstance(operation, (bytes, bytearray, memoryview)):
            operation = WorkerOperation.FromString(bytes(operation))
        if self.closed:
            raise ValueError("operation on a closed state")
        which = operation.WhichOneof()
        job = operation.job_id if operation.job_id is not None else ""
        if which == "close":
            self.state.close()
            self.closed = True
            return None
        if which == "kronprod":
            mats = {}
            for matop in operation.kronprod.matrices:
                indices, mat = pbmatop_to_matop(matop)
                mats[indices] = mat
            self.state.kronselect_dot(mats)
            return WorkerConfirm(job_id=job)
        if which == "total_prob":
            return WorkerConfirm(job_id=job, measure_result=MeasureResult(measured_prob=self.state.total_prob()))
        if which == "sync":
            return WorkerConfirm(job_id=job)
        if which == "measure":
            m = operation.measure
            indices = pbindices_to_indices(m.indices if m.indices is not None else Indices())
            res = m.measure_result
            measured = res.measured_bits if res is not None else None
            measured_prob = res.measured_prob if res is not None else None
            if m.soft:
                bits, p = self.state.soft_measure(indices, measured=measured)
            elif m.reduce:
                bits, p = self.state.reduce_measure(indices, measured=measured, measured_prob=measured_prob)
            elif m.top_k:
                top, probs = self.state.measure_probabilities(indices, top_k=m.top_k)
                out = MeasureResult(top_k_indices=indices_to_pbindices(top))
                out.top_k_probs = numpy.asarray(probs, dtype=numpy.float64)
                return WorkerConfirm(job_id=self.job_id, measure_result=out)
            else:
                bits, p = self.state.measure(indices, measured=measured, measured_prob=measured_prob)
            return WorkerConfirm(job_id=job, measure_result=MeasureResult(measured_bits=int(bits), measured_prob=float(p)))
        raise ValueError("unknown operation: {!r}".format(operation))

    def handle_bytes(self, data: bytes) -> bytes:
        """``handle`` on serialised messages; an empty reply for ``close``."""
        conf = self.handle(data)
        return b"" if conf is None else conf.SerializeToString()
