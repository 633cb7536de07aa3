"""Gate catalogue (``qip/operators.py``).  Each gate turns the global indices of its
inputs into a ``{indices: matrix}`` dictionary that the backend applies with
``kronselect_dot``; controlled gates wrap their inner matrices in ``CMat`` and register
swaps use ``SwapMat``, recognised by the backend through their ``_kron_struct`` tags."""
from __future__ import annotations

from typing import Any, Callable, Mapping, Sequence, Tuple, Union, cast

import numpy

from .qip import OpConstructor, Qubit
from .qubit_util import QubitOpWrapper
from .util import IndexType, MatrixType, flatten


class MatrixOp(Qubit):
    """A gate given by matrices; ``dagger=True`` applies the conjugate transpose."""

    def __init__(self, *inputs: Qubit, **kwargs):
        super().__init__(*inputs, **kwargs)
        self.ms = None
        self.dagger = kwargs.get("dagger", False)

    def feed_indices(self, state, index_groups: Sequence[Sequence[int]], n: int) -> Tuple[int, int]:
        if self.ms is None:
            ms = self.makemats(index_groups)
            if self.dagger:
                ms = {k: v.conj().T for k, v in ms.items()}
            self.ms = ms
        state.kronselect_dot(self.ms)
        return 0, 0

    def makemats(self, index_groups: Sequence[Sequence[int]]) -> Mapping[IndexType, MatrixType]:
        raise NotImplementedError("This method should never be called.")


def _per_qubit(index_groups, mat) -> dict:
    return {i: mat for i in flatten(index_groups)}


class NotOp(MatrixOp):
    def makemats(self, index_groups):
        return _per_qubit(index_groups, numpy.array([[0.0, 1.0], [1.0, 0.0]]))

    def __repr__(self) -> str:
        return "Not({})".format(self.qid)


Not = QubitOpWrapper(NotOp)


class XOp(NotOp):
    def __repr__(self):
        return "X({})".format(self.qid)


X = QubitOpWrapper(XOp)


class YOp(MatrixOp):
    def makemats(self, index_groups):
        return _per_qubit(index_groups, numpy.array([[0.0, -1.0j], [1.0j, 0.0]]))

    def __repr__(self) -> str:
        return "Y({})".format(self.qid)


Y = QubitOpWrapper(YOp)


class ZOp(MatrixOp):
    def makemats(self, index_groups):
        return _per_qubit(index_groups, numpy.array([[1.0, 0.0], [0.0j, -1.0]]))

    def __repr__(self) -> str:
        return "Z({})".format(self.qid)


Z = QubitOpWrapper(ZOp)


class HOp(MatrixOp):
    def makemats(self, index_groups):
        return _per_qubit(index_groups, (1 / numpy.sqrt(2)) * numpy.array([[1, 1], [1, -1]]))

    def __repr__(self) -> str:
        return "H({})".format(self.qid)


H = QubitOpWrapper(HOp)


class ROp(MatrixOp):
    """Phase gate diag(1, e^{i phi})."""

    def __init__(self, phi: float, *inputs: Qubit, **kwargs):
        super().__init__(*inputs, **kwargs)
        self.exponented = numpy.exp(1.0j * phi)

    def makemats(self, index_groups):
        return _per_qubit(index_groups, numpy.array([[1, 0], [0, self.exponented]]))

    def __repr__(self) -> str:
        return "R({})".format(self.qid)


R = QubitOpWrapper(ROp)


class RmOp(ROp):
    """R(2 pi / 2^m), or R(-2 pi / 2^m) with ``negate``."""

    def __init__(self, m: int, *inputs: Qubit, negate: bool = False, **kwargs):
        super().__init__((-2 if negate else 2) * numpy.pi / pow(2.0, m), *inputs, **kwargs)
        self.m = m

    def __repr__(self) -> str:
        return "R[{}]({})".format(self.m, self.qid)


Rm = QubitOpWrapper(RmOp)


class RYOp(MatrixOp):
    """exp(-i theta Y / 2).  Not in the reference's catalogue; a plain MatrixOp."""

    def __init__(self, theta: float, *inputs: Qubit, **kwargs):
        super().__init__(*inputs, **kwargs)
        self.theta = float(theta)

    def makemats(self, index_groups):
        c, s = numpy.cos(self.theta / 2), numpy.sin(self.theta / 2)
        return _per_qubit(index_groups, numpy.array([[c, -s], [s, c]], dtype=numpy.complex128))

    def __repr__(self) -> str:
        return "RY({})".format(self.qid)


RY = QubitOpWrapper(RYOp)


class RZOp(MatrixOp):
    """exp(-i phi Z / 2).  Not in the reference's catalogue; a plain MatrixOp."""

    def __init__(self, phi: float, *inputs: Qubit, **kwargs):
        super().__init__(*inputs, **kwargs)
        self.phi = float(phi)

    def makemats(self, index_groups):
        e = numpy.exp(-0.5j * self.phi)
        return _per_qubit(index_groups, numpy.array([[e, 0], [0, numpy.conj(e)]], dtype=numpy.complex128))

    def __repr__(self) -> str:
        return "RZ({})".format(self.qid)


RZ = QubitOpWrapper(RZOp)


class UOp(MatrixOp):
    """An arbitrary 2x2 (or 2^k x 2^k on a k-qubit input) unitary."""

    def __init__(self, mat, *inputs: Qubit, **kwargs):
        super().__init__(*inputs, **kwargs)
        self.mat = numpy.asarray(mat, dtype=numpy.complex128)

    def makemats(self, index_groups):
        idx = flatten(index_groups)
        if self.mat.shape[0] == 2:
            return {i: self.mat for i in idx}
        return {tuple(idx): self.mat}

    def __repr__(self) -> str:
        return "U({})".format(self.qid)


U = QubitOpWrapper(UOp)


class SwapOp(MatrixOp):
    def __init__(self, *inputs: Qubit, **kwargs):
        super().__init__(*inputs, **kwargs)
        if len(self.inputs) != 2:
            raise Exception("Swap can only take two inputs")
        if self.inputs[0].n != self.inputs[1].n:
            raise Exception("Inputs must be of equal size {}/{}".format(self.inputs[0], self.inputs[1]))

    def makemats(self, index_groups):
        return {tuple(flatten([index_groups[0], index_groups[1]])): SwapMat(self.inputs[0].n)}

    def __repr__(self) -> str:
        return "Swap({})".format(self.qid)


Swap = QubitOpWrapper(SwapOp)


class SwapMat(object):
    """2^(2n) x 2^(2n) permutation exchanging two n-qubit registers; the backend
    recognises it by ``_kron_struct == 3`` and moves data instead of multiplying."""

    _kron_struct = 3

    def __init__(self, n: int):
        self.n = n
        self.shape = (2 ** (2 * n), 2 ** (2 * n))

    def __getitem__(self, item):
        if type(item) == tuple and len(item) == 2:  # noqa: E721
            low = (1 << self.n) - 1
            r, c = item
            return 1.0 if (r & low) == (c >> self.n) and (c & low) == (r >> self.n) else 0.0
        raise ValueError("SwapMat can only be indexed with M[i,j] not M[{}]".format(item))

    def __repr__(self):
        return "SwapMat({})".format(self.n)


def C(op: OpConstructor) -> OpConstructor:
    """Controlled version of ``op``: the first input is the (1-qubit) control."""
    if hasattr(op, "wrap_op_hook"):
        return op.wrap_op_hook(C, consumed_inputs=[0]) or QubitOpWrapper(COp, op)
    return QubitOpWrapper(COp, op)


def _check_control_inputs(inputs: Sequence[Qubit]) -> None:
    """Argument rules of a controlled op (messages as QIP's, which callers catch)."""
    if len(inputs) < 2:
        raise ValueError("Not enough input values given.")
    if inputs[0].n != 1:
        raise ValueError("Control bit can only be of size n=1")
    if len(set(inputs)) != len(inputs):
        raise ValueError("Cannot have repeated qubits in COp")


class COp(MatrixOp):
    """``op`` controlled by the first input (a single qubit, active at |1>).

    The wrapped op is built on the other inputs without registering itself as their
    consumer or splitting its output; this node takes over its qid, so it runs where
    the plain op would.  Its dictionary is the op's, each key prefixed by the control
    index and each matrix wrapped in ``CMat`` (nested ``C(C(...))`` nest CMats)."""

    def __init__(self, op: OpConstructor, *inputs: Qubit, **kwargs):
        _check_control_inputs(inputs)
        # A fresh dict per call: the caller's kwargs go unchanged to this node.
        self.op = cast(MatrixOp, self.make_op(op, inputs, {**kwargs, "nosink": True, "nosplit": True}))
        if not isinstance(self.op, MatrixOp):
            raise ValueError("C(Op) may only be applied to matrix ops and swaps, not {}".format(type(self.op)))
        super().__init__(*inputs, qid=self.op.qid, **kwargs)

    def make_op(self, op: OpConstructor, inputs: Sequence[Qubit], nkwargs: Mapping[str, Any]):
        """The controlled op, on every input but the control."""
        target_regs = inputs[1:]
        return op(*target_regs, **nkwargs)

    def makemats(self, index_groups):
        control = list(index_groups[0])
        return {tuple(control + list(flatten([key]))): CMat(m)
                for key, m in self.op.makemats(index_groups[1:]).items()}

    def __repr__(self):
        return "C{}".format(self.op)


def _as_dense(m) -> numpy.ndarray:
    """A numpy matrix of ``m``: an array, a ``CMat`` or a ``SwapMat``."""
    if isinstance(m, CMat):
        return m.numpy()
    if isinstance(m, SwapMat):
        rows = numpy.arange(m.shape[0])
        low = (1 << m.n) - 1
        out = numpy.zeros(m.shape, dtype=numpy.complex128)
        out[rows, ((rows & low) << m.n) | (rows >> m.n)] = 1.0
        return out
    return numpy.asarray(m)


class CMat(object):
    """Block-diagonal matrix diag(I, m) of twice m's size: identity while the leading
    (control) index bit is 0, ``m`` when it is 1.  The backend recognises it by
    ``_kron_struct == 2`` and visits only the control-satisfied half."""

    _kron_struct = 2

    def __init__(self, mat):
        self.m = numpy.array(mat) if type(mat) == list else mat  # noqa: E721 (other sequences are kept as given)
        rows, cols = self.m.shape[0], self.m.shape[1]
        self.shape = (2 * rows, 2 * cols)

    def __getitem__(self, item):
        if not (type(item) == tuple and len(item) == 2):  # noqa: E721
            raise ValueError("CMat can only be indexed with M[i,j] not M[{}]".format(item))
        r, c = item
        hr, hc = self.shape[0] // 2, self.shape[1] // 2
        if (r >= hr) != (c >= hc):
            return 0.0  # off-diagonal blocks
        if r >= hr:
            return self.m[r - hr, c - hc]
        return 1.0 if r == c else 0.0

    def conj(self):
        """Element-wise conjugate (a CMat again)."""
        return CMat(self.m.conj())

    @property
    def T(self):
        """Transpose (a CMat again)."""
        return CMat(self.m.T)

    def numpy(self) -> numpy.ndarray:
        inner = _as_dense(self.m).astype(numpy.complex128)
        hr, hc = inner.shape
        out = numpy.zeros(self.shape, dtype=numpy.complex128)
        out[:hr, :hc] = numpy.eye(hr, hc)
        out[hr:, hc:] = inner
        return out


class FOp(Qubit):
    """|x>|q> -> |x>|f(x) xor q> for registers (reg1, reg2)."""

    def __init__(self, func: Callable[[int], int], reg1: Qubit, reg2: Qubit, **kwargs):
        super().__init__(reg1, reg2, **kwargs)
        self.func = func
        self.reg1 = reg1
        self.reg2 = reg2

    def feed_indices(self, state, index_groups: Sequence[Sequence[int]], n: int) -> Tuple[int, int]:
        reg1 = numpy.array(index_groups[0], dtype=numpy.int32)
        reg2 = numpy.array(index_groups[1], dtype=numpy.int32)
        state.func_apply(reg1, reg2, self.func)
        return 0, 0

    def __repr__(self) -> str:
        return "F({}, {})".format(self.reg1, self.reg2)


F = QubitOpWrapper(FOp)
