"""Quantum Fourier transform circuit (``qip/qfft.py``): per qubit an H, then controlled
phase rotations from every later qubit, then a register reversal by Swaps."""
from __future__ import annotations

from typing import MutableSequence, Tuple, Union

from .operators import C, H, Rm, Swap
from .qip import Qubit
from .qubit_util import QubitFuncWrapper
from .util import flatten


@QubitFuncWrapper.wrap
def QFFT(*inputs: Qubit, rev: bool = True) -> Union[Qubit, Tuple[Qubit, ...]]:
    qarr = flatten([inp.split(range(inp.n)) for inp in inputs])
    recQFFT(qarr)
    if rev:
        half = len(qarr) // 2
        for i in range(half):
            qarr[i], qarr[-1 - i] = Swap(qarr[i], qarr[-1 - i])
    if len(inputs) < len(qarr):
        outputs = []
        start = 0
        for qubit in inputs:
            outputs.append(Qubit(*(qarr[start:start + qubit.n])))
            start += qubit.n
    else:
        outputs = qarr
    return tuple(outputs) if len(outputs) > 1 else outputs[0]


def recQFFT(qarr: MutableSequence[Qubit], offset: int = 0):
    """Iterative form of the reference's recursion (``qip/qfft.py:33-39``): same gates in
    the same order, without Python's recursion limit at large n."""
    for off in range(offset, len(qarr)):
        qarr[off] = H(qarr[off])
        for i in range(off + 1, len(qarr)):
            m = 1 + i - off
            qarr[i], qarr[off] = C(makeR(m))(qarr[i], qarr[off])


def makeR(m: int):
    return lambda *inputs, **kwargs: Rm(m, *inputs, negate=True, **kwargs)
