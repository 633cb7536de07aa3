"""Small host helpers of the QIP API surface (``qip/util.py``): type aliases, bit-array
conversion, flattening and state printing.  The reference's CPU kron kernels of that
module (``kronselect_dot``/``dot_loop``) are not part of this package: gates run on
the GPU through ``GpuBackend``."""
from __future__ import annotations

import collections.abc
from typing import Any, Iterable, List, MutableSequence, Sequence, Tuple, TypeVar, Union

import numpy

InitialState = Union[MutableSequence[complex], int, numpy.ndarray]
IndexType = Union[int, Tuple[int, ...]]
MatrixType = Any
T = TypeVar("T")


def flatten(lst: Iterable[Any]) -> List[Any]:
    """One level of flattening: iterable items are expanded, others kept
    (``qip/util.py:152-154``)."""
    out: List[Any] = []
    for item in lst:
        if isinstance(item, collections.abc.Iterable):
            out.extend(item)
        else:
            out.append(item)
    return out


def uint_to_bitarray(num: int, n: int) -> List[int]:
    """Bits of ``num`` as a length-n list, most significant first."""
    return [(num >> (n - 1 - i)) & 1 for i in range(n)]


def bitarray_to_uint(bits: Sequence[int]) -> int:
    """Inverse of ``uint_to_bitarray`` (first element is the MSB)."""
    v = 0
    for b in bits:
        v = (v << 1) | (1 if b else 0)
    return v


def qubit_index_notation(i: int, *qns: int, n: int = None) -> List[int]:
    """Split basis index i into per-register values (registers of qns qubits, first
    register most significant)."""
    if n is None:
        n = sum(qns)
    out = []
    shift = n
    for size in qns:
        shift -= size
        out.append((i >> shift) & ((1 << size) - 1))
    return out


def gen_qubit_prints(state: Sequence[complex], *qs: Union[int, Any]):
    """Yield ``|a,b,...> = amplitude`` lines for the non-zero amplitudes."""
    sizes = [q if isinstance(q, int) else q.n for q in qs]
    n = sum(sizes)
    for i, amp in enumerate(state):
        if amp == 0:
            continue
        yield "|" + ",".join(map(str, qubit_index_notation(i, *sizes, n=n))) + "> = {}".format(amp)
