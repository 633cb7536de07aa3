"""Reusable page-locked host arrays for state readback.

``GpuBackend.get_state`` returns a numpy array backed by page-locked memory
(``qsv_host_alloc``): the device-to-host copy is then one DMA, with neither a staging
copy nor first-touch page faults (which cost as much as the copy for a fresh 2 GiB
array).  Buffers are pooled by size.  A buffer goes back to the pool only when no array
refers to it any more (the arrays keep their owner alive through ``.base``), so an
array handed to a caller is never overwritten behind its back.  States larger than
``PINNED_LIMIT_BYTES`` (or ``QSV_PINNED_READBACK=0``) get ordinary numpy memory.
"""
from __future__ import annotations

import ctypes
import os
import threading
from typing import Dict, List

import numpy

from . import _native as nat

PINNED_LIMIT_BYTES = 8 << 30
POOL_PER_SIZE = 2

_lock = threading.Lock()
_free: Dict[int, List[int]] = {}
# How each pinned request was served: a pooled buffer reused, a new buffer allocated, or
# ordinary numpy memory because the page-locked allocation failed.
counts = {"reused": 0, "allocated": 0, "alloc_failed": 0}


class _PinnedOwner:
    """Owns one page-locked buffer; numpy arrays view it through __array_interface__."""

    def __init__(self, ptr: int, nbytes: int, shape, dtype: numpy.dtype):
        self.ptr = ptr
        self.nbytes = nbytes
        self.__array_interface__ = {"data": (ptr, False), "shape": tuple(shape), "typestr": dtype.str,
                                    "version": 3}

    def __del__(self):
        try:
            _release(self.ptr, self.nbytes)
        except Exception:
            pass


def _release(ptr: int, nbytes: int) -> None:
    with _lock:
        lst = _free.setdefault(nbytes, [])
        if len(lst) < POOL_PER_SIZE:
            lst.append(ptr)
            return
    nat.load().qsv_host_free(ctypes.c_void_p(ptr))


def is_pooled(arr) -> bool:
    """True when ``arr`` is a view of one of this pool's page-locked buffers."""
    base = arr
    while base is not None and not isinstance(base, _PinnedOwner):
        base = getattr(base, "base", None)
    return base is not None


def enabled() -> bool:
    return os.environ.get("QSV_PINNED_READBACK", "1") != "0"


def empty(count: int, dtype) -> numpy.ndarray:
    """An uninitialised 1-D array of ``count`` elements, page-locked when allowed."""
    dtype = numpy.dtype(dtype)
    nbytes = int(count) * dtype.itemsize
    if nbytes == 0 or nbytes > PINNED_LIMIT_BYTES or not enabled():
        return numpy.empty(count, dtype=dtype)
    with _lock:
        lst = _free.get(nbytes)
        ptr = lst.pop() if lst else None
        if ptr is not None:
            counts["reused"] += 1
    if ptr is None:
        p = ctypes.c_void_p()
        if nat.load().qsv_host_alloc(nbytes, ctypes.byref(p)) != nat.QSV_OK or not p.value:
            counts["alloc_failed"] += 1
            return numpy.empty(count, dtype=dtype)
        counts["allocated"] += 1
        ptr = p.value
    return numpy.asarray(_PinnedOwner(ptr, nbytes, (count,), dtype))
