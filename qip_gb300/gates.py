"""Host-side translation of a ``kronselect_dot`` dictionary into device operations.

The reference applies ``{indices: matrix}`` dictionaries with one generic kernel that
enumerates, for every output amplitude, all 2^|union of indices| input columns and
multiplies the matching sub-matrix entries (``qip/ext/kronprod.pyx:155-197``, entry
rules ``kronprod.pyx:203-235``).  Here each entry becomes one structured operation:

* ``CMat`` nesting (``qip/operators.py:233-268``) becomes explicit controls — the first
  indices of the entry, active when 1 (``kronprod.pyx:215-225``);
* ``SwapMat`` (``qip/operators.py:157-179``, ``kronprod.pyx:227-231``) becomes a
  register exchange (pure data movement);
* a numpy matrix becomes a diagonal, monomial (one non-zero per row) or dense
  operation, whichever matches its structure.

Entries of one dictionary act as a Kronecker product.  When their qubit sets are
disjoint, or overlap only in qubits that are controls of every entry that names them,
applying them one after another is the same operator.  Other overlaps keep the
reference's entry-product semantics by expanding the dictionary into one dense
matrix on the union of its indices.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Dict, List, Mapping, Sequence, Tuple

import numpy

KRON_CMAT = 2  # ``_kron_struct`` tag of CMat (qip/operators.py:234)
KRON_SWAP = 3  # ``_kron_struct`` tag of SwapMat (qip/operators.py:159)
MAX_DENSE = 5  # widest dense matrix the per-gate kernel takes


@dataclass
class GateOp:
    """One structured operation on a state.

    kind: ``dense`` (mat 2^k x 2^k), ``diag`` (diag vector 2^k), ``mono``
    (perm/phase, out[r] = phase[r] * in[perm[r]]) or ``swap`` (register a <-> b).
    ``targets``/``controls`` are global qubit indices (0 = most significant bit);
    targets[0] is the most significant bit of the matrix index.
    """

    kind: str
    targets: Tuple[int, ...]
    controls: Tuple[int, ...] = ()
    mat: Any = None
    perm: Any = None
    swap_b: Tuple[int, ...] = ()
    qubits: frozenset = field(default_factory=frozenset)
    qmask: int = 0  # the qubits as a bit mask (bit q <-> qubit q), for the planner

    def __post_init__(self):
        self.qubits = frozenset(self.targets) | frozenset(self.controls) | frozenset(self.swap_b)
        m = 0
        for q in self.qubits:
            m |= 1 << int(q)
        self.qmask = m

    @property
    def width(self) -> int:
        return len(self.qubits)

    def amp_update_weight(self) -> float:
        """Fraction of the 2^n amplitudes one application rewrites (2^-controls)."""
        return 2.0 ** (-len(self.controls))

    def matrix(self) -> Tuple[Tuple[int, ...], numpy.ndarray]:
        """Dense matrix of the whole operation on ``order`` (controls first); read-only
        for callers.  Copies of a cached decomposition build it once (``shared``)."""
        shared = getattr(self, "shared", None)
        if shared is None:
            return self._dense()
        hit = shared.get("matrix")
        if hit is None:
            hit = shared["matrix"] = self._dense()
        return hit

    def _dense(self) -> Tuple[Tuple[int, ...], numpy.ndarray]:
        if self.kind == "swap":
            a, b = self.targets, self.swap_b
            m = len(a)
            core_q = tuple(a) + tuple(b)
            dim = 1 << (2 * m)
            core = numpy.zeros((dim, dim), dtype=numpy.complex128)
            for col in range(dim):
                x, y = col >> m, col & ((1 << m) - 1)
                core[(y << m) | x, col] = 1.0
        elif self.kind == "dense":
            core_q, core = tuple(self.targets), numpy.asarray(self.mat, dtype=numpy.complex128)
        elif self.kind == "diag":
            core_q, core = tuple(self.targets), numpy.diag(numpy.asarray(self.mat, dtype=numpy.complex128))
        elif self.kind == "mono":
            d = len(self.perm)
            core = numpy.zeros((d, d), dtype=numpy.complex128)
            core[numpy.arange(d), numpy.asarray(self.perm)] = numpy.asarray(self.mat, dtype=numpy.complex128)
            core_q = tuple(self.targets)
        else:
            raise ValueError(self.kind)
        c = len(self.controls)
        if c == 0:
            return core_q, core
        dim = core.shape[0] << c
        full = numpy.eye(dim, dtype=numpy.complex128)
        full[dim - core.shape[0]:, dim - core.shape[0]:] = core
        return tuple(self.controls) + core_q, full


def normalize_mats(mats: Mapping[Any, Any]) -> Dict[Tuple[int, ...], Any]:
    """Key/shape validation of ``qip.util.kronselect_dot`` (``qip/util.py:35-58``):
    int keys become 1-tuples, list matrices become numpy arrays, and the square
    sub-matrix must be 2^len(indices) wide."""
    out: Dict[Tuple[int, ...], Any] = {}
    for indices in mats:
        m = mats[indices]
        if type(indices) == tuple:  # noqa: E721 - the reference checks exact types
            key = indices
        elif type(indices) == int:  # noqa: E721
            key = (indices,)
        else:
            raise Exception("Type of indices must be tuple: {}".format(indices))
        if type(m) == list:  # noqa: E721
            m = numpy.array(m)
        n = len(key)
        if 2 ** n != m.shape[0] or 2 ** n != m.shape[1]:
            raise Exception("Shape of square submatrix must equal 2**(number of indices): "
                            "{}: {}".format(indices, m))
        out[key] = m
    return out


def classify_matrix(targets: Tuple[int, ...], controls: Tuple[int, ...], m: numpy.ndarray) -> List[GateOp]:
    m = numpy.asarray(m)
    if m.dtype.kind not in "biufc":
        raise ValueError("Cannot pass matrices which are not numpy, SwapMat, or CMat")
    m = m.astype(numpy.complex128, copy=False)
    d = m.shape[0]
    off = m.copy()
    off[numpy.arange(d), numpy.arange(d)] = 0
    if not off.any():
        diag = numpy.ascontiguousarray(numpy.diag(m))
        if numpy.all(diag == 1.0):
            return []  # identity: nothing to do
        return [GateOp("diag", targets, controls, mat=diag)]
    nz = m != 0
    if len(targets) <= 3 and numpy.all(nz.sum(axis=1) == 1) and numpy.all(nz.sum(axis=0) == 1):
        perm = numpy.argmax(nz, axis=1).astype(numpy.int32)
        phase = m[numpy.arange(d), perm]
        return [GateOp("mono", targets, controls, mat=numpy.ascontiguousarray(phase), perm=perm)]
    if len(targets) > MAX_DENSE:
        raise NotImplementedError(f"dense matrix on {len(targets)} qubits (max {MAX_DENSE})")
    return [GateOp("dense", targets, controls, mat=numpy.ascontiguousarray(m))]


def _entry_ops(indices: Tuple[int, ...], m: Any) -> List[GateOp]:
    controls: List[int] = []
    while getattr(m, "_kron_struct", None) == KRON_CMAT:
        controls.append(indices[len(controls)])
        m = m.m
    rest = tuple(indices[len(controls):])
    tag = getattr(m, "_kron_struct", None)
    if tag == KRON_SWAP:
        k = int(m.n)
        if len(rest) != 2 * k:
            raise Exception("SwapMat({}) needs {} indices, got {}".format(k, 2 * k, rest))
        return [GateOp("swap", rest[:k], tuple(controls), swap_b=rest[k:])]
    if tag is None and isinstance(m, numpy.ndarray):
        return classify_matrix(rest, tuple(controls), m)
    raise ValueError("Cannot pass matrices which are not numpy, SwapMat, or CMat")


def _entry_value(m: Any, i: int, j: int) -> complex:
    """Entry (i, j) of a numpy / CMat / SwapMat, as ``calc_mat_entry`` defines it."""
    tag = getattr(m, "_kron_struct", None)
    if tag == KRON_CMAT:
        half = m.shape[0] >> 1
        if i < half and j < half:
            return 1.0 if i == j else 0.0
        if i >= half and j >= half:
            return _entry_value(m.m, i - half, j - half)
        return 0.0
    if tag == KRON_SWAP:
        k = m.n
        low = (1 << k) - 1
        return 1.0 if (i & low) == (j >> k) and (j & low) == (i >> k) else 0.0
    return complex(m[i, j])


def union_matrix(entries: Dict[Tuple[int, ...], Any]) -> Tuple[Tuple[int, ...], numpy.ndarray]:
    """Dense matrix of a whole dictionary on the sorted union of its indices, with the
    reference's product-of-entries rule (``kronprod.pyx:164-196``)."""
    flat = tuple(sorted({q for key in entries for q in key}))
    u = len(flat)
    if u > MAX_DENSE:
        raise NotImplementedError(f"overlapping kron entries spanning {u} qubits")
    where = {q: u - 1 - i for i, q in enumerate(flat)}
    dim = 1 << u
    out = numpy.ones((dim, dim), dtype=numpy.complex128)
    rows = numpy.arange(dim)
    for key, m in entries.items():
        L = len(key)
        sub = numpy.zeros(dim, dtype=numpy.int64)
        for pos, q in enumerate(key):
            sub |= ((rows >> where[q]) & 1) << (L - 1 - pos)
        dense = numpy.empty((1 << L, 1 << L), dtype=numpy.complex128)
        for i in range(1 << L):
            for j in range(1 << L):
                dense[i, j] = _entry_value(m, i, j)
        out *= dense[sub[:, None], sub[None, :]]
    return flat, out


def _mat_key(m: Any):
    """Content key of a matrix value (numpy, CMat, SwapMat), or None when it has none."""
    tag = getattr(m, "_kron_struct", None)
    if tag == KRON_CMAT:
        inner = _mat_key(m.m)
        return None if inner is None else ("C", inner)
    if tag == KRON_SWAP:
        return ("S", int(m.n))
    if type(m) is numpy.ndarray and m.dtype.kind in "biufc" and m.size <= 1024:
        return (m.dtype.str, m.shape, m.tobytes())
    return None


_CACHE_MAX = 4096
_cache: Dict[Any, List[GateOp]] = {}


def decompose(mats: Mapping[Any, Any], copy: bool = True) -> List[GateOp]:
    """Turn one ``kronselect_dot`` dictionary into a list of GateOps (in order).

    Graph ops hand the same matrices to every run (the reference caches them per node,
    ``qip/operators.py:17-18``), so results are cached by content: the dictionary's keys
    and each matrix's dtype, shape and bytes.  A hit returns fresh copies of the cached
    ops (callers own what they get; the matrix arrays are shared and never written);
    ``copy=False`` returns the cached ops themselves, for callers that only read them
    (the backend's gate path)."""
    key = []
    for indices in mats:
        if type(indices) not in (tuple, int):
            key = None
            break
        mk = _mat_key(mats[indices])
        if mk is None:
            key = None
            break
        key.append((indices, mk))
    if key is not None:
        key = tuple(key)
        hit = _cache.get(key)
        if hit is not None:
            return [_clone(op) for op in hit] if copy else hit
    ops = _decompose(mats)
    if key is not None:
        if len(_cache) >= _CACHE_MAX:
            _cache.clear()
        for op in ops:
            # The cached op must not alias the caller's arrays, which may change later.
            if op.mat is not None:
                op.mat = numpy.array(op.mat, copy=True)
            if op.perm is not None:
                op.perm = numpy.array(op.perm, copy=True)
            op.finite = op.mat is None or bool(numpy.all(numpy.isfinite(op.mat)))
            op.shared = {}  # per-template data the copies share (the backend's call arguments)
        _cache[key] = ops
        return [_clone(op) for op in ops] if copy else ops
    return ops


def _clone(op: GateOp) -> GateOp:
    """A shallow copy of a cached op (its attributes, the arrays and ``shared`` shared)."""
    new = object.__new__(GateOp)
    new.__dict__.update(op.__dict__)
    return new


def _decompose(mats: Mapping[Any, Any]) -> List[GateOp]:
    entries = normalize_mats(mats)
    ops_per_entry = [(_entry_ops(key, m), key, m) for key, m in entries.items()]
    if len(entries) > 1:
        # Qubits named by more than one entry must be controls of every entry naming them.
        owners: Dict[int, List[Tuple[List[GateOp], Tuple[int, ...]]]] = {}
        for ops, key, _ in ops_per_entry:
            for q in key:
                owners.setdefault(q, []).append((ops, key))
        for q, lst in owners.items():
            if len(lst) < 2:
                continue
            for ops, key in lst:
                ok = all(q in op.controls for op in ops) if ops else True
                if not ok or not ops:
                    qubits, dense = union_matrix(entries)
                    return classify_matrix(qubits, (), dense)
    out: List[GateOp] = []
    for ops, _, _ in ops_per_entry:
        out.extend(ops)
    return out
