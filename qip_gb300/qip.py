"""Graph nodes of the circuit API: registers, register splits and measurements.

The names, constructor arguments, exception types and messages, and the qid rules are
the interface of QIP's ``qip/qip.py`` (``Qubit``, ``SplitQubit``, ``Measure``,
``StochasticMeasure``, ``OpConstructor``, ``Q``), because circuits written against QIP
must build the same graph here:

* a node's qid is its creation number (``Qubit.QID`` counts them); the executor orders
  ready nodes by qid and assigns global qubit indices in that order
  (``qip/pipeline.py:111-122,203``);
* the registers cut from one node share one qid, so they stay adjacent;
* a plain ``Qubit`` feeds at most one downstream plain ``Qubit`` (no cloning).

Measurement nodes hand the state their global qubit indices as an int32 array, as the
reference's ``feed_indices`` do (``qip/qip.py:148-155,177-182``).
"""
from __future__ import annotations

from itertools import accumulate
from typing import Any, Callable, Iterable, List, Optional, Sequence, Tuple, Type, Union

import numpy

from .pipeline import PipelineObject
from .util import InitialState, flatten


def _claim_qid(requested: Optional[int]) -> int:
    """``requested`` when given (registers cut from one node share it), else the next
    creation number."""
    if requested is not None:
        return requested
    qid = Qubit.QID
    Qubit.QID = qid + 1
    return qid


def _cut(parent: "Qubit", groups: Sequence[Sequence[int]]) -> Tuple["SplitQubit", ...]:
    """One ``SplitQubit`` per group of the parent's local indices, all with one qid."""
    pieces: List[SplitQubit] = []
    for group in groups:
        pieces.append(SplitQubit(list(group), parent, qid=pieces[0].qid if pieces else None))
    return tuple(pieces)


class Qubit(PipelineObject):
    """A register of ``n`` qubits (default: the inputs' total, or 1).  As an operation
    on its inputs it is the identity: ``Qubit(a, b)`` joins two registers into one."""

    QID = 0

    def __init__(self, *inputs: "Qubit", n: int = None, qid: int = None, nosink: bool = False,
                 default: InitialState = None, quantum: bool = True, **kwargs):
        super().__init__(quantum, default=default)
        width = n if n is not None else max(1, sum(reg.n for reg in inputs))
        if type(default) == list and len(default) != 2 ** width:  # noqa: E721 (only plain lists are checked)
            raise ValueError("Default state length must be 2**n")
        if width <= 0:
            raise Exception("Number of qubits must be greater than 0")
        self.n = width
        self.qid = _claim_qid(qid)
        self.inputs = inputs
        if not nosink:
            for reg in inputs:
                reg.set_sink(self)

    def split(self, indices: Optional[Iterable[int]] = None) -> Tuple["Qubit", ...]:
        """Cut the register at the given local positions (default: where one input ends
        and the next begins; a single input gives ``(self,)``)."""
        if indices is None:
            cuts = list(accumulate(reg.n for reg in self.inputs))
            if len(cuts) == 1:
                return (self,)
        else:
            cuts = sorted(indices)
        edges = ([] if 0 in cuts else [0]) + cuts + ([] if self.n in cuts else [self.n])
        return _cut(self, [range(lo, hi) for lo, hi in zip(edges, edges[1:])])

    def extract_index(self, indices: Union[int, Iterable[int]]) -> Tuple["SplitQubit", "SplitQubit"]:
        """(the register of the given local positions, the register of the others)."""
        chosen = [indices] if isinstance(indices, int) else list(indices)
        inside = [i for i in chosen if 0 <= i < self.n]
        return _cut(self, [inside, [i for i in range(self.n) if i not in chosen]])

    def set_sink(self, sink: PipelineObject):
        """Record a consumer.  Plain ``Qubit`` consumers must all be the same register
        (they may be several cuts of it, which share its qid)."""
        clones = type(sink) == Qubit and self.sink and self.sink[0].qid != sink.qid  # noqa: E721
        if clones:
            raise Exception("Qubits may only sink to one output (no cloning)")
        self.sink += [sink]

    def __repr__(self):
        return "Q({})".format(self.qid)


class OpConstructor:
    """Callable that builds an op node; ``wrap_op_hook`` lets ``C(...)`` and contexts
    re-wrap it (None: no special handling)."""

    def __init__(self, op: Union[Type[Qubit], Callable[..., Qubit]]):
        self.op = op

    def __call__(self, *args, **kwargs) -> Qubit:
        return self.op(*args, **kwargs)

    def wrap_op_hook(self, opconstructor, consumed_inputs: Optional[Sequence[int]] = None):
        return None

    def __repr__(self):
        return "Wrap({!r})".format(self.op)


Q = OpConstructor(Qubit)


class SplitQubit(Qubit):
    """The register of some local positions (``indices``) of its parent."""

    def __init__(self, indices: Sequence[int], *inputs: Qubit, **kwargs):
        super().__init__(*inputs, n=len(indices), **kwargs)
        self.indices = indices

    def select_index(self, indices: Sequence[int]) -> Sequence[int]:
        """Global indices of this register, given the parent's."""
        return [indices[pos] for pos in self.indices]

    def __repr__(self) -> str:
        return "SplitQubit({})".format(",".join(repr(reg) for reg in self.inputs))


def _measured_indices(index_groups: Sequence[Sequence[int]]) -> numpy.ndarray:
    return numpy.asarray(flatten(index_groups), dtype=numpy.int32)


class Measure(Qubit):
    """Measures its inputs and collapses the state; classical result (outcome, p)."""

    def __init__(self, *inputs: Qubit, measure_by: int = None, nosink: bool = False):
        super().__init__(*inputs, nosink=nosink)
        self.measure = measure_by

    def feed_indices(self, state, index_groups: Sequence[Sequence[int]], n: int) -> Tuple[int, Any]:
        outcome = state.measure(_measured_indices(index_groups))
        return 0, tuple(outcome)

    def __repr__(self):
        return "M({})".format(",".join(repr(reg) for reg in self.inputs))


class StochasticMeasure(Qubit):
    """The outcome distribution of its inputs, state unchanged; with ``top_k`` the
    (outcomes, probabilities) of the k likeliest outcomes.  Classical only."""

    def __init__(self, *inputs: Qubit, nosink: bool = False, top_k: int = 0):
        super().__init__(*inputs, quantum=False, nosink=nosink)
        self.top_k = top_k

    def feed_indices(self, state, index_groups: Sequence[Sequence[int]], n: int) -> Tuple[int, object]:
        dist = state.measure_probabilities(_measured_indices(index_groups), top_k=self.top_k)
        return 0, dist[:]

    def __repr__(self) -> str:
        return "SM({})".format(",".join(repr(reg) for reg in self.inputs))
