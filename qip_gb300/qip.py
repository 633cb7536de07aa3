"""Graph nodes: qubit registers, splits and measurements (``qip/qip.py``)."""
from __future__ import annotations

from typing import Any, Callable, Iterable, Optional, Sequence, Tuple, Type, Union

import numpy

from .pipeline import PipelineObject
from .util import InitialState, flatten


class Qubit(PipelineObject):
    """A register of ``n`` qubits.  Applying a qubit node to other nodes is the
    identity on them.  Qids give creation order; global qubit indices follow it, and a
    plain ``Qubit`` may feed only one downstream ``Qubit`` (no cloning)."""

    QID = 0

    def __init__(self, *inputs: "Qubit", n: int = None, qid: int = None, nosink: bool = False,
                 default: InitialState = None, quantum: bool = True, **kwargs):
        super().__init__(quantum, default=default)
        if n is None:
            n = sum(q.n for q in inputs) if inputs else 1
        if type(default) == list and len(default) != 2 ** n:  # noqa: E721
            raise ValueError("Default state length must be 2**n")
        if n <= 0:
            raise Exception("Number of qubits must be greater than 0")
        self.n = n
        if qid is None:
            qid = Qubit.QID
            Qubit.QID += 1
        self.qid = qid
        self.inputs = inputs
        if not nosink:
            for item in inputs:
                item.set_sink(self)

    def split(self, indices: Optional[Iterable[int]] = None) -> Tuple["Qubit", ...]:
        """Split the output into registers.  Without ``indices`` the cut points are the
        input boundaries; a single input returns ``(self,)``.  Pieces share one qid."""
        if indices is None:
            cuts = []
            acc = 0
            for q in self.inputs:
                acc += q.n
                cuts.append(acc)
            if len(cuts) == 1:
                return self,
        else:
            cuts = sorted(indices)
        if 0 not in cuts:
            cuts = [0] + cuts
        if self.n not in cuts:
            cuts = cuts + [self.n]
        pieces = []
        qid = None
        for lo, hi in zip(cuts[:-1], cuts[1:]):
            sq = SplitQubit(list(range(lo, hi)), self, qid=qid)
            pieces.append(sq)
            qid = sq.qid
        return tuple(pieces)

    def extract_index(self, indices: Union[int, Iterable[int]]):
        """(selected, remaining) registers for the given local indices."""
        if isinstance(indices, int):
            indices = [indices]
        indices = list(indices)
        sq = SplitQubit([i for i in indices if 0 <= i < self.n], self)
        rest = SplitQubit([i for i in range(self.n) if i not in indices], self, qid=sq.qid)
        return sq, rest

    def set_sink(self, sink: PipelineObject):
        if type(sink) == Qubit:  # noqa: E721 - only plain Qubits enforce no-cloning
            if len(self.sink) == 0 or self.sink[0].qid == sink.qid:
                self.sink += [sink]
            else:
                raise Exception("Qubits may only sink to one output (no cloning)")
        else:
            self.sink += [sink]

    def __repr__(self):
        return "Q({})".format(self.qid)


class OpConstructor:
    def __init__(self, op: Union[Type[Qubit], Callable[..., Qubit]]):
        self.op = op

    def __call__(self, *args, **kwargs) -> Qubit:
        return self.op(*args, **kwargs)

    def wrap_op_hook(self, opconstructor, consumed_inputs: Optional[Sequence[int]] = None):
        return None

    def __repr__(self):
        return "Wrap({})".format(repr(self.op))


Q = OpConstructor(Qubit)


class SplitQubit(Qubit):
    """A register made of a subset of the parent's qubits (local indices)."""

    def __init__(self, indices: Sequence[int], *inputs: Qubit, **kwargs):
        super().__init__(*inputs, n=len(indices), **kwargs)
        self.indices = indices

    def select_index(self, indices: Sequence[int]) -> Sequence[int]:
        return [indices[i] for i in self.indices]

    def __repr__(self) -> str:
        return "SplitQubit({})".format(",".join(map(repr, self.inputs)))


class Measure(Qubit):
    """Measures and collapses its inputs; the classical result is (outcome, prob)."""

    def __init__(self, *inputs: Qubit, measure_by: int = None, nosink: bool = False):
        super().__init__(*inputs, nosink=nosink)
        self.inputs = inputs
        self.n = sum(q.n for q in inputs)
        self.measure = measure_by
        # The reference registers the sink a second time here (qip/qip.py:144-146).
        if not nosink:
            for item in inputs:
                item.set_sink(self)

    def feed_indices(self, state, index_groups: Sequence[Sequence[int]], n: int) -> Tuple[int, Any]:
        indices = numpy.array(flatten(index_groups), dtype=numpy.int32)
        bits, prob = state.measure(indices)
        return 0, (bits, prob)

    def __repr__(self):
        return "M({})".format(",".join(repr(i) for i in self.inputs))


class StochasticMeasure(Qubit):
    """Outcome distribution of its inputs without collapsing the state; with ``top_k``
    the (outcomes, probabilities) of the k most likely outcomes."""

    def __init__(self, *inputs: Qubit, nosink: bool = False, top_k: int = 0):
        super().__init__(*inputs, quantum=False, nosink=nosink)
        self.top_k = top_k
        if not nosink:
            for item in inputs:
                item.set_sink(self)

    def feed_indices(self, state, index_groups: Sequence[Sequence[int]], n: int) -> Tuple[int, object]:
        indices = numpy.array(flatten(index_groups), dtype=numpy.int32)
        probs = state.measure_probabilities(indices, top_k=self.top_k)[:]
        return 0, probs

    def __repr__(self) -> str:
        return "SM({})".format(",".join(repr(i) for i in self.inputs))
