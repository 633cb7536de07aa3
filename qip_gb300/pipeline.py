"""Graph executor: turns a DAG of qubit nodes into backend calls.

Same contract as the reference executor (``qip/pipeline.py``):

* ``run`` resolves the leaf qubits, assigns global qubit indices in creation (qid)
  order, builds the state through ``backend_constructor`` and walks the graph;
* nodes run in qid order among those whose inputs are complete; equal qids keep the
  order in which they became ready (the reference re-sorts a list stably,
  ``qip/pipeline.py:202-204``; here a heap keyed by (qid, arrival) gives the same order
  in O(log n) per node);
* every node's ``feed`` result lands in the classic map when it is not None.

The default backend is the GB300 ``GpuBackend``.
"""
from __future__ import annotations

import heapq
import itertools
import os
from collections import OrderedDict
from typing import Any, Callable, Dict, List, Mapping, Sequence, Set, Tuple, Type, Union

import numpy

from .util import InitialState, flatten


class PipelineObject(object):
    """Base of every graph node (``qip/pipeline.py:7-68``)."""

    def __init__(self, quantum: bool, default: InitialState = None, n: int = 0):
        self.quantum = quantum
        self.inputs = []
        self.sink = []
        self.default = default
        self.n = n

    def run(self, feed: Mapping["PipelineObject", InitialState] = None, **kwargs):
        return run(self, feed=feed, **kwargs)

    def feed(self, state, qbitindex: Mapping["PipelineObject", Sequence[int]], n: int) -> Tuple[int, object]:
        return self.feed_indices(state, [qbitindex[q] for q in self.inputs], n)

    def feed_indices(self, state, index_groups: Sequence[Sequence[int]], n: int) -> Tuple[int, Any]:
        """Operate on the state; returns (qubits removed, classical annotation)."""
        return 0, 0

    def select_index(self, indices: Sequence[int]) -> Sequence[int]:
        return indices

    def remap_index(self, index_map: Mapping["PipelineObject", int], n: int) -> Mapping["PipelineObject", int]:
        return index_map

    def set_sink(self, sink: "PipelineObject"):
        self.sink += [sink]

    def get_inputs(self) -> Sequence["PipelineObject"]:
        return self.inputs


def _default_backend():
    from .backend import GpuBackend

    return GpuBackend.make_state


def run(*args: PipelineObject,
        feed: Mapping[Union[PipelineObject, Tuple[PipelineObject, ...]], InitialState] = None,
        strict: bool = False,
        backend_constructor: Callable = None,
        statetype: Type = numpy.complex128,
        **kwargs):
    """Run the graph ending in ``args`` (``qip/pipeline.py:71-135``).

    :param feed: {qubit or tuple of qubits: initial vector}
    :param strict: every leaf qubit must be fed
    :param backend_constructor: ``make_state``-style factory (default GpuBackend)
    :param statetype: numpy complex dtype of the state
    :return: (state array, {node: classical result})
    """
    feed = {} if feed is None else {(k if type(k) == tuple else (k,)): feed[k] for k in feed}  # noqa: E721
    fed_qubits = list(flatten(feed.keys()))
    if backend_constructor is None:
        backend_constructor = _default_backend()

    walk_key = (args, tuple(feed.keys()))
    walk = _WALKS.get(walk_key)
    if walk is not None:
        _WALKS.move_to_end(walk_key)
        frontier, graphnodes = walk.frontier, walk.graphnodes
    else:
        frontier, graphnodes = get_deps(*args, feed=feed)
    for qubit in frontier:
        if qubit not in fed_qubits and qubit.default is not None:
            if type(qubit.default) == int:  # noqa: E721
                if 0 < qubit.default < 2 ** qubit.n:
                    vec = numpy.zeros((2 ** qubit.n,))
                    vec[qubit.default] = 1.0
                    feed[(qubit,)] = vec
            else:
                feed[(qubit,)] = qubit.default

    frontier = sorted(frontier, key=lambda q: q.qid)
    if strict:
        missing = [q for q in frontier if q not in fed_qubits]
        if missing:
            raise ValueError("Missing Qubit states for: {}".format(missing))

    qbitindex: Dict[PipelineObject, List[int]] = {}
    n = 0
    for q in frontier:
        qbitindex[q] = list(range(n, n + q.n))
        n += q.n

    feed_index_groups = [sum((qbitindex[q] for q in qs), []) for qs in feed]
    feed_states = [feed[qs] for qs in feed]
    if kwargs.get("state") is not None and _truthy(kwargs["state"]):
        # Deprecated full-state argument: one feed over every qubit (a vector, or an
        # int naming a basis state, which is how make_circuit_mat uses it).
        feed_index_groups = [tuple(range(n))]
        feed_states = [kwargs["state"]]

    state = backend_constructor(n, feed_index_groups, feed_states, statetype=statetype)
    if walk is not None:
        return walk.replay(state, n)
    if not _walk_is_structural(graphnodes):
        return feed_forward(frontier, state, graphnodes)
    acc = _RecordingFeeder(state, n)
    run_graph(frontier, graphnodes, acc)
    _WALKS[walk_key] = _Walk(frontier, graphnodes, acc.schedule)
    if len(_WALKS) > _WALKS_MAX:
        _WALKS.popitem(last=False)
    return acc.state.get_state(), acc.classic_map


def _truthy(v) -> bool:
    if isinstance(v, numpy.ndarray):
        return v.size > 0
    return bool(v)


def get_deps(*args: PipelineObject, feed: Mapping[PipelineObject, InitialState] = None):
    """Leaf nodes and all nodes reachable backwards from ``args``
    (``qip/pipeline.py:138-160``)."""
    if feed is None:
        feed = {}
    seen: Set[PipelineObject] = set()
    deps: Set[PipelineObject] = set()
    stack = list(args)
    while stack:
        node = stack.pop()
        if node in seen:
            continue
        seen.add(node)
        if node in feed or len(node.inputs) == 0:
            deps.add(node)
        else:
            stack.extend(node.inputs)
    return list(deps), seen


def make_circuit_mat(*args: PipelineObject, **kwargs) -> numpy.ndarray:
    """Matrix of the quantum part of the circuit, one basis column per run
    (``qip/pipeline.py:163-178``); column i is the output for input basis state i."""
    o, _ = run(*args, **kwargs)
    n = int(numpy.log2(len(o)))
    mat = numpy.zeros((2 ** n, 2 ** n), dtype=numpy.complex128)
    mat[:, 0] = o
    for i in range(1, 2 ** n):
        o, _ = run(*args, state=i, **kwargs)
        mat[:, i] = o
    return mat


class GraphAccumulator:
    def feed(self, qbitindex: Mapping[PipelineObject, Sequence[int]], node: PipelineObject) -> None:
        raise NotImplementedError("Method not implemented.")


def run_graph(frontier: Sequence[PipelineObject], graphnodes, graphacc: GraphAccumulator):
    """Feed every node to ``graphacc`` in execution order (``qip/pipeline.py:186-222``)."""
    qbitindex: Dict[PipelineObject, List[int]] = {}
    n = 0
    ordered = sorted(frontier, key=lambda q: q.qid)
    for q in ordered:
        qbitindex[q] = list(range(n, n + q.n))
        n += q.n
    arrival = itertools.count()
    heap = [(q.qid, next(arrival), q) for q in ordered]
    heapq.heapify(heap)
    queued: Set[PipelineObject] = set(ordered)
    seen: Set[PipelineObject] = set()
    while heap:
        _, _, node = heapq.heappop(heap)
        queued.discard(node)
        graphacc.feed(qbitindex, node)
        qbitindex = node.remap_index(qbitindex, n)
        seen.add(node)
        for nxt in node.sink:
            if nxt in graphnodes and nxt not in seen and nxt not in queued:
                if all(p in seen for p in nxt.inputs):
                    heapq.heappush(heap, (nxt.qid, next(arrival), nxt))
                    queued.add(nxt)
                    qbitindex[nxt] = nxt.select_index(flatten(qbitindex[j] for j in nxt.inputs))


# QSV_NVTX=1: one NVTX range per graph node (named after its operator class), visible on
# a profiler's timeline around that node's kernels.
TRACE = os.environ.get("QSV_NVTX", "0") not in ("", "0")


def _trace_lib():
    from . import _native as nat

    return nat.load()


class NodeFeeder(GraphAccumulator):
    """Feeds nodes to the state and records classical results (``qip/pipeline.py:225-240``)."""

    def __init__(self, state, n: int):
        self.state = state
        self.n = n
        self.classic_map = {}

    def feed(self, qbitindex, node):
        if TRACE:
            _trace_lib().qsv_trace_push(type(node).__name__.encode())
        try:
            n_bits, bits = node.feed(self.state, qbitindex, self.n)
        finally:
            if TRACE:
                _trace_lib().qsv_trace_pop()
        if n_bits > 0 or bits is not None:
            self.classic_map[node] = bits
            self.n -= n_bits


class _RecordingFeeder(NodeFeeder):
    """A NodeFeeder that also records each node with the index groups it was given."""

    def __init__(self, state, n: int):
        super().__init__(state, n)
        self.schedule: List[Tuple[PipelineObject, List[Sequence[int]]]] = []

    def feed(self, qbitindex, node):
        self.schedule.append((node, [qbitindex[q] for q in node.inputs]))
        super().feed(qbitindex, node)


# Compiled walks.  The executor's node order, and the global indices each node is given,
# depend only on the graph's structure (qids, inputs, sinks, register sizes), not on the
# state or the feeds' values, as long as every node keeps the base ``feed`` and
# ``remap_index``.  ``run`` records the walk of a graph (keyed by its output nodes and
# fed registers) and later runs of the same graph replay it: the same ``feed_indices``
# calls in the same order, without re-deriving the order.  The most recent graphs are
# kept (the entries hold references to their nodes).
_WALKS_MAX = 32
_WALKS: "OrderedDict[Any, _Walk]" = OrderedDict()


def _walk_is_structural(graphnodes) -> bool:
    base_feed, base_remap = PipelineObject.feed, PipelineObject.remap_index
    return all(type(node).feed is base_feed and type(node).remap_index is base_remap for node in graphnodes)


class _Walk:
    def __init__(self, frontier, graphnodes, schedule):
        self.frontier = frontier
        self.graphnodes = graphnodes
        # Nodes with the base feed_indices (register joins and cuts) do nothing but
        # record (0, 0); the replay records that without the call.
        base = PipelineObject.feed_indices
        self.schedule = [(node, groups, type(node).feed_indices is base) for node, groups in schedule]

    def replay(self, state, n: int):
        classic = {}
        for node, groups, noop in self.schedule:
            if noop and not TRACE:
                classic[node] = 0
                continue
            if TRACE:
                _trace_lib().qsv_trace_push(type(node).__name__.encode())
            try:
                n_bits, bits = node.feed_indices(state, groups, n)
            finally:
                if TRACE:
                    _trace_lib().qsv_trace_pop()
            if n_bits > 0 or bits is not None:
                classic[node] = bits
                n -= n_bits
        return state.get_state(), classic


def clear_compiled_walks() -> None:
    """Forget the recorded walks (and release the graphs they reference)."""
    _WALKS.clear()


def feed_forward(frontier: Sequence[PipelineObject], state, graphnodes):
    n = sum(f.n for f in frontier)
    acc = NodeFeeder(state, n)
    run_graph(frontier, graphnodes, acc)
    return acc.state.get_state(), acc.classic_map


class PrintFeeder(GraphAccumulator):
    """ASCII circuit drawing (``qip/pipeline.py:251-302``)."""

    BLACKLIST = ["SplitQubit", "Q"]

    def __init__(self, n: int, opwidth: int = 1, linespacing: int = 1, outputfn: Callable[[str], None] = print):
        self.opwidth = opwidth
        self.linespacing = linespacing
        self.outputfn = outputfn
        self.n = n
        self.qubit_line = (" " * opwidth) + "|" + (" " * opwidth)

    def _emit(self, line):
        self.outputfn((" " * self.linespacing).join(line))

    def feed(self, qbitindex, node):
        indices = flatten([qbitindex[q] for q in node.inputs])
        if not indices:
            return
        name = repr(node)
        cut = name.find("(")
        if cut > 0:
            name = name[:cut]
        if name in PrintFeeder.BLACKLIST:
            return
        blank = [self.qubit_line] * self.n
        self._emit(blank)
        line = list(blank)
        for i in indices:
            line[i] = "-" * (2 * self.opwidth + 1)
        self._emit(line)
        pad = " " * (self.opwidth - 1)
        for ch in name:
            line = list(blank)
            for i in indices:
                line[i] = "|" + pad + ch + pad + "|"
            self._emit(line)
        width = max(len(str(i)) for i in range(len(indices)))
        labels = [str(i).rjust(width) for i in range(len(indices))]
        for row in range(width):
            for k, i in enumerate(indices):
                line[i] = "|" + pad + labels[k][row] + pad + "|"
            self._emit(line)
        for i in indices:
            line[i] = "-" * (2 * self.opwidth + 1)
        self._emit(line)


def print_circuit(*args, opwidth: int = 1, linespacing: int = 1, outputfn: Callable[[str], None] = print):
    frontier, graphnodes = get_deps(*args)
    frontier = sorted(frontier, key=lambda q: q.qid)
    n = sum(f.n for f in frontier)
    run_graph(frontier, graphnodes, PrintFeeder(n, opwidth, linespacing, outputfn))
