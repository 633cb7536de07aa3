"""Op-wrapping machinery (``qip/qubit_util.py``): ops that split their outputs,
``with``-contexts that turn every op built inside into a controlled op, and functions
wrapped into first-class ops so that ``C(circuit)`` works.

Two behaviours of the reference are kept because they change which circuit is
built:
* ``QubitOpWrapper.__call__`` passes only the construction-time keyword arguments to
  the op; keyword arguments given at call time are dropped
  (``qip/qubit_util.py:142-143``).  E.g. ``Rm(m, q, negate=True)`` through a wrapper
  call builds a positive-angle Rm, which is why ``QFFT`` equals the inverse DFT.
* ``C(f)`` on a wrapped function registers the control on that function object
  itself (``qip/qubit_util.py:198-201``).
"""
from __future__ import annotations

import collections.abc
from typing import Any, Callable, List, Mapping, Optional, Sequence, Tuple, Type, Union

from .qip import OpConstructor, Qubit
from .util import flatten


class QubitWrapperContext:
    """Within ``with QubitWrapperContext(C, [q]):`` every op built through a
    ``QubitOpWrapper`` is wrapped by ``C`` and receives ``q`` as its first input."""

    TOTAL_CONTEXT_QUBITS = 0
    CONTEXT_STACK: List[list] = []

    def __init__(self, *args):
        super().__init__()
        self.context = []
        self.context_size = 0
        pending: list = []
        for arg in args:
            if isinstance(arg, collections.abc.Iterable):
                pending.append(list(arg))
            else:
                if pending:
                    self.add_context(*pending)
                    pending = []
                pending.append(arg)
        if pending:
            self.add_context(*pending)

    def add_context(self, constructor, qubits: Sequence[Qubit], indices: Optional[Sequence[int]] = None):
        if indices is None:
            indices = list(range(len(qubits)))
        self.context.append((constructor, qubits, indices))
        self.context_size += len(qubits)

    @staticmethod
    def get_context():
        return flatten(QubitWrapperContext.CONTEXT_STACK)

    @staticmethod
    def apply_to_qubits_in_context(op_func, *qubits: Qubit, op_args=None, op_kwargs=None) -> Tuple[Qubit, ...]:
        qubits_list = list(qubits)
        active = len(QubitWrapperContext.CONTEXT_STACK) > 0
        if active:
            qubits_list = QubitWrapperContext.put_qubits_in_context_order(*qubits_list)
            op_func = QubitWrapperContext.make_context_constructor(op_func)
        outputs = op_func(*qubits_list, nocontext=True, nosplit=True).split()
        if active:
            controls, outputs = QubitWrapperContext.split_context_and_circuit_qubits(*outputs)
            QubitWrapperContext.set_qubits(controls)
        return outputs

    def put_qubits_in_local_context_order(self, *qubits: Qubit) -> Tuple[Qubit, ...]:
        return self._insert(self.context, qubits)

    @staticmethod
    def put_qubits_in_context_order(*qubits: Qubit) -> Tuple[Qubit, ...]:
        return QubitWrapperContext._insert(QubitWrapperContext.get_context(), qubits)

    @staticmethod
    def _insert(contexts, qubits) -> Tuple[Qubit, ...]:
        out = list(qubits)
        for _, cq, ci in reversed(contexts):
            for q, i in zip(cq, ci):
                out.insert(i, q)
        return tuple(out)

    @staticmethod
    def split_context_and_circuit_qubits(*qubits: Qubit):
        rest = list(qubits)
        controls = []
        for _, _, ci in QubitWrapperContext.get_context():
            for i in ci:
                controls.append(rest.pop(i))
        return controls, rest

    @staticmethod
    def make_context_constructor(op_func, op_args=None, op_kwargs=None):
        for ctor, _, _ in reversed(QubitWrapperContext.get_context()):
            op_func = ctor(op_func)
        return op_func

    @staticmethod
    def set_qubits(qubits_list: Sequence[Qubit]):
        if len(qubits_list) != QubitWrapperContext.TOTAL_CONTEXT_QUBITS:
            raise ValueError("Size of qubits_list incorrect: {} is not required {}".format(
                len(qubits_list), QubitWrapperContext.TOTAL_CONTEXT_QUBITS))
        pos = 0
        for level in QubitWrapperContext.CONTEXT_STACK:
            for i, (ctor, cq, ci) in enumerate(level):
                level[i] = (ctor, qubits_list[pos:pos + len(cq)], ci)
                pos += len(cq)

    def __enter__(self):
        QubitWrapperContext.CONTEXT_STACK.append(self.context)
        QubitWrapperContext.TOTAL_CONTEXT_QUBITS += self.context_size
        return self

    def __exit__(self, exc_type, exc_val, exc_tb):
        QubitWrapperContext.CONTEXT_STACK.pop()
        QubitWrapperContext.TOTAL_CONTEXT_QUBITS -= self.context_size


class QubitOpWrapper(OpConstructor):
    """Wraps an op class so a call splits its output per input register."""

    def __init__(self, op, *args, **kwargs):
        super().__init__(op)
        self.args = args
        self.kwargs = kwargs

    def __call__(self, *inputs: Qubit, nosplit: bool = False, nocontext: bool = False, **kwargs):
        kwargs = dict(self.kwargs)  # call-time keyword arguments are not forwarded
        if nocontext:
            q = self.op(*self.args, *inputs, nocontext=nocontext, **kwargs)
            if len(q.inputs) == 1 or nosplit:
                return q
            if len(q.inputs) > 1:
                return q.split()
            return None
        outs = QubitWrapperContext.apply_to_qubits_in_context(self, *inputs)
        if len(outs) > 1:
            return outs
        if len(outs) == 1:
            return outs[0]
        raise ValueError("Somehow ended up with zero output qubits.")

    def wrap_op_hook(self, opconstructor, consumed_inputs=None):
        return None

    def __repr__(self):
        if not self.args:
            return "OpWrap({})".format(self.op)
        return "OpWrap({},+{} args)".format(self.op, len(self.args))


class QubitFuncWrapper(OpConstructor):
    """Makes a circuit-building function a first-class op (``C(f)`` works)."""

    def __init__(self, func):
        super().__init__(func)
        self.wrapper_funcs = []

    def __call__(self, *inputs: Qubit, **kwargs):
        remaining = list(inputs)
        layers = []
        for ctor, consumed in reversed(self.wrapper_funcs):
            taken = [remaining.pop(i) for i in reversed(consumed)]
            layers.append((ctor, list(reversed(taken)), consumed))
        layers.reverse()
        with QubitWrapperContext(*flatten(layers)) as context:
            outputs = self.op(*remaining, **kwargs)
            if isinstance(outputs, Qubit):
                outputs = (outputs,)
            ordered = context.put_qubits_in_local_context_order(*outputs)
            return ordered[0] if len(ordered) == 1 else ordered

    def wrap_op_hook(self, opconstructor, consumed_inputs=None):
        self.wrapper_funcs.append((opconstructor, consumed_inputs))
        return self

    @staticmethod
    def wrap(op_func):
        return QubitFuncWrapper(op_func)
