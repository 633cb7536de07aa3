"""qip_gb300: a GB300 (sm_103a) state-vector backend for the QIP circuit API.

The graph/operator API (``Qubit``, ``H``/``X``/``Y``/``Z``, ``Swap``, ``Rm``, ``C(...)``,
``Measure``, ``StochasticMeasure``, ``run``) mirrors QIP's; ``GpuBackend.make_state`` is
the backend constructor, usable with this package's ``run`` or with QIP's own
(``run(..., backend_constructor=GpuBackend.make_state)``).  All state-vector work runs
in libqsv.so (hand-written CUDA, see ``csrc/``); there is no CPU fallback.
"""
from .backend import GpuBackend, StateType
from .operators import (C, CMat, COp, F, FOp, H, HOp, MatrixOp, Not, NotOp, R, RmOp, ROp, Rm, RY, RYOp, RZ,
                        RZOp, Swap, SwapMat, SwapOp, U, UOp, X, XOp, Y, YOp, Z, ZOp)
from .pipeline import (GraphAccumulator, NodeFeeder, PipelineObject, PrintFeeder, feed_forward, get_deps,
                       make_circuit_mat, print_circuit, run, run_graph)
from .qfft import QFFT
from .qip import Measure, OpConstructor, Q, Qubit, SplitQubit, StochasticMeasure
from .qubit_util import QubitFuncWrapper, QubitOpWrapper, QubitWrapperContext

__all__ = [
    "GpuBackend", "StateType", "C", "CMat", "COp", "F", "FOp", "H", "HOp", "MatrixOp", "Not", "NotOp", "R",
    "RmOp", "ROp", "Rm", "RY", "RYOp", "RZ", "RZOp", "Swap", "SwapMat", "SwapOp", "U", "UOp", "X", "XOp", "Y",
    "YOp", "Z", "ZOp", "GraphAccumulator", "NodeFeeder", "PipelineObject", "PrintFeeder", "feed_forward",
    "get_deps", "make_circuit_mat", "print_circuit", "run", "run_graph", "QFFT", "Measure", "OpConstructor",
    "Q", "Qubit", "SplitQubit", "StochasticMeasure", "QubitFuncWrapper", "QubitOpWrapper",
    "QubitWrapperContext",
]
