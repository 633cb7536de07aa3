"""The quantum Fourier transform as a graph op (QIP's ``qip/qfft.py:8-43``).

``QFFT(*registers, rev=True)`` cuts every input register into single-qubit wires and
applies ``circuits.qft_schedule``: per wire an H, then an Rm controlled by each later
wire, then (``rev``) Swaps that reverse the wire order.  The outputs are regrouped into
registers of the inputs' sizes.  The controlled phase is built as QIP builds it,
``C(lambda *q, **kw: Rm(m, *q, negate=True, **kw))``: QIP's op wrapper drops call-time
keyword arguments (``qip/qubit_util.py:142-143``), so ``negate`` has no effect there
and none here — the transform is the inverse DFT, as in the reference.
"""
from __future__ import annotations

from itertools import accumulate
from typing import Tuple, Union

from .circuits import qft_schedule
from .operators import C, H, Rm, Swap
from .qip import Qubit
from .qubit_util import QubitFuncWrapper


def _controlled_rm(m: int):
    return C(lambda *inputs, **kwargs: Rm(m, *inputs, negate=True, **kwargs))


@QubitFuncWrapper.wrap
def QFFT(*inputs: Qubit, rev: bool = True) -> Union[Qubit, Tuple[Qubit, ...]]:
    wires = [w for reg in inputs for w in reg.split(range(reg.n))]
    for step in qft_schedule(len(wires), rev):
        if step[0] == "h":
            wires[step[1]] = H(wires[step[1]])
        elif step[0] == "cphase":
            _, c, t, m = step
            wires[c], wires[t] = _controlled_rm(m)(wires[c], wires[t])
        else:
            _, a, b = step
            wires[a], wires[b] = Swap(wires[a], wires[b])
    if len(wires) == len(inputs):
        outputs = wires
    else:
        ends = list(accumulate(reg.n for reg in inputs))
        outputs = [Qubit(*wires[lo:hi]) for lo, hi in zip([0] + ends[:-1], ends)]
    return outputs[0] if len(outputs) == 1 else tuple(outputs)
