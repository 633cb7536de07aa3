"""Circuit scenarios written once against "an API namespace" so the same code builds
the circuit with the reference's QIP package (when fixtures are generated) and with
qip_gb300 (when they are checked).  Most follow the reference's own unit tests
(tests/qiptest.py, tests/qfttest.py, tests/qubit_util_test.py of Renmusxd/QIP); the last
ones are the QFT workload at larger sizes.

Each scenario returns a list of runs; a run is (outputs, feed, measured_nodes) and is
executed as ``api.run(*outputs, feed=feed)``.
"""
from __future__ import annotations

import numpy

S2 = pow(2, -0.5)


def _q(api, n=1, **kw):
    return api.Qubit(n=n, **kw)


def not_simple(api):
    runs = []
    for v in ([1.0, 0.0], [0.0, 1.0]):
        q = _q(api)
        n = api.Not(q)
        runs.append(([n], {q: v}, []))
    return runs


def bell(api):
    runs = []
    for v in ([1.0, 0.0], [0.0, 1.0]):
        q = _q(api)
        h = api.H(q)
        runs.append(([h], {q: v}, []))
    return runs


def h_first(api):
    q1, q2 = _q(api), _q(api)
    h1, h2 = api.H(q1), api.H(q2)
    q3, q4 = api.Qubit(h1, h2).split()
    h3 = api.H(q3)
    r1 = ([h3], {q1: [1.0, 0.0], q2: [1.0, 0.0]}, [])
    q1, q2 = _q(api), _q(api)
    h3 = api.H(q2)
    q3, q4 = api.Qubit(q1, h3).split()
    r2 = ([q3], {q1: [1.0, 0.0], q2: [1.0, 0.0]}, [])
    return [r1, r2]


def multi_not(api):
    q1, q2 = _q(api), _q(api)
    s = api.NotOp(q1, q2)
    return [([s], {q1: [1.0, 0.0], q2: [1.0, 0.0]}, [])]


def swap(api):
    q1, q2 = _q(api), _q(api)
    s = api.SwapOp(q1, q2)
    feeds = [([1.0, 0.0], [1.0, 0.0]), ([1.0, 0.0], [0.0, 1.0]), ([0.0, 1.0], [1.0, 0.0]), ([0.0, 1.0], [0.0, 1.0])]
    return [([s], {q1: a, q2: b}, []) for a, b in feeds]


def swap_twobit(api):
    q1, q2 = _q(api, 2), _q(api, 2)
    s = api.SwapOp(q1, q2)
    return [([s], {q1: [0.0, 1.0, 0.0, 0.0], q2: [1.0, 0.0, 0.0, 0.0]}, [])]


def split(api):
    q1, q2 = _q(api), _q(api)
    n1, n2 = api.Not(q1, q2)
    f1, f2 = api.Not(n1), api.Not(n2)
    feed = {q1: [1.0, 0.0], q2: [1.0, 0.0]}
    return [([f1], feed, []), ([f2], feed, []), ([f1, f2], feed, [])]


def allsplit(api):
    n = 5
    q = _q(api, n)
    qs = q.split(range(n + 1))
    newq = api.Qubit(*qs)
    state = numpy.cos(numpy.linspace(0, numpy.pi, 2 ** n))
    return [([newq], {q: state}, [])]


def cnot(api):
    q1, q2 = _q(api), _q(api)
    c1, c2 = api.C(api.Not)(q1, q2)
    return [([c1, c2], {q1: [1.0, 0.0], q2: [1.0, 0.0]}, []), ([c1, c2], {q1: [0.0, 1.0], q2: [1.0, 0.0]}, [])]


def defaults(api):
    q1 = _q(api, default=[0.0, 1.0])
    q2 = _q(api)
    r1 = ([q1, q2], {q2: [1.0, 0.0]}, [])
    a = _q(api, 2, default=[1, 2, 3, 4])
    b = _q(api, 2, default=[1, 0, 0, 0])
    r2 = ([a, b], {}, [])
    c = _q(api, 2, default=[1, 2, 3, 4])
    d = _q(api, 2)
    r3 = ([c, d], {d: [1, 0, 0, 0]}, [])
    return [r1, r2, r3]


def _cswap(api, n, s2, s3):
    q1, q2, q3 = _q(api), _q(api, n), _q(api, n)
    h1 = api.H(q1)
    c1, c2, c3 = api.C(api.Swap)(h1, q2, q3)
    m1 = api.H(c1)
    return ([m1], {q1: [1.0, 0.0], q2: s2, q3: s3}, [])


def cswap(api):
    runs = [_cswap(api, 1, [0.0, 1.0], [1.0, 0.0]), _cswap(api, 1, [1.0, 0.0], [1.0, 0.0]),
            _cswap(api, 2, [0.0, 0.0, 0.0, 1.0], [1.0, 0.0, 0.0, 0.0]),
            _cswap(api, 2, [1.0, 0.0, 0.0, 0.0], [1.0, 0.0, 0.0, 0.0])]
    a, b = numpy.zeros(32), numpy.zeros(32)
    a[0], b[1] = 1.0, 1.0
    runs.append(_cswap(api, 5, a, b))
    a, b = numpy.zeros(32), numpy.zeros(32)
    a[0], b[0] = 1.0, 1.0
    runs.append(_cswap(api, 5, a, b))
    return runs


def not_ordered(api):
    q1, q2, q3 = _q(api), _q(api), _q(api, 3)
    n1, n2, n3 = api.Not(q1), api.H(q2), api.Not(q3)
    feed = {q1: [1.0, 0.0], q2: [1.0, 0.0], q3: [1.0] + [0.0] * 7}
    return [([n1, n2, n3], feed, [])]


def stochastic(api):
    q1, q2 = _q(api, 2), _q(api, 2)
    m1 = api.StochasticMeasure(q2)
    r1 = ([m1, q1], {q1: [0.0, 0.0, 1.0, 0.0], q2: [0.5, 0.5, 0.5, 0.5]}, [m1])
    q1, q2 = _q(api, 2), _q(api, 2)
    m2 = api.StochasticMeasure(q2, top_k=4)
    r2 = ([m2, q1], {q1: [0.0, 0.0, 1.0, 0.0], q2: [0.6, 0.8, 0.0, 0.0]}, [m2])
    return [r1, r2]


def fop(api):
    runs = []
    r1 = _q(api, 2, default=[1, 2, 3, 4])
    r2 = _q(api, 2, default=[1, 0, 0, 0])
    f1, f2 = api.F(lambda x: 1, r1, r2)
    runs.append(([f1, f2], {}, []))
    r1 = _q(api, 2, default=[1, 2, 3, 4])
    r2 = _q(api, 2, default=[0, 1, 0, 0])
    f1, f2 = api.F(lambda x: 1, r1, r2)
    runs.append(([f1, f2], {}, []))
    r1 = _q(api, 4, default=numpy.ones(16) * pow(16, -0.5))
    r2 = _q(api, 2)
    f1, f2 = api.F(lambda x: pow(3, x, 4), r1, r2)
    runs.append(([f1, f2], {}, []))
    return runs


def rop(api):
    q1, q2 = _q(api), _q(api)
    r2 = api.Rm(2, q2)
    a = ([q1, r2], {}, [])
    q1, q2 = _q(api), _q(api, default=1)
    r2 = api.Rm(2, q2)
    b = ([q1, r2], {}, [])
    q1, q2 = _q(api), _q(api)
    r2 = api.Rm(2, q2)
    c = ([q1, r2], {q1: [1.0, 0.0], q2: [0.0, 1.0]}, [])
    d = ([q1, r2], {(q1, q2): [0.0, 1.0, 0.0, 0.0]}, [])
    e = ([q1, r2], {(q2, q1): [0.0, 0.0, 1.0, 0.0]}, [])
    return [a, b, c, d, e]


def toffoli(api):
    q1, q2, q3 = _q(api), _q(api), _q(api)
    c1, c2, c3 = api.C(api.C(api.Not))(q1, q2, q3)
    return [([c1, c2, c3], {q1: [S2, S2], q2: [S2, S2]}, [])]


def qft_small(api):
    q = _q(api, 2)
    a = ([api.QFFT(q)], {q: [0.5, 0.5, 0.5, 0.5]}, [])
    n = 6
    q = _q(api, n)
    st = numpy.cos(numpy.linspace(0, 2 * 5 * numpy.pi, 2 ** n))
    st = st / numpy.linalg.norm(st)
    b = ([api.QFFT(q)], {q: st}, [])
    return [a, b]


def contexts(api):
    runs = []
    # basic context
    q3, q4 = _q(api, default=[S2, S2]), _q(api)
    with api.QubitWrapperContext(api.C, [q3]):
        h = api.H(q4)
    runs.append(([h], {}, []))
    # explicit context
    q4, q5, q6 = _q(api, default=[S2, S2]), _q(api, default=[S2, S2]), _q(api)
    with api.QubitWrapperContext(api.C, [q4]):
        c4, c5 = api.C(api.H)(q5, q6)
    runs.append(([c4, c5], {}, []))
    # function wrapper
    circuit = api.QubitFuncWrapper.wrap(lambda *args: api.H(*args))
    q3, q4 = _q(api, default=[S2, S2]), _q(api, 2)
    c3, c4 = api.C(circuit)(q3, q4)
    runs.append(([c3, c4], {}, []))
    # nested C inside a wrapped function
    circuit = api.QubitFuncWrapper.wrap(lambda *args: api.C(api.H)(*args))
    q4, q5, q6 = _q(api, default=[S2, S2]), _q(api, default=[S2, S2]), _q(api)
    c4, c5, c6 = api.C(circuit)(q4, q5, q6)
    runs.append(([c4, c5, c6], {}, []))
    # double nesting
    circuit = api.QubitFuncWrapper.wrap(lambda *args: api.C(api.C(api.H))(*args))
    q5, q6, q7, q8 = _q(api, default=[S2, S2]), _q(api, default=[S2, S2]), _q(api, default=[S2, S2]), _q(api)
    c5, c6, c7, c8 = api.C(circuit)(q5, q6, q7, q8)
    runs.append(([c5, c6, c7, c8], {}, []))
    # reference circuit for the double nesting
    q1, q2, q3, q4 = _q(api, default=[S2, S2]), _q(api, default=[S2, S2]), _q(api, default=[S2, S2]), _q(api)
    c1, c2, c3, c4 = api.C(api.C(api.C(api.H)))(q1, q2, q3, q4)
    runs.append(([c1, c2, c3, c4], {}, []))
    return runs


def qft_config1(api, n=16, seed=2024):
    """QFT on n qubits of a seeded N(0,1) complex state, then the outcome distribution
    of the top 4 qubits."""
    rng = numpy.random.default_rng(seed)
    st = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    st = st / numpy.linalg.norm(st)
    q = _q(api, n)
    out = api.QFFT(q)
    top = out.split([4])
    sm = api.StochasticMeasure(top[0])
    sk = api.StochasticMeasure(top[0], top_k=16)
    return [([sm, sk, top[1]], {q: st}, [sm, sk])]


def qft_medium(api):
    return qft_config1(api, n=10, seed=5)


SCENARIOS = {
    "not_simple": not_simple, "bell": bell, "h_first": h_first, "multi_not": multi_not, "swap": swap,
    "swap_twobit": swap_twobit, "split": split, "allsplit": allsplit, "cnot": cnot, "defaults": defaults,
    "cswap": cswap, "not_ordered": not_ordered, "stochastic": stochastic, "fop": fop, "rop": rop,
    "toffoli": toffoli, "qft_small": qft_small, "contexts": contexts, "qft_medium": qft_medium,
    "qft_config1": qft_config1,
}
