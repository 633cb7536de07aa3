"""Generate the golden fixtures of tests/golden from the reference itself.

Runs only where the reference checkout exists (it imports Renmusxd/QIP through
``oracle/ref_qip.py``, with its Cython kernels built by ``oracle/build_ref.py``).  Writes:

* ``kron_cases.npz``  — ``kronselect_dot`` through the reference's ``cdot_loop`` on
  seeded states: random numpy / CMat / SwapMat dictionaries, n = 3..8;
* ``measure_cases.npz`` — ``measure_probabilities``, ``measure_top_probabilities``
  (top_k >= number of outcomes), ``measure``/``reduce_measure`` with an explicit
  outcome and probability, and ``soft_measure`` with an explicit outcome;
* ``func_cases.npz`` — ``func_apply`` where every qubit is in reg1 or reg2;
* ``scenarios.npz`` — every scenario of ``scenarios.py`` run through the reference's
  own ``run()``;
* ``workloads.npz`` — small brickwork / Grover / random / ansatz gate lists of
  ``qip_gb300.circuits`` applied with the reference's ``kronselect_dot``.

Usage: ``python tests/golden/make_golden.py`` from the repository root.
"""
from __future__ import annotations

import json
import os
import sys
import types

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)


def reference_api():
    import ref_qip

    qip = ref_qip.import_reference()
    ns = types.SimpleNamespace()
    for mod in (qip.qip, qip.operators, qip.pipeline, qip.qfft, qip.qubit_util):
        for k in dir(mod):
            if not k.startswith("_"):
                setattr(ns, k, getattr(mod, k))
    return qip, ns


# ---- encoding of kron dictionaries --------------------------------------------------------

def encode(mats, arrays, prefix):
    """JSON description of a dict of numpy / CMat / SwapMat entries; numpy payloads go to
    ``arrays`` under ``prefix``-derived keys."""
    desc = []
    for j, (key, m) in enumerate(mats.items()):
        ctrl = 0
        while getattr(m, "_kron_struct", None) == 2:
            ctrl += 1
            m = m.m
        item = {"idx": list(int(x) for x in (key if isinstance(key, tuple) else (key,))),
                "int_key": not isinstance(key, tuple), "ctrl": ctrl}
        if getattr(m, "_kron_struct", None) == 3:
            item["swap"] = int(m.n)
        else:
            name = f"{prefix}_m{j}"
            arrays[name] = numpy.asarray(m, dtype=numpy.complex128)
            item["mat"] = name
        desc.append(item)
    return desc


def decode(desc, arrays, CMat, SwapMat):
    out = {}
    for item in desc:
        m = SwapMat(item["swap"]) if "swap" in item else numpy.asarray(arrays[item["mat"]])
        for _ in range(item["ctrl"]):
            m = CMat(m)
        key = item["idx"][0] if item.get("int_key") else tuple(item["idx"])
        out[key] = m
    return out


def rand_unitary(rng, k):
    z = rng.standard_normal((2 ** k, 2 ** k)) + 1j * rng.standard_normal((2 ** k, 2 ** k))
    q, r = numpy.linalg.qr(z)
    return q * (numpy.diag(r) / numpy.abs(numpy.diag(r)))[None, :]


def rand_state(rng, n):
    v = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    return v / numpy.linalg.norm(v)


def kron_dicts(rng, n, CMat, SwapMat):
    """A list of varied kron dictionaries on n qubits."""
    pick = lambda k: [int(x) for x in rng.choice(n, size=k, replace=False)]  # noqa: E731
    out = []
    q = pick(1)
    out.append({q[0]: rand_unitary(rng, 1)})                     # int key
    out.append({tuple(pick(1)): rand_unitary(rng, 1)})
    out.append({tuple(pick(2)): rand_unitary(rng, 2)})            # random order pair
    if n >= 3:
        out.append({tuple(pick(3)): rand_unitary(rng, 3)})
    a, b = pick(2)
    out.append({(a,): rand_unitary(rng, 1), (b,): rand_unitary(rng, 1)})  # disjoint entries
    if n >= 3:
        a, b, c = pick(3)
        out.append({(a, b): rand_unitary(rng, 2), (c,): rand_unitary(rng, 1)})
        out.append({(a, b, c): CMat(rand_unitary(rng, 2))})        # 1 control, 2 targets
        out.append({(a, b, c): CMat(CMat(rand_unitary(rng, 1)))})  # 2 controls
        out.append({(a, b, c): CMat(SwapMat(1))})                  # C(Swap)
        out.append({(a, b): CMat(numpy.diag(numpy.exp(1j * rng.uniform(0, 6, 2))))})  # controlled phase
        out.append({(a, b): CMat(numpy.array([[0, 1], [1, 0]], dtype=float))})      # CNOT
        out.append({(a, b): CMat(rand_unitary(rng, 1)), (a, c): CMat(rand_unitary(rng, 1))})  # shared control
    a, b = pick(2)
    out.append({(a, b): SwapMat(1)})
    out.append({(a,): numpy.array([[0, -1j], [1j, 0]])})                           # Y
    out.append({(b,): numpy.array([[1, 0], [0, -1.0]])})                           # Z
    out.append({(a,): numpy.eye(2)})                                               # identity
    if n >= 4:
        w = pick(4)
        out.append({tuple(w): SwapMat(2)})
        out.append({(w[0], w[1]): rand_unitary(rng, 2), (w[1], w[2]): rand_unitary(rng, 2)})  # overlapping
    if n >= 5:
        w = pick(5)
        out.append({tuple(w): CMat(SwapMat(2))})
        out.append({(w[0], w[1], w[2]): CMat(CMat(numpy.array([[1, 0], [0, -1.0]]))), (w[3], w[4]): rand_unitary(rng, 2)})
    return out


def main():
    qip, api = reference_api()
    kp = sys.modules["qip.ext.kronprod"]
    fa = sys.modules["qip.ext.func_apply"]
    from qip.util import kronselect_dot as ref_kron

    CMat, SwapMat = api.CMat, api.SwapMat
    rng = numpy.random.default_rng(20261203)

    # ---- kron cases -------------------------------------------------------------------
    arrays, cases = {}, []
    # The reference unit tests' known answers (utiltest.py:9-66) as golden cases.
    h = numpy.array([[1, 1], [1, -1]], dtype=complex)
    a_ = numpy.array([[1, 2], [3, 4]], dtype=complex)
    b_ = numpy.array([[5, 6], [7, 8]], dtype=complex)
    fixed = [{0: h, 2: h}, {(0, 2): numpy.kron(h, h)}, {0: a_, 2: b_}, {(0, 2): numpy.kron(a_, b_)},
             {(2, 0): numpy.kron(b_, a_)}]
    ci = 0
    for mats in fixed:
        for col in range(8):
            vec = numpy.zeros(8, dtype=numpy.complex128)
            vec[col] = 1.0
            out = numpy.zeros(8, dtype=numpy.complex128)
            ref_kron(mats, vec, 3, out, dot_impl=kp.cdot_loop)
            arrays[f"k{ci}_in"], arrays[f"k{ci}_out"] = vec, out
            cases.append({"n": 3, "mats": encode(mats, arrays, f"k{ci}"), "id": ci})
            ci += 1
    skipped = 0
    for n in range(3, 9):
        for mats in kron_dicts(rng, n, CMat, SwapMat):
            vec = rand_state(rng, n)
            out = numpy.zeros(2 ** n, dtype=numpy.complex128)
            try:
                ref_kron(mats, vec, n, out, dot_impl=kp.cdot_loop)
            except ValueError:
                # Mixed key lengths / mixed matrix kinds in one dictionary: the
                # reference cannot pack them into its 2-D index array on current
                # numpy (qip/util.py:62-64); such dictionaries are checked against
                # the oracle instead.
                skipped += 1
                continue
            arrays[f"k{ci}_in"], arrays[f"k{ci}_out"] = vec, out
            cases.append({"n": n, "mats": encode(mats, arrays, f"k{ci}"), "id": ci})
            ci += 1
    arrays["meta"] = numpy.array(json.dumps(cases))
    numpy.savez_compressed(os.path.join(HERE, "kron_cases.npz"), **arrays)
    print("kron cases:", len(cases), "skipped (reference raises):", skipped)

    # ---- measurement cases ------------------------------------------------------------
    arrays, cases = {}, []
    ci = 0
    for n in (3, 5, 6, 8):
        for _ in range(5):
            vec = rand_state(rng, n)
            if ci % 3 == 0:
                vec[rng.choice(2 ** n, size=2 ** (n - 1), replace=False)] = 0.0  # sparse states
                vec /= numpy.linalg.norm(vec)
            k = int(rng.integers(1, min(4, n - 1) + 1))
            idx = numpy.array(rng.choice(n, size=k, replace=False), dtype=numpy.int32)
            probs = kp.measure_probabilities(idx, n, vec)
            tm, tp = kp.measure_top_probabilities(idx, n, 2 ** k, vec)
            m = int(rng.integers(0, 2 ** k))
            sm, sp = kp.soft_measure(idx, n, vec, measured=m)
            out = numpy.zeros(2 ** n, dtype=numpy.complex128)
            p = float(sp) if sp > 0 else 0.5
            cm, cp = kp.measure(idx, n, vec, out, measured=m, measured_prob=p)
            red = numpy.zeros(2 ** n, dtype=numpy.complex128)
            kp.reduce_measure(idx, n, vec, red, measured=m, measured_prob=p)
            arrays[f"c{ci}_vec"] = vec
            arrays[f"c{ci}_probs"] = numpy.asarray(probs)
            arrays[f"c{ci}_topm"] = numpy.asarray(tm, dtype=numpy.int64)
            arrays[f"c{ci}_topp"] = numpy.asarray(tp, dtype=numpy.float64)
            arrays[f"c{ci}_collapse"] = out
            arrays[f"c{ci}_reduce"] = red[: 2 ** (n - k)]
            cases.append({"n": n, "idx": [int(x) for x in idx], "m": m, "soft": [int(sm), float(sp)], "p": p,
                          "id": ci})
            ci += 1
    arrays["meta"] = numpy.array(json.dumps(cases))
    numpy.savez_compressed(os.path.join(HERE, "measure_cases.npz"), **arrays)
    print("measure cases:", len(cases))

    # ---- func_apply cases (every qubit in reg1 or reg2) ----------------------------------
    arrays, cases = {}, []
    for ci, (n1, n2) in enumerate([(2, 2), (1, 3), (3, 2), (4, 2), (2, 4)]):
        n = n1 + n2
        perm = [int(x) for x in rng.permutation(n)]
        r1 = numpy.array(perm[:n1], dtype=numpy.int32)
        r2 = numpy.array(perm[n1:], dtype=numpy.int32)
        table = [int(x) for x in rng.integers(0, 2 ** n2, size=2 ** n1)]
        vec = rand_state(rng, n)
        out = numpy.zeros(2 ** n, dtype=numpy.complex128)
        fa.func_apply(r1, r2, lambda x, t=table: t[x], vec, n, out)
        arrays[f"f{ci}_vec"], arrays[f"f{ci}_out"] = vec, out
        cases.append({"n": n, "reg1": [int(x) for x in r1], "reg2": [int(x) for x in r2], "table": table,
                      "id": ci})
    arrays["meta"] = numpy.array(json.dumps(cases))
    numpy.savez_compressed(os.path.join(HERE, "func_cases.npz"), **arrays)
    print("func cases:", len(cases))

    # ---- scenarios through the reference's run() -----------------------------------------
    import scenarios

    arrays, meta = {}, {}
    for name, fn in scenarios.SCENARIOS.items():
        runs = fn(api)
        meta[name] = []
        for r, (outs, feed, measured) in enumerate(runs):
            o, classic = api.run(*outs, feed=feed)
            arrays[f"{name}_{r}_state"] = numpy.asarray(o)
            rec = {"measured": []}
            for j, node in enumerate(measured):
                val = classic[node]
                if isinstance(val, tuple):
                    arrays[f"{name}_{r}_m{j}_idx"] = numpy.asarray(val[0], dtype=numpy.int64)
                    arrays[f"{name}_{r}_m{j}_p"] = numpy.asarray(val[1], dtype=numpy.float64)
                    rec["measured"].append("topk")
                else:
                    arrays[f"{name}_{r}_m{j}_p"] = numpy.asarray(val, dtype=numpy.float64)
                    rec["measured"].append("probs")
            meta[name].append(rec)
    arrays["meta"] = numpy.array(json.dumps(meta))
    numpy.savez_compressed(os.path.join(HERE, "scenarios.npz"), **arrays)
    print("scenarios:", len(meta))

    # ---- workload gate lists through the reference kernel --------------------------------
    from qip_gb300 import circuits

    def run_ref(gates, n, vec):
        out = numpy.zeros(2 ** n, dtype=numpy.complex128)
        for g in gates:
            ref_kron(g, vec, n, out, dot_impl=kp.cdot_loop)
            vec, out = out, vec
        return vec

    arrays = {}
    n = 10
    v0 = numpy.zeros(2 ** n, dtype=numpy.complex128)
    v0[0] = 1
    arrays["brickwork_n10"] = run_ref(circuits.brickwork(n, 12, seed=11), n, v0.copy())
    gates, marked = circuits.grover_gates(8, iterations=2, seed=3)
    v0 = numpy.zeros(2 ** 8, dtype=numpy.complex128)
    v0[0] = 1
    arrays["grover_n8"] = run_ref(gates, 8, v0)
    arrays["grover_n8_marked"] = numpy.array(marked)
    wrng = numpy.random.default_rng(99)
    for i in range(6):
        nn = int(wrng.integers(4, 11))
        depth = int(wrng.integers(20, 61))
        gl = circuits.random_circuit(wrng, nn, depth)
        feeds = circuits.random_product_feed(wrng, nn)
        st = numpy.ones(1, dtype=numpy.complex128)
        for f in feeds:
            st = numpy.kron(st, f)
        arrays[f"random_{i}_state"] = run_ref(gl, nn, st.astype(numpy.complex128))
        arrays[f"random_{i}_shape"] = numpy.array([nn, depth])
    thetas = numpy.random.default_rng(5).uniform(0, 2 * numpy.pi, 2 * 6 * 3)
    v0 = numpy.zeros(2 ** 6, dtype=numpy.complex128)
    v0[0] = 1
    arrays["ansatz_n6"] = run_ref(circuits.ansatz_layers(6, 3, thetas), 6, v0)
    arrays["ansatz_n6_thetas"] = thetas
    # Parameter-shift gradient of <sum Z> for the RY/RZ/CNOT-ring ansatz through the
    # reference kernel (E(theta + pi/2) - E(theta - pi/2)) / 2 per angle.
    def sumz(vec, nq):
        idx = numpy.arange(2 ** nq)
        w = nq - 2 * numpy.array([bin(i).count("1") for i in idx])
        return float(numpy.sum(w * numpy.abs(vec) ** 2))

    def energy(th, nq, layers):
        v = numpy.zeros(2 ** nq, dtype=numpy.complex128)
        v[0] = 1
        return sumz(run_ref(circuits.ansatz_layers(nq, layers, th), nq, v), nq)

    nq, layers = 6, 2
    trng = numpy.random.default_rng(77)
    thetas = trng.uniform(0, 2 * numpy.pi, (3, 2 * nq * layers))
    energies, grads = [], []
    for th in thetas:
        energies.append(energy(th, nq, layers))
        g = []
        for j in range(th.size):
            tp, tm = th.copy(), th.copy()
            tp[j] += numpy.pi / 2
            tm[j] -= numpy.pi / 2
            g.append((energy(tp, nq, layers) - energy(tm, nq, layers)) / 2)
        grads.append(g)
    arrays["ansatz_ps_thetas"] = thetas
    arrays["ansatz_ps_energies"] = numpy.array(energies)
    arrays["ansatz_ps_grads"] = numpy.array(grads)
    arrays["ansatz_ps_shape"] = numpy.array([nq, layers])
    numpy.savez_compressed(os.path.join(HERE, "workloads.npz"), **arrays)
    print("workloads written")


if __name__ == "__main__":
    main()
