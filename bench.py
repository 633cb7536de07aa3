"""Benchmark: random brickwork circuit, n=28, depth 40 (amp-updates/s).

Our arm (default):
  value      complex64 state, gates fused into <=6-qubit blocks run on the tensor cores
             (tcgen05, split-bf16 products, FP32 accumulation); device time per step
             (state reset to |0...0> + the whole circuit), inputs resident in HBM.
  plain_fp64 the same circuit on the complex128 per-gate kernels (one launch per gate).
  infidelity 1 - |<psi_fused|psi_fp64>|^2 computed on the GPU in FP64.
  e2e        the same metric through the backend plugin with host buffers: build the
             state, one kronselect_dot per gate with host numpy matrices, get_state()
             back to host memory; host<->device copies inside the timed region.  Each
             step submits the same circuit structure, so the whole-circuit plan kept
             after the first circuit is replayed; e2e.streamed times the same steps
             with keep_plans=False (planned window by window, as a circuit run once).
  roofline   the fused block kernel: algorithmic bytes per launch (read + write of the
             2^n complex64 state) over its mean CUDA-event launch time.
  cpu_baseline  the reference's own Cython/OpenMP kernel (cdot_loop) on the host's cores,
             a bounded sample of the same gate list at the same n.
  hbm_n32    QFT + 8 Grover iterations at n=32 complex64 (fused) and n=31 complex128
             (per-gate): per-pass GB/s and fraction of the HBM peak, every single-qubit
             marginal, the marked probability against Grover's closed form.
  adjoint    adjoint gradients of the n=24, 960-angle ansatz for 64 parameter sets:
             gradient vectors/s, backward/forward, error against central differences.
  batched    4096 uneven circuits in one persistent launch: circuits/s, p50/p99 latency.
  Each of the last three has its own CUDA-event timing and clock record.
--impl reference: the reference CPU kernel alone, same metric/config, one JSON line.

Multi-GPU: every rank runs an independent replica (the state vector is not sharded);
value = total amp-updates of all ranks / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import ctypes
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT, DEPTH_DEFAULT, SEED = 28, 40, 1234
# DRAM bytes (read + write) of one fused-block launch on a 2^25 complex64 state, from an
# ncu capture (dram__bytes_read.sum 268.57 MB + dram__bytes_write.sum 207.09 MB); the
# traffic of a launch grows with the state, so it is scaled by 2^(n-25).
NCU_BLOCK_TRAFFIC_N25 = 268.574464e6 + 207.090944e6
METRIC = "amp-updates/s (brickwork circuit, fused FP32 tensor-core blocks vs plain FP64 per-gate)"
THROTTLE_REASONS = {
    0x1: "gpu_idle", 0x2: "applications_clocks_setting", 0x4: "sw_power_cap", 0x8: "hw_slowdown",
    0x10: "sync_boost", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown",
    0x100: "display_clock_setting",
}


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while the timed region runs."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sms, mx, reasons = [], None, set()
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 3:
                continue
            try:
                sms.append(float(parts[0]))
                mx = float(parts[1])
                mask = int(parts[2], 16) if parts[2].startswith("0x") else int(parts[2])
            except ValueError:
                continue
            for bit, name in THROTTLE_REASONS.items():
                if mask & bit and name != "gpu_idle":
                    reasons.add(name)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sms)}


# ---- reference CPU kernel --------------------------------------------------------------------

def load_reference_kernels():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_ref

    if not build_ref.available():
        build_ref.build()
    if not build_ref.available():
        return None
    kronprod, _ = build_ref.load()
    return kronprod


def ref_pack(mats):
    """Pack a kron dictionary the way the reference's util.kronselect_dot hands it to
    cdot_loop: an int32 index array and an array of complex128 / CMat / SwapMat."""
    keys = [k if isinstance(k, tuple) else (k,) for k in mats]
    vals = [mats[k] for k in mats]
    cind = numpy.array([numpy.array(k, dtype=numpy.int32) for k in keys])
    cm = numpy.empty(len(vals), dtype=object)
    for i, m in enumerate(vals):
        cm[i] = m.astype(numpy.complex128) if isinstance(m, numpy.ndarray) else m
    return cind, cm


def cpu_reference_sample(n, gates, seconds_cap=30.0):
    """Time the reference cdot_loop over a bounded prefix-sample of the gate list at full
    n (state + arena ping-pong as CythonBackend does).  Returns (amp_updates/s, info)."""
    from qip_gb300 import circuits

    kp = load_reference_kernels()
    if kp is None:
        return None, {"kind": "unavailable", "why": "reference kernels not built"}
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    # A representative sample: 3 Haar single-qubit gates and 2 controlled-Z gates.
    haar = [g for g in gates if len(next(iter(g))) == 1][:3]
    cz = [g for g in gates if len(next(iter(g))) == 2][:2]
    sample = haar + cz
    vec = numpy.zeros(2 ** n, dtype=numpy.complex128)
    vec[0] = 1.0
    out = numpy.zeros(2 ** n, dtype=numpy.complex128)
    packed = [ref_pack(g) for g in sample]
    done = 0.0
    t0 = time.perf_counter()
    used = []
    for g, (ci, cm) in zip(sample, packed):
        kp.cdot_loop(ci, cm, vec, n, out)
        vec, out = out, vec
        done += circuits.gate_amp_updates([g], n)
        used.append(g)
        if time.perf_counter() - t0 > seconds_cap:
            break
    dt = time.perf_counter() - t0
    info = {"kind": "reference", "cores": int(os.environ.get("OMP_NUM_THREADS", cores)),
            "sample": f"{len(used)} gates of the n={n} brickwork ({sum(len(next(iter(g))) == 1 for g in used)} "
                      f"Haar 1-qubit, {sum(len(next(iter(g))) == 2 for g in used)} CZ) through the reference "
                      f"Cython cdot_loop, complex128, {dt:.1f} s"}
    return done / dt, info


# ---- GPU arm -----------------------------------------------------------------------------------

def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch

    if ws > 1:
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return ws, rank, local


def barrier_max(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def run_ours(args):
    import torch

    from qip_gb300 import GpuBackend, _native as nat, circuits, fusion, gates as gmod
    from qip_gb300.autotune import MODES as MODE_NAMES, default_tuner, placement_class

    ws, rank, local = dist_setup(args)
    n, depth = args.n, args.depth
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    gl = circuits.brickwork(n, depth, seed=SEED)
    amp_updates = circuits.gate_amp_updates(gl, n)
    ops = [op for g in gl for op in gmod.decompose(g)]
    lib = nat.load()
    st = GpuBackend.make_state(n, [], [], statetype=numpy.complex64, fusion=True)
    st.set_stream(stream.cuda_stream)
    t_plan0 = time.perf_counter()
    tuner = default_tuner()
    if args.kmax:
        kmax, width_report = args.kmax, {}
        steps = tuner.place(st.handle, n, fusion.plan(ops, kmax=kmax, beam=fusion.BEAM_WIDE))
    else:
        # Measured fusion width and block access modes (scratch-state timings).
        kmax, steps, width_report = tuner.choose_width(st.handle, n, ops)
    t_plan = time.perf_counter() - t_plan0
    blocks = [s for s in steps if isinstance(s, fusion.Block) and len(s.qubits) >= 4]
    mode_counts = {}
    for b in blocks:
        meas = tuner.measured(n, *placement_class(b.qubits, n))
        name = MODE_NAMES[meas[1]] if meas else "rule"
        mode_counts[name] = mode_counts.get(name, 0) + 1
    # Device-resident plan: block images uploaded once; a step launches kernels only.
    ks = nat.int_array([len(b.qubits) for b in blocks])
    tg = nat.int_array([q for b in blocks for q in b.qubits])
    mats = numpy.ascontiguousarray(numpy.concatenate([b.matrix.reshape(-1) for b in blocks])).view(numpy.float64)
    plan = ctypes.c_void_p()
    nat.check(lib.qsv_plan_create(st.handle, len(blocks), nat.ip(ks), nat.ip(tg), nat.dp(mats), ctypes.byref(plan)),
              st.handle, "plan_create")
    block_index = {id(b): i for i, b in enumerate(blocks)}
    seq = []  # ("block", i) | ("op", GateOp)
    for s_ in steps:
        if isinstance(s_, fusion.Block) and id(s_) in block_index:
            seq.append(("block", block_index[id(s_)]))
        elif isinstance(s_, fusion.Block):
            for op in gmod.classify_matrix(s_.qubits, (), s_.matrix):
                seq.append(("op", op))
        else:
            seq.append(("op", s_))

    def reset():
        nat.check(lib.qsv_set_product_state(st.handle, 0, None, None, None), st.handle, "reset")

    ev_pairs = []

    def fused_step(record):
        reset()
        for kind, x in seq:
            if kind == "block":
                if record:
                    a = torch.cuda.Event(enable_timing=True)
                    b = torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    nat.check(lib.qsv_plan_launch(st.handle, plan, x, 1), st.handle, "plan_launch")
                    b.record(stream)
                    ev_pairs.append((a, b))
                else:
                    nat.check(lib.qsv_plan_launch(st.handle, plan, x, 1), st.handle, "plan_launch")
            else:
                st.apply_op(x)

    for _ in range(args.warmup):
        fused_step(False)
    torch.cuda.synchronize()
    barrier(ws)
    launches0 = nat.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            fused_step(True)
        e1.record(stream)
        e1.synchronize()
    launches = nat.launch_count() - launches0
    st.synchronize()
    t_fused = e0.elapsed_time(e1) * 1e-3 / args.steps
    t_fused = barrier_max(t_fused, ws)
    block_ms = [a.elapsed_time(b) for a, b in ev_pairs]
    mean_block_s = statistics.mean(block_ms) * 1e-3 if block_ms else float("nan")
    value = ws * amp_updates / t_fused

    parts = set(args.parts.split(","))
    if "plain" not in parts:
        lib.qsv_plan_destroy(plan)
        st.close()
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "amp-updates/s", "n_gpus": ws,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_fused * 1e3,
                              "partial": sorted(parts), "mean_block_ms": mean_block_s * 1e3,
                              "gpu_launches": int(launches), "fusion_kmax": kmax, "fused_blocks": len(blocks),
                              "autotune": {"width_predicted_ms": {str(k): round(v, 3)
                                                                  for k, v in width_report.items()},
                                           "block_modes": mode_counts, "plan_seconds": t_plan}}), flush=True)
        return
    # The end-to-end leg runs right after the fused leg, before the complex128 per-gate leg:
    # device-to-host copies measured just after seconds of heavy GPU work ran slower (the
    # same copy loop in a fresh process: 11 ms on an idle GPU, 45-180 ms right after one),
    # and the fused value it is compared with was also taken first.
    # e2e through the plugin (StateType calls with host buffers).  Every step submits the
    # same circuit structure, so from the second circuit on the stream replays the
    # whole-circuit plan kept after the first (qip_gb300.plancache); the blocks per step
    # are reported.
    e2e_stats = {}
    stage_log = {True: [], False: []}

    def e2e_step(keep_plans=True):
        # Stages: create, submit (one kronselect_dot per gate; blocks launch while gates
        # arrive), drain (the last blocks; synchronize), readback (get_state: one DMA into
        # a pooled page-locked array), close.  The step's time is their sum.
        t0 = time.perf_counter()
        s2 = GpuBackend.make_state(n, [], [], statetype=numpy.complex64, fusion=True, max_block=kmax,
                                   keep_plans=keep_plans)
        t1 = time.perf_counter()
        for g in gl:
            s2.kronselect_dot(g)
        t2 = time.perf_counter()
        s2.synchronize()
        t3 = time.perf_counter()
        out = s2.get_state()
        t4 = time.perf_counter()
        e2e_stats.update(s2.stats)
        s2.close()
        t5 = time.perf_counter()
        stage_log[keep_plans].append((t1 - t0, t2 - t1, t3 - t2, t4 - t3, t5 - t4,
                                      s2.stats["readback_buffer_ms"] * 1e-3, s2.stats["readback_copy_ms"] * 1e-3,
                                      float(s2.stats["readback_page_locked"])))
        return out

    # Every timed step counts (up to 10): a single slow readback (host memory shared with
    # other work on the machine) then moves the mean less.
    e2e_steps = max(1, min(args.steps, 10))
    # Warm-up holds two results at once, as the timed loop does (the previous step's
    # array is alive while the next one runs): both page-locked readback buffers exist
    # before timing starts.
    w1 = e2e_step()
    w2 = e2e_step()
    del w1, w2
    stage_log[True].clear()
    # The objects this benchmark built for the other legs live on; keep the collector's
    # full scans from walking them during the timed steps (collection itself stays on).
    gc.collect()
    gc.freeze()
    barrier(ws)
    with ClockSampler(local) as clk_e2e:
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            host = e2e_step()
        t_e2e = barrier_max((time.perf_counter() - t0) / e2e_steps, ws)
    replay_stats = dict(e2e_stats)
    # The same circuits as a program that runs each once sees them: planned window by
    # window while the gates stream in (no kept plan); reported beside the value.
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        host = e2e_step(keep_plans=False)
    t_streamed = barrier_max((time.perf_counter() - t0) / e2e_steps, ws)
    streamed_blocks = e2e_stats.get("blocks")
    gc.unfreeze()
    h2d = sum(fusion_image_bytes(len(b.qubits)) for b in blocks) + sum(
        numpy.asarray(op.mat).nbytes for kind, op in seq if kind == "op" and op.mat is not None)
    d2h = host.nbytes
    del host
    # Plain complex128 per-gate path (the FP64 baseline of the metric).
    ref = GpuBackend.make_state(n, [], [], statetype=numpy.complex128, fusion=False)
    ref.set_stream(stream.cuda_stream)
    plain_ops = ops

    def plain_step():
        nat.check(lib.qsv_set_product_state(ref.handle, 0, None, None, None), ref.handle, "reset")
        for op in plain_ops:
            ref.apply_op(op)

    plain_step()
    torch.cuda.synchronize()
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    psteps = max(1, min(2, args.steps))
    p0.record(stream)
    for _ in range(psteps):
        plain_step()
    p1.record(stream)
    p1.synchronize()
    t_plain = barrier_max(p0.elapsed_time(p1) * 1e-3 / psteps, ws)
    # Infidelity of the fused FP32 result against the FP64 result.
    fused_step(False)
    st.synchronize()
    re_, im_ = ctypes.c_double(), ctypes.c_double()
    nat.check(lib.qsv_inner_product(st.handle, ref.handle, ctypes.byref(re_), ctypes.byref(im_)), st.handle, "inner")
    nrm = numpy.zeros(1)
    nrm_ref = numpy.zeros(1)
    nat.check(lib.qsv_norm2(st.handle, nat.dp(nrm)), st.handle)
    nat.check(lib.qsv_norm2(ref.handle, nat.dp(nrm_ref)), ref.handle)
    infid = 1.0 - (re_.value ** 2 + im_.value ** 2) / (nrm[0] * nrm_ref[0])
    # Largest amplitude difference, read back in chunks (outside any timed region).
    max_err = 0.0
    chunk = 1 << min(n, 24)
    a64 = numpy.empty(chunk, dtype=numpy.complex64)
    a128 = numpy.empty(chunk, dtype=numpy.complex128)
    for start in range(0, 1 << n, chunk):
        nat.check(lib.qsv_read_range(st.handle, a64.ctypes.data_as(ctypes.c_void_p), start, chunk), st.handle)
        nat.check(lib.qsv_read_range(ref.handle, a128.ctypes.data_as(ctypes.c_void_p), start, chunk), ref.handle)
        max_err = max(max_err, float(numpy.max(numpy.abs(a64.astype(numpy.complex128) - a128))))
    del a64, a128
    ref.close()
    lib.qsv_plan_destroy(plan)
    st.close()
    torch.cuda.synchronize()


    peak, peak_src = read_peaks()
    alg_bytes = 2 * (2 ** n) * 8
    achieved = alg_bytes / mean_block_s / 1e9
    traffic = NCU_BLOCK_TRAFFIC_N25 * 2.0 ** (n - 25)
    result = {
        "metric": METRIC, "value": value, "unit": "amp-updates/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_fused * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64",
        "data": "synthetic: seeded Haar-random brickwork, |0...0> input",
        "config": {"workload": f"brickwork n={n} depth {depth} (Haar 2x2 on every qubit, CZ even/odd pairs, "
                               f"C(Swap) every 10 layers)", "n": n, "depth": depth, "gates": len(gl),
                   "amp_updates_per_step": amp_updates, "fusion_kmax": kmax,
                   "autotune": {"width_predicted_ms": {str(k): round(v, 3) for k, v in width_report.items()},
                                "block_modes": mode_counts},
                   "fused_blocks": len(blocks), "standalone_ops": sum(1 for k, _ in seq if k == "op"),
                   "plan_seconds": t_plan, "parallelism": f"replicas x{ws}",
                   "l2": f"state {2 ** n * 8 / 2 ** 30:.0f} GiB > L2; no flush needed"},
        "plain_fp64": {"value": ws * amp_updates / t_plain, "ms_per_step": t_plain * 1e3, "steps": psteps,
                       "launches_per_step": len(ops)},
        "speedup_fused_vs_plain_fp64": t_plain / t_fused,
        "infidelity_vs_fp64": infid,
        "max_abs_err_vs_fp64": max_err,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum "
                     "of one k_block_tc launch at n=25, scaled by 2^(n-25)",
                     "kernel": "k_block_tc (fused block, k<=6)",
                     "per_launch_bytes": alg_bytes, "mean_launch_ms": mean_block_s * 1e3,
                     "peak_source": f"{peak_src} hbm_gbs"},
        "e2e": {"value": ws * amp_updates / t_e2e, "unit": "amp-updates/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "seconds_per_step": t_e2e, "steps": e2e_steps,
                "blocks_per_step": replay_stats.get("blocks"), "replayed_steps": replay_stats.get("replayed_steps"),
                "streamed": {"seconds_per_step": t_streamed, "value": ws * amp_updates / t_streamed,
                             "blocks_per_step": streamed_blocks,
                             "stages_ms": stage_summary(stage_log[False], len(gl)),
                             "note": "the same circuits with keep_plans=False: each planned window by window "
                                     "as a circuit run once is"},
                "stages_ms": stage_summary(stage_log[True], len(gl)),
                "clocks": clk_e2e.summary()},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    # Configs 3, 4 and 5 on the same GPU, each with its own CUDA-event timing and clocks.
    if "hbm" in parts:
        result["hbm_n32"] = measure_hbm(args)
    if "adjoint" in parts:
        result["adjoint"] = measure_adjoint(args)
    if "batched" in parts:
        result["batched"] = measure_batched(args, cpu_seconds=0 if args.no_cpu or "cpu" not in parts
                                            else min(args.cpu_seconds, 8.0))
    if rank == 0 and ws == 1 and not args.no_cpu and "cpu" in parts:
        v, info = cpu_reference_sample(n, gl, seconds_cap=args.cpu_seconds)
        info = dict(info)
        info["value"] = v
        info["unit"] = "amp-updates/s"
        result["cpu_baseline"] = info
        # Precision-matched: the GPU's complex128 per-gate path against the reference's
        # complex128 CPU kernel.
        if v:
            result["plain_fp64"]["vs_cpu_reference_c128"] = result["plain_fp64"]["value"] / v
    if rank == 0:
        print(json.dumps(result), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def stage_summary(rows, ngates):
    """Median milliseconds per e2e stage over the timed steps, and host microseconds per
    gate while submitting."""
    if not rows:
        return None
    names = ("create", "submit", "drain", "readback", "close", "readback_buffer", "readback_copy")
    med = [statistics.median(r[i] for r in rows) * 1e3 for i in range(len(names))]
    out = {k: round(v, 3) for k, v in zip(names, med)}
    out["submit_us_per_gate"] = round(med[1] * 1e3 / ngates, 2)
    out["readback_page_locked_steps"] = int(sum(r[7] for r in rows))
    out["readback_copy_ms_each"] = [round(r[6] * 1e3, 1) for r in rows]
    from qip_gb300 import hostbuf

    out["host_buffers"] = dict(hostbuf.counts)
    out["gc"] = "collector frozen over the setup objects; collection stays on"
    out["readback_note"] = "pooled page-locked array (no first-touch faults after warm-up)"
    return out


def fusion_image_bytes(k):
    kd = 2 << k
    return 2 * kd * kd * 2


def run_reference(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from qip_gb300 import circuits

    n, depth = args.n, args.depth
    gl = circuits.brickwork(n, depth, seed=SEED)
    kp = load_reference_kernels()
    if kp is None:
        print(json.dumps({"impl": "reference", "unavailable": "reference Cython kernels could not be built here"}))
        return
    vals = []
    info = None
    for i in range(args.warmup + args.steps):
        v, info = cpu_reference_sample(n, gl, seconds_cap=max(5.0, args.cpu_seconds / 2))
        if i >= args.warmup:
            vals.append(v)
    value = statistics.mean(vals)
    amp = circuits.gate_amp_updates(gl, n)
    info = dict(info)
    info["value"] = value
    info["unit"] = "amp-updates/s"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "amp-updates/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": amp / value * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic: seeded Haar-random brickwork, |0...0> input",
        "config": {"workload": f"brickwork n={n} depth {depth}", "n": n, "depth": depth,
                   "note": "reference CPU kernel timed on a bounded gate sample per step; ms_per_step "
                           "extrapolates the full circuit"},
        "cpu_baseline": info,
        "e2e": {"value": value, "unit": "amp-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# ---- supplementary workloads (one JSON line each; not the headline) -----------------------

def _events():
    import torch

    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def run_qft16(args):
    """QFT on n=16 qubits of a seeded N(0,1) state, complex128, through the graph API
    run() (state in, full state and top-4-qubit distribution out), against the inverse
    DFT (the QFT's known answer) and the reference's Cython kernel."""
    import torch

    from qip_gb300 import GpuBackend, QFFT, Qubit, StochasticMeasure, circuits, run

    n = 16
    rng = numpy.random.default_rng(2024)
    x = rng.standard_normal(2 ** n) + 1j * rng.standard_normal(2 ** n)
    x /= numpy.linalg.norm(x)
    q = Qubit(n=n)
    out = QFFT(q)
    top = out.split([4])
    sm = StochasticMeasure(top[0])
    want = numpy.fft.ifft(x, norm="ortho")
    i = numpy.arange(2 ** n)
    outcome = sum(((i >> (n - 1 - j)) & 1) << j for j in range(4))  # bit j <-> qubit j
    want_p = numpy.bincount(outcome, weights=numpy.abs(want) ** 2, minlength=16)
    amp = circuits.gate_amp_updates(circuits.qft_gates(n), n)
    for _ in range(args.warmup):
        run(sm, top[1], feed={q: x}, backend_constructor=GpuBackend.make_state)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o, classic = run(sm, top[1], feed={q: x}, backend_constructor=GpuBackend.make_state)
    dt = (time.perf_counter() - t0) / args.steps
    err = float(numpy.max(numpy.abs(o - want)))
    perr = float(numpy.max(numpy.abs(classic[sm] - want_p)))
    res = {"metric": "amp-updates/s (QFT n=16 complex128 through run(), e2e)", "value": amp / dt,
           "unit": "amp-updates/s", "ms_per_run": dt * 1e3, "steps": args.steps, "dtype": "c128",
           "config": {"workload": "QFT n=16 on a seeded N(0,1) state + distribution of the top 4 qubits"},
           "max_abs_err_vs_inverse_dft": err, "max_abs_err_top4_probs": perr}
    kp = load_reference_kernels()
    if kp is not None:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        gl = circuits.qft_gates(n)
        packed = [ref_pack(g) for g in gl]
        vec = x.astype(numpy.complex128).copy()
        o2 = numpy.zeros_like(vec)
        t0 = time.perf_counter()
        for ci, cm in packed:
            kp.cdot_loop(ci, cm, vec, n, o2)
            vec, o2 = o2, vec
        rt = time.perf_counter() - t0
        res["cpu_baseline"] = {"kind": "reference", "value": amp / rt, "unit": "amp-updates/s",
                               "cores": int(os.environ["OMP_NUM_THREADS"]),
                               "sample": f"the full QFT gate list through the reference cdot_loop ({rt:.2f} s)",
                               "max_abs_diff_vs_ours": float(numpy.max(numpy.abs(vec - o)))}
    print(json.dumps(res), flush=True)


def op_touched(op, n: int) -> float:
    """Amplitudes a per-gate pass rewrites: its control-satisfied subspace, restricted to
    the entries that are not the identity (diagonal: entries != 1; monomial: rows that
    move or change phase; swap: the a != b half, 1 - 2^-m of the subspace)."""
    sub = 2.0 ** (n - len(op.controls))
    k = len(op.targets)
    if op.kind == "diag":
        d = numpy.asarray(op.mat)
        return sub * numpy.count_nonzero(d != 1) / d.size
    if op.kind == "mono":
        perm, ph = numpy.asarray(op.perm), numpy.asarray(op.mat)
        moved = numpy.count_nonzero((perm != numpy.arange(perm.size)) | (ph != 1))
        return sub * moved / perm.size
    if op.kind == "swap":
        return sub * (1.0 - 2.0 ** (-k))
    return sub


def measure_hbm(args):
    """Config 3: QFT + 8 amplitude-amplification iterations at n=32 complex64 (fused) and
    n=31 complex128 (per-gate); every single-qubit marginal; per-pass achieved GB/s by
    CUDA events on the launching stream.  Checked against Grover's closed form (the QFT
    of |0...0> is the uniform state)."""
    import torch

    from qip_gb300 import GpuBackend, circuits, fusion, gates as gmod
    from qip_gb300.autotune import default_tuner

    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    peak, peak_src = read_peaks()
    out = {"metric": "achieved HBM GB/s per pass and amp-updates/s (QFT + 8 Grover iterations)",
           "unit": "GB/s", "peak": peak, "peak_source": f"{peak_src} hbm_gbs", "runs": []}
    for n, dt, fusion_on in ((args.hbm_n64, numpy.complex64, True), (args.hbm_n128, numpy.complex128, False)):
        gl, marked = circuits.grover_gates(n, 8, seed=7)
        amp = circuits.gate_amp_updates(gl, n)
        ops = [op for g in gl for op in gmod.decompose(g)]
        st = GpuBackend.make_state(n, [], [], statetype=dt, fusion=fusion_on)
        st.set_stream(stream.cuda_stream)
        size = 8 if dt == numpy.complex64 else 16
        per_kind = {}
        if fusion_on:
            steps = default_tuner().place(st.handle, n, fusion.plan(ops, kmax=6))
        else:
            steps = ops
        t_all0, t_all1 = _events()
        with ClockSampler(torch.cuda.current_device()) as clk:
            torch.cuda.synchronize()
            t_all0.record(stream)
            for stp in steps:
                a, b = _events()
                a.record(stream)
                if isinstance(stp, fusion.Block) and len(stp.qubits) >= 4:
                    st.apply_blocks([stp])
                    kind, touched = "fused_block", 2 ** n
                elif isinstance(stp, fusion.Block):
                    for op in gmod.classify_matrix(stp.qubits, (), stp.matrix):
                        st.apply_op(op)
                    kind, touched = "small_block", 2 ** n
                else:
                    st.apply_op(stp)
                    kind = f"{stp.kind}{len(stp.targets)}c{len(stp.controls)}"
                    touched = op_touched(stp, n)
                b.record(stream)
                per_kind.setdefault(kind, []).append((a, b, touched))
            t_all1.record(stream)
            t_all1.synchronize()
        total_s = t_all0.elapsed_time(t_all1) * 1e-3
        kinds = {}
        for k, lst in per_kind.items():
            ms = [a.elapsed_time(b) for a, b, _ in lst]
            byt = sum(2 * t * size for _, _, t in lst)
            gbs = byt / (sum(ms) * 1e-3) / 1e9
            kinds[k] = {"passes": len(lst), "mean_ms": round(statistics.mean(ms), 4), "GB_s": round(gbs, 1),
                        "frac": round(gbs / peak, 4)}
        marg, nrm = st.qubit_marginals()
        N = 2.0 ** n
        th = numpy.arcsin(1 / numpy.sqrt(N))
        pm = numpy.sin(17 * th) ** 2
        pu = (1 - pm) / (N - 1)
        bits = numpy.array([(marked >> (n - 1 - q)) & 1 for q in range(n)])
        want = pm * bits + pu * (N / 2 - bits)
        amp_m = st.get_relative_range(marked, marked + 1)[0]
        st.close()
        out["runs"].append({
            "n": n, "dtype": "c64" if dt == numpy.complex64 else "c128", "fused": fusion_on,
            "gates": len(gl), "passes": len(steps), "seconds": total_s, "amp_updates_per_s": amp / total_s,
            "per_pass": kinds, "marginals_p1": [float(f"{x:.10g}") for x in marg],
            "max_abs_err_marginals": float(numpy.max(numpy.abs(marg - want))),
            "norm2": nrm, "marked_index": marked, "marked_prob": float(abs(amp_m) ** 2),
            "marked_prob_expected": float(pm), "clocks": clk.summary()})
        torch.cuda.synchronize()
    fb = out["runs"][0]["per_pass"].get("fused_block")
    out["value"] = fb["GB_s"] if fb else None
    out["frac"] = fb["frac"] if fb else None
    out["kernel"] = "k_block_tc at n=32 (fused blocks of the QFT + Grover plan)"
    return out


def run_hbm(args):
    print(json.dumps(measure_hbm(args)), flush=True)


def measure_batched(args, cpu_seconds=None):
    """Config 4: 4096 independent circuits (n ~ U[8,20], depth ~ U[20,100]) in one
    persistent launch, replayed from a CUDA graph: circuits/s (CUDA events) and
    per-circuit device latency percentiles (%globaltimer stamps)."""
    import torch

    from qip_gb300 import batch

    circs, feeds, sizes = batch.random_batch(args.batch_count, seed=4096)
    b = batch.CircuitBatch(circs, feeds, sizes)
    stream = torch.cuda.Stream()
    for _ in range(max(3, args.warmup)):
        b.run(stream.cuda_stream)
    stream.synchronize()
    e0, e1 = _events()
    steps = max(5, args.steps)
    with ClockSampler(torch.cuda.current_device()) as clk:
        e0.record(stream)
        for _ in range(steps):
            b.run(stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
    dt = e0.elapsed_time(e1) * 1e-3 / steps
    lat = b.latencies_ns() / 1e6
    p50, p99 = float(numpy.percentile(lat, 50)), float(numpy.percentile(lat, 99))
    res = {"metric": "circuits/s (batched uneven circuits, one persistent launch)", "value": args.batch_count / dt,
           "unit": "circuits/s", "ms_per_step": dt * 1e3, "steps": steps, "dtype": "c64",
           "config": {"workload": f"{args.batch_count} circuits, n~U[8,20], depth~U[20,100], "
                                  "gates H/X/Rm/CNOT/C(Swap)/Haar, random product feeds"},
           "latency_ms": {"p50": p50, "p99": p99, "max": float(lat.max()), "p99_over_p50": p99 / p50},
           "clocks": clk.summary()}
    b.close()
    cap = args.cpu_seconds if cpu_seconds is None else cpu_seconds
    kp = load_reference_kernels() if cap > 0 else None
    if kp is not None:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        t0 = time.perf_counter()
        done = 0
        for gl, f, n in zip(circs, feeds, sizes):
            st = numpy.ones(1, dtype=numpy.complex128)
            for v in f:
                st = numpy.kron(st, v)
            o2 = numpy.zeros_like(st)
            for g in gl:
                ci, cm = ref_pack(g)
                kp.cdot_loop(ci, cm, st, n, o2)
                st, o2 = o2, st
            done += 1
            if time.perf_counter() - t0 > cap:
                break
        rt = time.perf_counter() - t0
        res["cpu_baseline"] = {"kind": "reference", "value": done / rt, "unit": "circuits/s",
                               "cores": int(os.environ["OMP_NUM_THREADS"]),
                               "sample": f"first {done} circuits of the same list through the reference cdot_loop"}
    return res


def run_batched(args):
    print(json.dumps(measure_batched(args)), flush=True)


def measure_adjoint(args):
    """Config 5: adjoint gradients, n=24, 20 layers of RY/RZ on every qubit + CNOT ring
    (960 angles), objective <sum Z>, batch of 64 parameter sets, complex64.  Forward and
    backward timed by CUDA events on the current stream; the gradient is spot-checked
    against complex128 central differences (h=1e-3) on seeded angles."""
    import torch

    from qip_gb300 import adjoint

    n, L, B = args.adj_n, args.adj_layers, args.adj_batch
    a = adjoint.Ansatz(n, L)
    th = torch.tensor(numpy.random.default_rng(2025).uniform(0, 2 * numpy.pi, (B, a.nparams)), device="cuda")
    fwd, bwd = [], []
    reps = max(1, min(args.steps, 2))
    with ClockSampler(torch.cuda.current_device()) as clk:
        for rep in range(1 + reps):
            thr = th.clone().requires_grad_(True)
            e0, e1 = _events()
            e2 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            e = adjoint.SumZExpectation.apply(thr, a, torch.complex64)
            e1.record()
            e.sum().backward()
            e2.record()
            e2.synchronize()
            if rep >= 1:
                fwd.append(e0.elapsed_time(e1) * 1e-3)
                bwd.append(e1.elapsed_time(e2) * 1e-3)
    g = thr.grad
    tf, tb = statistics.mean(fwd), statistics.mean(bwd)
    # The same gradients on the CUDA-core segment kernels (one timed repetition), for scale.
    thr2 = th.clone().requires_grad_(True)
    s0, s1 = _events()
    s2 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s0.record()
    e_seg = adjoint.SumZExpectation.apply(thr2, a, torch.complex64, "segmented")
    s1.record()
    e_seg.sum().backward()
    s2.record()
    s2.synchronize()
    seg = {"forward_s": s0.elapsed_time(s1) * 1e-3, "backward_s": s1.elapsed_time(s2) * 1e-3}
    seg["value"] = B / (seg["forward_s"] + seg["backward_s"])
    seg["max_abs_grad_diff_vs_tensor"] = float((thr2.grad - g).abs().max())
    rng = numpy.random.default_rng(77)
    idx = sorted({0, a.nparams - 1, *(int(x) for x in rng.choice(a.nparams, 4, replace=False))})
    errs = []
    for j in idx:
        tp, tm = th[:1].clone(), th[:1].clone()
        tp[0, j] += 1e-3
        tm[0, j] -= 1e-3
        with torch.no_grad():
            ep = adjoint.SumZExpectation.apply(tp, a, torch.complex128)
            em = adjoint.SumZExpectation.apply(tm, a, torch.complex128)
        fd = float((ep - em).item() / 2e-3)
        errs.append(abs(fd - float(g[0, j].item())))
    return {
        "metric": "gradient vectors/s (adjoint method, batch of parameter sets)", "value": B / (tf + tb),
        "unit": "gradients/s", "dtype": "c64", "steps": reps,
        "config": {"workload": f"ansatz n={n}, {L} layers RY/RZ + CNOT ring, {a.nparams} angles, batch {B}, "
                               "objective <sum Z>"},
        "forward_s": tf, "backward_s": tb, "backward_over_forward": tb / tf,
        "grad_components_per_s": B * a.nparams / (tf + tb),
        "method": "tensor cores: 6-qubit blocks, per-set block images, correlation GEMM + FP64 walk per block",
        "blocks": len(adjoint.tensor_core_plan(a).blocks),
        "fused_backward_blocks": adjoint.tensor_core_plan(a).fused_blocks, "cuda_core_segmented": seg,
        "max_abs_grad": float(g.abs().max()),
        "fd_checked_angles": idx, "max_abs_err_vs_fd_c128": max(errs),
        "cpu_baseline": None, "cpu_baseline_note": "the reference has no gradient code (qip/backend.py:14-65)",
        "clocks": clk.summary()}


def run_adjoint(args):
    print(json.dumps(measure_adjoint(args)), flush=True)


def run_block_placements(args):
    """One fused k-qubit block per target placement (high bits, low bits, mixed), timed
    with CUDA events: the fused kernel's achieved HBM bandwidth by placement."""
    import torch

    from qip_gb300 import GpuBackend, _native as nat

    n = args.n
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    st = GpuBackend.make_state(n, [], [], statetype=numpy.complex64, fusion=True)
    st.set_stream(stream.cuda_stream)
    lib = nat.load()
    rng = numpy.random.default_rng(3)
    k = args.kmax or 6
    bits_list = [list(range(n - k, n)), list(range(k)), [0, 1] + list(range(n - k + 2, n)),
                 [0, 1, 2, 3] + list(range(n - k + 4, n)), [1, 2, 3] + list(range(n - k + 3, n)),
                 [0, 2, 4, 6, 8, 10][:k], sorted(int(x) for x in rng.choice(n, k, replace=False))]
    for low in ([3, 4], [1, 2], [4, 5, 6], [1, 2, 3, 4], [5, 6]):
        bits_list.append(low + list(range(n - k + len(low), n)))
    peak, _ = read_peaks()
    rows = []
    for bits in bits_list:
        tg = [n - 1 - b for b in bits]  # qubit indices
        u = numpy.linalg.qr(rng.standard_normal((2 ** k, 2 ** k)) + 1j * rng.standard_normal((2 ** k, 2 ** k)))[0]
        ks, tgt = nat.int_array([k]), nat.int_array(sorted(tg))
        mats = numpy.ascontiguousarray(u.astype(numpy.complex128)).view(numpy.float64)
        p = ctypes.c_void_p()
        nat.check(lib.qsv_plan_create(st.handle, 1, nat.ip(ks), nat.ip(tgt), nat.dp(mats), ctypes.byref(p)), st.handle)
        for _ in range(args.warmup):
            nat.check(lib.qsv_plan_launch(st.handle, p, 0, 1), st.handle)
        e0, e1 = _events()
        e0.record(stream)
        for _ in range(args.steps):
            nat.check(lib.qsv_plan_launch(st.handle, p, 0, 1), st.handle)
        e1.record(stream)
        e1.synchronize()
        lib.qsv_plan_destroy(p)
        ms = e0.elapsed_time(e1) / args.steps
        gbs = 2 * (2 ** n) * 8 / (ms * 1e-3) / 1e9
        rows.append({"target_bits": bits, "ms": ms, "GB_s": gbs, "frac": gbs / peak})
    st.close()
    print(json.dumps({"metric": "fused block kernel GB/s by target placement", "unit": "GB/s", "n": n, "k": k,
                      "placements": rows}), flush=True)


def run_gate_placements(args):
    """Per-gate kernels by gate kind and target bit position (complex64 and complex128),
    CUDA-event timed: algorithmic GB/s = 2 x amplitudes the gate rewrites x amp size."""
    import torch

    from qip_gb300 import GpuBackend, circuits
    from qip_gb300.gates import GateOp

    n = args.n
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    peak, _ = read_peaks()
    rng = numpy.random.default_rng(5)
    h = numpy.array([[1, 1], [1, -1]]) / numpy.sqrt(2)
    u4 = numpy.linalg.qr(rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4)))[0]
    u8 = numpy.linalg.qr(rng.standard_normal((8, 8)) + 1j * rng.standard_normal((8, 8)))[0]

    def q(bit):
        return n - 1 - bit

    def kinds(p):
        p2 = p + 1 if p + 1 < n else p - 1
        p3 = p + 2 if p + 2 < n else p - 2
        return [
            ("haar1", GateOp("dense", (q(p),), (), circuits.haar_2x2(rng)), 1.0),
            ("h1", GateOp("dense", (q(p),), (), h), 1.0),
            ("phase1", GateOp("diag", (q(p),), (), numpy.array([1, numpy.exp(0.3j)])), 0.5),
            ("x1", GateOp("mono", (q(p),), (), numpy.array([1, 1]), perm=numpy.array([1, 0])), 1.0),
            ("cnot", GateOp("mono", (q(p),), (q(p2),), numpy.array([1, 1]), perm=numpy.array([1, 0])), 0.5),
            ("cz", GateOp("diag", (q(p), q(p2)), (), numpy.array([1, 1, 1, -1])), 0.25),
            ("dense2", GateOp("dense", (q(p), q(p2)), (), u4), 1.0),
            ("dense3", GateOp("dense", (q(p), q(p2), q(p3)), (), u8), 1.0),
            ("swap", GateOp("swap", (q(p),), (), swap_b=(q(p2),)), 0.5),
        ]

    rows = []
    for dt, size in ((numpy.complex64, 8), (numpy.complex128, 16)):
        st = GpuBackend.make_state(n, [], [], statetype=dt, fusion=False)
        st.set_stream(stream.cuda_stream)
        for p in (0, 1, 2, 3, 4, 5, 8, 16, n - 1):
            for name, op, frac in kinds(p):
                for _ in range(args.warmup):
                    st.apply_op(op)
                e0, e1 = _events()
                e0.record(stream)
                for _ in range(args.steps):
                    st.apply_op(op)
                e1.record(stream)
                e1.synchronize()
                ms = e0.elapsed_time(e1) / args.steps
                gbs = 2 * frac * (2 ** n) * size / (ms * 1e-3) / 1e9
                rows.append({"dtype": numpy.dtype(dt).name, "kind": name, "bit": p, "ms": round(ms, 4),
                             "GB_s": round(gbs, 1), "frac": round(gbs / peak, 3)})
        st.close()
    print(json.dumps({"metric": "per-gate kernel GB/s by kind and target bit", "unit": "GB/s", "n": n,
                      "peak": peak, "rows": rows}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--depth", type=int, default=DEPTH_DEFAULT)
    ap.add_argument("--kmax", type=int, default=0, help="fusion width; 0 = measured by the autotuner")
    ap.add_argument("--tune-cache", default=None,
                    help="JSON file of autotuner decisions: loaded if present, written after tuning")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--parts", default="fused,plain,e2e,cpu,hbm,adjoint,batched",
                    help="comma list of fused,plain,e2e,cpu,hbm,adjoint,batched (profiling runs use fused only)")
    ap.add_argument("--workload", default="brickwork", choices=["brickwork", "qft16", "hbm", "batched", "adjoint", "blocks", "gates"])
    ap.add_argument("--hbm-n64", type=int, default=32)
    ap.add_argument("--hbm-n128", type=int, default=31)
    ap.add_argument("--batch-count", type=int, default=4096)
    ap.add_argument("--adj-n", type=int, default=24)
    ap.add_argument("--adj-layers", type=int, default=20)
    ap.add_argument("--adj-batch", type=int, default=64)
    args = ap.parse_args()
    if args.tune_cache:
        os.environ["QSV_TUNE_CACHE"] = args.tune_cache
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "brickwork":
        run_ours(args)
    else:
        {"qft16": run_qft16, "hbm": run_hbm, "batched": run_batched, "adjoint": run_adjoint,
         "blocks": run_block_placements, "gates": run_gate_placements}[args.workload](args)


if __name__ == "__main__":
    main()
