"""Benchmark: seeded random brickwork circuit on n=30 qubits, depth 20.

Workload: every layer applies U3(t, p, l) (angles i.i.d. uniform [0, 2pi) from the
seed) to all 30 qubits, then CZ on disjoint nearest-neighbour pairs alternating even
and odd offsets: 600 U3 + 290 CZ = 890 gates, starting from |0...0>.

One step = |0...0> followed by the 890 gates, run by the GB300 engine's fused
(cache-blocked) path in complex64 — the precision mode whose bulk gate arithmetic is
complex64 and whose reductions are FP64 — on a state resident in HBM (8 GiB, larger
than the 129 MB L2, so no flush is needed between steps).  ``value`` is whole-job
gate-applications/s.  The same run also times, once each, the complex128 fused path,
the complex64 and complex128 per-gate (plain) paths, and reports the complex64
result's infidelity and max amplitude error against the complex128 state.

``roofline`` covers the dominant kernel (the fused pass): achieved = algorithmic bytes
of one pass (2 x 8 B x 2^30, one read and one write of the state) / its mean duration
from CUDA events over the timed region; FP32 arithmetic is reported beside it
(16 flops per amplitude per dense one-qubit gate).  ``e2e`` repeats the metric
through the public backend API (``execute_circuit_stream``) with every step's initial
state uploaded from pinned host memory and its final state read back, the copies of
neighbouring steps overlapped with the passes; ``sequential_value`` is the same through
``execute_circuit`` one call at a time.
``cpu_baseline`` and ``--impl reference`` time the CPU restatement of the reference's
Numba kernels (per-gate, OpenMP, all host threads) on the first layer of the circuit.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_QUBITS = 30
DEPTH = 20
SEED = 1234
FALLBACK_HBM_GBS = 6800.0
FP32_PEAK_TFLOPS = 73.3  # FP32 FMA rate measured on this GPU type by a probe (2 flops per FMA)


def metric_name(n: int) -> str:
    return f"gate-applications/s (brickwork n={n} depth {DEPTH})"


UNIT = "gates/s"


def _peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def _traffic_from_profiles(key: str):
    """DRAM bytes per launch recorded in the committed ncu summary, or None."""
    try:
        for line in open(os.path.join(ROOT, "profiles", f"{key}.md")):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sms)}


def _dist():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0"))


def cpu_baseline_oracle(n: int, dtype: str, sample_layers: int = 1):
    """The oracle's per-gate restatement of the reference kernels, first layer(s) of the circuit."""
    from oracle import pyoracle as O
    from qibojit_gb300 import circuits
    from qibojit_gb300.matrices import CustomMatrices

    cores = O.max_threads()
    circ = circuits.brickwork(n, DEPTH, SEED)
    gates = circ.queue[: (n + n // 2) * sample_layers]
    cm = CustomMatrices(dtype)
    ob = O.OracleBackend()
    state = np.empty(1 << n, dtype=dtype)
    O.initial_state_vector(state)
    t0 = time.perf_counter()
    for g in gates:
        q = ob.qubits_tensor(n, g.target_qubits, g.control_qubits)
        if type(g).__name__ == "U3":
            ob._one_qubit_base(state, n, g.target_qubits[0], "apply_gate", cm.U3(*g.parameters), q)
        else:
            ob._one_qubit_base(state, n, g.target_qubits[0], "apply_z", None, q)
    dt = time.perf_counter() - t0
    del state
    return {"value": len(gates) / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"first {sample_layers} layer(s) ({len(gates)} gates) of the n={n} {dtype} circuit, per-gate "
                      f"C/OpenMP restatement of the reference Numba kernels, {dt:.2f} s"}


def run_reference(args):
    ws, rank = _dist()
    if rank != 0:
        return
    n = args.nqubits
    for _ in range(max(0, args.warmup)):
        pass  # the CPU sample has no warm-up state; each step is a fresh bounded sample
    vals, last = [], None
    for _ in range(max(1, args.steps)):
        last = cpu_baseline_oracle(n, args.dtype, 1)
        vals.append(last["value"])
    v = statistics.median(vals)
    last["value"] = v
    line = {"impl": "reference", "metric": metric_name(n), "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * (n + n // 2) / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64" if args.dtype == "complex64" else "c128", "data": "synthetic",
            "config": {"workload": f"brickwork n={n} depth {DEPTH} {args.dtype} (seed {SEED})",
                       "sample": "one layer (45 gates) per step, per-gate"},
            "cpu_baseline": last,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def replicas_throughput(elapsed_ms: float, units_per_rank: float, device: str = "cuda"):
    """Whole-job throughput of N independent replicas (one circuit per rank, no data
    exchange): the units of all ranks over the slowest rank's time.  Returns
    (max elapsed ms, units/s)."""
    import torch

    dist = torch.distributed
    ws = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    if ws > 1:
        t = torch.tensor([float(elapsed_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    return elapsed_ms, ws * units_per_rank / (elapsed_ms / 1000.0)


def _fp32_issue(arith_per_amp: float, n: int, ms: float) -> dict:
    """The fused passes against their own bound: the plan's arithmetic lane instructions
    (FFMA and FMUL, counted from its pass blocks by sv_program_arith_per_amplitude) over
    the step's pass time, against the FP32 FMA rate a probe measured on this GPU type
    (one lane instruction per FMA)."""
    return _fp32_issue_total(arith_per_amp * (1 << n), ms) | {"instructions_per_amplitude_per_step": arith_per_amp}


def _fp32_issue_total(instructions: float, ms: float) -> dict:
    achieved = instructions / (ms / 1000.0) / 1e12
    peak = FP32_PEAK_TFLOPS / 2.0
    return {"instructions": instructions, "achieved": achieved, "peak": peak, "unit": "T lane-instructions/s",
            "frac": achieved / peak, "peak_kind": "FP32 FMA rate of a probe"}


def _time_program(torch, prog, backend, state, dcode, n, steps, stream):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        backend.lib.sv_zero_state(backend.ctx.handle, state.data_ptr(), dcode, n)
        prog.run(state)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def run_engine(args):
    import torch

    ws, rank = _dist()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from qibojit_gb300 import MetaBackend, circuits
    from qibojit_gb300 import _lib

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    backend = MetaBackend.load("gb300", device=dev)
    n = args.nqubits
    dtype = args.dtype
    dcode = _lib.DTYPE_CODES[dtype]
    itemsize = 16 if dtype == "complex128" else 8
    circ = circuits.brickwork(n, DEPTH, SEED + rank)
    ngates = len(circ.queue)
    n_u3 = sum(1 for g in circ.queue if type(g).__name__ == "U3")
    # the headline program: the autotuner times the cache-blocked passes on each tile
    # size (pass kernels specialised to this circuit's structure at run time, compiled
    # once, outside the timed region) and the fastest is the one measured
    from qibojit_gb300.autotune import autotune

    specialize = True
    t_tune = time.perf_counter()
    tiles = (11, 12, 13) if dtype == "complex64" else (10, 11, 12)
    best, tune_rows = autotune(backend, circ, dtype, candidates=[("passes", t) for t in tiles], reps=1)
    t_tune = time.perf_counter() - t_tune
    torch.cuda.empty_cache()
    t_spec = time.perf_counter()
    prog = backend.compile(circ, dtype, tile_bits=best[1], specialize=specialize)
    t_spec = time.perf_counter() - t_spec
    st = prog.stats()
    # lane instructions (FFMA, FMUL) per amplitude of one step as planned: the bound of
    # the fused complex64 passes is FP32 issue, not HBM
    arith_per_amp = prog.arith_per_amplitude()
    state = backend.zero_state(n, dtype=dtype)
    stream = torch.cuda.current_stream()

    # ---- warm-up, then the timed region (events on the launching stream)
    for _ in range(args.warmup):
        backend.lib.sv_zero_state(backend.ctx.handle, state.data_ptr(), dcode, n)
        prog.run(state)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    # the zero-state kernel is timed alone so the fused passes' share is exact
    zs_ms = _time_program(torch, type("Z", (), {"run": staticmethod(lambda s: s)}), backend, state, dcode, n, 3, stream)
    with ClockSampler(dev) as clocks:
        ms_step = _time_program(torch, prog, backend, state, dcode, n, args.steps, stream)
    elapsed_ms, value = replicas_throughput(ms_step * args.steps, ngates * args.steps, "cuda")
    if ws > 1:
        torch.distributed.barrier()
    pass_ms = (ms_step - zs_ms) / st["passes"]

    # ---- end to end through the public API.  Each step starts from |0...0> prepared on
    # the device (config 2's initial state), its inputs are the gate coefficients sent
    # with the pass launches, and its result, the final state, is read back into pinned
    # host memory; execute_circuit_stream overlaps step k-1's read-back with step k's
    # passes.  The variant beside it also uploads a host initial state every step.
    host_in = backend.host_buffer(n, dtype)  # pinned, on the GPU's local memory node
    host_in[0] = 1
    host_out = backend.host_buffer(n, dtype)
    for _ in range((backend.specialize_after or 0) + 1):  # plans, caches and specialises the program
        backend.execute_circuit(circ, host_in)
    torch.cuda.synchronize()
    nbytes_state = (1 << n) * itemsize
    link = _link_rates(torch, backend, host_out, nbytes_state)
    e2e_steps = max(3, min(2 * args.steps, 8))
    backend.execute_circuit_stream(circ, None, [host_out])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    backend.execute_circuit_stream(circ, None, [host_out] * e2e_steps)
    e2e_value = ws * ngates * e2e_steps / (time.perf_counter() - t0)
    param_bytes = backend._cached_program(circ, dtype).param_bytes()
    # the same with the initial state uploaded from pinned host memory every step
    t0 = time.perf_counter()
    backend.execute_circuit_stream(circ, [host_in] * e2e_steps, [host_out] * e2e_steps)
    e2e_roundtrip = ws * ngates * e2e_steps / (time.perf_counter() - t0)
    # one call at a time: upload, passes and read-back in sequence
    seq_steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(seq_steps):
        s = backend.execute_circuit(circ, host_in)
        host_out.copy_(s)
        del s
    torch.cuda.synchronize()
    e2e_seq_value = ws * ngates * seq_steps / (time.perf_counter() - t0)
    backend.execute_circuit_stream(circ, [host_in], [host_out])
    torch.cuda.synchronize()
    final64 = host_out  # |psi> of the complex64 fused run, on the host

    # ---- variants, timed once each after one warm-up (same circuit)
    variants = {}
    if not args.quick and rank == 0:
        plain_ms = {}
        for vdt in ("complex64", "complex128"):
            s = backend.zero_state(n, dtype=vdt)
            backend.execute_circuit(circ, s, fuse=False)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            backend.execute_circuit(circ, backend.zero_state(n, dtype=vdt), fuse=False)
            e1.record(stream)
            torch.cuda.synchronize()
            plain_ms[vdt] = e0.elapsed_time(e1)
            del s
            torch.cuda.empty_cache()
        # the same circuit on the interpreting tile kernel (default tile), complex64
        pint = backend.compile(circ, "complex64")
        sint = backend.zero_state(n, dtype="complex64")
        _time_program(torch, pint, backend, sint, _lib.SV_C64, n, 1, stream)
        int_ms = _time_program(torch, pint, backend, sint, _lib.SV_C64, n, 2, stream)
        del pint, sint
        torch.cuda.empty_cache()
        # complex128 passes in double-word arithmetic: the interpreting kernel (shared op
        # code) outruns the compiled passes, whose unrolled double-word ops overflow the
        # instruction cache; both are timed, the faster is reported
        p128 = backend.compile(circ, "complex128", specialize=True)
        s128 = backend.zero_state(n, dtype="complex128")
        f128_spec_ms = _time_program(torch, p128, backend, s128, _lib.SV_C128, n, 1, stream)
        del p128
        p128 = backend.compile(circ, "complex128")
        f128_int_ms = _time_program(torch, p128, backend, s128, _lib.SV_C128, n, 1, stream)
        f128_ms = min(f128_spec_ms, f128_int_ms)
        s64 = backend.cast(final64, dtype="complex64")
        ip = backend.inner_product(s128, s64, n)
        variants = {
            "c64_fused_gates_per_s": value,
            "c64_fused_interpreted_gates_per_s": ngates / ((int_ms - zs_ms) / 1000.0),
            "c128_fused_gates_per_s": ngates / (f128_ms / 1000.0),
            "c128_fused_compiled_gates_per_s": ngates / (f128_spec_ms / 1000.0),
            "c128_fused_interpreted_gates_per_s": ngates / (f128_int_ms / 1000.0),
            "c64_plain_gates_per_s": ngates / (plain_ms["complex64"] / 1000.0),
            "c128_plain_gates_per_s": ngates / (plain_ms["complex128"] / 1000.0),
            "precision": {
                "infidelity_c64_vs_c128": 1.0 - abs(ip) ** 2,
                "infidelity_normalised": 1.0 - abs(ip) ** 2 / (backend.norm2(s64, n) * backend.norm2(s128, n)),
                "max_abs_err_c64_vs_c128": backend.max_abs_diff(s64, s128, n),
                "norm2_fp64_c64": backend.norm2(s64, n),
                "zz01_c64": backend.expectation_z(s64, [0, 1], n),
                "zz01_c128": backend.expectation_z(s128, [0, 1], n),
            },
        }
        variants["measurement_n30"] = _measurement_variants(torch, backend, stream, n, {"complex64": s64,
                                                                                       "complex128": s128})
        del s128, s64
        torch.cuda.empty_cache()
        variants["dense_gates_n30_c64"] = _dense_gate_variants(torch, backend, stream, n)
        variants["c128_gates_n30"] = _c128_gate_variants(torch, backend, stream, n)
        variants["fusion_k_sweep_n30_c64"] = _fusion_sweep(backend, circ)
        torch.cuda.empty_cache()
        variants.update(_extra_workloads(torch, backend, stream, args))
        variants["precision_n32_depth40"] = precision_report(backend, 32, 40)

    peak, peak_kind = _peak_hbm()
    kname = "sv_pass" if specialize else "k_fused_pass"
    pass_bytes = 2 * itemsize * (1 << n)
    achieved = pass_bytes / (pass_ms / 1000.0) / 1e9
    # the gates' flops counted as dense complex 2x2s (16 per amplitude and U3; CZ sign flips
    # carry none); phase-folded passes do fewer operations than this for the same unitary
    flops_per_step = 16.0 * (1 << n) * n_u3
    fp32_tflops = flops_per_step / ((ms_step - zs_ms) / 1000.0) / 1e12
    nbytes = (1 << n) * itemsize
    if rank == 0:
        cb = cpu_baseline_oracle(n, dtype, 1) if (not args.skip_cpu and ws == 1) else None
        line = {
            "metric": metric_name(n), "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64" if dtype == "complex64" else "c128",
            "data": "synthetic",
            "config": {"workload": f"brickwork n={n} depth {DEPTH} {dtype} (seed {SEED}), fused cache-blocked passes",
                       "gates_per_step": ngates, "passes_per_step": st["passes"], "tile_bits": st["tile_bits"],
                       "pass_kernels": "specialised at run time" if specialize else "interpreting tile kernel",
                       "specialise_seconds": round(t_spec, 2) if specialize else None,
                       "autotuned": {"pick": f"{best[0]}:{best[1]}", "seconds": round(t_tune, 2),
                                     "candidates": tune_rows},
                       "state_bytes": nbytes, "l2": "state larger than the 129 MB L2; no flush needed",
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": _traffic_from_profiles(f"{kname}_{dtype}"), "peak_kind": peak_kind,
                         "kernel": kname, "algorithmic_bytes_per_launch": pass_bytes,
                         "avg_launch_ms": pass_ms, "dense_u3_equivalent_fp32_tflops": fp32_tflops,
                         "dense_u3_equivalent_frac_of_fp32_probe_peak": fp32_tflops / FP32_PEAK_TFLOPS,
                         "fp32_issue": _fp32_issue(arith_per_amp, n, ms_step - zs_ms)},
            "cpu_baseline": cb,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": param_bytes, "d2h_bytes_per_step": nbytes,
                    "steps": e2e_steps,
                    "api": "execute_circuit_stream from |0...0> on the device, final state read back into pinned "
                           "host memory (read-back of step k-1 overlapped with step k's passes); h2d = the pass "
                           "parameter blocks sent with the launches",
                    "state_upload_value": e2e_roundtrip, "state_upload_h2d_bytes_per_step": nbytes,
                    "sequential_value": e2e_seq_value, "sequential_steps": seq_steps, "link": link},
            "gpu_launches": args.steps * (st["passes"] + 1),
            "clocks": clocks.summary(),
            "variants": variants,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def _unitary(d, seed):
    """Seeded Haar-random d x d unitary (QR of a complex Gaussian matrix, phases fixed)."""
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d)))
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _events_ms(torch, stream, fn, reps=3):
    """Mean device time of fn() over reps calls (CUDA events on the launching stream),
    after one untimed call."""
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _frac(nbytes, ms):
    peak, _ = _peak_hbm()
    gbs = nbytes / (ms / 1000.0) / 1e9
    return {"ms": ms, "algorithmic_bytes": nbytes, "achieved_gbs": gbs, "frac_of_hbm": gbs / peak}


def _link_rates(torch, backend, host, nbytes):
    """Achieved pinned host <-> device copy rates for one state (CUDA events on the
    current stream), with the CPUs next to the GPU that the pinned pages were placed on."""
    from qibojit_gb300.backend import _gpu_local_cpus

    dev = torch.empty(host.numel(), dtype=host.dtype, device="cuda")
    stream = torch.cuda.current_stream()
    h2d = _events_ms(torch, stream, lambda: dev.copy_(host, non_blocking=True), reps=2)
    d2h = _events_ms(torch, stream, lambda: host.copy_(dev, non_blocking=True), reps=2)
    del dev
    torch.cuda.empty_cache()
    cpus = _gpu_local_cpus(torch.cuda.current_device())
    return {"h2d_gbs": nbytes / (h2d / 1000.0) / 1e9, "d2h_gbs": nbytes / (d2h / 1000.0) / 1e9,
            "pinned_on_gpu_local_cpus": sorted(cpus)[:1] + sorted(cpus)[-1:] if cpus else None}


def _measurement_variants(torch, backend, stream, n, states):
    """Config 2's measurement stage at n=30 on the brickwork's final states: the full
    2^n-entry probabilities, 10^6 Metropolis shots over all qubits (the reference's
    branch above SHOT_METROPOLIS_THRESHOLD, one chain per host thread, cpu.py:383-394,
    ops.py:82-108) and the normalised collapse on qubits 0-3 (ops.py:63-79)."""
    out = {}
    for dt, s in states.items():
        b = 16 if dt == "complex128" else 8
        pb = 8 if dt == "complex128" else 4
        r = {}
        holder = {}

        def probs():
            holder["p"] = backend.calculate_probabilities(s, list(range(n)), n)

        r["probabilities_all_qubits"] = _frac(b * (1 << n) + pb * (1 << n), _events_ms(torch, stream, probs))
        p = holder["p"]
        freqs = torch.zeros(1 << n, dtype=torch.int64, device=s.device)

        def shots():
            freqs.zero_()
            backend.measure_frequencies_op(freqs, p, 10**6, n, 1234, backend.nthreads)

        ms = _events_ms(torch, stream, shots, reps=2)
        r["metropolis_1e6_shots"] = {"ms": ms, "chains": backend.nthreads, "shots_per_s": 1e6 / (ms / 1000.0),
                                     "shots_counted": int(freqs.sum().item()),
                                     "note": "one dependent random 8-byte probability read per proposal: latency-bound"}
        del freqs, p
        holder.clear()
        work = torch.empty_like(s)

        def collapse():
            work.copy_(s)
            backend.collapse_state(work, [0, 1, 2, 3], 5, n, normalize=True)

        copy_ms = _events_ms(torch, stream, lambda: work.copy_(s))
        ms = _events_ms(torch, stream, collapse) - copy_ms
        r["collapse_qubits_0_3"] = _frac(b * (1 << n) + 2 * b * (1 << (n - 4)), ms)
        r["collapse_qubits_0_3"]["norm2_after"] = backend.norm2(work, n)
        del work
        torch.cuda.empty_cache()
        out[dt] = r
    return out


def _dense_gate_variants(torch, backend, stream, n):
    """Dense k-target complex64 gates at n=30 on the tensor cores (tcgen05, TF32 split
    in two) and on the CUDA-core kernels, targets on the highest and lowest qubits."""
    s = backend.zero_state(n, dtype="complex64")
    out = {}
    for k in (4, 5, 6):
        g = _unitary(2**k, k).astype(np.complex64)
        for where, targets in (("high_bits", list(range(k))), ("low_bits", list(range(n - k, n)))):
            row = {}
            for mode in ("tensor", "simt"):
                backend.ctx.set_dense_mode(mode)
                ms = _events_ms(torch, stream, lambda: backend._multi_qubit_base(s, n, targets, g, None))
                row[mode] = _frac(2 * 8 * (1 << n), ms)
            backend.ctx.sync()
            out[f"k{k}_{where}"] = row
    backend.ctx.set_dense_mode("auto")
    del s
    torch.cuda.empty_cache()
    return out


def _c128_gate_variants(torch, backend, stream, n):
    """complex128 per-gate passes at n=30: double-word arithmetic on the FP32 pipe
    against FP64 instructions."""
    s = backend.zero_state(n, dtype="complex128")
    u2, u4, u8, u16, u32 = _unitary(2, 1), _unitary(4, 2), _unitary(8, 3), _unitary(16, 4), _unitary(32, 5)
    cases = {
        "u3_target0": (lambda: backend._one_qubit_base(s, n, 0, "apply_gate", u2, None), 32 << n),
        "u3_target29": (lambda: backend._one_qubit_base(s, n, n - 1, "apply_gate", u2, None), 32 << n),
        "u1_target15": (lambda: backend._one_qubit_base(s, n, 15, "apply_z_pow", np.array(np.exp(0.3j)), None),
                        16 << n),
        "two_target_3_17": (lambda: backend._two_qubit_base(s, n, 3, 17, "apply_two_qubit_gate", u4, None), 32 << n),
        "three_target_0_1_2": (lambda: backend._multi_qubit_base(s, n, [0, 1, 2], u8, None), 32 << n),
        "four_target_0_1_2_3": (lambda: backend._multi_qubit_base(s, n, [0, 1, 2, 3], u16, None), 32 << n),
        "five_target_0_to_4": (lambda: backend._multi_qubit_base(s, n, [0, 1, 2, 3, 4], u32, None), 32 << n),
    }
    out = {}
    for name, (fn, nbytes) in cases.items():
        row = {}
        for mode in ("double-word", "fp64"):
            backend.ctx.set_c128_arithmetic(mode)
            row[mode] = _frac(nbytes, _events_ms(torch, stream, fn))
        out[name] = row
    backend.ctx.set_c128_arithmetic("double-word")
    del s
    torch.cuda.empty_cache()
    return out


def _fusion_sweep(backend, circ):
    """The brickwork fused into dense blocks of k = 2..6 qubits (one HBM pass per block,
    qibo Circuit.fuse-style; 5- and 6-qubit complex64 blocks on the tensor cores)
    against the cache-blocked passes, each timed once by the autotuner."""
    from qibojit_gb300.autotune import autotune

    t0 = time.perf_counter()
    best, rows = autotune(backend, circ, "complex64",
                          candidates=[("blocks", k) for k in range(2, 7)] + [("passes", 13)], reps=1)
    return {"pick": f"{best[0]}:{best[1]}", "table": rows, "seconds": round(time.perf_counter() - t0, 1)}


def _extra_workloads(torch, backend, stream, args):
    """The other configurations of the same engine, one bounded measurement each:
    QFT n=20 complex128 (parity against sqrt(N) * ifft), the batched VQE forward pass
    (4096 hardware-efficient-ansatz circuits, n ~ U{10..22}, L ~ U{4..12}, TFIM
    energies) and adjoint TFIM gradients (n=26, 20 layers, 1040 parameters)."""
    from oracle import pyoracle as O
    from qibojit_gb300 import circuits
    from qibojit_gb300.adjoint import AdjointTFIM
    from qibojit_gb300.batch import BatchedCircuits, hea_batch

    out = {}
    # ---- QFT n=20, complex128
    n = 20
    q = circuits.qft(n)
    x = np.random.default_rng(SEED).standard_normal(2**n) + 1j * np.random.default_rng(SEED + 1).standard_normal(2**n)
    x /= np.linalg.norm(x)
    xd = backend.cast(x)
    res = {}
    for mode in ("plain", "fused"):
        # warm-up past the program cache's specialisation point (compiled once, untimed)
        for _ in range((backend.specialize_after or 0) + 1):
            s = backend.execute_circuit(q, xd, fuse=(mode == "fused"))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(5):
            s = backend.execute_circuit(q, xd, fuse=(mode == "fused"))
        e1.record(stream)
        torch.cuda.synchronize()
        res[f"qft_n20_c128_{mode}_gates_per_s"] = len(q.queue) * 5 / (e0.elapsed_time(e1) / 1000.0)
        res[f"qft_n20_c128_{mode}_max_abs_err_vs_ifft"] = float(
            np.abs(backend.to_numpy(s) - np.sqrt(2**n) * np.fft.ifft(x)).max())
    ob = O.OracleBackend()
    ref = x.copy()
    cm = backend.custom_matrices
    t0 = time.perf_counter()
    for g in q.queue:
        qt = ob.qubits_tensor(n, g.target_qubits, g.control_qubits)
        name = type(g).__name__
        if name == "H":
            ob._one_qubit_base(ref, n, g.target_qubits[0], "apply_gate", cm.H, qt)
        elif name == "CU1":
            ob._one_qubit_base(ref, n, g.target_qubits[0], "apply_z_pow", cm.CU1(*g.parameters), qt)
        else:
            ob._two_qubit_base(ref, n, *g.target_qubits, "apply_swap", None, qt)
    res["qft_n20_c128_cpu_reference_gates_per_s"] = len(q.queue) / (time.perf_counter() - t0)
    out["qft"] = res
    # ---- batched VQE forward, 4096 circuits
    specs = hea_batch(4096, seed=SEED)
    vq = {}
    batches = {}
    for dt, reps in (("complex64", 3), ("complex128", 1)):
        t0 = time.perf_counter()
        bat = BatchedCircuits.from_hea(backend, specs, dt)
        create_s = time.perf_counter() - t0

        def timed_runs():
            bat.run()  # eager run + CUDA graph capture
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                bat.run()
            e1.record(stream)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / reps

        ms_interp = timed_runs()  # interpreting pass kernel
        # the whole batch in one cooperative launch (interpreting kernel), then back to
        # the graph of per-group launches
        bat.set_executor("persistent")
        ms_persist = timed_runs()
        e_persist = bat.tfim_energies(1.0)
        bat.set_executor("graph")
        ms, spec_s = ms_interp, None
        # complex128 batches run the interpreting double-word kernel: compiling every
        # group's double-word passes takes minutes and measured no faster (3.87 against
        # 3.65 s per batch of 4096)
        if dt == "complex64":
            t0 = time.perf_counter()
            bat.specialize()  # one compiled kernel per group and pass
            spec_s = time.perf_counter() - t0
            ms = timed_runs()
        t0 = time.perf_counter()
        en = bat.tfim_energies(1.0)
        st = bat.stats()
        vq[dt] = {"circuits_per_s": 4096 / (ms / 1000.0), "ms_per_batch": ms, "energy_ms":
                  1000 * (time.perf_counter() - t0), "plan_s": create_s, "specialise_s": spec_s,
                  "interpreted_circuits_per_s": 4096 / (ms_interp / 1000.0),
                  "persistent_single_launch_circuits_per_s": 4096 / (ms_persist / 1000.0),
                  "persistent_max_abs_energy_diff": float(np.abs(e_persist - en).max()), "stats": st,
                  # every circuit's plan passes, each one read and one write of its state
                  "roofline": _frac(st["pass_bytes"], ms)}
        if dt == "complex64":  # the passes' arithmetic against the FP32 issue bound
            vq[dt]["fp32_issue"] = _fp32_issue_total(st["arith_instructions"], ms)
        vq[dt]["energies_head"] = [float(v) for v in en[:3]]
        batches[dt] = (bat, en)
    (b64, e64), (b128, e128) = batches["complex64"], batches["complex128"]
    vq["max_abs_energy_diff_c64_vs_c128"] = float(np.abs(e64 - e128).max())
    infid = []
    for i, nq in enumerate(b64.nqubits):
        a, b = b128.state(i), b64.state(i)
        ip = backend.inner_product(a, b, nq)
        infid.append(1.0 - abs(ip) ** 2 / (backend.norm2(a, nq) * backend.norm2(b, nq)))
    infid = np.array(infid)
    vq["infidelity_c64_vs_c128_per_circuit"] = {"max": float(infid.max()), "median": float(np.median(infid)),
                                                "circuits": len(infid), "normalised": True}
    for bat, _ in batches.values():
        bat.close()
    del batches, b64, b128
    torch.cuda.empty_cache()
    # CPU baseline on a sample: the oracle's per-gate kernels on the first 8 circuits
    from qibojit_gb300.batch import hea_circuit

    t0 = time.perf_counter()
    ngates = 0
    for nq, L, prm in specs[:8]:
        c = hea_circuit(nq, L, prm)
        st = ob.zero_state(nq, "complex64")
        for g in c.queue:
            qt = ob.qubits_tensor(nq, g.target_qubits, g.control_qubits)
            name = type(g).__name__
            if name == "CNOT":
                ob._one_qubit_base(st, nq, g.target_qubits[0], "apply_x", None, qt)
            else:
                ob._one_qubit_base(st, nq, g.target_qubits[0], "apply_gate", g.base_matrix("complex64"), qt)
            ngates += 1
    vq["cpu_reference_sample"] = {"circuits_per_s": 8 / (time.perf_counter() - t0),
                                  "sample": "first 8 circuits, per-gate C/OpenMP restatement, complex64"}
    out["vqe_forward_4096"] = vq
    # ---- adjoint gradients: one wave of 64 circuits, n=26, 20 layers, complex64
    nq, L, wave = 26, 20, 64
    prm = np.random.default_rng(SEED).uniform(0, 2 * np.pi, size=(wave, L, nq, 2))
    eng = AdjointTFIM(backend, nq, L, wave, "complex64", checkpoint_every=5, specialize=True)
    eng(prm)  # plans and allocates
    t0 = time.perf_counter()
    E, G = eng(prm)
    dt_s = time.perf_counter() - t0
    eng.close()
    del eng
    torch.cuda.empty_cache()
    # complex128 on a smaller wave (its fused passes are FP64-bound), against the complex64
    # gradients, energies and final states of the same circuits
    w128 = 4
    ad = {}
    for dt in ("complex128", "complex64"):
        e = AdjointTFIM(backend, nq, L, w128, dt, checkpoint_every=5, specialize=True)
        e(prm[:w128])
        t0 = time.perf_counter()
        Ew, Gw = e(prm[:w128])
        ad[dt] = (Ew, Gw, time.perf_counter() - t0, [e.state(i).clone() for i in range(w128)])
        e.close()
        del e
    infid = []
    for a, b in zip(ad["complex128"][3], ad["complex64"][3]):
        ip = backend.inner_product(a, b, nq)
        infid.append(1.0 - abs(ip) ** 2 / (backend.norm2(a, nq) * backend.norm2(b, nq)))
    c128 = {"gradient_vectors_per_s": w128 / ad["complex128"][2], "wave": w128,
            "c64_same_wave_gradient_vectors_per_s": w128 / ad["complex64"][2],
            "max_abs_gradient_diff_c64_vs_c128": float(np.abs(ad["complex64"][1] - ad["complex128"][1]).max()),
            "max_abs_energy_diff_c64_vs_c128": float(np.abs(ad["complex64"][0] - ad["complex128"][0]).max()),
            "max_final_state_infidelity_c64_vs_c128": float(max(infid))}
    del ad
    torch.cuda.empty_cache()
    # HBM traffic estimate: the forward plan's passes on psi, the reverse sweep's passes
    # on psi and lambda together (its plan has one pass per forward pass), each pass one
    # read and one write of the state; checkpoint copies left out
    fwd_passes = backend.compile(hea_circuit(nq, L, prm[0]), "complex64").stats()["passes"]
    adj_bytes = wave * 3 * fwd_passes * 2 * 8 * (1 << nq)
    # CPU: one forward evaluation of two layers on the oracle, scaled to a parameter-shift gradient
    c = hea_circuit(nq, 2, prm[0, :2])
    st = ob.zero_state(nq, "complex64")
    t0 = time.perf_counter()
    for g in c.queue:
        qt = ob.qubits_tensor(nq, g.target_qubits, g.control_qubits)
        if type(g).__name__ == "CNOT":
            ob._one_qubit_base(st, nq, g.target_qubits[0], "apply_x", None, qt)
        else:
            ob._one_qubit_base(st, nq, g.target_qubits[0], "apply_gate", g.base_matrix("complex64"), qt)
    t_two = time.perf_counter() - t0
    del st
    t_eval = t_two * L / 2
    out["adjoint_n26_L20"] = {"gradient_vectors_per_s": wave / dt_s, "wave": wave, "params_per_circuit": 2 * L * nq,
                              "s_per_wave": dt_s, "energy_head": [float(v) for v in E[:2]],
                              "cpu_parameter_shift_gradient_vectors_per_s_estimate": 1.0 / (2 * 2 * L * nq * t_eval),
                              "cpu_sample": f"2 of {L} layers forward on the oracle ({t_two:.1f} s), scaled to "
                                            f"{2 * 2 * L * nq} shifted evaluations",
                              "roofline_estimate": {**_frac(adj_bytes, 1000.0 * dt_s), "forward_passes": fwd_passes},
                              "complex128": c128}
    return out


def precision_report(backend, n: int, depth: int) -> dict:
    """The precision configuration: brickwork n=32, depth 40 (1280 U3 + 620 CZ), the
    complex64 state (32 GiB) on specialised fused passes against the complex128 state
    (64 GiB) on fused passes, both on this GPU; the complex128 run is the reference
    precision (its passes are pinned to the oracle at n <= 28 by the tests)."""
    import torch

    from qibojit_gb300 import circuits

    circ = circuits.brickwork(n, depth, SEED)
    ngates = len(circ.queue)
    stream = torch.cuda.current_stream()
    out = {}
    states = {}
    # complex128 on the interpreting kernel: its double-word passes outrun the compiled ones
    for dt, spec in (("complex64", True), ("complex128", False)):
        t0 = time.perf_counter()
        prog = backend.compile(circ, dt, specialize=spec)
        plan_s = time.perf_counter() - t0
        s = backend.zero_state(n, dtype=dt)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        prog.run(s)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        out[dt] = {"gates_per_s": ngates / (ms / 1000.0), "ms": ms, "passes": prog.stats()["passes"],
                   "tile_bits": prog.stats()["tile_bits"], "plan_and_compile_s": round(plan_s, 2),
                   "pass_kernels": "specialised" if spec else "interpreting"}
        states[dt] = s
        del prog
    s64, s128 = states["complex64"], states["complex128"]
    ip = backend.inner_product(s128, s64, n)
    rep = {
        "workload": f"brickwork n={n} depth {depth} (seed {SEED})", "gates": ngates,
        "state_bytes": {"c64": 8 << n, "c128": 16 << n},
        # 1 - |<psi128|psi64>|^2 (raw: includes the complex64 state's norm drift) and
        # the infidelity of the normalised states
        "infidelity_c64_vs_c128": 1.0 - abs(ip) ** 2,
        "infidelity_normalised": 1.0 - abs(ip) ** 2 / (backend.norm2(s64, n) * backend.norm2(s128, n)),
        "max_abs_err_c64_vs_c128": backend.max_abs_diff(s64, s128, n),
        "norm2_fp64_c64": backend.norm2(s64, n),
        "norm2_fp64_c128": backend.norm2(s128, n),
        "zz01_c64": backend.expectation_z(s64, [0, 1], n),
        "zz01_c128": backend.expectation_z(s128, [0, 1], n),
        "runs": out,
    }
    del states, s64, s128
    torch.cuda.empty_cache()
    return rep


def run_precision(args):
    """``--precision``: the precision configuration on its own (one JSON line)."""
    from qibojit_gb300 import MetaBackend

    backend = MetaBackend.load("gb300")
    rep = precision_report(backend, args.precision_nqubits, 40)
    line = {"metric": f"precision (brickwork n={args.precision_nqubits} depth 40)", "n_gpus": 1,
            "dtype": "c64 vs c128", "data": "synthetic", **rep}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--nqubits", type=int, default=N_QUBITS)
    ap.add_argument("--dtype", default="complex64", choices=["complex128", "complex64"])
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--quick", action="store_true", help="skip the variants and the precision report")
    ap.add_argument("--precision", action="store_true",
                    help="run only the precision configuration (brickwork depth 40, c64 against c128)")
    ap.add_argument("--precision-nqubits", type=int, default=32)
    args = ap.parse_args()
    if args.precision:
        run_precision(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
