#!/usr/bin/env python3
"""Benchmark of the GB300 state-vector engine on the 30-qubit gate sweep.

Workload (one step): a seeded depth-40 random circuit on 30 qubits — each
layer H/RX/RY/RZ on every qubit, then 15 disjoint CNOT/CZ/SWAP pairs, half
nearest-neighbour, half long-range — applied to a resident complex64 state
(8 GiB, larger than L2, so no flush is needed between steps). The metric is
whole-job gates/s; the roofline is HBM bandwidth of the tile-pass kernels
(2 * 2^30 * 8 bytes per pass, one kernel launch per pass). Also reported: end-to-end gates/s through the
C ABI with host buffers (qf_run_circuit: upload f64 amplitudes, run, download),
the CPU baseline (the oracle restating the reference's rayon path, on every
host core, on a bounded sample of the same circuit), and 24-qubit VQE
adjoint vs parameter-shift gradients/s.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "30q gates/s (HBM GB/s vs peak); adjoint vs param-shift grads/s at 1e-5 err"
UNIT = "gates/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--depth", type=int, default=40)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--dtype", default="c64")
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--mode", default="auto", choices=["auto", "unfused", "fused"])
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true")
    ap.add_argument("--no-parity", dest="parity", action="store_false",
                    help="skip the complex128 run of the headline circuit (error of the complex64 result)")
    ap.add_argument("--extras", default="vqe24,qaoa4096,shots20,shots_ff,noise_shots,density14,vqe32,c2_matrix",
                    help="comma-separated extra workloads to run after the headline")
    ap.add_argument("--vqe-qubits", type=int, default=32, help="qubits of the checkpointed-adjoint extra (vqe32)")
    ap.add_argument("--qaoa-instances", type=int, default=4096, help="instances of the batched QAOA extra (qaoa4096)")
    ap.add_argument("--vqe24-adjoint-only", action="store_true",
                    help="vqe24 extra: only the adjoint gradient with a checkpoint every four layers, twice (profiling runs)")
    ap.add_argument("--density-qubits", type=int, default=14, help="qubits of the density-matrix extra (density14)")
    ap.add_argument("--noise-shots", type=int, default=100_000, help="shots of the noisy-shot extra (noise_shots)")
    ap.add_argument("--c2-modes", default="unfused,passes,k2,k3,k4,k5,k5_simt",
                    help="modes of the c2_matrix extra (unfused, passes, k2..k5, k5_simt)")
    ap.add_argument("--c2-dtypes", default="c64,c128", help="state types of the c2_matrix extra")
    ap.add_argument("--extras-only", action="store_true",
                    help="run only the extras (small profiling runs); prints {\"extra\": ...} instead of the headline")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def hbm_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample_ops(ops):
    """A bounded sample of the circuit keeping its 1q:2q mix: the first two
    one-qubit gates, then the first two-qubit gate, repeated down the list."""
    from quantumforge_gb300 import _abi as A

    one = [i for i, r in enumerate(ops) if r["kind"] == A.OP_GATE]
    two = [i for i, r in enumerate(ops) if r["kind"] != A.OP_GATE]
    seq = []
    for k in range(len(two)):
        seq += one[2 * k: 2 * k + 2] + [two[k]]
    return seq


def time_cpu_oracle(n, ops, seconds, threads):
    """The oracle's restatement of the reference CPU path (rayon clone/map/
    collect for one-qubit gates on `threads` threads, single-threaded two-qubit
    loops), timed on the same circuit until `seconds` have elapsed."""
    import numpy as np

    import oracle as O

    a = np.zeros(1 << n, dtype=np.complex128)
    a.view(np.float64)[::512] = 0.0  # touch every page before timing
    a[0] = 1.0
    seq = cpu_sample_ops(ops)
    done = 0
    t0 = time.perf_counter()
    for idx in seq:
        rec = ops[idx: idx + 1]
        st = O.lib().qfo_run_ops(O._p(a), n, O._p(rec), 1, None, 0, None, 0, -1, 0.0, threads)
        if st:
            raise RuntimeError(f"oracle failed with status {st}")
        done += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    n1 = sum(1 for i in seq[:done] if ops[i]["kind"] == 0)
    return done / dt, f"first {done} gates ({n1} one-qubit, {done - n1} two-qubit, in circuit order, 1q:2q = 2:1) " \
                      f"of the {n}-qubit circuit, complex128 as the reference, {dt:.1f} s"


def reference_arm(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    from quantumforge_gb300 import workloads as W

    ops = W.random_circuit(args.qubits, args.depth, args.seed, two_qubit="mixed")
    threads = os.cpu_count() or 1
    import numpy as np

    import oracle as O

    n = args.qubits
    a = np.zeros(1 << n, dtype=np.complex128)
    a.view(np.float64)[::512] = 0.0
    a[0] = 1.0
    seq = cpu_sample_ops(ops)
    step_times = []
    for s in range(args.warmup + args.steps):
        idx = seq[s % len(seq)]
        rec = ops[idx: idx + 1]
        t0 = time.perf_counter()
        st = O.lib().qfo_run_ops(O._p(a), n, O._p(rec), 1, None, 0, None, 0, -1, 0.0, threads)
        dt = time.perf_counter() - t0
        if st:
            raise RuntimeError(f"oracle failed with status {st}")
        if s >= args.warmup:
            step_times.append(dt)
    total = sum(step_times)
    value = len(step_times) / total
    sample = f"one gate per step, cycling the circuit's gates with its 1q:2q = 2:1 mix; {n} qubits complex128"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * total / len(step_times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "complex128", "data": "synthetic",
        "config": {"workload": f"{n}q depth-{args.depth} mixed random circuit (seed {args.seed})", "qubits": n,
                   "depth": args.depth, "gates": len(ops)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is Rust (no toolchain on this box): its CPU path is timed through the oracle's C "
                "restatement of StateVector::apply/apply_cnot/apply_cz/apply_swap",
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import ctypes as C

    import numpy as np
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import quantumforge_gb300 as qf
    from quantumforge_gb300 import _abi as A
    from quantumforge_gb300 import _native
    from quantumforge_gb300 import workloads as W

    n = args.qubits
    backend = qf.CudaBackend(local)
    ops = W.random_circuit(n, args.depth, args.seed, two_qubit="mixed")
    n_gates = len(ops)
    dcode = A.C64 if args.dtype in ("c64", "complex64") else A.C128
    amp_bytes = 8 if dcode == A.C64 else 16
    mode = {"auto": A.EXEC_AUTO, "unfused": A.EXEC_UNFUSED, "fused": A.EXEC_FUSED}[args.mode]
    exec_opts = {"mode": args.mode, "tile_qubits": args.tile}
    lib = _native.load()
    npass, ngate = C.c_uint64(), C.c_uint64()
    eo = A.ExecOpts(mode, args.tile, 0, 0)
    _native.check(lib.qf_plan_stats(n, dcode, _native.ptr(ops), len(ops), None, 0, None, 0, C.byref(eo),
                                    C.byref(npass), C.byref(ngate)))
    n_passes = npass.value

    sv = qf.StateVector.zero(n, dtype=args.dtype, backend=backend)
    sp = C.c_void_p()
    lib.qf_ctx_stream(backend.handle, C.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value, device=torch.device("cuda", local))

    for _ in range(args.warmup):
        sv.apply_ops(ops, exec_opts=exec_opts)
    backend.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    backend.synchronize()
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.4)  # let the sampler attach before the timed region
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        sv.apply_ops(ops, exec_opts=exec_opts)
    ev1.record(stream)
    ev1.synchronize()
    backend.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    t = ev0.elapsed_time(ev1) / 1000.0
    if world > 1:
        tt = torch.tensor([t], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t = float(tt.item())
    value = world * args.steps * n_gates / t
    ms_per_step = 1000.0 * t / args.steps
    # roofline of the dominant kernels (one launch per tile pass): every launch
    # is one full read + write sweep of the state
    bytes_per_launch = 2 * (1 << n) * amp_bytes
    launches = args.steps * n_passes
    avg_launch_s = t / launches
    achieved = bytes_per_launch / avg_launch_s / 1e9
    peak, peak_kind = hbm_peak()
    if dcode == A.C64 and n >= 24:
        kernel = f"compiled tile passes p0..p{n_passes - 1} (one NVRTC sm_103a kernel per pass)"
    elif dcode == A.C64 and n >= 12:
        kernel = "k_rs_pass (register-tiled pass interpreter)"
    else:
        kernel = "k_tile_pass<double2,false>" if dcode == A.C128 else "k_tile_pass<float2,false>"
    # DRAM bytes per launch from one ncu capture of this workload (see profiles/)
    traffic = None
    tf = ROOT / "profiles" / "tile_pass_traffic.json"
    if tf.exists():
        try:
            traffic = json.loads(tf.read_text()).get(f"{n}q_d{args.depth}_s{args.seed}_{args.dtype}_bytes_per_launch")
        except Exception:
            traffic = None

    # end to end through the C ABI with host buffers (pinned), copies timed
    e2e = None
    if args.e2e_steps > 0:
        host_in = torch.zeros(2 << n, dtype=torch.float64, pin_memory=True)
        host_in[0] = 1.0
        host_out = torch.empty(2 << n, dtype=torch.float64, pin_memory=True)
        eo2 = A.ExecOpts(mode, args.tile, 0, 0)
        _native.check(lib.qf_run_circuit(backend.handle, n, dcode, _native.ptr(ops), len(ops),
                                         C.c_void_p(host_in.data_ptr()), C.c_void_p(host_out.data_ptr()), 2 << n,
                                         C.byref(eo2)))
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            _native.check(lib.qf_run_circuit(backend.handle, n, dcode, _native.ptr(ops), len(ops),
                                             C.c_void_p(host_in.data_ptr()), C.c_void_p(host_out.data_ptr()), 2 << n,
                                             C.byref(eo2)))
        te = time.perf_counter() - t0
        if world > 1:
            tt = torch.tensor([te], device="cuda")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            te = float(tt.item())
        e2e = {"value": world * args.e2e_steps * n_gates / te, "unit": UNIT, "h2d_bytes_per_step": 16 << n,
               "d2h_bytes_per_step": 16 << n,
               "api": "qf_run_circuit (CudaBackend::run_circuit): f64 host amplitudes in and out, pinned"}
        del host_in, host_out

    parity = None
    if rank == 0 and args.parity and dcode == A.C64:
        del sv
        parity = c128_parity(backend, n, ops, exec_opts)
    extra = {}
    cpu = None
    if rank == 0 and not args.no_extra:
        wanted = set(args.extras.split(","))
        if "vqe24" in wanted:
            extra["vqe24"] = vqe_gradients(backend, cpu=not args.no_cpu_baseline, adjoint_only=args.vqe24_adjoint_only)
        if "qaoa4096" in wanted:
            extra["qaoa4096"] = qaoa_batch(backend, cpu=not args.no_cpu_baseline, count=args.qaoa_instances)
        if "shots20" in wanted:
            extra["shots20"] = shots20(backend, cpu=not args.no_cpu_baseline)
        if "shots_ff" in wanted:
            extra["shots_ff"] = shots_feedforward(backend, cpu=not args.no_cpu_baseline)
        if "density14" in wanted:
            extra["density14"] = density14(backend, cpu=not args.no_cpu_baseline, n=args.density_qubits)
        if "noise_shots" in wanted:
            extra["noise_shots"] = noise_shots(backend, cpu=not args.no_cpu_baseline, shots=args.noise_shots)
        if "vqe32" in wanted:
            extra["vqe32"] = vqe32_checkpointed(backend, args.vqe_qubits)
        if "c2_matrix" in wanted:
            extra["c2_matrix"] = c2_matrix(backend, modes_wanted=args.c2_modes.split(","), dtypes=args.c2_dtypes.split(","))
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, sample = time_cpu_oracle(n, ops, args.cpu_seconds, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "complex64" if dcode == A.C64 else "complex128", "data": "synthetic",
            "config": {"workload": f"{n}q depth-{args.depth} mixed random circuit (seed {args.seed}), "
                                   f"{args.dtype} state, {args.mode} execution",
                       "qubits": n, "depth": args.depth, "gates": n_gates, "passes_per_step": n_passes,
                       "tile_qubits": args.tile or "auto", "l2": "state larger than L2 (no flush needed)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "peak_kind": f"of {peak_kind}", "kernel": kernel,
                         "bytes_per_launch": bytes_per_launch, "avg_launch_ms": 1000 * avg_launch_s},
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": launches,
            "parity_vs_c128": parity, "extra": extra,
        }
        print(json.dumps(line), flush=True)
    backend.close()
    if world > 1:
        torch.distributed.destroy_process_group()


class _DeviceArray:
    """A flat device buffer seen by torch through __cuda_array_interface__."""

    def __init__(self, ptr: int, count: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (count,), "typestr": typestr, "data": (ptr, False), "version": 3}


def state_tensor(sv):
    """The interleaved (re, im) reals of a device state as a torch tensor (no copy)."""
    import ctypes as C

    import torch

    from quantumforge_gb300 import _native

    p = C.c_void_p()
    _native.check(_native.load().qf_sv_device_ptr(sv._h, C.byref(p)))
    from quantumforge_gb300 import _abi as A

    typestr = "<f4" if sv.dtype == A.C64 else "<f8"  # StateVector.dtype holds the qf_dtype code
    return torch.as_tensor(_DeviceArray(p.value, 2 << sv.qubits, typestr), device="cuda")


def c128_parity(backend, n, ops, exec_opts):
    """The headline circuit once from |0...0> on a complex64 and on a
    complex128 state (the reference's precision; the complex128 tile passes
    agree with the oracle to 1e-10 where it can run): the largest amplitude
    and <Z_q> differences, computed on the device in chunks."""
    import torch

    import quantumforge_gb300 as qf

    sv64 = qf.StateVector.zero(n, dtype="c64", backend=backend)
    sv64.apply_ops(ops, exec_opts=exec_opts)
    z64 = np.asarray(sv64.expectation_z_all())
    sv128 = qf.StateVector.zero(n, dtype="c128", backend=backend)
    sv128.apply_ops(ops)  # warm (plans the passes)
    sv128 = qf.StateVector.zero(n, dtype="c128", backend=backend)
    backend.synchronize()
    t0 = time.perf_counter()
    sv128.apply_ops(ops)
    backend.synchronize()
    t128 = time.perf_counter() - t0
    z128 = np.asarray(sv128.expectation_z_all())
    a, b = state_tensor(sv64), state_tensor(sv128)
    err, norm_err, chunk = 0.0, 0.0, 1 << 26
    for i in range(0, a.numel(), chunk):
        d = (a[i:i + chunk].double() - b[i:i + chunk]).view(-1, 2)
        err = max(err, float(torch.sqrt((d * d).sum(1)).max()))
    max_amp = 0.0
    for i in range(0, b.numel(), chunk):
        v = b[i:i + chunk].view(-1, 2)
        max_amp = max(max_amp, float(torch.sqrt((v * v).sum(1)).max()))
    torch.cuda.synchronize()
    del a, b, sv64, sv128
    return {"reference": "the same circuit on a complex128 state", "max_abs_amp_err_vs_c128": err,
            "max_abs_amp_c128": max_amp, "max_z_err_vs_c128": float(np.abs(z64 - z128).max()),
            "c128_step_s": t128, "c128_gates_per_s": len(ops) / t128}


def max_amp_diff(sv_a, sv_b) -> float:
    """max_i |a_i - b_i| over two device states of the same size (on the device, in chunks)."""
    import torch

    a, b = state_tensor(sv_a), state_tensor(sv_b)
    err, chunk = 0.0, 1 << 26
    for i in range(0, a.numel(), chunk):
        d = (a[i:i + chunk].double() - b[i:i + chunk].double()).view(-1, 2)
        err = max(err, float(torch.sqrt((d * d).sum(1)).max()))
    return err


def unfused_bytes(ops, n, amp_bytes) -> int:
    """Algorithmic bytes of one gate per sweep (dense or RZ-type 2Nb, Z/S/T Nb,
    CNOT/SWAP Nb, CZ Nb/2) summed over the circuit."""
    from quantumforge_gb300 import _abi as A

    N = 1 << n
    tot = 0
    for r in ops:
        k, g = int(r["kind"]), int(r["gate"])
        if k == A.OP_GATE:
            tot += N * amp_bytes if g in (A.GATE_Z, A.GATE_S, A.GATE_SDG, A.GATE_T, A.GATE_TDG) else 2 * N * amp_bytes
        elif k in (A.OP_CNOT, A.OP_SWAP):
            tot += N * amp_bytes
        else:
            tot += N * amp_bytes // 2
    return tot


def c2_matrix(backend, n64: int = 30, n128: int = 26, depth: int = 40, seed: int = 1, modes_wanted=None, dtypes=("c64", "c128")):
    """The headline circuit generator run unfused (one sweep per gate, the
    reference's structure), as per-gate tile passes (the default), and fused
    into dense k-qubit blocks for k = 2..5 (k = 5 on the tensor cores and on
    the FP32 pipe), in complex64 at 30 qubits and complex128 at 26 qubits
    (FP64 dense blocks of 5 qubits take minutes at 30; complex128 unfused and
    per-gate passes also at 30). Per mode: gates/s, HBM
    passes, the fraction of the measured copy peak over the passes'
    algorithmic bytes, and the largest amplitude error against the complex128
    per-gate result of the same circuit."""
    import ctypes as C

    import torch

    import quantumforge_gb300 as qf
    from quantumforge_gb300 import _abi as A
    from quantumforge_gb300 import _native
    from quantumforge_gb300 import workloads as W

    lib = _native.load()
    peak, peak_kind = hbm_peak()
    sp = C.c_void_p()
    lib.qf_ctx_stream(backend.handle, C.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value)
    modes = [("unfused", {"mode": "unfused"}), ("passes", {}), ("k2", {"block_qubits": 2}), ("k3", {"block_qubits": 3}),
             ("k4", {"block_qubits": 4}), ("k5", {"block_qubits": 5}),
             ("k5_simt", {"block_qubits": 5, "blocks_engine": "simt"})]
    out = {"metric": "gates/s", "peak": peak, "peak_kind": f"of {peak_kind}",
           "reference_state": "complex128 per-gate tile passes of the same circuit"}
    if modes_wanted:
        modes = [m for m in modes if m[0] in modes_wanted]
    runs = [("c64", n64), ("c128", n128)]
    if n128 < n64:  # complex128 at the full size too, for the unfused sweeps and the per-gate passes
        runs.append(("c128", n64))
    all_modes = modes
    for dtype, n in runs:
        if dtype not in dtypes:
            continue
        modes = [m for m in all_modes if m[0] in ("unfused", "passes")] if (dtype == "c128" and n > n128) else all_modes
        ops = W.random_circuit(n, depth, seed, two_qubit="mixed")
        b = 8 if dtype == "c64" else 16
        ref = qf.StateVector.zero(n, dtype="c128", backend=backend)
        ref.apply_ops(ops)
        rows = {}
        for name, eo in modes:
            if dtype == "c128" and name == "k5_simt":
                continue  # complex128 blocks always run on the FP64 pipe
            npass, ngate = C.c_uint64(), C.c_uint64()
            o = A.exec_opts(eo)
            _native.check(lib.qf_plan_stats(n, A.C64 if dtype == "c64" else A.C128, _native.ptr(ops), len(ops), None, 0,
                                            None, 0, C.byref(o), C.byref(npass), C.byref(ngate)))
            sv = qf.StateVector.zero(n, dtype=dtype, backend=backend)
            try:
                sv.apply_ops(ops, exec_opts=eo)  # from |0...0>: plans, compiles; the error check
            except Exception as e:  # a mode that fails is reported, not fatal to the bench
                rows[name] = {"error": str(e)[:300]}
                del sv
                continue
            backend.synchronize()
            err = max_amp_diff(sv, ref)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0 = time.perf_counter()
            e0.record(stream)
            sv.apply_ops(ops, exec_opts=eo)
            e1.record(stream)
            e1.synchronize()
            t_wall = time.perf_counter() - t0
            t = e0.elapsed_time(e1) / 1000.0
            algo = unfused_bytes(ops, n, b) if name == "unfused" else npass.value * 2 * (1 << n) * b
            rows[name] = {"gates_per_s": len(ops) / t, "step_s": t, "wall_s": t_wall, "hbm_passes": npass.value,
                          "algorithmic_gb": algo / 1e9, "frac": algo / t / 1e9 / peak,
                          "max_abs_amp_err_vs_c128": err}
            del sv
        timed = {m: r["gates_per_s"] for m, r in rows.items() if "gates_per_s" in r}
        out[f"{dtype}_{n}q"] = {"gates": len(ops), "fastest": max(timed, key=timed.get) if timed else None, **rows}
        del ref
        torch.cuda.empty_cache()
    return out


def shots20(backend, cpu: bool):
    """20 qubits complex128, depth-20 random circuit with CNOT ladders:
    probabilities, <Z_i> for all i and 10^5 seeded shots (measure(q, q) for
    every qubit), checked against the oracle's exact memoised sampler."""
    import numpy as np

    import oracle as O
    import quantumforge_gb300 as qf
    from quantumforge_gb300 import workloads as W

    n, shots, seed = 20, 100_000, 42
    ops = W.random_circuit(n, 20, 7)
    mops = W.with_terminal_measurements(ops, n)
    circ = qf.Circuit.from_ops(mops)
    res = circ.run_shots(n, shots, seed, dtype="c128", backend=backend, tie_eps=1e-12)  # warm
    t0 = time.perf_counter()
    sv = qf.StateVector.zero(n, dtype="c128", backend=backend)
    sv.apply_ops(ops)
    probs = sv.probabilities()
    zs = sv.expectation_z_all()
    t_state = time.perf_counter() - t0
    t0 = time.perf_counter()
    circ.run_shots_packed(n, shots, seed, dtype="c128", backend=backend, tie_eps=1e-12)
    t_engine = time.perf_counter() - t0
    t0 = time.perf_counter()
    res = circ.run_shots(n, shots, seed, dtype="c128", backend=backend, tie_eps=1e-12)
    t_shots = time.perf_counter() - t0
    out = {"qubits": n, "gates": len(ops), "shots": shots, "seed": seed, "run_probs_z_s": t_state,
           "engine_call_s": t_engine, "engine_shots_per_s": shots / t_engine,
           "api_call_s": t_shots, "api_shots_per_s": shots / t_shots,
           "api": "engine: qf_run_shots (simulate, sample, packed outcomes to host); api: Circuit.run_shots incl. the "
                  "counts map keyed by bit tuples",
           "ties": res.ties, "distinct_outcomes": len(res.counts)}
    exp_packed, width = O.run_shots(mops, n, shots, seed, threads=os.cpu_count() or 1)
    out["counts_bit_exact_vs_oracle"] = res.counts == O.counts(exp_packed, width)
    out["more_seeds"] = {}
    for s2 in (43, 44):  # two more seeds of the same circuit
        t0 = time.perf_counter()
        r2 = circ.run_shots(n, shots, s2, dtype="c128", backend=backend, tie_eps=1e-12)
        t2 = time.perf_counter() - t0
        e2, w2 = O.run_shots(mops, n, shots, s2, threads=os.cpu_count() or 1)
        out["more_seeds"][str(s2)] = {"api_shots_per_s": shots / t2, "ties": r2.ties,
                                      "counts_bit_exact_vs_oracle": r2.counts == O.counts(e2, w2)}
    a = O.run(ops, n, threads=os.cpu_count() or 1)
    out["max_prob_err_vs_oracle"] = float(np.abs(probs - O.probabilities(a)).max())
    out["max_z_err_vs_oracle"] = float(max(abs(zs[q] - O.expectation(a, 2, q)) for q in range(n)))
    if cpu:
        # the reference re-simulates every shot (run_shots_impl); 2 shots timed
        t0 = time.perf_counter()
        O.run_shots(mops, n, 2, seed, literal=True)
        t2 = time.perf_counter() - t0
        out["cpu_literal_shots_per_s"] = 2 / t2
        out["cpu_sample"] = "2 shots of the literal per-shot re-simulation (oracle restating run_shots_impl, one thread)"
    return out


def feedforward_circuit(n=20, seed=7):
    """C1's circuit (depth-20 random H/RX/RY/RZ + CNOT ladders) cut into four
    parts by three mid-circuit measurements, each followed by classically
    conditioned corrections (X, H, Rz) on other qubits, then measure(q, q) for
    every qubit."""
    import quantumforge_gb300 as qf
    from quantumforge_gb300 import workloads as W

    body = W.random_circuit(n, 20, seed)
    c = qf.Circuit()
    parts = np.array_split(np.arange(len(body)), 4)
    for k, idx in enumerate(parts):
        for i in idx:
            r = body[i]
            c.operations.append((int(r["kind"]), int(r["gate"]), int(r["q0"]), int(r["q1"]), 0, float(r["theta"]), 0))
        if k < 3:
            q = (5 * k + 3) % n
            c.measure(q, q)
            c.if_classical_bit(q, 1, qf.Gate.X, (q + 1) % n)
            c.if_classical_bit(q, 0, qf.Gate.H, (q + 7) % n)
            c.if_classical_bit(q, 1, qf.Gate.Rz(0.7), (q + 11) % n)
    for q in range(n):
        c.measure(q, q)
    return c


def shots_feedforward(backend, cpu: bool):
    """10^5 seeded shots of a 20-qubit complex128 circuit with three mid-circuit
    measurements and feed-forward: the branching shot engine, its first shots
    against the oracle's literal per-shot engine (run_shots_impl)."""
    import oracle as O

    n, shots, seed = 20, 100_000, 42
    c = feedforward_circuit(n)
    c.run_shots_packed(n, shots, seed, dtype="c128", backend=backend, tie_eps=1e-12)  # warm (compiles nothing; allocs)
    t0 = time.perf_counter()
    got, width, ties = c.run_shots_packed(n, shots, seed, dtype="c128", backend=backend, tie_eps=1e-12)
    dt = time.perf_counter() - t0
    out = {"qubits": n, "ops": len(c.operations), "mid_circuit_measurements": 3, "shots": shots, "seed": seed,
           "engine_call_s": dt, "engine_shots_per_s": shots / dt, "ties": int(ties),
           "distinct_outcomes": int(len(np.unique(got)))}
    k = 3  # the literal engine re-simulates every shot: compare the first shots
    t0 = time.perf_counter()
    want, _ = O.run_shots(c.ops(), n, k, seed, literal=True)
    tl = time.perf_counter() - t0
    out["first_shots_equal_oracle"] = bool(np.array_equal(got[:k], want))
    if cpu:
        out["cpu_literal_shots_per_s"] = k / tl
        out["cpu_sample"] = f"{k} shots of the literal per-shot re-simulation (oracle restating run_shots_impl, one thread)"
    return out


def noisy_layers(n, layers, seed, gamma, dep):
    """`layers` of random H/RX/RY/RZ + CNOT ladders, each followed by
    amplitude damping (gamma) on every qubit and depolarizing (dep) on every
    other qubit."""
    import quantumforge_gb300 as qf
    from quantumforge_gb300 import workloads as W

    c = qf.Circuit()
    for layer in range(layers):
        for r in W.random_circuit(n, 1, seed + layer):
            c.operations.append((int(r["kind"]), int(r["gate"]), int(r["q0"]), int(r["q1"]), 0, float(r["theta"]), 0))
        for q in range(n):
            c.channel(q, qf.NoiseChannel.AmplitudeDamping(gamma))
        for q in range(0, n, 2):
            c.channel(q, qf.NoiseChannel.Depolarizing(dep))
    return c


def density14(backend, cpu: bool, n: int = 14):
    """A 14-qubit density matrix (4^14 complex128 entries, 4 GiB) through 6
    noisy layers (`noisy_layers`): Circuit.run_density on the resident matrix,
    timed with CUDA events on the engine's stream; the channel kernel timed
    alone; the same workload at 8 qubits against the oracle."""
    import ctypes as C

    import torch

    import oracle as O
    import quantumforge_gb300 as qf
    from quantumforge_gb300 import _abi as A
    from quantumforge_gb300 import _native

    c = noisy_layers(n, 6, 5, 0.02, 0.01)
    ops = c.ops()
    n_ch = int((ops["kind"] == A.OP_CHANNEL).sum())
    sp = C.c_void_p()
    _native.load().qf_ctx_stream(backend.handle, C.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value)
    rho = qf.DensityMatrix.zero(n, backend=backend)
    c.run_density(rho)  # warm
    reps = 3
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        c.run_density(rho)
    e1.record(stream)
    e1.synchronize()
    t = e0.elapsed_time(e1) / 1000.0 / reps
    # channel kernels alone: one channel per launch (k_dm_channel), and a layer
    # of n channels fused into 12-bit tile passes (k_dm_channel_tile)
    one = qf.Circuit()
    one.channel(n // 2, qf.NoiseChannel.AmplitudeDamping(0.02))
    one.run_density(rho)
    e0.record(stream)
    for _ in range(n):
        one.run_density(rho)
    e1.record(stream)
    e1.synchronize()
    t_ch = e0.elapsed_time(e1) / 1000.0 / n
    bytes_ch = 2 * (4 ** n) * 16
    peak, peak_kind = hbm_peak()
    chan = qf.Circuit()
    for q in range(n):
        chan.channel(q, qf.NoiseChannel.AmplitudeDamping(0.02))
    groups, mask = 1, 31  # the engine's grouping: add while the tile stays within 12 bits
    for q in range(n):
        m = mask | (1 << q) | (1 << (n + q))
        if bin(m).count("1") > 12:
            groups, mask = groups + 1, 31 | (1 << q) | (1 << (n + q))
        else:
            mask = m
    fused = {}
    for dt, b in (("c64", 8),):  # complex128 channels stay one kernel each (FP64-bound)
        r = qf.DensityMatrix.zero(n, dtype=dt, backend=backend)
        chan.run_density(r)
        reps_ch = 8  # calls back to back: the host prepares one call while the GPU runs the previous one
        e0.record(stream)
        for _ in range(reps_ch):
            chan.run_density(r)
        e1.record(stream)
        e1.synchronize()
        tf = e0.elapsed_time(e1) / 1000.0 / (groups * reps_ch)
        fused[dt] = {"passes_for_n_channels": groups, "avg_launch_ms": 1000 * tf, "bytes_per_launch": 2 * (4 ** n) * b,
                     "achieved_gbs": 2 * (4 ** n) * b / tf / 1e9, "frac": 2 * (4 ** n) * b / tf / 1e9 / peak}
        del r
    rho64 = qf.DensityMatrix.zero(n, dtype="c64", backend=backend)
    c.run_density(rho64)  # warm (compiles the 2n-qubit passes); one run from |0><0|
    d64 = None
    if n <= 12:
        ref = qf.DensityMatrix.zero(n, backend=backend)
        c.run_density(ref)
        d64 = float(np.abs(rho64.entries() - ref.entries()).max())
        del ref
    e0.record(stream)
    c.run_density(rho64)
    e1.record(stream)
    e1.synchronize()
    t64 = e0.elapsed_time(e1) / 1000.0
    del rho64
    tr = rho.trace()
    out = {"qubits": n, "entries": 4 ** n, "dtype": "complex128", "ops": len(ops), "gates": len(ops) - n_ch,
           "channels": n_ch, "run_density_s": t, "ops_per_s": len(ops) / t,
           "channel_kernel": {"kernel": "k_dm_channel<double2>", "avg_launch_ms": 1000 * t_ch,
                              "bytes_per_launch": bytes_ch, "achieved_gbs": bytes_ch / t_ch / 1e9,
                              "frac": bytes_ch / t_ch / 1e9 / peak, "peak": peak, "peak_kind": f"of {peak_kind}"},
           "fused_channel_passes": {"kernel": "k_dm_channel_pairs (complex64, two channels per shared-memory round)", **fused},
           "trace_re": tr.real, "purity": rho.purity(),
           "c64_run_density_s": t64, "c64_ops_per_s": len(ops) / t64}
    if d64 is not None:
        out["c64_max_abs_diff_vs_c128"] = d64
    m = 8
    cs = noisy_layers(m, 6, 5, 0.02, 0.01)
    small = qf.DensityMatrix.zero(m, backend=backend)
    cs.run_density(small)
    want = O.run_density(cs.ops(), m)
    out["max_abs_err_vs_oracle_8q"] = float(np.abs(small.entries() - want).max())
    if cpu:
        k = 9
        ck = noisy_layers(k, 6, 5, 0.02, 0.01)
        t0 = time.perf_counter()
        O.run_density(ck.ops(), k)
        tk = time.perf_counter() - t0
        scale = 4 ** (n - k)
        out["cpu_ops_per_s_extrapolated"] = len(ck.ops()) / (tk * scale)
        out["cpu_sample"] = (f"the same layers at {k} qubits through the oracle's DensityMatrix restatement (one thread), "
                             f"time scaled by 4^{n - k} entries (extrapolated)")
    return out


def noise_shots(backend, cpu: bool, n: int = 12, shots: int = 100_000):
    """run_shots_with_noise: 12 qubits complex128, 4 noisy layers
    (`noisy_layers`, gamma 0.01, depolarizing 0.005) then measure(q, q) for
    every qubit, 10^5 shots through the engine's default (per-shot
    shared-memory trajectories) and 10^4 through the branch tree; the first
    shots against the oracle's literal per-shot trajectories."""
    import oracle as O

    c = noisy_layers(n, 4, 9, 0.01, 0.005)
    for q in range(n):
        c.measure(q, q)
    seed = 42
    c.run_shots_packed(n, 64, seed, backend=backend, tie_eps=1e-12, noise=True)  # warm
    t0 = time.perf_counter()
    got, width, ties = c.run_shots_packed(n, shots, seed, backend=backend, tie_eps=1e-12, noise=True)
    dt = time.perf_counter() - t0
    out = {"qubits": n, "ops": len(c.operations), "shots": shots, "engine": "per-shot trajectories (k_trajectories)",
           "engine_call_s": dt, "engine_shots_per_s": shots / dt, "ties": int(ties),
           "distinct_outcomes": int(len(np.unique(got)))}
    t_shots = min(10_000, shots)
    t0 = time.perf_counter()
    tree, _, _ = c.run_shots_packed(n, t_shots, seed, backend=backend, tie_eps=1e-12, noise=True,
                                    exec_opts={"shots_engine": "tree"})
    out["tree_engine_shots_per_s"] = t_shots / (time.perf_counter() - t0)
    out["tree_equals_trajectories"] = bool(np.array_equal(tree, got[:t_shots]))
    t0 = time.perf_counter()
    g64, _, ties64 = c.run_shots_packed(n, shots, seed, dtype="c64", backend=backend, tie_eps=2e-5, noise=True)
    d64 = time.perf_counter() - t0
    out["c64_engine_shots_per_s"] = shots / d64
    out["c64_ties"] = int(ties64)
    out["c64_shots_differing_from_c128"] = int((g64 != got).sum())
    k = 200
    t0 = time.perf_counter()
    want, _ = O.run_shots(c.ops(), n, k, seed, noise=True)
    tl = time.perf_counter() - t0
    out["first_shots_equal_oracle"] = bool(np.array_equal(got[:k], want))
    if cpu:
        out["cpu_literal_shots_per_s"] = k / tl
        out["cpu_sample"] = f"{k} shots of the oracle's literal noisy trajectories (run_shots_impl, one thread)"
    return out


def qaoa_batch(backend, cpu: bool, count: int = 4096):
    """`count` (4096) random 3-regular MaxCut instances, n uniform in
    {12..20}, p = 4: cost and 8-parameter adjoint gradient per instance,
    replayed from a CUDA graph (batched tile passes per qubit count above 12
    qubits, one CTA per instance up to 12 qubits, tiles autotuned there)."""
    import numpy as np

    from quantumforge_gb300 import workloads as W
    from quantumforge_gb300.qaoa import QaoaBatch, autotune_tiles

    problems, gam, bet = W.qaoa_batch_problems(count)
    t0 = time.perf_counter()
    tiles = autotune_tiles(problems, 4, candidates=(9, 10, 11, 12), large_candidates=(0, 12), reps=1, backend=backend)
    t_tune = time.perf_counter() - t0
    batch = QaoaBatch(problems, 4, tile_qubits=tiles, backend=backend, use_graph=True)
    batch.run(gam, bet)
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        cost, grad = batch.run(gam, bet)
    dt = (time.perf_counter() - t0) / reps
    # algorithmic HBM bytes of the instances in batched passes (above 12
    # qubits, tiles of 0 = batched): per layer a forward pass A (psi + cost
    # bytes) and B, one lambda write, per reverse layer passes B and A on psi
    # and lambda (+ cost bytes); smaller instances stay in L2 / shared memory
    p = 4
    algo = 0
    for n, _ in problems:
        if n > 12 and tiles.get(n, 0) == 0:
            N = 1 << n
            algo += p * (2 * 16 * N + N) + 8 * N + p * (2 * 32 * N + N)
    peak, peak_kind = hbm_peak()
    out = {"instances": len(problems), "sizes": [12, 14, 16, 18, 20], "p": 4, "batch_s": dt,
           "instances_per_s": len(problems) / dt, "gradient_params_per_instance": 8, "tiles": tiles,
           "tiles_meaning": "per qubit count: up to 12 the tile width of the one-CTA-per-instance kernel; above 12, "
                            "0 = batched tile passes, else one CTA per instance with that tile width",
           "autotune_s": t_tune, "dtype": "complex64", "host_copies_in_timing": True, "mean_cost": float(np.mean(cost)),
           "roofline": {"bound": "hbm", "algorithmic_gb": algo / 1e9, "achieved_gbs": algo / dt / 1e9, "peak": peak,
                        "frac": algo / dt / 1e9 / peak, "peak_kind": f"of {peak_kind}",
                        "note": "batched-pass bytes over the whole batch time (small instances, host copies and "
                                "launch gaps included): a lower bound of the passes' own fraction"}}
    if cpu:
        out["cpu_estimate"] = qaoa_cpu_estimate(problems)
    return out


def qaoa_cpu_estimate(problems):
    """The reference's per-instance route — run qaoa_maxcut and
    maxcut_expectation, central finite differences for 8 parameters (17
    circuit evaluations) — with the oracle on every host core: one evaluation
    timed per n in {12, 14, 16}, n = 18 and 20 extrapolated by the observed
    per-qubit growth; averaged over the batch's size mix."""
    import numpy as np

    import oracle as O
    from quantumforge_gb300 import workloads as W

    threads = os.cpu_count() or 1
    t_eval = {}
    for n in (12, 14, 16):
        edges = W.random_3_regular(n, 1)
        ops = W.qaoa_maxcut(n, edges, 4, [0.3] * 4, [0.5] * 4)
        t0 = time.perf_counter()
        a = O.run(ops, n, threads=threads)
        O.maxcut_expectation(a, edges)
        t_eval[n] = time.perf_counter() - t0
    growth = (t_eval[16] / t_eval[12]) ** (1 / 4)  # per qubit
    t_eval[18] = t_eval[16] * growth ** 2
    t_eval[20] = t_eval[16] * growth ** 4
    per_inst = np.mean([17 * t_eval[n] for n, _ in problems])
    return {"instances_per_s": 1.0 / per_inst, "cores": threads, "kind": "port",
            "sample": "one circuit evaluation timed at n = 12, 14, 16 (18, 20 extrapolated); 17 evaluations per "
                      "instance (cost + 8-parameter central differences)",
            "eval_s": {str(k): v for k, v in t_eval.items()}}


def vqe_gradients(backend, cpu: bool = True, adjoint_only: bool = False):
    """24-qubit VQE (RY.RZ per qubit + CZ ring, 8 layers, 384 params, TFIM
    ring h = 1): adjoint (checkpoint per layer) vs GPU parameter shift, both
    complex64; the energy and gradient error against a complex128 adjoint run
    of the same circuit (the reference's precision), and central finite
    differences (h = 1e-4, complex128 energies) on a few parameters. The CPU
    baseline is the oracle's parameter shift (two energy evaluations timed,
    scaled to the 2 x 384 evaluations of one gradient)."""
    import numpy as np

    import quantumforge_gb300 as qf
    from quantumforge_gb300 import workloads as W
    from quantumforge_gb300.gradients import GradientOptions, GradientStrategy, gradient_with_inputs

    n = 24
    ops, params, H = W.vqe_tfim(n, 8, seed=3)
    pc = qf.ParameterizedCircuit(params.size)
    for r in ops:
        pc.operations.append((int(r["kind"]), int(r["gate"]), int(r["q0"]), int(r["q1"]), int(r["param"]),
                              float(r["theta"])))
    # checkpoint policies: psi stored at every layer, every four layers, or
    # never (pure uncompute); each timed over 5 gradients, with its algorithmic
    # HBM bytes from the adjoint's own plan (qf_adjoint_plan_stats)
    import ctypes as C

    from quantumforge_gb300 import _abi as A
    from quantumforge_gb300 import _native

    if adjoint_only:  # a warm-up and one timed gradient, nothing else launched
        kw = dict(dtype="c64", backend=backend, checkpoint_every=12 * n)
        gradient_with_inputs(pc, GradientOptions(strategy=GradientStrategy.Adjoint), [], params, n, H, **kw)
        t0 = time.perf_counter()
        gradient_with_inputs(pc, GradientOptions(strategy=GradientStrategy.Adjoint), [], params, n, H, **kw)
        return {"qubits": n, "params": int(params.size), "adjoint_policy": "every_4_layers",
                "s_per_gradient": time.perf_counter() - t0}
    peak, peak_kind = hbm_peak()
    policies = {}
    for name, every in (("per_layer", 3 * n), ("every_4_layers", 12 * n), ("uncompute", 0)):
        kw = dict(dtype="c64", backend=backend, checkpoint_every=every)
        adj = gradient_with_inputs(pc, GradientOptions(strategy=GradientStrategy.Adjoint), [], params, n, H, **kw)
        reps = 5
        t0 = time.perf_counter()
        for _ in range(reps):
            adj = gradient_with_inputs(pc, GradientOptions(strategy=GradientStrategy.Adjoint), [], params, n, H, **kw)
        t = (time.perf_counter() - t0) / reps
        o = A.GradientOpts()
        o.strategy, o.dtype, o.checkpoint_every = A.GRAD_ADJOINT, A.C64, every
        st = A.AdjointStats()
        pp = np.ascontiguousarray(params, dtype=np.float64)
        terms = H.array()
        _native.check(_native.load().qf_adjoint_plan_stats(n, A.C64, _native.ptr(ops), len(ops), _native.ptr(pp), pp.size,
                                                           None, 0, _native.ptr(terms), len(terms), C.byref(o),
                                                           C.byref(st)))
        policies[name] = {"checkpoint_every_ops": every, "grads_per_s": 1.0 / t, "s_per_gradient": t,
                          "launches": {"forward": st.forward_passes, "pauli": st.pauli_passes,
                                       "backward": st.backward_passes, "state_copies": st.state_copies},
                          "algorithmic_gb": st.hbm_bytes / 1e9,
                          "roofline_frac": st.hbm_bytes / t / 1e9 / peak, "grad": np.asarray(adj.gradient), "est": adj}
    best = min(policies, key=lambda k: policies[k]["s_per_gradient"])
    adj = policies[best]["est"]
    t_adj = policies[best]["s_per_gradient"]
    pc.expectation_pauli_sum(params, n, H, dtype="c64", backend=backend)  # warm: compiles the forward passes
    t0 = time.perf_counter()
    sh = gradient_with_inputs(pc, GradientOptions(strategy=GradientStrategy.ParameterShift), [], params, n, H,
                              dtype="c64", backend=backend)
    t_sh = time.perf_counter() - t0
    # complex128 reference run and finite differences
    t0 = time.perf_counter()
    ref = gradient_with_inputs(pc, GradientOptions(strategy=GradientStrategy.Adjoint), [], params, n, H,
                               dtype="c128", backend=backend, checkpoint_every=3 * n)
    t_ref = time.perf_counter() - t0
    g64, g128 = np.asarray(adj.gradient), np.asarray(ref.gradient)
    h = 1e-4
    fd_params = [0, 97, 191, 288, 383]
    fd = []
    for k in fd_params:
        pp, pm = params.copy(), params.copy()
        pp[k] += h
        pm[k] -= h
        ep = pc.expectation_pauli_sum(pp, n, H, dtype="c128", backend=backend)
        em = pc.expectation_pauli_sum(pm, n, H, dtype="c128", backend=backend)
        fd.append((ep - em) / (2 * h))
    fd = np.asarray(fd)
    pol = {}
    for name, v in policies.items():
        pol[name] = {k: v[k] for k in ("checkpoint_every_ops", "grads_per_s", "launches", "algorithmic_gb", "roofline_frac")}
        pol[name]["max_abs_grad_err_vs_c128"] = float(np.abs(v["grad"] - g128).max())
    out = {"qubits": n, "params": int(params.size), "ops": len(ops), "adjoint_grads_per_s": 1.0 / t_adj,
           "adjoint_policy": best, "adjoint_policies": pol,
           "roofline": {"bound": "hbm", "algorithmic_gb_per_gradient": policies[best]["algorithmic_gb"],
                        "achieved_gbs": policies[best]["algorithmic_gb"] / t_adj, "peak": peak,
                        "frac": policies[best]["roofline_frac"], "peak_kind": f"of {peak_kind}",
                        "note": "the gradient's algorithmic HBM bytes (forward, Pauli and backward passes, checkpoint "
                                "copies) over its wall time, host work included"},
           "param_shift_grads_per_s": 1.0 / t_sh, "ratio": t_sh / t_adj,
           "max_abs_grad_diff_adjoint_vs_shift": float(np.abs(adj.gradient - sh.gradient).max()),
           "energy_adjoint": adj.expectation, "energy_shift_run": sh.expectation, "dtype": "complex64",
           "vs_c128": {"energy_c128": ref.expectation, "energy_err_vs_c128": abs(adj.expectation - ref.expectation),
                       "max_abs_grad_err_vs_c128": float(np.abs(g64 - g128).max()),
                       "shift_max_abs_grad_err_vs_c128": float(np.abs(np.asarray(sh.gradient) - g128).max()),
                       "target": 1e-6, "c128_adjoint_s": t_ref},
           "central_fd": {"step": h, "params": fd_params, "energies": "complex128",
                          "max_abs_diff_vs_c128_adjoint": float(np.abs(fd - g128[fd_params]).max()),
                          "max_abs_diff_vs_c64_adjoint": float(np.abs(fd - g64[fd_params]).max())}}
    if cpu:
        import oracle as O

        threads = os.cpu_count() or 1
        m = 20  # one 24-qubit evaluation takes about a minute on the host: time the same ansatz at 20 qubits
        ops_m, params_m, H_m = W.vqe_tfim(m, 8, seed=3)
        t0 = time.perf_counter()
        O.energy(ops_m, m, params_m, H_m.array(), threads=threads)
        te = (time.perf_counter() - t0) * (1 << (n - m))
        out["cpu_baseline"] = {"value": 1.0 / (2 * params.size * te), "unit": "gradients/s", "cores": threads,
                               "kind": "port",
                               "sample": f"one energy evaluation of the same 8-layer ansatz at {m} qubits through the "
                                         f"oracle (complex128, {threads} threads), scaled by 2^{n - m} amplitudes and "
                                         f"by the 2 x {params.size} evaluations of a parameter-shift gradient "
                                         f"(extrapolated)"}
    return out


def vqe32_checkpointed(backend, n=32):
    """n-qubit (default 32) XXZ-ring VQE (RX.RY per qubit + CNOT ring, 4
    layers, 8n params, H = sum XX + YY + 0.5 ZZ, 3n terms): complex64 adjoint
    gradient with a checkpoint per layer (psi, lambda + 3 checkpoints = 160 GiB
    at 32 qubits) and with pure uncompute (64 GiB), both against a complex128
    uncompute run (128 GiB) of the same circuit."""
    import numpy as np

    import quantumforge_gb300 as qf
    from quantumforge_gb300 import workloads as W
    from quantumforge_gb300.gradients import GradientOptions, GradientStrategy, gradient_with_inputs

    layers = 4
    ops, params, H = W.vqe_xxz(n, layers, seed=5)
    pc = qf.ParameterizedCircuit.from_ops(ops, params.size)
    opts = GradientOptions(strategy=GradientStrategy.Adjoint)
    runs = {}
    for name, every in (("checkpoint_per_layer", 3 * n), ("uncompute", 0)):
        gradient_with_inputs(pc, opts, [], params, n, H, dtype="c64", checkpoint_every=every, backend=backend)
        t0 = time.perf_counter()
        est = gradient_with_inputs(pc, opts, [], params, n, H, dtype="c64", checkpoint_every=every, backend=backend)
        runs[name] = (time.perf_counter() - t0, est)
    t0 = time.perf_counter()
    ref = gradient_with_inputs(pc, opts, [], params, n, H, dtype="c128", checkpoint_every=0, backend=backend)
    t_ref = time.perf_counter() - t0
    out = {"qubits": n, "params": int(params.size), "ops": len(ops), "terms": len(H.terms),
           "energy_c128": ref.expectation, "c128_uncompute_s_per_gradient": t_ref}
    for name, (t, est) in runs.items():
        out[name] = {"s_per_gradient": t, "gradients_per_s": 1.0 / t,
                     "max_abs_grad_err_vs_c128": float(np.abs(np.asarray(est.gradient) - np.asarray(ref.gradient)).max()),
                     "energy_err_vs_c128": abs(est.expectation - ref.expectation), "dtype": "complex64"}
    return out


def extras_only(args):
    import torch

    import quantumforge_gb300 as qf

    torch.cuda.set_device(0)
    backend = qf.CudaBackend(0)
    wanted = set(args.extras.split(","))
    cpu = not args.no_cpu_baseline
    extra = {}
    if "vqe24" in wanted:
        extra["vqe24"] = vqe_gradients(backend, cpu=not args.no_cpu_baseline, adjoint_only=args.vqe24_adjoint_only)
    if "qaoa4096" in wanted:
        extra["qaoa4096"] = qaoa_batch(backend, cpu=cpu, count=args.qaoa_instances)
    if "shots20" in wanted:
        extra["shots20"] = shots20(backend, cpu=cpu)
    if "shots_ff" in wanted:
        extra["shots_ff"] = shots_feedforward(backend, cpu=cpu)
    if "density14" in wanted:
        extra["density14"] = density14(backend, cpu=cpu, n=args.density_qubits)
    if "noise_shots" in wanted:
        extra["noise_shots"] = noise_shots(backend, cpu=cpu, shots=args.noise_shots)
    if "vqe32" in wanted:
        extra["vqe32"] = vqe32_checkpointed(backend, args.vqe_qubits)
    if "c2_matrix" in wanted:
        extra["c2_matrix"] = c2_matrix(backend, n64=args.qubits, n128=min(args.qubits, 26),
                                       modes_wanted=args.c2_modes.split(","), dtypes=args.c2_dtypes.split(","))
    print(json.dumps({"extra": extra}), flush=True)
    backend.close()


def main():
    args = parse_args()
    if args.impl == "reference":
        reference_arm(args)
    elif args.extras_only:
        extras_only(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
