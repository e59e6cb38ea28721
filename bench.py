#!/usr/bin/env python3
"""Benchmark of the GB300 ICM quadrature engine.

One step = one full quadrature solve (Q = 256 nodes) of the drop-in workload:
n = k = 65536 players, stacks log-uniform over [1, 1e9], quadratic payouts
(k-j+1)^2 normalised, FP64.  Prints one JSON line:

  value     ms per solve, CUDA-event time of the kernel sequence with the
            plan (sorted stacks, buffers) resident on the device
  e2e       ms per solve through icm_equity (the reference's C entry point):
            host stacks and payouts in, host equities out, plan set-up,
            copies and synchronisation inside the timed region
  roofline  dominant kernel: algorithmic FP64 flops per launch / its mean
            CUDA-event duration over the timed region, against the FP64
            peak measured on this GPU by a DFMA microbenchmark
  cpu_baseline  the CPU oracle (this project's C port of the reference
            engine) on the host cores, a bounded sample of the same
            workload, scaled to one full solve

--impl reference times the reference's own CPU implementation instead
(oracle/_ref when it was compiled on this host, else the C port), with all
host threads, on the same workload and metric.

Multi-GPU (torchrun, N ranks): each rank solves its own copy (replicas; the
solve does not shard across GPUs), times are maxed over ranks and the whole
job's ms per solve is the max time / (K * N).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms @n=k=65536 Q=256"
UNIT = "ms/solve"
WORKLOAD = "drop-in: one tournament n=k=65536, Q=256, stacks log-uniform [1,1e9], payout (k-j+1)^2 normalised"
B200_PUBLISHED_MS = 20.26   # reference RESULTS.md:551, B200, n=k=65536, Q=256 (uniform [1,100] stacks)
# the reference's block size for these configurations: its B200 lookup table
# (devices/b200/gpu_fft_config.h:2373-, read by gpu_empirical_best_B,
# src/gpu/gpu_cost_model.cu:833)
REF_B = {(65536, 65536): 64, (1 << 20, 1 << 20): 32, (1 << 20, 1000): 144, (16384, 2000): 64}


def canonical_work(n: int, k: int, B: int, Q: int = 256):
    """The reference GPU engine's work per solve, (FP64 flops, HBM bytes), for
    (n, k, B, Q): its tree geometry (src/gpu/gpu_cost_model.cu:517-572: nblocks
    leaves of degree B, psz = min(B 2^(l+1), k_pad), g_needed, below_sat) and
    per level the effective lengths of src/gpu/gpu_plan.cu:97-114 (p_eff,
    g_eff, conv_build).  Per parent: schoolbook (conv_build <= 128) build
    2 p_eff^2, propagate 4 out p_eff; FFT with N = nextpow2(max(conv_build,
    g_eff)), T = 2.5 N log2 N: build 3T + 3N, propagate 5T + 6N; no build at
    the root.  Leaves n (2B + 4B) + 20 n.  Bytes: per parent 8 (psz + 2 cps)
    for the build, 8 (psz + 4 cps) for the propagate, plus 48 n.  Times Q.
    k_pad = k (the reference's own padding for a power-of-two k; other k it
    pads to a nearby smooth length, a difference of a few percent here)."""
    def npow2(x):
        p = 1
        while p < x:
            p <<= 1
        return p
    nb = -(-n // B)
    L = npow2(nb).bit_length()
    nreal = [nb]
    for _ in range(1, L):
        nreal.append((nreal[-1] + 1) // 2)
    psz = [min(B << (l + 1), k) for l in range(L)]
    gneed = [min(B, psz[0])]
    for l in range(1, L):
        gneed.append(min(gneed[-1] + psz[l - 1] - 1, psz[l]))
    flop = byte = 0.0
    for l in range(1, L):
        cps, pg, P, root = psz[l - 1], psz[l], nreal[l], l == L - 1
        doubled = (psz[l - 1] == 2 * psz[l - 2]) if l >= 2 else (psz[0] == 2 * B)
        below = doubled and cps >= 2
        p_eff = cps // 2 + 1 if below else cps
        out = gneed[l - 1]
        g_eff = min(out + p_eff - 1, min(cps + cps // 2, pg) if below else pg)
        conv = 2 * (cps // 2) + 1 if below else 2 * cps - 1
        if conv <= 128:
            build, prop = 2.0 * p_eff * p_eff, 4.0 * out * p_eff
        else:
            N = npow2(max(conv, g_eff))
            T = 2.5 * N * np.log2(N)
            build, prop = 3 * T + 3 * N, 5 * T + 6 * N
        flop += P * ((0.0 if root else build) + prop)
        byte += P * 8.0 * ((0 if root else pg + 2 * cps) + pg + 4 * cps)
    flop += n * 6.0 * B + 20.0 * n
    byte += 48.0 * n
    return flop * Q, byte * Q


def hbm_peak_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json"
    except (OSError, ValueError, KeyError):
        return 6806.5, "fallback (copy bandwidth measured earlier on this pool)"


def canonical_rates(n, k, ms, fp64_tflops):
    """The reference's canonical work for (n, k) over this run's time: as a
    fraction of the measured FP64 peak (above 1: this engine does that much
    less FP64 work than the reference's algorithm) and of the HBM peak."""
    B = REF_B.get((n, k))
    if B is None:
        return None
    W, D = canonical_work(n, k, B)
    hbm, src = hbm_peak_gbs()
    t = ms * 1e-3
    return {"B_ref": B, "W_ref_flop": float(W), "D_ref_bytes": float(D),
            "achieved_fp64": float(W / (t * fp64_tflops * 1e12)), "achieved_hbm": float(D / (t * hbm * 1e9)),
            "fp64_peak_tflops": fp64_tflops, "hbm_peak_gbs": hbm, "hbm_peak_source": src}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--n", type=int, default=65536)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--q-chunk", type=int, default=0, help="quadrature nodes per launch sequence (0 = auto)")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-tournaments leg")
    ap.add_argument("--batch-count", type=int, default=4096, help="tournaments in the batched leg")
    ap.add_argument("--no-vjp", action="store_true", help="skip the VJP leg")
    ap.add_argument("--no-gpu-scale", action="store_true", help="skip the n = 2^20 leg")
    ap.add_argument("--no-b200", action="store_true", help="skip the leg on the B200 figures' inputs")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="reference arm: skip the reference's own GPU library")
    ap.add_argument("--case", default="",
                    help="run one small workload once, untimed, and exit (for profilers): "
                         "vjp_batch:T (T tournaments of the VJP leg's batch), batch:T[:Q] (T of the batched leg), "
                         "small:n:k (20 single solves), dropin:n:Q (one drop-in solve), linear:n:k (linear engine)")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self.proc = None
        self.n0, self.n1 = 0, None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t0 = time.perf_counter()   # the timed region starts once sampling runs
            while not self.samples and self.proc.poll() is None and time.perf_counter() - t0 < 5.0:
                time.sleep(0.01)
        except (OSError, FileNotFoundError):
            self.proc = None
        self.n0 = len(self.samples)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        self.n1 = len(self.samples)
        if self.proc:
            if self.n1 == self.n0:   # region shorter than the sampling period: take the next sample
                t0 = time.perf_counter()
                while len(self.samples) == self.n0 and self.proc.poll() is None and time.perf_counter() - t0 < 1.0:
                    time.sleep(0.005)
                self.n1 = len(self.samples)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        ss = self.samples[self.n0:self.n1] if self.n1 is not None else self.samples
        if not ss:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in ss if len(s) > 2 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in ss if len(s) > 2 and s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in ss:
            for nm, v in zip(names, s[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(ss)}


def _median(xs):
    return float(np.median(np.asarray(xs, dtype=np.float64)))


def detail(name, obj):
    """One detail record on its own stdout line, ahead of the JSON result
    line (which stays compact); '#'-prefixed so that only the result line
    parses as JSON."""
    print(f"# {name}: " + json.dumps(obj), flush=True)


def cpu_reference(S, P, steps=1, warmup=1, budget_s=30.0, single_thread=True):
    """The reference's own CPU icm_equity (oracle/_ref, built from its
    unmodified src/cpu/icm.c) on this host: the OpenMP build on all cores,
    `steps` timed solves after `warmup`, median as the reference's bench.c
    (bench/bench.c:57-59) reports; plus the serial build on one core.  A solve
    is all 256 nodes while one takes at most budget_s, else a sample of
    q nodes (the per-node tree work does not depend on the node), scaled by
    256 / q.  Falls back to the C port (kind "port") where the reference
    library was not built."""
    from oracle.oracle import Oracle, ReferenceLib, build
    build()
    cores = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(cores)
    if ReferenceLib.available(openmp=True):
        kind = "reference"
        ref = ReferenceLib(openmp=True)

        def solve(q):
            t0 = time.perf_counter()
            ref.equity(S, P, Q=q)
            return time.perf_counter() - t0
    else:
        kind = "port"
        orc = Oracle()

        def solve(q):
            t0 = time.perf_counter()
            orc.equity(S, P, Q=q, B=8, fft_min_deg=64, threads=cores)
            return time.perf_counter() - t0
    q = 256
    t = solve(q)                                  # first warm-up decides the sample
    first_s = t
    if t > budget_s:
        q = max(8, 1 << int(np.floor(np.log2(256 * budget_s / t))))
    for _ in range(max(0, warmup - 1)):
        solve(q)
    times = [solve(q) * 256.0 / q for _ in range(max(1, steps))]
    out = {"value": 1e3 * _median(times), "unit": UNIT, "cores": cores, "kind": kind,
           "sample": (f"median of {len(times)} full solves (256 nodes, n={len(S)}, k={len(P)}) "
                      f"on {cores} threads (OpenMP build)" if q == 256 else
                      f"median of {len(times)} runs of {q} of 256 quadrature nodes (full n={len(S)}, "
                      f"k={len(P)} tree each) on {cores} threads (OpenMP build), scaled by 256/{q}"),
           "steps": len(times), "first_solve_s": round(first_s, 3)}
    if single_thread and kind == "reference" and ReferenceLib.available(openmp=False):
        # serial build: two node samples, extrapolated linearly to 256 nodes
        # (the difference gives the per-node cost, free of the per-call set-up)
        ser = ReferenceLib(openmp=False)
        ser.equity(S[:2048], P[:min(len(P), 2048)], Q=4)
        q1 = 8 if len(S) >= 32768 else 32
        ts1 = []
        for q in (q1, 2 * q1):
            t0 = time.perf_counter()
            ser.equity(S, P, Q=q)
            ts1.append(time.perf_counter() - t0)
        per_node = max(ts1[1] - ts1[0], 0.0) / q1
        est = ts1[0] + per_node * (256 - q1)
        out["single_thread"] = {"value": 1e3 * est, "unit": UNIT, "cores": 1,
                                "sample": f"serial build, {q1}- and {2 * q1}-node runs ({ts1[0]:.2f} s, "
                                          f"{ts1[1]:.2f} s) extrapolated to 256 nodes"}
    return out


def reference_gpu_leg(W, cpu_equity=None, batch_sample=16):
    """The reference's own GPU library (oracle/_ref/libicm_ref_gpu.so: its
    src/gpu/*.cu, cuFFT tier, B200 calibration data) on this GPU: ms per
    solve through icm_gpu_equity_with_plan (median of the library's own
    total_ns, host wall time including its synchronisation, as its
    tools/heatmap_gpu.cu reports the published figures; plan created once, the
    reference benchmarks' options) for
    the drop-in workload and for the inputs of its published B200 timings,
    one-shot icm_gpu_equity, and the plain loop of one-shot calls over a
    1-in-`batch_sample` sample of the batched workload, scaled to the whole
    batch."""
    from oracle.oracle import ReferenceGpu, build
    try:
        build(gpu=True)
    except Exception as e:   # noqa: BLE001 -- report, do not fail the arm
        return {"unavailable": f"reference GPU library did not build: {e}"}
    if not ReferenceGpu.available():
        return {"unavailable": "reference GPU sources not present on this host"}
    ref = ReferenceGpu(0)
    out = {"library": "reference src/gpu/*.cu (cuFFT tier; cuFFTDx/MathDx absent), devices/b200 data, sm_103a"}

    def with_plan(S, P, reps):
        t0 = time.perf_counter()
        plan = ref.plan(S, len(P))
        create = time.perf_counter() - t0
        E, _ = ref.equity_with_plan(plan, len(S), P)
        ts, wall = [], []
        for _ in range(reps):
            t0 = time.perf_counter()
            E, ns = ref.equity_with_plan(plan, len(S), P)
            wall.append(time.perf_counter() - t0)
            ts.append(ns * 1e-9)
        ref.destroy(plan)
        return E, {"ms": 1e3 * _median(ts), "wall_ms": 1e3 * _median(wall), "runs": reps,
                   "plan_create_ms": 1e3 * create}

    S, P, _ = W.dropin()
    E, rec = with_plan(S, P, 3)
    if cpu_equity is not None:
        rec["max_rel_diff_vs_reference_cpu"] = float(np.max(np.abs(E - cpu_equity) /
                                                           np.maximum(np.abs(cpu_equity), 1e-300)))
    t0 = time.perf_counter()
    ref.equity(S, P)
    rec["one_shot_ms"] = 1e3 * (time.perf_counter() - t0)
    out["dropin_65536"] = rec
    S, P = W.b200_heatmap(65536)
    out["b200_inputs_65536"] = with_plan(S, P, 3)[1]
    out["b200_inputs_65536"]["published_b200_ms"] = B200_PUBLISHED_MS
    if out["dropin_65536"]["ms"] < 2000.0:
        S, P = W.b200_heatmap(1 << 20)
        out["b200_inputs_1048576"] = with_plan(S, P, 1)[1]
        out["b200_inputs_1048576"]["published_b200_ms"] = 507.90
    ts = W.batched()
    sample = ts[::batch_sample]
    for S, P in sample[:4]:
        ref.equity(S, P)
    t0 = time.perf_counter()
    for S, P in sample:
        ref.equity(S, P)
    dt = time.perf_counter() - t0
    out["batch_loop"] = {"tournaments_timed": len(sample), "of": len(ts), "sample_s": dt,
                         "ms_per_batch_est": 1e3 * dt * len(ts) / len(sample),
                         "path": f"one icm_gpu_equity call per tournament, every {batch_sample}th tournament "
                                 f"of the batched workload, time scaled by {len(ts)}/{len(sample)}"}
    return out


def run_reference(args):
    """The reference's own CPU implementation (all host cores; its serial
    build on one core beside it) on the drop-in workload, and its own GPU
    library on this GPU beside that."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from icm_gb300 import workloads as W
    S, P, _ = W.dropin(n=args.n)
    cpu = cpu_reference(S, P, steps=args.steps, warmup=max(args.warmup, 1))
    ms = cpu["value"]
    gpu = None
    if not args.no_reference_gpu and args.n == 65536:
        cpu_E = None
        try:
            from oracle.oracle import ReferenceLib
            if cpu["kind"] == "reference":
                cpu_E = ReferenceLib(openmp=True).equity(S, P)
        except OSError:
            cpu_E = None
        gpu = reference_gpu_leg(W, cpu_E)
    line = {"metric": METRIC, "value": ms, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": cpu["steps"], "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded splitmix64)",
            "config": {"workload": WORKLOAD, "n": args.n, "k": args.n, "Q": 256},
            "cpu_baseline": cpu,
            "e2e": {"value": ms, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference_gpu": gpu}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    rank, world, local = dist_info()
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        pg = dist

    def barrier():
        if pg:
            pg.barrier()

    from icm_gb300 import build as b
    if rank == 0:   # one rank compiles (a no-op when the library is up to date); the others wait
        b.build()
    barrier()
    import ctypes
    import icm_gb300 as icm
    from icm_gb300 import workloads as W
    from icm_gb300._lib import lib

    L = lib()
    if L.icm_gpu_init(local) != 1:
        raise SystemExit(f"icm_gpu_init({local}) failed: {L.icm_gpu_last_error().decode()}")
    icm.init()
    if args.case:
        run_case(icm, W, args.case)
        return
    if args.q_chunk:
        icm.configure(q_chunk=args.q_chunk)
    S, P, T = W.dropin(n=args.n)
    n, k = len(S), len(P)
    fp64_peak_gflops = icm.measure_fp64_gflops()

    plan = icm.GpuPlan(S, k)
    summ = plan.summary()
    for _ in range(max(args.warmup, 3)):
        plan.equity(P)

    barrier()
    dev_ms = []
    launches = 0
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            plan.equity(P)
            dev_ms.append(L.icm_gb300_plan_device_ms(plan._p))
            launches += icm.last_launch_count()
        wall = time.perf_counter() - t0
    barrier()
    clocks = clk.summary()

    # per-kernel table from a profiled pass after the timed region (profiling
    # brackets every launch with events and keeps the run on one stream)
    L.icm_gb300_plan_set_profiling(plan._p, 1)
    prof_dev = 0.0
    for _ in range(args.steps):
        plan.equity(P)
        prof_dev += L.icm_gb300_plan_device_ms(plan._p)
    kst = []
    cnt = L.icm_gb300_plan_kernel_stats(plan._p, -1, None, 0, None, None, None)
    for i in range(cnt):
        nm = ctypes.create_string_buffer(64)
        ms, nl, fl = ctypes.c_double(), ctypes.c_long(), ctypes.c_double()
        L.icm_gb300_plan_kernel_stats(plan._p, i, nm, 64, ctypes.byref(ms), ctypes.byref(nl), ctypes.byref(fl))
        kst.append({"kernel": nm.value.decode(), "ms": ms.value, "launches": nl.value, "flops": fl.value})
    kst.sort(key=lambda r: -r["ms"])
    # the drop-in workload's 64-target subset on the same resident plan
    L.icm_gb300_plan_set_profiling(plan._p, 0)
    plan.set_targets(T)
    plan.equity(P)
    sub_dev = []
    for _ in range(max(3, args.steps // 2)):
        plan.equity(P)
        sub_dev.append(L.icm_gb300_plan_device_ms(plan._p))
    plan.set_targets(None)
    plan.close()

    # the drop-in workload's subset query (64 targets) against the full query,
    # both one-shot through the reference's GPU entry points
    sub_ms, full_ms = [], []
    for i in range(4):
        t1 = time.perf_counter()
        icm.gpu_equity_subset(S, P, T)
        t2 = time.perf_counter()
        icm.gpu_equity(S, P)
        t3 = time.perf_counter()
        if i:
            sub_ms.append((t2 - t1) * 1e3)
            full_ms.append((t3 - t2) * 1e3)

    subset = {"targets": int(len(T)), "device_ms": _r(_median(sub_dev)),
              "device_ratio_to_full": _r(_median(sub_dev) / (float(np.sum(dev_ms)) / args.steps)),
              "one_shot_ms": _r(_median(sub_ms)), "one_shot_full_ms": _r(_median(full_ms)),
              "path": "resident plan with targets (icm_gb300_plan_set_targets) vs the full solve; "
                      "one-shot icm_gpu_equity_subset vs icm_gpu_equity"}
    b200 = None if args.no_b200 else b200_inputs_leg(icm, W, 5)
    batched = (None if args.no_batched else
               batched_leg(icm, W, max(2, args.steps // 3), args.batch_count, fp64_peak_gflops / 1e3))
    vjp = None if args.no_vjp else vjp_leg(icm, W, 3, fp64_peak_gflops / 1e3)
    gscale = None if args.no_gpu_scale else gpu_scale_leg(icm, W, 2, fp64_peak_gflops / 1e3)

    # end to end through icm_equity (host buffers, plan set-up inside)
    e2e = []
    for _ in range(2):
        icm.equity(S, P)
    barrier()
    for _ in range(max(1, args.steps // 2)):
        t1 = time.perf_counter()
        icm.equity(S, P)
        e2e.append(time.perf_counter() - t1)
    barrier()

    total_dev = float(np.sum(dev_ms))
    if pg:
        import torch
        t = torch.tensor([total_dev, float(np.mean(e2e))], device=f"cuda:{local}", dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        total_dev, e2e_mean = float(t[0]), float(t[1])
    else:
        e2e_mean = float(np.mean(e2e))
    if rank != 0:
        return
    ms_per_solve = total_dev / (args.steps * world)
    top = kst[0] if kst else None
    roofline = None
    if top:
        per_launch_s = top["ms"] / top["launches"] * 1e-3
        ach = top["flops"] / top["launches"] / per_launch_s / 1e12
        peak = fp64_peak_gflops / 1e3
        roofline = {"bound": "fp64", "kernel": top["kernel"], "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                    "frac": ach / peak,
                    "peak_source": "measured on this GPU (register-resident DFMA loop); MEASURED_PEAKS.json has no FP64 figure",
                    "traffic": traffic_for(top["kernel"]),
                    "share_of_device_time": top["ms"] / prof_dev,
                    "timing": "kernel durations from a profiled pass (events around every launch, one stream)"}
    total_flops = sum(r["flops"] for r in kst) / args.steps
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_reference(S, P, steps=1, warmup=1)
        cpu.pop("steps", None)
    kernels = [{**r, "ms_per_solve": r["ms"] / args.steps} for r in kst]
    detail("kernels (drop-in solve, profiled pass)", kernels)
    canon = canonical_rates(n, k, ms_per_solve, fp64_peak_gflops / 1e3)
    metric = METRIC if n == 65536 else f"ms @n=k={n} Q=256"
    b200_ms = b200["n65536"]["device_ms"] if b200 else None
    line = {
        "metric": metric, "value": ms_per_solve, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": total_dev / args.steps, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": (b200_ms / B200_PUBLISHED_MS) if b200_ms else None, "dtype": "f64",
        "data": "synthetic (seeded splitmix64; the reference publishes no dataset)",
        "config": {"workload": WORKLOAD, "n": n, "k": k, "Q": 256, "B": summ["B"],
                   "l2": "inputs larger than L2: the plan's working set exceeds 129 MB",
                   "parallelism": f"replicas x{world}",
                   "vs_baseline_note": "this engine on the inputs of the published B200 figure (stacks 1+99U, "
                                       "payout n-m, n=k=65536; RESULTS.md:551, tools/heatmap_gpu.cu:15-25) "
                                       "over that figure, 20.26 ms"},
        "e2e": {"value": e2e_mean * 1e3, "unit": UNIT, "h2d_bytes_per_step": 8 * (n + k), "d2h_bytes_per_step": 8 * n,
                "path": "icm_equity (C ABI, host buffers)"},
        "gpu_launches": launches,
        "roofline": roofline,
        "cpu_baseline": cpu, "clocks": clocks,
        "algorithmic_tflops_per_s": total_flops / (ms_per_solve * 1e-3) / 1e12,
        "fp64_peak_tflops_measured": fp64_peak_gflops / 1e3,
        "canonical": {"W_ref_flop": canon["W_ref_flop"], "achieved_fp64": canon["achieved_fp64"]} if canon else None,
        "b200_inputs": b200,
        "subset": subset,
        "batched": compact_batched(batched),
        "vjp": compact_vjp(vjp),
        "gpu_scale": compact_scale(gscale),
    }
    print(json.dumps(line), flush=True)


def _r(x, d=4):
    return None if x is None else float(f"{x:.{d}g}")


def compact_batched(b):
    """The batched leg's headline figures (the full record is a detail line)."""
    if not b:
        return None
    detail("batched", b)
    return {"tourn_per_s": _r(b["value"]), "ms_per_batch": _r(b["ms_per_batch"]),
            "e2e_tourn_per_s": _r(b["e2e"]["value"]), "loop_ms": _r(b["plain_loop"]["ms_per_batch"]),
            "speedup_vs_loop": {"device": _r(b["speedup_vs_loop"]["device"]), "e2e": _r(b["speedup_vs_loop"]["e2e"])},
            "max_rel_err_vs_loop": _r(b["max_rel_err_vs_loop"], 3),
            "achieved_fp64_canonical": _r((b.get("canonical") or {}).get("achieved_fp64"))}


def compact_vjp(v):
    if not v:
        return None
    detail("vjp", v)
    out = {}
    for shape in ("linear", "quadratic", "untruncated_262144"):
        if shape in v:
            out[shape] = {"ratio": _r(v[shape]["ratio"]), "vjp_ms": _r(v[shape]["vjp_ms"]),
                          "fwd_ms": _r(v[shape]["fwd_ms"])}
    if "batched_256" in v:
        out["batched_256_device_ratio"] = _r(v["batched_256"]["device_ratio"])
    return out


def compact_scale(g):
    if not g:
        return None
    detail("gpu_scale", g)
    out = {}
    for shape in ("linear", "geometric"):
        if shape in g:
            r = g[shape]
            out[shape] = {"k": r["k"], "device_ms": _r(r["device_ms"]), "e2e_ms": _r(r["e2e_ms"])}
            if "max_rel_err_vs_closed_form_64_players" in r:
                out[shape]["rel_err_closed_form"] = _r(r["max_rel_err_vs_closed_form_64_players"], 3)
    return out


def b200_inputs_leg(icm, W, steps):
    """This engine on the inputs of the reference's published B200 timings
    (stacks 1 + 99 U, payout n - m; tools/heatmap_gpu.cu:15-25): device ms per
    solve with the plan resident, at n = k = 65536 (published 20.26 ms,
    RESULTS.md:551) and n = k = 2^20 (507.90 ms, RESULTS.md:553)."""
    from icm_gb300._lib import lib
    out = {}
    for n, reps, pub in ((65536, steps, B200_PUBLISHED_MS), (1 << 20, 2, 507.90)):
        S, P = W.b200_heatmap(n)
        plan = icm.GpuPlan(S, n)
        plan.equity(P)
        dev = []
        for _ in range(max(2, reps)):
            plan.equity(P)
            dev.append(lib().icm_gb300_plan_device_ms(plan._p))
        plan.close()
        out[f"n{n}"] = {"device_ms": _r(_median(dev)), "published_b200_ms": pub,
                        "ratio_to_b200": _r(_median(dev) / pub)}
    return out


def batched_leg(icm, W, steps, count, fp64_tflops=None):
    """Batched form: `count` tournaments, n log-uniform in [9, 20000],
    k = ceil(0.15 n), lognormal(sigma=1) stacks x 1e4, geometric payouts 0.8,
    Q = 256.  Device time of the work-list engine (graph replay, stacks and
    buffers resident), end to end through icm_gpu_equity_batched (host arrays,
    set-up inside), and the plain loop of icm_gpu_equity calls on the same
    GPU, with the largest relative difference between the two."""
    ts = W.batched(count=count)
    Ss = [S for S, _ in ts]
    Ps = [P for _, P in ts]
    ks = [len(P) for P in Ps]
    players = int(sum(len(S) for S in Ss))
    b = icm.GpuBatch(Ss, ks)
    info = b.info()
    for _ in range(2):
        b.equity(Ps, split=False)
    dev, wall = [], []
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        out = b.equity(Ps, split=False)
        wall.append(time.perf_counter() - t0)
        dev.append(b.info()["device_ms"])
    launches = icm.last_launch_count()
    b.set_options(graphs=False, profiling=True)
    b.equity(Ps, split=False)
    kst = sorted(b.kernel_stats(), key=lambda r: -r["ms"])
    b.close()
    # end to end through the C entry point: create + run + destroy per call
    icm.equity_batched(ts[:64])
    e2e = []
    for _ in range(2):
        t0 = time.perf_counter()
        res = icm.equity_batched(ts)
        e2e.append(time.perf_counter() - t0)
    # the plain loop: one icm_gpu_equity call per tournament
    for S, P in ts[:16]:
        icm.gpu_equity(S, P)
    t0 = time.perf_counter()
    loop = [icm.gpu_equity(S, P) for S, P in ts]
    loop_s = time.perf_counter() - t0
    err = 0.0
    for a, r in zip(res, loop):
        err = max(err, float(np.max(np.abs(a - r) / np.maximum(np.abs(r), 1e-300))))
    split = np.split(out, np.cumsum([len(S) for S in Ss])[:-1])
    err_replay = max(float(np.max(np.abs(a - r) / np.maximum(np.abs(r), 1e-300))) for a, r in zip(split, loop))
    dev_ms = float(np.mean(dev))
    tot = sum(r["ms"] for r in kst)
    return {
        "metric": "batched tourn/s", "value": count / (dev_ms * 1e-3), "unit": "tournaments/s",
        "ms_per_batch": dev_ms, "tournaments": count, "players": players, "Q": 256,
        "q_chunk": info["q_chunk"], "device_bytes": info["device_bytes"], "fallback_tournaments": info["fallbacks"],
        "gpu_launches_per_batch": launches,
        "replay_wall_ms": 1e3 * float(np.mean(wall)),
        "e2e": {"value": count / float(np.mean(e2e)), "unit": "tournaments/s", "ms_per_batch": 1e3 * float(np.mean(e2e)),
                "h2d_bytes_per_step": 8 * (players + sum(ks)) + 8 * count, "d2h_bytes_per_step": 8 * players,
                "path": "icm_gpu_equity_batched (C ABI, host arrays, batch set-up inside)"},
        "plain_loop": {"value": count / loop_s, "unit": "tournaments/s", "ms_per_batch": 1e3 * loop_s,
                       "path": "one icm_gpu_equity call per tournament (host arrays)"},
        "speedup_vs_loop": {"device": (loop_s * 1e3) / dev_ms, "e2e": loop_s / float(np.mean(e2e))},
        "max_rel_err_vs_loop": max(err, err_replay),
        "kernels": [{"kernel": r["name"], "ms": r["ms"], "launches": r["launches"], "flops": r["flops"],
                     "share": r["ms"] / tot if tot else None} for r in kst],
        "config": "n log-uniform [9,20000], k=ceil(0.15n), stacks 1e4*lognormal(0,1), payout 0.8^j normalised",
        "canonical": batch_canonical(Ss, ks, dev_ms, fp64_tflops),
    }


def batch_canonical(Ss, ks, ms, fp64_tflops):
    """The reference's canonical work of the whole batch (each member with
    the block size min(64, max(8, n/4))) over the batch's device time, as a
    fraction of the measured FP64 peak."""
    if not fp64_tflops:
        return None
    W = sum(canonical_work(len(S), k, min(64, max(8, len(S) // 4)))[0] for S, k in zip(Ss, ks))
    return {"W_ref_flop": float(W), "achieved_fp64": float(W / (ms * 1e-3 * fp64_tflops * 1e12)),
            "fp64_peak_tflops": fp64_tflops, "B_ref": "min(64, max(8, n/4)) per member"}


def gpu_scale_leg(icm, W, steps, fp64_tflops=None):
    """GPU-only scale: n = 2^20 players, stacks 1e4 exp(1.5 N(0,1)), Q = 256;
    (a) k = n linear payout, (b) k = 1000 geometric 0.97.  Device ms per solve
    with the plan resident, end-to-end ms through icm_equity, and the
    closed-form error of (a) on 64 sampled players (E = V1 / sum(n - m))."""
    out = {"config": "n=1048576, stacks 1e4*exp(1.5 N(0,1)), Q=256"}
    from icm_gb300._lib import lib
    for shape in ("linear", "geometric"):
        S, P = W.gpu_scale(shape=shape)
        plan = icm.GpuPlan(S, len(P))
        E = plan.equity(P)
        dev = []
        for _ in range(max(2, steps)):
            plan.equity(P)
            dev.append(lib().icm_gb300_plan_device_ms(plan._p))
        summ = plan.summary()
        plan.close()
        t0 = time.perf_counter()
        icm.equity(S, P)
        e2e = time.perf_counter() - t0
        rec = {"k": len(P), "device_ms": float(np.median(dev)), "e2e_ms": e2e * 1e3,
               "q_chunk": summ["q_batch"], "device_bytes": summ["planned_peak_vram_bytes"]}
        if fp64_tflops:
            rec["canonical"] = canonical_rates(len(S), len(P), rec["device_ms"], fp64_tflops)
        if shape == "linear":   # V1_i = 1 + sum_{j != i} S_i / (S_i + S_j); payout (n - m) / sum
            idx = np.random.default_rng(3).choice(len(S), 64, replace=False)
            n = len(S)
            ref = np.array([0.5 + np.sum(S[i] / (S[i] + S)) for i in idx]) * (P[0] / n)
            rec["max_rel_err_vs_closed_form_64_players"] = float(np.max(np.abs(E[idx] - ref) / np.abs(ref)))
        out[shape] = rec
    return out


def vjp_leg(icm, W, steps, fp64_tflops=None):
    """Differentiated form: n = 16384, k = 2000, Q = 256, gamma(2, 5000)
    stacks, N(0, 1) cotangent, linear and quadratic payouts.  Device time of
    the VJP (forward tree recomputed inside) against the forward solve on the
    same stacks, both with plans resident; e2e through icm_gb300_equity_vjp;
    the same at n = k = 2^18 (linear payout: every level untruncated, so the
    tree's top levels are spectral in both directions); and the batched VJP
    over 256 tournaments with n in [100, 4000]."""
    out = {"metric": "VJP/fwd time", "config": "n=16384, k=2000, Q=256, stacks gamma(2,5000), cotangent N(0,1)"}
    for shape in ("linear", "quadratic", "untruncated_262144"):
        S, P, cot = W.vjp(payout=shape) if shape != "untruncated_262144" else W.vjp(n=1 << 18, k=1 << 18)
        k = len(P)
        fplan = icm.GpuPlan(S, k)
        vplan = icm.VjpPlan(S, k)
        for _ in range(2):
            fplan.equity(P)
            vplan.run(P, cot)
        fwd, vjp = [], []
        from icm_gb300._lib import lib
        for _ in range(max(2, steps)):
            fplan.equity(P)
            fwd.append(lib().icm_gb300_plan_device_ms(fplan._p))
            vplan.run(P, cot)
            vjp.append(vplan.device_ms())
        fplan.close()
        vplan.close()
        t0 = time.perf_counter()
        icm.equity_vjp(S, P, cot)
        e2e = time.perf_counter() - t0
        if fp64_tflops:
            out.setdefault("canonical_fwd", canonical_rates(len(S), k, float(np.median(fwd)), fp64_tflops))
        out[shape] = {"fwd_ms": float(np.median(fwd)), "vjp_ms": float(np.median(vjp)),
                      "ratio": float(np.median(vjp) / np.median(fwd)), "vjp_e2e_ms": e2e * 1e3}
    ts, cots = vjp_batch_tournaments(256)
    icm.equity_vjp_batched(ts[:4], cots[:4])
    t0 = time.perf_counter()
    icm.equity_vjp_batched(ts, cots)
    tv = time.perf_counter() - t0
    t0 = time.perf_counter()
    icm.equity_batched(ts)
    tf = time.perf_counter() - t0
    # resident batches: device time of one graph replay each
    stacks, ks, pays = [S for S, _ in ts], [len(P) for _, P in ts], [P for _, P in ts]
    fb, vb = icm.GpuBatch(stacks, ks), icm.GpuVjpBatch(stacks, ks)
    fdev, vdev = [], []
    for i in range(max(2, steps) + 2):
        fb.equity(pays)
        vb.vjp(pays, cots)
        if i >= 2:
            fdev.append(fb.info()["device_ms"])
            vdev.append(vb.info()["device_ms"])
    fb.close()
    vb.close()
    out["batched_256"] = {"vjp_ms": tv * 1e3, "fwd_ms": tf * 1e3, "ratio": tv / tf,
                          "vjp_device_ms": float(np.median(vdev)), "fwd_device_ms": float(np.median(fdev)),
                          "device_ratio": float(np.median(vdev) / np.median(fdev)),
                          "config": "256 tournaments, n uniform [100,4000], k=ceil(0.15n), payout 0.8^j; one-shot "
                                    "wall time, and device time of resident batches (graph replay)"}
    return out


def vjp_batch_tournaments(count, seed=77):
    """The VJP leg's batch: n uniform in [100, 4000], k = ceil(0.15 n),
    1e4 lognormal(0, 1) stacks, payouts 0.8^j, N(0, 1) cotangents."""
    rng = np.random.default_rng(seed)
    ts, cots = [], []
    for _ in range(count):
        n = int(rng.integers(100, 4001))
        k = max(1, int(np.ceil(0.15 * n)))
        ts.append((1e4 * np.exp(rng.standard_normal(n)), 0.8 ** np.arange(k)))
        cots.append(rng.standard_normal(n))
    return ts, cots


def run_case(icm, W, case):
    """One untimed run of a named small workload (the target of an ncu capture)."""
    kind, *rest = case.split(":")
    if kind == "vjp_batch":
        ts, cots = vjp_batch_tournaments(int(rest[0]))
        vb = icm.GpuVjpBatch([S for S, _ in ts], [len(P) for _, P in ts])
        vb.set_options(graphs=False)
        vb.vjp([P for _, P in ts], cots)
        vb.close()
    elif kind == "batch":   # batch:T[:Q] -- Q nodes in one chunk (default 256)
        ts = W.batched(count=int(rest[0]))
        Q = int(rest[1]) if len(rest) > 1 else 256
        icm.configure(q_chunk=Q)
        b = icm.GpuBatch([S for S, _ in ts], [len(P) for _, P in ts])
        b.set_options(graphs=False)
        b.equity([P for _, P in ts], Q=Q)
        b.close()
        icm.configure()
    elif kind == "small":
        n, k = int(rest[0]), int(rest[1])
        rng = np.random.default_rng(n)
        S, P = 1e4 * np.exp(rng.standard_normal(n)), 0.8 ** np.arange(k)
        for _ in range(20):
            icm.gpu_equity(S, P)
    elif kind == "dropin":   # the drop-in distribution at n players and Q nodes (one chunk), one solve
        n, Q = int(rest[0]), int(rest[1])
        S, P, _ = W.dropin(n=n)
        icm.configure(q_chunk=Q)
        icm.gpu_equity(S, P, Q=Q)
        icm.configure()
    elif kind == "linear":   # the linear engine, one solve
        n, k = int(rest[0]), int(rest[1])
        rng = np.random.default_rng(n)
        S, P = 1e4 * np.exp(rng.standard_normal(n)), 0.8 ** np.arange(k)
        icm.configure(engine="linear")
        icm.gpu_equity(S, P)
        icm.configure()
    else:
        raise SystemExit(f"unknown case {case!r}")
    print(json.dumps({"case": case, "status": "ok"}))


def traffic_for(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary
    (profiles/traffic.txt: '<kernel> <bytes_per_launch> <workload note>'),
    or None when no capture covers it."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.isfile(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel and not line.startswith("#"):
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


if __name__ == "__main__":
    main()
