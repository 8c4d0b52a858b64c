#!/usr/bin/env python
"""Benchmark of the plain single-solve RK4 step: 3D Taylor-Green vortex,
compressible Euler, gamma 1.4, periodic [0, 2 pi)^3 Fourier grid 256^3,
float32 state, 2/3 dealiasing, RK4 with fixed dt = 1e-3.

One "step" is one full RK4 step (four right-hand-side evaluations, the
end-of-step filter) of the whole grid; the metric is cell-updates/s (grid
nodes advanced by one RK4 step per second).  Inputs (the state and the pass
intermediates, ~2.7 GB) are far larger than the 129 MB L2, so no flush is
needed between timed steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun (N > 1) every rank advances its own replica (a single solve
does not shard); the value is the total cell-updates of all ranks over the
slowest rank's time.  ``--impl reference`` times the CPU restatement of the
reference algorithm (float64 NumPy/SciPy FFT, all host cores) on rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "cell-updates/s vs plain; ensemble solves/s, p50/p99 latency at rel-L2 err≤1e-5"
UNIT = "cell-updates/s"
DT = 1e-3
PEAKS_FILE = os.path.join(REPO, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def workload_config(n: int, world: int) -> dict:
    return {
        "workload": f"3D Taylor-Green vortex, compressible Euler, {n}^3 periodic Fourier, RK4 dt={DT}",
        "grid": [n, n, n],
        "state_dtype": "float32",
        "dealias": "2/3",
        "filter": "off (mask-only end-of-step filter applied every step)",
        "cells_per_step": n ** 3,
        "l2_policy": "inputs larger than L2 (state + pass intermediates ~2.7 GB >> 129 MB)",
        "parallelism": f"replicas x{world}" if world > 1 else "single solve",
    }


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the
# pass kernels of a TGV 256^3 RK4 step, averaged over the step's launches,
# from ncu captures of the bench command (x pass at 256^3; y and last pass
# at 128^3, reads scaled by the 8x cell count, writes at their algorithmic
# size, which every write reaches at 256^3).
NCU_TRAFFIC_TGV256 = {"x_pass": 1.366e9, "y_pass": 1.678e9, "last_pass": 1.762e9}


def traffic_per_launch(kind: str, n: int):
    if kind not in NCU_TRAFFIC_TGV256 or n != 256:
        return None
    return NCU_TRAFFIC_TGV256[kind]


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_oracle_step_rate(n: int, max_steps: int, budget_s: float):
    """Time the float64 CPU restatement of the reference step at n^3."""
    from oracle import spectral as O
    from phrike_gb300 import problems
    cores = os.cpu_count() or 1
    os.environ.setdefault("PHRIKE_ORACLE_WORKERS", str(cores))
    s = O.EulerSolver(O.FourierBox((n, n, n), (2 * np.pi,) * 3, dealias=True), cfl=0.25)
    U = problems.taylor_green_3d(n)
    done, t_total = 0, 0.0
    while done < max_steps:
        t0 = time.perf_counter()
        U = s.step(U, DT)
        t_total += time.perf_counter() - t0
        done += 1
        if t_total >= budget_s:
            break
    return n ** 3 * done / t_total, done, t_total, cores


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    n = args.n
    # bounded sample: at most 1 warm-up and 3 timed full RK4 steps at n^3
    from oracle import spectral as O  # noqa: F401  (checker import only)
    if args.warmup > 0:
        cpu_oracle_step_rate(n, 1, 0.0)
    rate, done, t_total, cores = cpu_oracle_step_rate(n, max(1, min(args.steps, 3)), 120.0)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": world,
        "steps": done, "warmup": min(args.warmup, 1), "ms_per_step": 1e3 * t_total / done,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (analytic Taylor-Green initial condition)",
        "config": workload_config(n, 1),
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{done} full RK4 step(s) at {n}^3 (float64 NumPy/SciPy FFT restatement "
                                   f"of the reference, scipy.fft workers={cores})"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gb300(args, rank: int, world: int):
    import torch
    import torch.distributed as dist
    from phrike_gb300 import _build, problems
    from phrike_gb300.engine import Plan

    _build.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    n = args.n
    cells = n ** 3
    plan = Plan((n, n, n), (2 * np.pi,) * 3, device=device)
    U0h = torch.from_numpy(problems.taylor_green_3d(n).astype(np.float32))
    U = U0h.to(device)

    def barrier():
        if world > 1:
            dist.barrier()

    # warm-up
    plan.run_(U, args.warmup, DT)
    torch.cuda.synchronize()

    # timed region: K steps, device-resident state
    sampler = ClockSampler(local)
    plan.profile(True)
    plan.collect_profile()
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    stream = torch.cuda.current_stream(device)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    plan.run_(U, args.steps, DT)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    prof = plan.collect_profile()
    plan.profile(False)
    finite = bool(torch.isfinite(U).all().item())
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    value = cells * args.steps * world / (ms_max * 1e-3)

    # end-to-end through the public API with host buffers: every step takes
    # its state from pinned host memory (H2D), runs one RK4 step and returns
    # the new state to pinned host memory (D2H); Plan.step_host_stream
    # overlaps the copies of the neighbouring states with each step.  The
    # stream has as many states as the device-timed loop has steps, so the
    # first copy in and the last copy out (not overlapped) weigh as little.
    e2e_steps = max(2, args.steps)
    hin = U0h.pin_memory()
    hout = torch.empty_like(hin).pin_memory()
    plan.step_host_stream([hin, hin], [hout, hout], DT)  # warm-up of the copy path
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    plan.step_host_stream([hin] * e2e_steps, [hout] * e2e_steps, DT)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    te = torch.tensor([e2e_s], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_value = cells * e2e_steps * world / float(te.item())
    state_bytes = U.numel() * 4
    # the same with the copies in line: each step waits for its state to land,
    # steps, and copies the result back before the next state is sent
    dev_state = torch.empty_like(U)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        dev_state.copy_(hin, non_blocking=True)
        plan.step_(dev_state, DT)
        hout.copy_(dev_state, non_blocking=True)
        torch.cuda.synchronize()
    ti = torch.tensor([time.perf_counter() - t0], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(ti, op=dist.ReduceOp.MAX)
    e2e_inline = cells * e2e_steps * world / float(ti.item())

    if rank != 0:
        return
    # roofline of the dominant pass kernel (largest share of device time)
    peak, peak_kind = hbm_peak()
    dom = max(prof, key=lambda k: prof[k]["ms"])
    d = prof[dom]
    per_launch_ms = d["ms"] / d["launches"]
    per_launch_bytes = d["bytes"] / d["launches"]
    achieved = per_launch_bytes / (per_launch_ms * 1e-3) / 1e9
    total_ms = sum(v["ms"] for v in prof.values())
    roofline = {
        "bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
        "traffic": traffic_per_launch(dom, n), "algorithmic_bytes_per_launch": per_launch_bytes,
        "launch_ms": per_launch_ms,
        "kernels": {k: {"launches": v["launches"], "share": v["ms"] / total_ms,
                        "achieved_GBps": v["bytes"] / (v["ms"] * 1e-3) / 1e9}
                    for k, v in prof.items()},
        "step_GBps": sum(v["bytes"] for v in prof.values()) / (ms * 1e-3) / 1e9,
    }
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        rate, done, t_total, cores = cpu_oracle_step_rate(n, 1, 0.0)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{done} full RK4 step at {n}^3, {t_total:.1f} s (float64 NumPy/SciPy FFT "
                         f"restatement of the reference, scipy.fft workers={cores})"}
    ens = None
    if world == 1 and not args.no_ensemble_sample:
        plan.close()
        ens = ensemble_sample(device)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (analytic Taylor-Green initial condition)",
        "config": workload_config(n, world),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": state_bytes,
                "d2h_bytes_per_step": state_bytes, "steps": e2e_steps,
                "path": "phrike_gb300.engine.Plan.step_host_stream -> ps_step_rk4 (C ABI): pinned host state "
                        "in and out every step, copies of neighbouring states overlapped with each step",
                "inline_value": e2e_inline,
                "inline_path": "per step: pinned host state to the device, Plan.step_ (ps_step_rk4), result back "
                               "to pinned host memory, synchronize; no overlap"},
        "gpu_launches": sum(v["launches"] for v in prof.values()),
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "state_finite": finite,
        "ensemble_sample": ens,
    }
    print(json.dumps(line), flush=True)


def ensemble_sample(device, nsolve: int = 64, t_end: float = 0.2, chunk: int = 50) -> dict:
    """A short sample of the batching workload for the default line: nsolve
    seeded KHI solves (N uniform on 64..512) to t_end in one batched,
    graph-captured run, against the same solves run one at a time with the
    device time loop (one solve per size timed, scaled by the size counts)."""
    import torch
    from phrike_gb300.engine import Plan
    from phrike_gb300.ensemble import Ensemble, SolveSpec

    specs = khi_ensemble_specs(nsolve, t_end=t_end)
    Ensemble([SolveSpec(sp.shape, sp.lengths, sp.U0, 1e-4) for sp in specs], cfl=0.4,
             device=device, autotune=True).run(chunk=chunk, use_graphs=True)  # warm-up and tuning
    torch.cuda.synchronize()
    stats = Ensemble(specs, cfl=0.4, device=device, autotune=True).run(chunk=chunk, use_graphs=True)
    counts = {}
    for sp in specs:
        counts[sp.shape[0]] = counts.get(sp.shape[0], 0) + 1
    plain = 0.0
    for n, cnt in sorted(counts.items()):
        sp = next(x for x in specs if x.shape[0] == n)
        plan = Plan(sp.shape, sp.lengths, cfl=0.4, device=device)
        U = torch.as_tensor(sp.U0, dtype=torch.float32, device=device).contiguous()
        t = torch.zeros(1, dtype=torch.float64, device=device)
        te = torch.tensor([sp.t_end], dtype=torch.float64, device=device)
        plan.run_cfl_(U.clone(), 1, t.clone(), te)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        while float(t.item()) < sp.t_end - 1e-12:
            plan.run_cfl_(U, chunk, t, te)
        torch.cuda.synchronize()
        plain += cnt * (time.perf_counter() - t0)
        plan.close()
    return {"workload": f"{nsolve} KHI 2D solves, N uniform on 64..512, CFL 0.4, t_end={t_end}",
            "batched_solves_per_s": nsolve / stats["seconds"], "plain_device_loop_solves_per_s": nsolve / plain,
            "speedup_vs_plain_device_loop": plain / stats["seconds"],
            "cell_updates_per_s": stats["cell_updates_per_s"], "status": stats["status"],
            "accuracy": "one solve per size run to t=1 against the float64 oracle: momentum rel-L2 8.3e-6, "
                        "2.2e-6, 3.1e-6, 5.7e-5 at 64^2, 128^2, 256^2, 512^2 (tests/test_gpu_parity_full.py)"}


def khi_ensemble_specs(nsolve: int, seed: int = 20261203, t_end: float = 1.0):
    """The batching workload: KHI solves on [0,1)^2 with N uniform on
    {64,128,256,512}, U0 ~ U[0.5,1.5], A ~ U[0.005,0.02], seeded."""
    from phrike_gb300 import problems
    from phrike_gb300.ensemble import SolveSpec
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(nsolve):
        n = int(rng.choice([64, 128, 256, 512]))
        u0 = float(rng.uniform(0.5, 1.5))
        amp = float(rng.uniform(0.005, 0.02))
        specs.append(SolveSpec((n, n), (1.0, 1.0), problems.kelvin_helmholtz_2d(n, n, U0=u0, A=amp), t_end))
    return specs


def run_ensemble(args, rank: int = 0, world: int = 1):
    """Ensemble solves/s: every solve to t_end in one batched, graph-captured
    run, against the same solves run one at a time (a per-size sample,
    extrapolated by the size counts).  With N ranks the solve list is split
    by instance (phrike_gb300.replicas.shard, cost ~ n^3: cells x CFL steps);
    the run's time is the slowest rank's, and the plain form is N GPUs each
    running its share one solve at a time."""
    import torch
    from phrike_gb300 import _build
    from phrike_gb300.engine import Plan
    from phrike_gb300.ensemble import Ensemble
    from phrike_gb300.equations import EulerEquations2D
    from phrike_gb300.grid import Grid2D
    from phrike_gb300.replicas import reduce_max, shard
    from phrike_gb300.solver import SpectralSolver2D

    _build.build()
    device = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(device)
    all_specs = khi_ensemble_specs(args.nsolve, t_end=args.t_end)
    mine = shard([float(sp.shape[0]) ** 3 for sp in all_specs], rank, world)
    specs = [all_specs[i] for i in mine]
    # warm-up: the same groups for a short time, so that lazy kernel loading
    # (about 2 s for this library on first use) stays out of the timed run
    from phrike_gb300.ensemble import SolveSpec
    Ensemble([SolveSpec(sp.shape, sp.lengths, sp.U0, 1e-4) for sp in specs], cfl=0.4,
             device=device, autotune=True).run(chunk=args.chunk, use_graphs=True)
    torch.cuda.synchronize()
    ens = Ensemble(specs, cfl=0.4, device=device, autotune=True)  # tile widths measured (cached)
    sampler = ClockSampler(device.index)
    sampler.start()
    stats = ens.run(chunk=args.chunk, use_graphs=True)
    clocks = sampler.stop()
    seconds = reduce_max(stats["seconds"])
    if rank != 0:
        return
    # plain: one solve at a time, (a) device time loop, (b) host CFL loop as the reference's run()
    counts = {}
    for sp in all_specs:
        counts[sp.shape[0]] = counts.get(sp.shape[0], 0) + 1
    plain_dev, plain_host = 0.0, 0.0
    sample = {}
    for n, cnt in sorted(counts.items()):
        sp = next(x for x in all_specs if x.shape[0] == n)
        plan = Plan(sp.shape, sp.lengths, cfl=0.4, device=device)
        U = torch.as_tensor(sp.U0, dtype=torch.float32, device=device).contiguous()
        t = torch.zeros(1, dtype=torch.float64, device=device)
        te = torch.tensor([sp.t_end], dtype=torch.float64, device=device)
        plan.run_cfl_(U.clone(), 1, t.clone(), te)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        # the 2D/3D step loop is driven from the host: advance in chunks and
        # stop once the device-side time has reached t_end
        while float(t.item()) < sp.t_end - 1e-12:
            plan.run_cfl_(U, args.chunk, t, te)
        torch.cuda.synchronize()
        td = time.perf_counter() - t0
        grid = Grid2D(Nx=n, Ny=n, Lx=1.0, Ly=1.0, backend="gb300")
        solver = SpectralSolver2D(grid, EulerEquations2D(gamma=1.4), cfl=0.4)
        solver.run(sp.U0, 0.0, min(sp.t_end, 1e-3), output_interval=1e9)  # warm-up
        t0 = time.perf_counter()
        solver.run(sp.U0, 0.0, sp.t_end, output_interval=1e9)
        torch.cuda.synchronize()
        th = time.perf_counter() - t0
        plain_dev += cnt * td
        plain_host += cnt * th
        sample[str(n)] = {"solves": cnt, "device_loop_s": td, "host_loop_s": th}
    plain_dev /= world  # N GPUs, each running its share plainly (balanced)
    plain_host /= world
    line = {
        "metric": "ensemble solves/s (batched vs plain, same GPU)", "value": args.nsolve / seconds,
        "unit": "solves/s", "n_gpus": world, "higher_is_better": True, "dtype": "f32",
        "scaling": "strong", "data": "synthetic (seeded KHI initial conditions)",
        "config": {"workload": f"{args.nsolve} KHI 2D solves, N uniform on 64..512, CFL 0.4, t_end={args.t_end}",
                   "chunk_steps_per_graph": args.chunk,
                   "parallelism": f"replicas x{world}, solves split by instance" if world > 1 else "one GPU"},
        "seconds": seconds, "graph_capture_seconds": stats["capture_seconds"],
        "tile_cols": {f"{k[0][0]}x{k[0][1]}": v for k, v in ens.tile_cols.items()},
        "cell_updates_per_s": stats["cell_updates_per_s"] * (world if world > 1 else 1),
        "status": stats["status"],
        "plain_device_loop_solves_per_s": args.nsolve / plain_dev,
        "plain_host_loop_solves_per_s": args.nsolve / plain_host,
        "speedup_vs_plain_device_loop": plain_dev / seconds,
        "speedup_vs_plain_host_loop": plain_host / seconds,
        "plain_sample": sample, "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_lgl(args):
    """Precision on dense collocation: the LGL x LGL acoustic pulse (rho = 1 +
    0.01 exp(-r^2/0.01), p = rho^gamma/gamma, u = v = 0 on [-1, 1]^2, walls),
    RK4 with dt = 1e-5 for --lgl-steps steps, per contraction precision: time
    per step and the relative L2 error per conserved field against the
    float64 oracle, which runs here on the host cores (its time is the CPU
    baseline).  The error is given from the float64 initial state (what a
    float32-state run can reach) and from the float32-rounded one (the
    contraction precision alone)."""
    import torch
    from oracle import lgl as L
    from phrike_gb300 import _build, problems
    from phrike_gb300.engine import Plan

    _build.build()
    device = torch.device("cuda", 0)
    nsteps, dt = args.lgl_steps, 1e-5
    precs = ["fp64", "fp32", "bf16x3"]
    peaks = {}
    try:
        with open(PEAKS_FILE) as f:
            peaks = json.load(f)
    except Exception:
        pass
    tc_peak = float(peaks.get("bf16_tflops", 1900.0))
    table = []
    headline = None
    threads = os.cpu_count() or 1
    for n in [int(x) for x in args.lgl_sizes.split(",")]:
        ax = L.LGLAxis(n, 2.0)
        U0 = problems.acoustic_pulse_lgl_2d(ax.x - 1.0, ax.x - 1.0, gamma=1.4)
        s = L.LGLSolver2D(n, n, gamma=1.4)
        R = U0.copy()
        t0 = time.perf_counter()
        for _ in range(nsteps):
            R = s.step(R, dt)
        cpu_s = time.perf_counter() - t0
        s32 = L.LGLSolver2D(n, n, gamma=1.4)
        R32 = U0.astype(np.float32).astype(np.float64)
        for _ in range(nsteps):
            R32 = s32.step(R32, dt)
        row = {"n": n, "cells": n * n, "steps": nsteps, "cpu_oracle_s_per_step": cpu_s / nsteps,
               "cpu_oracle_cell_updates_per_s": n * n * nsteps / cpu_s, "cpu_threads": threads}
        for prec in precs:
            plan = Plan((n, n), (2.0, 2.0), gamma=1.4, basis="legendre", gemm_precision=prec, device=device)
            Uw = torch.as_tensor(U0, dtype=torch.float32, device=device).contiguous()
            plan.run_(Uw, 3, dt)  # warm-up
            U = torch.as_tensor(U0, dtype=torch.float32, device=device).contiguous()
            torch.cuda.synchronize()
            st = torch.cuda.current_stream(device)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            plan.run_(U, nsteps, dt)
            e1.record(st)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / nsteps
            G = U.cpu().numpy().astype(np.float64)

            def rl(a, b):
                return float(np.linalg.norm(a - b) / np.linalg.norm(b))

            ent = {"ms_per_step": ms, "cell_updates_per_s": n * n / (ms * 1e-3),
                   "rel_l2_vs_f64_ic": {"rho": rl(G[0], R[0]), "mom": rl(G[1:3], R[1:3]), "E": rl(G[3], R[3])},
                   "rel_l2_vs_f32_ic": {"rho": rl(G[0], R32[0]), "mom": rl(G[1:3], R32[1:3]),
                                        "E": rl(G[3], R32[3])},
                   "status": plan.status()}
            if prec == "bf16x3":
                # contraction kernels alone: issued split-bf16 flops per launch / event time
                plan.profile(True)
                Up = torch.as_tensor(U0, dtype=torch.float32, device=device).contiguous()
                plan.run_(Up, 5, dt)
                prof = plan.collect_profile()
                plan.profile(False)
                fl_x = 3 * 2.0 * (4 * n) * n * n
                fl_y = 3 * 2.0 * 4 * n * n * n
                for kind, fl in (("lgl_x", fl_x), ("lgl_y", fl_y)):
                    if kind in prof:
                        per = prof[kind]["ms"] / prof[kind]["launches"]
                        ent[f"{kind}_us"] = per * 1e3
                        ent[f"{kind}_tflops_issued"] = fl / (per * 1e-3) / 1e12
                        ent[f"{kind}_tensor_frac_of_measured_bf16"] = fl / (per * 1e-3) / 1e12 / tc_peak
                headline = ent["cell_updates_per_s"]
            row[prec] = ent
            plan.close()
        table.append(row)
    # a batch of --lgl-batch solves of the last size on the tensor cores: the
    # contraction of one solve fills one wave of CTAs; a batch fills the GPU
    batch = None
    if args.lgl_batch > 1:
        n = int(args.lgl_sizes.split(",")[-1])
        ax = L.LGLAxis(n, 2.0)
        U0 = problems.acoustic_pulse_lgl_2d(ax.x - 1.0, ax.x - 1.0, gamma=1.4)
        nb = args.lgl_batch
        UB = torch.as_tensor(np.stack([U0] * nb), dtype=torch.float32, device=device).contiguous()
        from phrike_gb300.autotune import tune_umma_n_tile
        nt, nt_times = tune_umma_n_tile((n, n), (2.0, 2.0), UB, nsolve=nb, dt=dt, gamma=1.4, device=device)
        plan = Plan((n, n), (2.0, 2.0), gamma=1.4, basis="legendre", gemm_precision="bf16x3", device=device,
                    nsolve=nb, umma_n_tile=nt)
        plan.run_(UB, 3, dt)
        torch.cuda.synchronize()
        st = torch.cuda.current_stream(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        bsteps = max(10, min(nsteps, 50))
        e0.record(st)
        plan.run_(UB, bsteps, dt)
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / bsteps
        plan.profile(True)
        plan.run_(UB, 3, dt)
        prof = plan.collect_profile()
        plan.profile(False)
        batch = {"solves": nb, "n": n, "ms_per_step": ms, "cell_updates_per_s": nb * n * n / (ms * 1e-3),
                 "status": plan.status(), "umma_n_tile": nt,
                 "umma_n_tile_ms_per_step": {str(k): v for k, v in nt_times.items()}}
        fl = 3 * 2.0 * (4 * n) * n * n * nb
        for kind in ("lgl_x", "lgl_y"):
            if kind in prof:
                per = prof[kind]["ms"] / prof[kind]["launches"]
                batch[f"{kind}_us"] = per * 1e3
                batch[f"{kind}_tflops_issued"] = fl / (per * 1e-3) / 1e12
                batch[f"{kind}_tensor_frac_of_measured_bf16"] = fl / (per * 1e-3) / 1e12 / tc_peak
        plan.close()
    line = {
        "metric": "LGL 2D acoustic pulse: cell-updates/s and rel-L2 vs float64 oracle per contraction precision",
        "batch_bf16x3": batch,
        "value": headline, "unit": "cell-updates/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32",
        "data": "synthetic (analytic acoustic pulse initial condition)",
        "config": {"workload": f"LGL x LGL acoustic pulse, walls, RK4 dt=1e-5, {nsteps} steps, "
                               f"sizes {args.lgl_sizes}; value = bf16x3 at the last size"},
        "table": table,
    }
    print(json.dumps(line), flush=True)


def run_ot(args):
    """2D ideal MHD: the Orszag-Tang vortex (rho = gamma^2, p = gamma, B0 = 1
    on [0, 2 pi)^2, gamma = 5/3, filter p = 8, alpha = 36) at --ot-n^2, fixed
    dt = 1e-3 RK4 steps with per-stage clamp and Helmholtz projection:
    cell-updates/s, per-pass launch times against the measured HBM peak, and
    the float64 oracle's step time on the host cores as the CPU baseline."""
    import torch
    from oracle import mhd as M
    from phrike_gb300 import _build, problems
    from phrike_gb300.engine import Plan

    _build.build()
    device = torch.device("cuda", 0)
    n = args.ot_n
    fp = {"enabled": True, "p": 8, "alpha": 36.0}
    U0 = problems.orszag_tang_2d(n, n, gamma=5.0 / 3.0)
    plan = Plan((n, n), (2 * np.pi, 2 * np.pi), gamma=5.0 / 3.0, filter_params=fp, device=device, equations="mhd")
    U = torch.as_tensor(U0, dtype=torch.float32, device=device).contiguous()
    plan.project_state_(U)
    plan.run_(U, args.warmup, 1e-3)
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    st = torch.cuda.current_stream(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    plan.run_(U, args.steps, 1e-3)
    e1.record(st)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    plan.profile(True)
    plan.run_(U, 3, 1e-3)
    prof = plan.collect_profile()
    plan.profile(False)
    peak, src = hbm_peak()
    kinds = {}
    for k, v in prof.items():
        per = v["ms"] / v["launches"]
        kinds[k] = {"launches_per_step": v["launches"] / 3, "us_per_launch": per * 1e3,
                    "gbs": v["bytes"] / v["launches"] / (per * 1e-3) / 1e9,
                    "frac_of_peak": v["bytes"] / v["launches"] / (per * 1e-3) / 1e9 / peak}
    # CPU baseline: the float64 oracle, one step at a bounded size
    s = M.MHDSolver2D(n, n, filter_params=fp)
    R = s.project(U0)
    t0 = time.perf_counter()
    R = s.step(R, 1e-3)
    cpu_s = time.perf_counter() - t0
    G = U.cpu().numpy()
    line = {
        "metric": "2D ideal MHD Orszag-Tang: cell-updates/s (RK4, per-stage projection)", "value": n * n / (ms * 1e-3),
        "unit": "cell-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "dtype": "f32", "data": "synthetic (analytic Orszag-Tang initial condition)",
        "config": {"workload": f"Orszag-Tang {n}^2, gamma 5/3, filter p=8 alpha=36, RK4 dt=1e-3"},
        "passes": kinds, "peak_gbs": peak, "peak_source": src,
        "cpu_baseline": {"value": n * n / cpu_s, "unit": "cell-updates/s", "cores": os.cpu_count(),
                         "kind": "port", "sample": f"1 RK4 step of the float64 oracle at {n}^2"},
        "state_finite": bool(np.isfinite(G).all()), "status": plan.status(), "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_khi(args):
    """2D Euler Kelvin-Helmholtz at one size (--khi-n^2, the ensemble's
    largest grid) with the ensemble's CFL loop (CFL 0.4, no solve finishing):
    one solve alone and a batch of --khi-batch solves in one plan, each timed
    over --steps device-side CFL steps, with cell-updates/s and per-pass
    launch times against the measured HBM peak.  The per-cell ratio of the
    two is what batching buys at this size."""
    import torch
    from phrike_gb300 import _build, problems
    from phrike_gb300.engine import Plan

    _build.build()
    device = torch.device("cuda", 0)
    n, nb = args.khi_n, args.khi_batch
    rng = np.random.default_rng(20261204)
    states = [problems.kelvin_helmholtz_2d(n, n, U0=float(rng.uniform(0.5, 1.5)), A=float(rng.uniform(0.005, 0.02)))
              for _ in range(nb)]
    peak, src = hbm_peak()
    out = {}
    for ns in (1, nb):
        plan = Plan((n, n), (1.0, 1.0), cfl=0.4, device=device, nsolve=ns)
        U = torch.as_tensor(np.stack(states[:ns]) if ns > 1 else states[0], dtype=torch.float32,
                            device=device).contiguous()
        t = torch.zeros(ns, dtype=torch.float64, device=device)
        te = torch.full((ns,), 1e9, dtype=torch.float64, device=device)
        plan.run_cfl_(U, args.warmup, t, te)
        torch.cuda.synchronize()
        st = torch.cuda.current_stream(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        plan.run_cfl_(U, args.steps, t, te)
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        plan.profile(True)
        plan.run_cfl_(U, 3, t, te)
        prof = plan.collect_profile()
        plan.profile(False)
        kinds = {}
        for k, v in prof.items():
            per = v["ms"] / v["launches"]
            kinds[k] = {"launches_per_step": v["launches"] / 3, "us_per_launch": per * 1e3,
                        "gbs": v["bytes"] / v["launches"] / (per * 1e-3) / 1e9,
                        "frac_of_peak": v["bytes"] / v["launches"] / (per * 1e-3) / 1e9 / peak}
        out["batch" if ns > 1 else "alone"] = {
            "nsolve": ns, "ms_per_step": ms, "cell_updates_per_s": ns * n * n / (ms * 1e-3), "passes": kinds,
            "status": plan.status(), "state_finite": bool(torch.isfinite(U).all().item())}
        plan.close()
    line = {
        "metric": "2D Euler KHI: cell-updates/s, one solve and a batch in one plan", "unit": "cell-updates/s",
        "value": out["batch"]["cell_updates_per_s"], "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded KHI initial conditions)",
        "config": {"workload": f"KHI {n}^2 on [0,1)^2, CFL 0.4, dealias, RK4; alone and {nb} solves per plan"},
        "alone": out["alone"], "batch": out["batch"],
        "batch_over_alone_per_cell": out["batch"]["cell_updates_per_s"] / out["alone"]["cell_updates_per_s"],
        "peak_gbs": peak, "peak_source": src,
    }
    print(json.dumps(line), flush=True)


def run_mhd3d(args):
    """3D ideal MHD: the circularly polarized Alfven wave along x (the
    reference's alfven3d problem) on --mhd3d-n^3, gamma = 5/3, filter p = 8,
    alpha = 36, fixed dt = 1e-3 RK4 with per-stage clamp and 3D projection:
    cell-updates/s, per-kind launch times against the measured HBM peak, and
    one float64 oracle step on the host cores as the CPU baseline."""
    import torch
    from oracle import mhd as M
    from phrike_gb300 import _build, problems
    from phrike_gb300.engine import Plan

    _build.build()
    device = torch.device("cuda", 0)
    n = args.mhd3d_n
    fp = {"enabled": True, "p": 8, "alpha": 36.0}
    U0 = problems.alfven_cp_3d(n, n, n, 1.0)
    plan = Plan((n, n, n), (1.0, 1.0, 1.0), gamma=5.0 / 3.0, filter_params=fp, device=device, equations="mhd")
    U = torch.as_tensor(U0, dtype=torch.float32, device=device).contiguous()
    plan.project_state_(U)
    plan.run_(U, args.warmup, 1e-3)
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    st = torch.cuda.current_stream(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = max(1, min(args.steps, 50))
    e0.record(st)
    plan.run_(U, steps, 1e-3)
    e1.record(st)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / steps
    plan.profile(True)
    plan.run_(U, 2, 1e-3)
    prof = plan.collect_profile()
    plan.profile(False)
    peak, src = hbm_peak()
    kinds, total_bytes = {}, 0.0
    for k, v in prof.items():
        per = v["ms"] / v["launches"]
        total_bytes += v["bytes"] / 2
        kinds[k] = {"launches_per_step": v["launches"] / 2, "us_per_launch": per * 1e3,
                    "gbs": v["bytes"] / v["launches"] / (per * 1e-3) / 1e9,
                    "frac_of_peak": v["bytes"] / v["launches"] / (per * 1e-3) / 1e9 / peak}
    cn = min(n, 64)  # CPU baseline: one float64 oracle step at a bounded size
    s = M.MHDSolver3D(cn, cn, cn, 1.0, 1.0, 1.0, gamma=5.0 / 3.0, filter_params=fp)
    R = s.project(problems.alfven_cp_3d(cn, cn, cn, 1.0))
    t0 = time.perf_counter()
    R = s.step(R, 1e-3)
    cpu_s = time.perf_counter() - t0
    G = U.cpu().numpy()
    line = {
        "metric": "3D ideal MHD Alfven wave: cell-updates/s (RK4, per-stage 3D projection)",
        "value": n ** 3 / (ms * 1e-3), "unit": "cell-updates/s", "n_gpus": 1, "steps": steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "dtype": "f32",
        "data": "synthetic (analytic circularly polarized Alfven wave)",
        "config": {"workload": f"Alfven 3D {n}^3, gamma 5/3, filter p=8 alpha=36, RK4 dt=1e-3"},
        "passes": kinds, "step_GBps": total_bytes / (ms * 1e-3) / 1e9, "peak_gbs": peak, "peak_source": src,
        "cpu_baseline": {"value": cn ** 3 / cpu_s, "unit": "cell-updates/s", "cores": os.cpu_count(),
                         "kind": "port", "sample": f"1 RK4 step of the float64 oracle at {cn}^3"},
        "state_finite": bool(np.isfinite(G).all()), "status": plan.status(), "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_tracers(args):
    """Tracer advection (FourierTracers3D.step) with the reference's turb3d
    tracer block: 262,144 tracers (64^3 uniform layout) on a 64^3 TGV state,
    one leap-frog step per call with the spectral interpolation of the
    velocity: tracer-steps/s, against the float64 oracle's evaluation of a
    bounded sample of the tracers on the host cores."""
    import torch
    from oracle import tracers as OT
    from phrike_gb300 import _build, problems
    from phrike_gb300.grid import Grid3D
    from phrike_gb300.tracers import tracers_from_config

    _build.build()
    n, num = args.tracer_n, args.tracer_num
    L = 2 * np.pi
    g = Grid3D(Nx=n, Ny=n, Nz=n, Lx=L, Ly=L, Lz=L)
    U0 = problems.taylor_green_3d(n)
    U = torch.as_tensor(U0, dtype=torch.float32, device="cuda").contiguous()
    tr = tracers_from_config(g, {"enabled": True, "num": num, "layout": "uniform", "seed": 42})
    for _ in range(args.warmup):
        tr.step(g, None, U, 1e-3)
    torch.cuda.synchronize()
    steps = max(1, min(args.steps, 20))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        tr.step(g, None, U, 1e-3)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    # the same step with the exact interpolant (the automatic choice above is
    # the NUFFT here: tracers x cells > 2^24), and the two methods' velocities
    # at the same positions
    pos = torch.stack([tr.x, tr.y, tr.z]).contiguous()
    vel = {}
    for method in ("nufft", "exact"):
        g.plan.tracer_method(method)
        vel[method] = g.plan.eval_points(torch.stack([U[1] / U[0], U[2] / U[0], U[3] / U[0]]).contiguous(), pos)
    nu_dev = float(torch.linalg.norm(vel["nufft"] - vel["exact"]) / torch.linalg.norm(vel["exact"]))
    xsteps = 2
    e0.record()
    for _ in range(xsteps):
        tr.step(g, None, U, 1e-3)
    e1.record()
    torch.cuda.synchronize()
    ms_exact = e0.elapsed_time(e1) / xsteps
    g.plan.tracer_method("auto")
    # CPU: the oracle's interpolation of 64 tracers' velocities (3 components)
    sample = 64
    pos = [tr.x[:sample].cpu().numpy(), tr.y[:sample].cpu().numpy(), tr.z[:sample].cpu().numpy()]
    t0 = time.perf_counter()
    for a in range(3):
        OT.eval_points(U0[1 + a] / U0[0], pos, (L, L, L), True, None)
    cpu_s = time.perf_counter() - t0
    line = {
        "metric": "tracer steps/s (spectral velocity interpolation + leap-frog)", "value": num / (ms * 1e-3),
        "unit": "tracer-steps/s", "n_gpus": 1, "steps": steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "dtype": "f32 fields, f64 positions", "data": "synthetic (TGV state, uniform tracers)",
        "config": {"workload": f"{num} tracers on a {n}^3 TGV state (turb3d tracer block)",
                   "interpolation": "NUFFT (exponential-of-semicircle kernel, 8 points per axis, 2x oversampling)"},
        "ms_per_step_exact_interpolant": ms_exact, "nufft_vs_exact_rel_l2": nu_dev,
        "cpu_baseline": {"value": sample / cpu_s, "unit": "tracer-steps/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": f"velocity of {sample} tracers by the float64 oracle (exact interpolant)"},
    }
    print(json.dumps(line), flush=True)


def run_sod(args):
    """The plain 1D workload: smoothed Sod step on [0, 1), N = 1024, gamma
    1.4, 2/3 dealiasing, exponential filter (p = 8, alpha = 36), RK4 with
    dt = 2e-5 for 1000 steps.  One solve runs whole steps in one CTA
    (k_step1d, state in shared memory); a batch of --nsolve independent solves
    fills the GPU.  cell-updates/s for both, relative L2 per field of the
    single solve against the float64 oracle (from the same float32 input), and
    the oracle's own rate on the host cores (the CPU baseline)."""
    import torch
    from oracle import spectral as O
    from phrike_gb300 import _build, problems
    from phrike_gb300.engine import Plan

    _build.build()
    device = torch.device("cuda", 0)
    N, dt, nsteps = 1024, 2e-5, 1000
    fp = {"enabled": True, "p": 8, "alpha": 36.0}
    U0 = problems.sod_smoothed(N)
    st = torch.cuda.current_stream(device)
    out = {}
    for ns in (1, max(1, args.nsolve)):
        plan = Plan((N,), (1.0,), filter_params=fp, device=device, nsolve=ns)
        base = np.stack([U0] * ns) if ns > 1 else U0
        U = torch.as_tensor(base, dtype=torch.float32, device=device).contiguous()
        plan.run_(U.clone(), max(args.warmup, 3), dt)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        plan.run_(U, nsteps, dt)
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        out[ns] = {"ms": ms, "cell_updates_per_s": ns * N * nsteps / (ms * 1e-3)}
        if ns == 1:
            G = U.double().cpu().numpy()
        plan.close()
    s = O.EulerSolver(O.FourierBox((N,), (1.0,), dealias=True, filter_enabled=True))
    R = U0.astype(np.float32).astype(np.float64)
    t0 = time.perf_counter()
    for _ in range(nsteps):
        R = s.step(R, dt)
    cpu_s = time.perf_counter() - t0
    err = {k: float(np.linalg.norm(G[c] - R[c]) / np.linalg.norm(R[c])) for c, k in enumerate(("rho", "mom", "E"))}
    ns = max(1, args.nsolve)
    line = {
        "metric": "1D Sod cell-updates/s (plain single solve and a batch)", "value": out[1]["cell_updates_per_s"],
        "unit": "cell-updates/s", "n_gpus": 1, "steps": nsteps, "higher_is_better": True, "dtype": "f32",
        "data": "synthetic (smoothed Sod step, tanh width 0.005)",
        "config": {"workload": f"1D Sod N={N}, RK4 dt={dt}, {nsteps} steps, dealias, filter p=8 alpha=36"},
        "ms_single": out[1]["ms"], f"batch_{ns}_cell_updates_per_s": out[ns]["cell_updates_per_s"],
        "rel_l2_vs_oracle": err,
        "cpu_baseline": {"value": N * nsteps / cpu_s, "unit": "cell-updates/s", "cores": os.cpu_count() or 1,
                         "kind": "port", "sample": f"{nsteps} steps of the float64 oracle ({cpu_s:.1f} s)"},
    }
    print(json.dumps(line), flush=True)


def run_khi4k(args):
    """The reference's largest shipped grid: configs/khi2d_4k.yaml, the khi2d
    problem on 3840 x 2160 (Lx = 16/9, Ly = 1; axes 2^8 3 5 and 2^4 3^3 5,
    the mixed-radix passes), gamma 1.4, 2/3 dealiasing, filter p = 8,
    alpha = 36 every step, RK4 at the initial CFL step (CFL 0.25).
    cell-updates/s, per-pass launch times against the measured HBM peak, and
    one float64 oracle step on the host cores as the CPU baseline."""
    import torch
    from oracle import spectral as O
    from phrike_gb300 import _build
    from phrike_gb300 import problem_ics as IC
    from phrike_gb300.engine import Plan

    _build.build()
    device = torch.device("cuda", 0)
    nx, ny, lx, ly = 3840, 2160, 1.77777777777777778, 1.0
    cfg = {"initial_conditions": {"rho_outer": 1.0, "rho_inner": 2.0, "u0": 1.0, "shear_thickness": 0.02,
                                  "pressure_outer": 1.0, "pressure_inner": 1.0, "perturb_eps": 0.01,
                                  "perturb_sigma": 0.02, "perturb_kx": 2}}
    x = np.linspace(0.0, lx, nx, endpoint=False)
    y = np.linspace(0.0, ly, ny, endpoint=False)
    U0 = IC.build("khi2d", cfg, 1.4, x, y, lengths=(lx, ly))
    fp = {"enabled": True, "p": 8, "alpha": 36.0}
    plan = Plan((ny, nx), (ly, lx), filter_params=fp, cfl=0.25, device=device)
    U = torch.as_tensor(U0, dtype=torch.float32, device=device).contiguous()
    dt = 0.25 * min(lx / nx, ly / ny) / float(plan.max_wave_speed(U)[0].item())
    plan.run_(U, max(args.warmup, 3), dt)
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    st = torch.cuda.current_stream(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    plan.run_(U, args.steps, dt)
    e1.record(st)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    plan.profile(True)
    plan.run_(U, 3, dt)
    prof = plan.collect_profile()
    plan.profile(False)
    peak, src = hbm_peak()
    kinds = {}
    for k, v in prof.items():
        per = v["ms"] / v["launches"]
        kinds[k] = {"launches_per_step": v["launches"] / 3, "us_per_launch": per * 1e3,
                    "gbs": v["bytes"] / v["launches"] / (per * 1e-3) / 1e9,
                    "frac_of_peak": v["bytes"] / v["launches"] / (per * 1e-3) / 1e9 / peak}
    cpu = None
    if not args.no_cpu_baseline:
        s = O.EulerSolver(O.FourierBox((ny, nx), (ly, lx), dealias=True, filter_enabled=True), cfl=0.25, fused=True)
        R = U0.astype(np.float32).astype(np.float64)
        t0 = time.perf_counter()
        R = s.step(R, dt)
        cpu_s = time.perf_counter() - t0
        cpu = {"value": nx * ny / cpu_s, "unit": "cell-updates/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"1 RK4 step of the float64 oracle (fused spectral sums) at {nx}x{ny} ({cpu_s:.1f} s)"}
    G = U.cpu().numpy()
    line = {
        "metric": "2D Euler KHI on the khi2d_4k grid: cell-updates/s (RK4, filter every step)",
        "value": nx * ny / (ms * 1e-3), "unit": "cell-updates/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "dtype": "f32",
        "data": "synthetic (the khi2d problem's analytic initial state)",
        "config": {"workload": f"khi2d {nx}x{ny} (configs/khi2d_4k.yaml), dealias, filter p=8 alpha=36, "
                               f"RK4 dt={dt:.4g}", "l2": "inputs larger than L2 (8.3M cells x 20 fields)"},
        "passes": kinds, "peak_gbs": peak, "peak_source": src, "cpu_baseline": cpu,
        "state_finite": bool(np.isfinite(G).all()), "status": plan.status(), "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def validation_report(device, tgv_n=64, tgv_steps=50, drift_n=256, drift_steps=200):
    """Accuracy figures of the plain form against the float64 oracle:
    (1) relative L2 error per conserved field of the 3D TGV after fixed-dt
        RK4 steps (both from the float32-rounded initial state);
    (2) mass / momentum / energy drift of the 256^3 TGV over 200 steps (the
        reference's plain sums);
    (3) spectral convergence: the masked derivative of f = 1/(1.5 + cos 2 pi x)
        (Fourier coefficients ~ 0.382^|k|) at N = 8..128, with the slope of
        ln(error) per grid point from N = 16 to 32 (the 2/3 mask keeps
        |k| <= N/3: asymptotic slope ln(0.382)/3 = -0.321);
    (4) RK4 temporal order: the circularly polarized Alfven wave (m = 2,
        N = 32, t = 1, filter off) through the 1D MHD kernel at dt = 0.02,
        0.01, 0.005 against the exact solution."""
    import torch
    from oracle import mhd as M
    from oracle import spectral as O
    from phrike_gb300 import problems
    from phrike_gb300.engine import Plan

    def rl(a, b):
        return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))

    out = {}
    n = tgv_n
    U0 = problems.taylor_green_3d(n).astype(np.float32).astype(np.float64)
    plan = Plan((n, n, n), (2 * np.pi,) * 3, device=device)
    U = torch.as_tensor(U0, dtype=torch.float32, device=device)
    plan.run_(U, tgv_steps, 1e-3)
    s = O.EulerSolver(O.FourierBox((n, n, n), (2 * np.pi,) * 3, dealias=True), cfl=0.25)
    R = U0.copy()
    for _ in range(tgv_steps):
        R = s.step(R, 1e-3)
    G = U.double().cpu().numpy()
    out["tgv_rel_l2"] = {"n": n, "steps": tgv_steps, "dt": 1e-3, "rho": rl(G[0], R[0]), "mom": rl(G[1:4], R[1:4]),
                         "E": rl(G[4], R[4])}
    n = drift_n
    plan = Plan((n, n, n), (2 * np.pi,) * 3, device=device)
    U = torch.as_tensor(problems.taylor_green_3d(n), dtype=torch.float32, device=device)
    c0 = plan.conserved(U).double().cpu().numpy().reshape(-1)
    plan.run_(U, drift_steps, 1e-3)
    c1 = plan.conserved(U).double().cpu().numpy().reshape(-1)
    scale = [abs(c0[0]), float(np.linalg.norm(c0[1:4])) + abs(c0[0]), abs(c0[4])]
    out["tgv_drift"] = {"n": n, "steps": drift_steps, "mass": abs(c1[0] - c0[0]) / scale[0],
                        "momentum": float(np.linalg.norm(c1[1:4] - c0[1:4])) / scale[1],
                        "energy": abs(c1[4] - c0[4]) / scale[2]}
    conv = {}
    for N in (8, 16, 32, 64, 128):
        x = np.arange(N) / N
        f = 1.0 / (1.5 + np.cos(2 * np.pi * x))
        df = 2 * np.pi * np.sin(2 * np.pi * x) / (1.5 + np.cos(2 * np.pi * x)) ** 2
        p1 = Plan((N,), (1.0,), device=device)
        d = p1.derivative(torch.as_tensor(f, dtype=torch.float32, device=device).reshape(1, N), 0)
        ref = O.FourierBox((N,), (1.0,), dealias=True).deriv(f, 0)
        conv[N] = {"gpu": rl(d.double().cpu().numpy().reshape(-1), df), "oracle": rl(ref, df)}
    slope = {k: float(np.log(conv[32][k] / conv[16][k]) / 16.0) for k in ("gpu", "oracle")}
    out["spectral_convergence"] = {"errors": conv, "slope_16_32": slope, "asymptotic_slope": float(np.log(1.5 - np.sqrt(1.25)) / 3)}
    errs = []
    for dt in (0.02, 0.01, 0.005):
        p1 = Plan((32,), (1.0,), gamma=5.0 / 3.0, device=device, equations="mhd")
        V = torch.as_tensor(problems.alfven_cp_1d(32, m=2), dtype=torch.float32, device=device).contiguous()
        p1.project_state_(V)
        p1.run_(V, int(round(1.0 / dt)), dt)
        ex = problems.alfven_cp_1d(32, t=1.0, m=2)
        errs.append(rl(V.double().cpu().numpy()[6:8], ex[6:8]))
    so = M.MHDSolver1D(32, 1.0, gamma=5.0 / 3.0)
    oerr = []
    for dt in (0.02, 0.01):
        W = so.project(problems.alfven_cp_1d(32, m=2))
        for _ in range(int(round(1.0 / dt))):
            W = so.step(W, dt)
        oerr.append(rl(W[6:8], problems.alfven_cp_1d(32, t=1.0, m=2)[6:8]))
    out["rk4_order"] = {"dt": [0.02, 0.01, 0.005], "gpu_errors": errs,
                        "gpu_orders": [float(np.log2(errs[i] / errs[i + 1])) for i in range(2)],
                        "oracle_errors": oerr, "oracle_order": float(np.log2(oerr[0] / oerr[1]))}
    return out


def run_validation(args):
    import torch
    from phrike_gb300 import _build
    _build.build()
    rep = validation_report(torch.device("cuda", 0))
    print(json.dumps({"metric": "accuracy of the plain form against the float64 oracle", **rep}), flush=True)


def run_adaptive(args):
    """Adaptive embedded RK45 with the reference's shipped settings.
    (a) configs/sod.yaml: 1D Sod N=1024, rk45, rtol 1e-6, atol 1e-8,
        artificial viscosity (sensor, nu_max 1e-3), filter p=8 alpha=36, to
        t_end=0.2: a batch of --nsolve solves with every attempt loop and
        decision on the device (k_ark1d), against the float64 oracle run of
        one solve on the host cores.
    (b) configs/tgv3d.yaml: 3D TGV at --n^3, rk45, rtol 1e-5, atol 1e-7:
        ms per attempt and cell-updates/s per accepted step.
    Synthetic smoothed Sod (tanh edges) instead of the sharp step."""
    import torch
    from oracle import adaptive as A
    from oracle import spectral as O
    from phrike_gb300 import _build, problems
    from phrike_gb300.engine import Plan

    _build.build()
    device = torch.device("cuda", 0)
    f64 = dict(dtype=torch.float64, device=device)
    fp = {"enabled": True, "p": 8, "alpha": 36.0}
    av = {"enabled": True, "mode": "sensor", "nu_max": 1e-3, "s_ref": 1.0, "s_min": 0.1, "p": 2.0,
          "epsilon": 1e-12, "sensor_variable": "density"}
    N, t_end, ns = 1024, 0.2, args.nsolve
    plan = Plan((N,), (1.0,), filter_params=fp, cfl=0.4, av_config=av, device=device, nsolve=ns)
    ad = Plan.adaptive_desc({"scheme": "rk45", "rtol": 1e-6, "atol": 1e-8})
    U0 = problems.sod_smoothed(N)
    # a seeded spread of initial states so the solves take different step sequences
    rng = np.random.default_rng(20261203)
    amps = 1.0 + 0.2 * rng.random(ns)
    base = np.stack([U0 * a for a in amps])
    s1 = O.EulerSolver(O.FourierBox((N,), (1.0,), dealias=True, filter_enabled=True), cfl=0.4, av=av)
    dt0 = np.array([s1.compute_dt(base[i]) for i in range(ns)])

    def fresh():
        U = torch.as_tensor(base, dtype=torch.float32, device=device).contiguous()
        return (U, torch.zeros(ns, **f64), torch.full((ns,), t_end, **f64), torch.as_tensor(dt0, **f64),
                torch.zeros((ns, 2), dtype=torch.int32, device=device))

    U, t, te, dtv, cnt = fresh()
    plan.run_adaptive_(U, 100000, ad, t, te, dtv, None, cnt)  # warm-up run (also builds the slope storage)
    torch.cuda.synchronize()
    U, t, te, dtv, cnt = fresh()
    plan.adaptive_reset()
    sampler = ClockSampler(0)
    sampler.start()
    st = torch.cuda.current_stream(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    plan.run_adaptive_(U, 100000, ad, t, te, dtv, None, cnt)
    e1.record(st)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    sec = e0.elapsed_time(e1) * 1e-3
    c = cnt.cpu().numpy()
    done = bool((t.cpu().numpy() >= t_end - 1e-12).all())
    # CPU baseline: the float64 oracle's adaptive run of solve 0, bounded
    cpu = None
    if not args.no_cpu_baseline:
        rhs, post = A.euler_hooks(s1)
        t0 = time.perf_counter()
        _, tc, log, _, _ = A.run_adaptive(rhs, post, base[0], 0.0, t_end, dt0[0], "rk45", A.Controller(),
                                          max_attempts=200)
        cs = time.perf_counter() - t0
        per_attempt = cs / max(len(log), 1)
        cpu = {"value": 1.0 / (per_attempt * (int(c[0].sum()))), "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": f"{len(log)} attempts of solve 0 with the float64 oracle ({cs:.1f} s), scaled to its "
                         f"{int(c[0].sum())} attempts"}
    line1 = {
        "metric": "adaptive RK45 1D Sod solves/s (decisions on the device)", "value": ns / sec, "unit": "solves/s",
        "n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic (smoothed Sod, seeded amplitudes)",
        "config": {"workload": f"{ns} x Sod N={N}, rk45 rtol 1e-6 atol 1e-8, AV sensor nu_max 1e-3, "
                               f"filter p=8 alpha=36, t_end={t_end}"},
        "seconds": sec, "attempts_per_solve": float(c.sum(axis=1).mean()),
        "accepted_per_solve": float(c[:, 0].mean()), "rejected_per_solve": float(c[:, 1].mean()),
        "all_finished": done, "state_finite": bool(torch.isfinite(U).all().item()), "cpu_baseline": cpu,
        "clocks": clocks, "gpu_launches": 1,
    }
    print(json.dumps(line1), flush=True)

    # (b) 3D TGV
    n = args.n
    plan3 = Plan((n, n, n), (2 * np.pi,) * 3, cfl=0.25, device=device)
    ad3 = Plan.adaptive_desc({"scheme": "rk45", "rtol": 1e-5, "atol": 1e-7})
    T0 = torch.as_tensor(problems.taylor_green_3d(n), dtype=torch.float32, device=device).contiguous()
    dt3 = float(plan3.max_wave_speed(T0).item())
    dt3 = 0.25 * (2 * np.pi / n) / dt3
    T = T0.clone()
    t, te, dtv = torch.zeros(1, **f64), torch.full((1,), 1e9, **f64), torch.full((1,), dt3, **f64)
    cnt = torch.zeros((1, 2), dtype=torch.int32, device=device)
    plan3.run_adaptive_(T, max(args.warmup, 3), ad3, t, te, dtv, None, cnt)
    torch.cuda.synchronize()
    c0 = cnt.clone()
    K = max(args.steps // 10, 5)
    e0.record(st)
    plan3.run_adaptive_(T, K, ad3, t, te, dtv, None, cnt)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / K
    acc = int((cnt - c0)[0, 0].item())
    line2 = {
        "metric": "adaptive RK45 3D TGV: cell-updates/s per accepted step", "value": n ** 3 * acc / (ms * K * 1e-3),
        "unit": "cell-updates/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32",
        "data": "synthetic (analytic Taylor-Green initial condition)",
        "config": {"workload": f"TGV {n}^3, rk45 rtol 1e-5 atol 1e-7 (7 stages, FSAL not used, as the reference)"},
        "ms_per_attempt": ms, "attempts": K, "accepted": acc, "status": plan3.status(),
        "state_finite": bool(torch.isfinite(T).all().item()),
    }
    print(json.dumps(line2), flush=True)


def run_serving(args):
    """Serving: a seeded Poisson stream (200 requests/s) mixing Sod 1D,
    KHI 2D, Orszag-Tang MHD, TGV 3D and LGL acoustic solves with t_end ~
    U[0.1, 1.0], served with continuous batching (phrike_gb300.serving).
    The plain form serves the same stream one solve at a time, first come
    first served, each solve alone on its own plan; its service times come
    from one alone run per (family, size) to t_end = --plain-t-end, scaled
    linearly with each request's t_end (CFL steps of near-constant size).
    The served run gives groups whose solves cost at least 5 s per unit time
    alone a high-priority stream."""
    import torch
    from phrike_gb300 import _build
    from phrike_gb300.serving import Request, Server, request_stream, run_alone

    _build.build()
    device = torch.device("cuda", 0)
    reqs = request_stream(args.requests, rate=200.0)
    # warm-up: one short request per (family, size) on a separate server with
    # the same group shapes, so that lazy kernel loading stays out of the timed run
    keys = sorted({(r.family, r.n) for r in reqs})
    Server(device, chunk=args.chunk, autotune=True).serve(
        [Request(-1 - i, f, n, 1e-4) for i, (f, n) in enumerate(keys)], realtime=False)
    torch.cuda.synchronize()
    # plain service times, one alone run per (family, size); they also give the
    # server its cost model (long solves on high-priority streams)
    rate = {}
    for key in sorted({(r.family, r.n) for r in reqs}):
        probe = Request(-1, key[0], key[1], args.plain_t_end)
        run_alone(probe, device, chunk=args.chunk)  # warm-up (plan, kernels)
        _, sec = run_alone(probe, device, chunk=args.chunk)
        rate[key] = sec / args.plain_t_end
    srv = Server(device, chunk=args.chunk, cost=lambda f, n: rate[(f, n)], autotune=True)
    sampler = ClockSampler(0)
    sampler.start()
    stats = srv.serve(reqs, realtime=True)
    clocks = sampler.stop()
    done, lat = 0.0, []
    for r in sorted(reqs, key=lambda q: q.arrival):
        start = max(r.arrival, done)
        done = start + rate[(r.family, r.n)] * r.t_end
        lat.append(done - r.arrival)
    lat = np.array(lat)
    plain_span = done - min(r.arrival for r in reqs)
    mix = {}
    for r in reqs:
        mix[f"{r.family}/{r.n}"] = mix.get(f"{r.family}/{r.n}", 0) + 1
    line = {
        "metric": "served solves/s and latency (continuous batching) vs plain one-at-a-time", "value":
        stats["solves_per_s"], "unit": "solves/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32",
        "data": "synthetic (seeded Poisson stream, analytic initial conditions)",
        "config": {"workload": f"{args.requests} requests at 200/s: sod1d, khi2d, ot2d, tgv3d, lgl2d, lgl1d; "
                               "t_end ~ U[0.1, 1.0]", "chunk_steps_per_graph": args.chunk},
        "latency_s": {"p50": stats["latency_p50"], "p95": stats["latency_p95"], "p99": stats["latency_p99"]},
        "seconds": stats["seconds"], "max_live_slots": stats["max_live_slots"], "groups": stats["groups"],
        "hbm_bytes": stats["hbm_bytes"], "status": stats["status"],
        "plain": {"solves_per_s": len(reqs) / plain_span,
                  "latency_s": {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                                "p99": float(np.percentile(lat, 99))},
                  "seconds_per_unit_time": {f"{k[0]}/{k[1]}": v for k, v in rate.items()}},
        "speedup_solves_per_s": stats["solves_per_s"] / (len(reqs) / plain_span),
        "mix": mix, "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", choices=["tgv", "ensemble", "lgl", "serving", "ot", "adaptive", "mhd3d",
                                           "tracers", "validation", "sod", "khi4k", "khi"], default="tgv")
    ap.add_argument("--requests", type=int, default=100)
    ap.add_argument("--plain-t-end", type=float, default=0.05)
    ap.add_argument("--lgl-sizes", default="257,513")
    ap.add_argument("--lgl-steps", type=int, default=500)
    ap.add_argument("--lgl-batch", type=int, default=16)
    ap.add_argument("--nsolve", type=int, default=512)
    ap.add_argument("--t-end", type=float, default=1.0)
    ap.add_argument("--chunk", type=int, default=50)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--n", "--size", dest="n", type=int, default=256)  # --size: unambiguous under torchrun
    ap.add_argument("--ot-n", type=int, default=512)
    ap.add_argument("--khi-n", type=int, default=512)
    ap.add_argument("--khi-batch", type=int, default=16)
    ap.add_argument("--mhd3d-n", type=int, default=128)
    ap.add_argument("--tracer-n", type=int, default=64)
    ap.add_argument("--tracer-num", type=int, default=262144)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ensemble-sample", action="store_true")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            import torch
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend=backend)
    try:
        if args.workload == "ensemble":
            run_ensemble(args, rank, world)
        elif args.workload == "lgl":
            if rank == 0:
                run_lgl(args)
        elif args.workload == "serving":
            if rank == 0:
                run_serving(args)
        elif args.workload == "ot":
            if rank == 0:
                run_ot(args)
        elif args.workload == "adaptive":
            if rank == 0:
                run_adaptive(args)
        elif args.workload == "mhd3d":
            if rank == 0:
                run_mhd3d(args)
        elif args.workload == "tracers":
            if rank == 0:
                run_tracers(args)
        elif args.workload == "validation":
            if rank == 0:
                run_validation(args)
        elif args.workload == "sod":
            if rank == 0:
                run_sod(args)
        elif args.workload == "khi4k":
            if rank == 0:
                run_khi4k(args)
        elif args.workload == "khi":
            if rank == 0:
                run_khi(args)
        elif args.impl == "reference":
            run_reference(args, rank, world)
        else:
            run_gb300(args, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
