"""Benchmark of the DG RHS / RK4 time-step path on GB300.

Workload (default): the density-wave Euler case -- [0,1]^2 periodic, 2 x 1024^2
= 2,097,152 triangles jittered by +-0.15h (seeded), Dubiner-order p = 3
(n_p = 10), 4 conserved variables in FP32, LLF flux, classic RK4 with the
reference's CFL rule (dt = 0.7 min diameter / max wave speed / (2p+1)) computed
on the device each step.  One "step" is one full RK4 time step (CFL reduction
plus four fused stage kernels); one DOF-update is one coefficient (element x
mode x variable) advanced by one step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  ``--impl reference`` times the reference's own CPU
Euler loops (built from its sources by oracle/Makefile; one serial process per
host core) on a bounded sample of the same workload -- or, without the
reference's sources, the CPU restatement in oracle/ -- and adds its CUDA solver
rebuilt for sm_103a on the full workload (``reference_gpu``).  Under torchrun (N > 1) every rank runs
an independent replica of the solve (the path has no data exchange between
solves) and value is the sum over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DOF-updates/s on 1 GB300, served/batched vs plain at L2≤1e-5; p50/p99 latency"
UNIT = "DOF-updates/s"
def workload(n: int, precision: str = "fp32") -> dict:
    """Labels of the density-wave workload on the 2 x n^2 mesh, computed in
    `precision` (the arithmetic of the arm that reports it)."""
    mb = 2 * n * n * 40 * 4 / 1e6
    return dict(workload=f"euler_density_wave_2x{n}^2_p3", equation="euler", order=3,
                num_elem=2 * n * n, mesh=f"periodic 2x{n}^2, jitter 0.15h, seed 12347",
                ic="rho=1+0.2 sin(2pi(x+y)), u=v=1, p=1, gamma=1.4", flux="LLF",
                integrator="RK4, CFL 0.7 on device", precision=precision,
                l2_flush=f"inputs larger than L2 (4 state vectors x {mb:.1f} MB)" if 4 * mb > 129
                else f"inputs of 4 x {mb:.1f} MB (not larger than L2)")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples (SM clock, reasons) taken while the bench runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0, period_ms: int = 100):
        self.samples = []
        self.proc = None
        self.index = index
        self.period = period_ms

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", f"-lms={self.period}"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), [x.strip() for x in line.split(",")]))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0: float, t1: float):
        win = [s for (t, s) in self.samples if t0 - 0.15 <= t <= t1 + 0.15]
        if not win:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(s[1]) for s in win if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in win if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in win for i in range(4) if len(s) > 5 + i and s[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(win)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("DGX_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend=backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def build_mesh(n: int):
    from dgcuda_gb300.mesh import periodic_square
    return periodic_square(n, jitter=0.15, seed=12347)


def run_reference(args, rank, world):
    """The reference's own implementations of the path, timed on this machine: its
    CPU Euler loops (src/2d/conservation/euler/cpu, built from the reference's
    sources by oracle/Makefile, serial, one process per host core on a bounded
    sub-problem) give `value`; its CUDA Euler solver rebuilt for sm_103a
    (oracle/ref_gpu_harness.cu around the reference's time_integrate_rk4) runs a
    few steps of the full workload on the GPU (`reference_gpu`).  Without the
    reference's sources the CPU figure falls back to the oracle port."""
    if rank != 0:
        return None
    from oracle import oracle as orc
    orc.build()
    wave = (0.2, 1.0, 1.0, 1.0, 1.0)
    out = {"metric": METRIC, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic", "config": workload(args.mesh_n, "fp64"), "impl": "reference"}
    if orc.build_ref() is not None:
        cores = os.cpu_count() or 1
        # size each process's sub-problem so that the timed steps take about a minute
        probe = build_mesh(16)
        po = orc.Oracle(probe, 3, orc.EULER, orc.LLF, 1.4)
        pc = po.project(orc.IC_DENSITY_WAVE, wave)
        per_elem = orc.time_ref_cpu(probe, 3, pc, po.cfl_dt(pc), 4)[0] / (4 * probe.num_elem)
        n_sample = 8
        for n in (256, 128, 64, 32, 16, 8):
            if per_elem * 2 * n * n * args.steps <= 60.0:
                n_sample = n
                break
        mesh = build_mesh(n_sample)
        o = orc.Oracle(mesh, 3, orc.EULER, orc.LLF, 1.4)
        c = o.project(orc.IC_DENSITY_WAVE, wave)
        secs = orc.time_ref_cpu(mesh, 3, c, o.cfl_dt(c), args.steps, procs=cores)
        dofs = 4 * 10 * mesh.num_elem
        el = max(secs)
        value = cores * dofs * args.steps / el
        kind = "reference"
        sample = (f"{args.steps} RK4 steps of the reference's own CPU Euler loops (serial FP64 C, "
                  f"built from its sources) on a 2x{n_sample}^2 periodic sub-problem ({mesh.num_elem} "
                  f"elements, p=3 density wave) of the 2x1024^2 workload, in {cores} processes side by "
                  f"side (one per host core)")
    else:
        cores = orc.set_threads(os.cpu_count() or 1)
        # size the per-step sample so that warm-up + timed steps take about two minutes
        probe = build_mesh(64)
        po = orc.Oracle(probe, 3, orc.EULER, orc.LLF, 1.4)
        pc = po.project(orc.IC_DENSITY_WAVE, wave)
        po.step(pc, po.cfl_dt(pc))
        t0 = time.perf_counter()
        po.step(pc, po.cfl_dt(pc))
        per_elem = (time.perf_counter() - t0) / probe.num_elem
        n_sample = 32
        for n in (512, 256, 128, 64, 32):
            if per_elem * 2 * n * n * (args.steps + args.warmup) <= 120.0:
                n_sample = n
                break
        mesh = build_mesh(n_sample)
        o = orc.Oracle(mesh, 3, orc.EULER, orc.LLF, 1.4)
        c = o.project(orc.IC_DENSITY_WAVE, wave)
        dofs = 4 * 10 * mesh.num_elem
        for _ in range(args.warmup):
            c = o.step(c, o.cfl_dt(c))
        t0 = time.perf_counter()
        for _ in range(args.steps):
            c = o.step(c, o.cfl_dt(c))
        el = time.perf_counter() - t0
        value = dofs * args.steps / el
        kind = "port"
        sample = (f"{args.steps} RK4 steps of the same scheme (p=3 Euler, LLF, CFL) on a 2x{n_sample}^2 "
                  f"periodic sub-problem ({mesh.num_elem} elements) of the 2x1024^2 workload, FP64")
    out.update({"value": value, "ms_per_step": 1e3 * el / args.steps,
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
    out["reference_gpu"] = run_reference_gpu(args.mesh_n)
    return out


def run_reference_gpu(mesh_n: int, steps: int = 3):
    """The reference's CUDA Euler solver (FP64, its own kernels and host loop,
    rebuilt for sm_103a) on the full workload: `steps` steps of its
    time_integrate_rk4 to an end time of `steps` CFL time steps."""
    try:
        import torch
        if not torch.cuda.is_available():
            return {"unavailable": "no GPU"}
        from oracle import ref_gpu
        if ref_gpu.build() is None:
            return {"unavailable": "the reference's CUDA sources are not at hand to build its solver"}
        from oracle import oracle as orc
        mesh = build_mesh(mesh_n)
        o = orc.Oracle(mesh, 3, orc.EULER, orc.LLF, 1.4)
        c0 = o.project(orc.IC_DENSITY_WAVE, (0.2, 1.0, 1.0, 1.0, 1.0))
        dt = o.cfl_dt(c0)
        r = ref_gpu.run(mesh, 3, c0, steps * dt * 0.999)
        dofs = 4 * 10 * mesh.num_elem
        return {"value": dofs * r["steps"] / r["seconds"], "unit": UNIT, "steps": r["steps"],
                "ms_per_step": 1e3 * r["seconds"] / r["steps"], "dtype": "f64",
                "what": "the reference's own CUDA kernels and RK4 host loop (time_integrate_rk4) rebuilt "
                        f"for sm_103a, 2x{mesh_n}^2 density wave p=3, wall time of the loop"}
    except Exception as exc:  # reported, never fatal to the bench line
        return {"unavailable": f"{type(exc).__name__}: {exc}"[:300]}


def cpu_baseline_sample(budget_s: float = 12.0):
    from oracle import oracle as orc
    orc.build()
    cores = orc.set_threads(os.cpu_count() or 1)
    mesh = build_mesh(512)               # 2 x 512^2 = 524,288 elements
    o = orc.Oracle(mesh, 3, orc.EULER, orc.LLF, 1.4)
    c = o.project(orc.IC_DENSITY_WAVE, (0.2, 1.0, 1.0, 1.0, 1.0))
    dofs = 4 * 10 * mesh.num_elem
    steps, t0 = 0, time.perf_counter()
    while True:
        c = o.step(c, o.cfl_dt(c))
        steps += 1
        el = time.perf_counter() - t0
        if el > budget_s or steps >= 20:
            break
    return {"value": dofs * steps / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{steps} RK4 steps of the oracle (FP64 C restatement, OpenMP) on a 2x512^2 "
                      f"periodic sub-problem ({mesh.num_elem} elements, p=3 Euler)"}


def _config4_requests(seed: int, count: int, n_lo: int, n_hi: int):
    """Solve specs drawn as in the batched configuration: equation 50/50, N
    log-uniform in [n_lo, n_hi] (2N^2 triangles, jitter 0.15h), p uniform in
    1..4, Gaussian pulses (width 0.05-0.2) for advection on [0,1]^2, isentropic
    vortices (beta 1-5) for Euler on [0,10]^2, at random centres."""
    from dgcuda_gb300 import _ffi
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        euler = rng.random() < 0.5
        n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        p = int(rng.integers(1, 5))
        if euler:
            params = (rng.uniform(0, 10), rng.uniform(0, 10), rng.uniform(1, 5), 1.0, 0.0, 10.0, 10.0)
            out.append(dict(n=n, order=p, equation=_ffi.EULER, ic=_ffi.IC_VORTEX, params=params,
                            lx=10.0, ly=10.0, jitter=0.15, seed=seed * 1000 + k))
        else:
            w = rng.uniform(0.05, 0.2)
            params = (rng.uniform(0, 1), rng.uniform(0, 1), w * w, 1.0, 1.0)
            out.append(dict(n=n, order=p, equation=_ffi.ADVECTION, ic=_ffi.IC_GAUSSIAN,
                            params=params, lx=1.0, ly=1.0, jitter=0.15, seed=seed * 1000 + k))
    return out


def _native_solver(spec, precision=None):
    from dgcuda_gb300 import _ffi
    from dgcuda_gb300.solver import DeviceMesh, Solver
    dm = DeviceMesh.periodic_square(spec["n"], spec["lx"], spec["ly"], spec["jitter"], spec["seed"])
    sv = Solver(dm, spec["order"], spec["equation"], _ffi.FLUX_LLF,
                _ffi.FP32 if precision is None else precision, 1.4)
    sv.project(spec["ic"], spec["params"])
    sv.set_dt(None, cfl=0.7)
    return sv


def run_accuracy(mesh_n: int, steps: int = 100, precision=None):
    """Config-3 accuracy: the FP32 path and the FP64 path on the same mesh and
    initial state for `steps` RK4 steps with the same fixed dt (the FP32 run's
    first CFL dt); relative L2 per conserved variable of FP32 against FP64, and
    the FP32 run's drift of the conserved totals (FP64 reductions).  The FP64
    path stands in for the FP64 oracle at this size: tests/test_gpu_parity.py
    holds it to 1e-11 of the CPU oracle on smaller meshes."""
    from dgcuda_gb300 import _ffi
    from dgcuda_gb300.solver import DeviceMesh, Solver
    if precision is None:
        precision = _ffi.FP32
    dm = DeviceMesh.periodic_square(mesh_n, 1.0, 1.0, 0.15, 12347)
    res = {}
    for prec in (precision, _ffi.FP64):
        sv = Solver(dm, 3, _ffi.EULER, _ffi.FLUX_LLF, prec, 1.4)
        sv.project(_ffi.IC_DENSITY_WAVE, (0.2, 1.0, 1.0, 1.0, 1.0))
        res[prec] = sv
    s32, s64 = res[precision], res[_ffi.FP64]
    s32.set_dt(None)
    s32.run(max_steps=1)
    _, dt = s32.time()
    s32.project(_ffi.IC_DENSITY_WAVE, (0.2, 1.0, 1.0, 1.0, 1.0))
    s32.reset_time(0.0)
    t0 = s32.totals()
    for sv in (s32, s64):
        sv.set_dt(dt)
        sv.run(max_steps=steps)
    c32, c64 = s32.get_state(), s64.get_state()
    t1 = s32.totals()
    nv = c32.shape[0]
    err = [float(np.linalg.norm(c32[n] - c64[n]) / np.linalg.norm(c64[n])) for n in range(nv)]
    drift = [float(abs(t1[n] - t0[n]) / max(abs(t0[n]), abs(t0[0]))) for n in range(nv)]
    return {"steps": steps, "dt": dt, "rel_l2_fp32_vs_fp64": err, "conserved_total_drift_fp32": drift,
            "max_rel_l2": max(err), "meets_1e-5": max(err) <= 1e-5,
            "reference": "FP64 path on the GPU (held to 1e-11 of the FP64 CPU oracle in the parity tests)"}


def run_batched(steps: int = 20):
    """Batched configuration: 256 independent solves advanced by the batched
    graph step, against the same solves stepped one by one on the plain path."""
    import torch
    from dgcuda_gb300.batch import Batch
    specs = _config4_requests(12349, 256, 16, 512)
    solvers = [_native_solver(sp) for sp in specs]
    dofs = sum(sv.nv * sv.np * sv.E for sv in solvers)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    with torch.cuda.stream(stream):
        for _ in range(3):
            for sv in solvers:
                sv.step(sh)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            for sv in solvers:
                sv.step(sh)
        b.record(stream)
        torch.cuda.synchronize()
        plain_ms = a.elapsed_time(b) / steps
        bt = Batch(solvers)
        bt.autotune(reps=2, stream=sh)
        chosen = bt.fused()[0]
        nsteps = 3 + steps

        def time_batch():
            nonlocal nsteps
            for _ in range(3):
                bt.step(sh)
            torch.cuda.synchronize()
            l0 = bt.launch_count()
            a.record(stream)
            for _ in range(steps):
                bt.step(sh)
            b.record(stream)
            torch.cuda.synchronize()
            nsteps += 3 + steps
            return a.elapsed_time(b) / steps, (bt.launch_count() - l0) / steps

        # every launch mode timed on its own (the per-class launches with the
        # tuned options, the fused launch's two variants), then the autotuner's
        # choice for the headline
        modes = {}
        sampled = None
        for mode in (0, 2, 3):
            bt.set_fused(mode)
            ms, lps = time_batch()
            if sampled is None:   # the accuracy sample after 2 x (3 + steps) steps
                sampled = (nsteps, {k: solvers[k].get_state() for k in range(0, len(solvers), 16)})
            modes[{0: "per_class", 2: "fused_2cta", 3: "fused_3cta"}[mode]] = {
                "ms_per_step": ms, "launches_per_step": lps, "value": dofs / (ms * 1e-3)}
        bt.set_fused(chosen)
        batch_ms, launches_per_step = time_batch()
        info = bt.info()
        opts = bt.class_options()
    bt.close()
    accuracy = _sample_accuracy(specs, solvers, sampled[0], states=sampled[1])
    for sv in solvers:
        sv.close()
    compensated = _batched_compensated(specs, steps)
    return {"workload": "256 solves: equation 50/50, N log-uniform [16,512] (2N^2 triangles), "
                        "p uniform 1..4, Gaussian pulses / isentropic vortices, FP32, CFL 0.7",
            "dofs_per_step": dofs, "elements": int(sum(2 * sp["n"] ** 2 for sp in specs)),
            "value": dofs / (batch_ms * 1e-3), "ms_per_step": batch_ms,
            "plain_value": dofs / (plain_ms * 1e-3), "plain_ms_per_step": plain_ms,
            "speedup_vs_plain": plain_ms / batch_ms, "classes": info["classes"],
            "work_items": info["items"], "launches_per_step": launches_per_step,
            "launch_mode": {0: "per_class", 2: "fused_2cta", 3: "fused_3cta"}[chosen],
            "launch_modes": modes, "tuned_options": opts, "accuracy": accuracy, "compensated": compensated,
            "unit": UNIT}


def _batched_compensated(specs, steps):
    """The batched configuration in the compensated FP32 precision
    (DGX_FP32_COMP): the same solves one by one and batched (autotuned),
    2 x (3 + steps) steps in all, then the same accuracy sample against the
    FP64 path as the FP32 run."""
    import torch
    from dgcuda_gb300 import _ffi
    from dgcuda_gb300.batch import Batch
    solvers = [_native_solver(sp, _ffi.FP32_COMP) for sp in specs]
    dofs = sum(sv.nv * sv.np * sv.E for sv in solvers)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        for _ in range(3):
            for sv in solvers:
                sv.step(sh)
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(steps):
            for sv in solvers:
                sv.step(sh)
        b.record(stream)
        torch.cuda.synchronize()
        plain_ms = a.elapsed_time(b) / steps
        bt = Batch(solvers)
        bt.autotune(reps=2, stream=sh)   # restores the solves' states and times
        for _ in range(3):
            bt.step(sh)
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(steps):
            bt.step(sh)
        b.record(stream)
        torch.cuda.synchronize()
        batch_ms = a.elapsed_time(b) / steps
        mode = bt.fused()[0]
    bt.close()
    accuracy = _sample_accuracy(specs, solvers, 2 * (3 + steps))
    for sv in solvers:
        sv.close()
    return {"precision": "fp32_comp (compensated accumulation of the RK4 increments)",
            "value": dofs / (batch_ms * 1e-3), "ms_per_step": batch_ms,
            "plain_value": dofs / (plain_ms * 1e-3), "plain_ms_per_step": plain_ms,
            "speedup_vs_plain": plain_ms / batch_ms,
            "launch_mode": {0: "per_class", 2: "fused_2cta", 3: "fused_3cta"}[mode],
            "accuracy": accuracy, "unit": UNIT}


def _sample_accuracy(specs, solvers, nsteps, every: int = 16, states=None):
    """Relative L2 per conserved variable of a sample of the FP32 solves
    (every `every`-th) against the same solve in FP64 (the FP64 path, held to
    1e-11 of the CPU oracle by the parity tests), both `nsteps` CFL steps from
    the same initial state; the FP32 run's dt comes from its FP32 state, so the
    two runs' times differ by FP32 rounding."""
    from dgcuda_gb300 import _ffi
    from dgcuda_gb300.solver import DeviceMesh, Solver
    worst, rows = [0.0] * 4, []
    for k in range(0, len(specs), every):
        sp, sv = specs[k], solvers[k]
        dm = DeviceMesh.periodic_square(sp["n"], sp["lx"], sp["ly"], sp["jitter"], sp["seed"])
        ref = Solver(dm, sp["order"], sp["equation"], _ffi.FLUX_LLF, _ffi.FP64, 1.4)
        ref.project(sp["ic"], sp["params"])
        ref.set_dt(None, cfl=0.7)
        ref.run(max_steps=nsteps)
        a = states[k] if states is not None else sv.get_state()
        b = ref.get_state()
        ref.close()
        nv = a.shape[0]
        err = [float(np.linalg.norm(a[n] - b[n]) / np.linalg.norm(b[n])) for n in range(nv)]
        for n in range(nv):
            worst[n] = max(worst[n], err[n])
        rows.append({"solve": k, "n": sp["n"], "order": sp["order"],
                     "equation": "euler" if sp["equation"] == _ffi.EULER else "advection", "rel_l2": err})
    return {"reference": f"the same solve in FP64 on the GPU, {nsteps} CFL steps from the same initial state",
            "max_rel_l2_per_variable": worst, "max_rel_l2": max(worst), "meets_1e-5": max(worst) <= 1e-5,
            "sample": rows}


def run_served(rates=(50, 200, 1000, 2000, 0), count: int = 400):
    """Served configuration scaled down so that every rate finishes in seconds
    (reported beside the stated-size prefixes of run_served_stated): Poisson
    arrivals of `count` requests per rate, sizes N log-uniform in [16,64],
    orders 1..4, equations 50/50, end times U[0.1,1] x 0.02 flow-through times
    (the stated configuration's N up to 512 and full flow-through end times
    need hours per rate).  Also runs the same requests one by one on the plain
    path for the throughput comparison.  Rate 0 submits every request at once:
    the server's capacity, where the swept rates measure the offered load."""
    from dgcuda_gb300.serve import Server, request
    out = []
    rng = np.random.default_rng(12350)
    plain = None
    for ri, rate in enumerate(rates):
        specs = _config4_requests(12350 + ri, count, 16, 64)
        for sp in specs:
            flow = sp["lx"] / 1.0            # flow-through time of the domain (unit speed)
            sp["t_end"] = flow * rng.uniform(0.1, 1.0) * 0.02
        srv = Server(budget_bytes=150 << 30, max_active=1024)
        srv.set_steps_per_check(4)
        gaps = rng.exponential(1.0 / rate, size=count) if rate > 0 else np.zeros(count)
        t0 = time.perf_counter()
        t_next = t0
        for sp, g in zip(specs, gaps):
            t_next += g
            while time.perf_counter() < t_next:
                pass
            srv.submit(request(**sp))
        srv.wait_idle(600.0)
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        out.append({"rate_req_s": rate if rate > 0 else "all at once", "requests": count, "completed": st["completed"],
                    "failed": st["failed"], "p50_s": st["p50_latency_s"],
                    "p99_s": st["p99_latency_s"], "dof_updates": st["dof_updates"],
                    "value": st["dof_updates"] / wall, "wall_s": wall, "repacks": st["repacks"],
                    "worker_s": {"admit": st["admit_seconds"], "repack": st["repack_seconds"],
                                 "step": st["busy_seconds"], "retire": st["retire_seconds"],
                                 "idle": st["idle_seconds"]}})
        if plain is None:
            # the same requests one by one on the plain path
            import torch
            tp0 = time.perf_counter()
            dof = 0.0
            for sp in specs:
                sv = _native_solver(sp)
                n, _ = sv.run(t_end=sp["t_end"])
                dof += n * sv.nv * sv.np * sv.E
                sv.close()
            torch.cuda.synchronize()
            plain = dof / (time.perf_counter() - tp0)
    return {"workload": "Poisson arrivals, N log-uniform [16,64], p 1..4, equations 50/50, "
                        "end times U[0.1,1] x 0.02 flow-through, 150 GB admission budget",
            "rates": out, "plain_value": plain, "unit": UNIT}


def _served_stream(seed: int = 12351, count: int = 10000):
    """The served configuration's request stream at its stated sizes: `count`
    requests drawn as in the batched configuration (N log-uniform in [16,512],
    p 1..4, equations 50/50) with end times U[0.1,1] domain flow-through times
    (advection: the unit square at speed 1 per axis; Euler: [0,10]^2 at the
    free-stream speed 1)."""
    specs = _config4_requests(seed, count, 16, 512)
    rng = np.random.default_rng(seed + 1)
    for sp in specs:
        sp["t_end"] = sp["lx"] * rng.uniform(0.1, 1.0)
    return specs


def _serve_window(specs, rate, arrive_s, serve_s, keep=()):
    """Submit specs in stream order at Poisson arrivals of `rate` per second
    (rate 0: all at once) for at most arrive_s seconds, serve until serve_s
    seconds after the first arrival (or until every submitted request is done),
    then stop the server.  Returns the window's record and the kept results."""
    from dgcuda_gb300.serve import Server, request
    rng = np.random.default_rng(12353 + int(rate))
    srv = Server(budget_bytes=150 << 30, max_active=1024)
    srv.set_steps_per_check(8)
    t0 = time.perf_counter()
    t_next, n_sub, ids = t0, 0, {}
    for k, sp in enumerate(specs):
        if rate > 0:
            t_next += rng.exponential(1.0 / rate)
            if t_next - t0 > arrive_s:
                break
            while time.perf_counter() < t_next:
                pass
        ids[k] = srv.submit(request(**sp, keep_state=k in keep))
        n_sub += 1
    srv.wait_idle(max(0.0, serve_s - (time.perf_counter() - t0)))
    wall = time.perf_counter() - t0
    st = srv.stats()
    kept = {}
    for k in keep:
        if k in ids:
            state, lat, _ = srv.status(ids[k])
            if state == 2:   # DGX_REQ_DONE
                sp = specs[k]
                nv = 4 if sp["equation"] == 1 else 1
                npm = (sp["order"] + 1) * (sp["order"] + 2) // 2
                c, _, steps, t = srv.result(ids[k], nv * npm * 2 * sp["n"] ** 2)
                kept[k] = (c.reshape(nv, npm, -1), steps, t)
    srv.close()
    rec = {"submitted": n_sub, "completed": st["completed"], "failed": st["failed"],
           "unfinished_at_stop": n_sub - st["completed"] - st["failed"],
           "p50_s": st["p50_latency_s"], "p99_s": st["p99_latency_s"], "max_s": st["max_latency_s"],
           "dof_updates": st["dof_updates"], "value": st["dof_updates"] / wall, "wall_s": wall,
           "repacks": st["repacks"],
           "worker_s": {"admit": st["admit_seconds"], "repack": st["repack_seconds"], "step": st["busy_seconds"],
                        "retire": st["retire_seconds"], "idle": st["idle_seconds"]}}
    return rec, kept


def run_served_stated(rates=(50, 200, 1000, 2000), arrive_s=6.0, serve_s=12.0, capacity_s=20.0, plain_s=15.0,
                      subset=96):
    """Served configuration at its stated sizes: the 10,000-request stream of
    _served_stream (N up to 512, end times up to a full flow-through).  Its
    work (~1e13 DOF-updates, hours of GPU time) cannot finish in a benchmark,
    so every part is a time-boxed prefix of the same stream, labelled as such:
      * per swept rate: Poisson arrivals for arrive_s seconds, served until
        serve_s seconds; value = DOF-updates done in the window / its length;
        p50/p99 over the requests that finished in it (the rest are counted as
        unfinished: at these sizes every swept rate exceeds the GPU's capacity,
        so latencies are queueing times);
      * capacity: the stream submitted at once, served for capacity_s seconds;
      * plain: the same stream solved one by one with the public single-solve
        calls for plain_s seconds (requests that start are run to their end),
        and the requests it finished served at once to their ends: the same
        work both ways at the stated sizes (the capacity window's admitted mix
        differs from those few requests, so its rate is not compared with
        theirs);
      * same requests: the stream's first `subset` requests with N <= 128,
        served (submitted at once, run to the last one's end) and solved one by
        one on the plain path, each to its full end time, so both paths do the
        same work;
      * accuracy: relative L2 per variable of the first 8 of those requests
        against the same request solved in FP64 on the GPU (the FP64 path, held
        to 1e-11 of the CPU oracle by the parity tests)."""
    import torch
    from dgcuda_gb300 import _ffi
    from dgcuda_gb300.solver import DeviceMesh, Solver
    base = _served_stream()
    # the stream's requests run hundreds to thousands of steps, where only the
    # compensated FP32 precision stays within 1e-5 of FP64 (the plain FP32
    # path reaches 1e-4): the windows, the capacity and the one-by-one path
    # run in it; the same-requests comparison below is made in both
    specs = [dict(sp, precision=_ffi.FP32_COMP) for sp in base]
    out = {"workload": "10,000 requests: N log-uniform [16,512], p 1..4, equations 50/50, end times U[0.1,1] "
                       "flow-through, Poisson arrivals, 150 GB admission budget (time-boxed prefixes)",
           "precision": "fp32_comp (compensated accumulation of the RK4 increments) for the windows, the "
                        "capacity and the plain path",
           "stream_requests": len(specs), "rates": []}
    for rate in rates:
        rec, _ = _serve_window(specs, rate, arrive_s, serve_s)
        rec["rate_req_s"] = rate
        rec["window"] = f"arrivals for {arrive_s:g} s, served until {serve_s:g} s"
        out["rates"].append(rec)
    cap, _ = _serve_window(specs, 0, 0.0, capacity_s)
    cap["window"] = f"the stream submitted at once, served for {capacity_s:g} s"
    out["capacity"] = cap
    # the plain path: one request after another through the single-solve calls
    t0, dof, done = time.perf_counter(), 0.0, 0
    for sp in specs:
        if time.perf_counter() - t0 > plain_s:
            break
        sv = _native_solver(sp, sp["precision"])
        n, _ = sv.run(t_end=sp["t_end"])
        dof += n * sv.nv * sv.np * sv.E
        sv.close()
        done += 1
    torch.cuda.synchronize()
    plain_wall = time.perf_counter() - t0
    first = [{"n": sp["n"], "order": sp["order"],
              "equation": "euler" if sp["equation"] == _ffi.EULER else "advection"} for sp in specs[:done]]
    out["plain"] = {"value": dof / plain_wall, "requests": done, "wall_s": plain_wall, "dof_updates": dof,
                    "which": first,
                    "path": "dgx_mesh_create_periodic_square + dgx_solver_create + dgx_project_ic + dgx_run per request"}
    # the same requests served at once, each to its end time
    same, _ = _serve_window(specs[:done], 0, 0.0, 600.0)
    out["plain_requests_served"] = {
        "wall_s": same["wall_s"], "value": same["dof_updates"] / same["wall_s"], "dof_updates": same["dof_updates"],
        "completed": same["completed"],
        "served_vs_plain": (same["dof_updates"] / same["wall_s"]) / (dof / plain_wall) if dof else None,
        "note": "the same requests as `plain`, submitted at once; large meshes fill the GPU alone, so batching "
                "them gains little"}
    # the same requests through both paths, each to its end time
    sel = [k for k, sp in enumerate(base) if sp["n"] <= 128][:subset]
    sub = [base[k] for k in sel]
    srv_rec, kept = _serve_window(sub, 0, 0.0, 600.0, keep=range(8))
    t0, pdof = time.perf_counter(), 0.0
    for sp in sub:
        sv = _native_solver(sp)
        n, _ = sv.run(t_end=sp["t_end"])
        pdof += n * sv.nv * sv.np * sv.E
        sv.close()
    torch.cuda.synchronize()
    pwall = time.perf_counter() - t0
    out["same_requests"] = {
        "requests": f"the stream's first {len(sub)} requests with N <= 128 (full end times)",
        "served": {"wall_s": srv_rec["wall_s"], "value": srv_rec["dof_updates"] / srv_rec["wall_s"],
                   "completed": srv_rec["completed"], "p50_s": srv_rec["p50_s"], "p99_s": srv_rec["p99_s"]},
        "plain": {"wall_s": pwall, "value": pdof / pwall},
        "served_vs_plain": (srv_rec["dof_updates"] / srv_rec["wall_s"]) / (pdof / pwall) if pdof else None}
    # the same requests in the compensated FP32 precision, both paths
    csub = [dict(sp, precision=_ffi.FP32_COMP) for sp in sub]
    csrv_rec, ckept = _serve_window(csub, 0, 0.0, 600.0, keep=range(8))
    t0, cdof = time.perf_counter(), 0.0
    for sp in sub:
        sv = _native_solver(sp, _ffi.FP32_COMP)
        n, _ = sv.run(t_end=sp["t_end"])
        cdof += n * sv.nv * sv.np * sv.E
        sv.close()
    torch.cuda.synchronize()
    cwall = time.perf_counter() - t0
    out["same_requests_compensated"] = {
        "precision": "fp32_comp (compensated accumulation of the RK4 increments)",
        "served": {"wall_s": csrv_rec["wall_s"], "value": csrv_rec["dof_updates"] / csrv_rec["wall_s"],
                   "completed": csrv_rec["completed"], "p50_s": csrv_rec["p50_s"], "p99_s": csrv_rec["p99_s"]},
        "plain": {"wall_s": cwall, "value": cdof / cwall},
        "served_vs_plain": (csrv_rec["dof_updates"] / csrv_rec["wall_s"]) / (cdof / cwall) if cdof else None}

    def accuracy_of(kept_states):
        rows, worst = [], [0.0] * 4
        for k, (c, steps, t) in kept_states.items():
            sp = sub[k]
            b = refs[k]
            err = [float(np.linalg.norm(c[n] - b[n]) / np.linalg.norm(b[n])) for n in range(c.shape[0])]
            for n, v in enumerate(err):
                worst[n] = max(worst[n], v)
            rows.append({"request": sel[k], "n": sp["n"], "order": sp["order"], "steps": steps,
                         "equation": "euler" if sp["equation"] == _ffi.EULER else "advection", "rel_l2": err})
        return {"reference": "the same request in FP64 on the GPU, to the same end time",
                "max_rel_l2_per_variable": worst, "max_rel_l2": max(worst) if rows else None,
                "meets_1e-5": (max(worst) <= 1e-5) if rows else None, "sample": rows}

    refs = {}
    for k in set(kept) | set(ckept):
        sp = sub[k]
        dm = DeviceMesh.periodic_square(sp["n"], sp["lx"], sp["ly"], sp["jitter"], sp["seed"])
        ref = Solver(dm, sp["order"], sp["equation"], _ffi.FLUX_LLF, _ffi.FP64, 1.4)
        ref.project(sp["ic"], sp["params"])
        ref.set_dt(None, cfl=0.7)
        ref.run(t_end=sp["t_end"])
        refs[k] = ref.get_state()
        ref.close()
    out["accuracy"] = accuracy_of(kept)
    out["accuracy_compensated"] = accuracy_of(ckept)
    return out


def time_steps(sv, steps, warmup, stream, world):
    """W untimed steps, then K steps timed with CUDA events on `stream`;
    returns (ms per step, mean ms of stages 2-4, kernel launches, wall start, wall end)."""
    import torch
    sh = stream.cuda_stream
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            sv.step(sh)
        torch.cuda.synchronize()
        launches0 = sv.launch_count()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
               torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        barrier(world)
        torch.cuda.synchronize()
        t_wall0 = time.time()
        for i in range(steps):
            ev[i][0].record(stream)
            sv.rk_stage(0, sh)        # CFL reduction + dt, then stage 1
            ev[i][1].record(stream)
            sv.rk_stage(1, sh)
            sv.rk_stage(2, sh)
            sv.rk_stage(3, sh)
            ev[i][2].record(stream)
        torch.cuda.synchronize()
        barrier(world)
        t_wall1 = time.time()
        launches = sv.launch_count() - launches0
    total_ms = ev[0][0].elapsed_time(ev[-1][2])
    ms_step = allreduce_max(total_ms / steps, world)
    stage_ms = sum(e[1].elapsed_time(e[2]) for e in ev) / (3 * steps)   # stages 2-4
    return ms_step, stage_ms, launches, t_wall0, t_wall1


def run_e2e(sv, mesh, prec, dofs, X, steps, world, in_flight: int = 3):
    """The step end to end through the C ABI with host buffers: every step
    copies its solve's state in from pinned host memory (dgx_set_state_f32),
    runs the RK4 step (dgx_step) and copies the state back out
    (dgx_get_state_f32), 335.5 MB each way at 2x1024^2.

    One solve alone serialises the three (the step needs the state in, the
    copy out needs the step).  The headline keeps `in_flight` solves of the
    same workload on their own streams, so one solve's copies run on the copy
    engines while another's step runs on the SMs: the host link (about
    200 GB/s each way) and the SMs work at once.  Both figures are reported."""
    import torch
    n_rounds = max(3, min(steps, 20))

    def host_buf(s, st):
        h = torch.empty(dofs, dtype=torch.float32, pin_memory=True)
        s.get_state_f32(h.numpy(), st.cuda_stream)
        return h

    def timed(solvers, streams, hosts, rounds):
        def one_round():
            for s, st, h in zip(solvers, streams, hosts):
                sh = st.cuda_stream
                s.set_state_f32(h.numpy(), sh)
                s.step(sh)
                s.get_state_f32(h.numpy(), sh)
        for _ in range(2):
            one_round()
        torch.cuda.synchronize()
        barrier(world)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(streams[0])
        for st in streams[1:]:
            st.wait_event(a)
        for _ in range(rounds):
            one_round()
        for st in streams[1:]:
            e = torch.cuda.Event()
            e.record(st)
            streams[0].wait_event(e)
        b.record(streams[0])
        torch.cuda.synchronize()
        return allreduce_max(a.elapsed_time(b) / (rounds * len(solvers)), world)

    st0 = torch.cuda.Stream()
    h0 = host_buf(sv, st0)
    serial_ms = timed([sv], [st0], [h0], n_rounds)
    solvers = [sv] + [density_wave_solver(mesh, prec) for _ in range(in_flight - 1)]
    streams = [st0] + [torch.cuda.Stream() for _ in range(in_flight - 1)]
    hosts = [h0] + [host_buf(s, st) for s, st in zip(solvers[1:], streams[1:])]
    torch.cuda.synchronize()
    ms = timed(solvers, streams, hosts, n_rounds)
    del solvers[1:]
    return {"value": dofs * world / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms,
            "h2d_bytes_per_step": X, "d2h_bytes_per_step": X,
            "path": "dgx_set_state_f32 (pinned host) + dgx_step + dgx_get_state_f32, every step",
            "solves_in_flight": in_flight,
            "how": f"{in_flight} solves of this workload, each on its own stream; one solve's state copies "
                   "overlap another's step",
            "serial": {"value": dofs * world / (serial_ms * 1e-3), "unit": UNIT, "ms_per_step": serial_ms,
                       "how": "one solve: state in, step, state out in sequence on one stream"}}


def density_wave_solver(mesh, precision):
    from dgcuda_gb300 import _ffi
    from dgcuda_gb300.solver import Solver
    sv = Solver(mesh, 3, _ffi.EULER, _ffi.FLUX_LLF, precision, 1.4)
    sv.project(_ffi.IC_DENSITY_WAVE, (0.2, 1.0, 1.0, 1.0, 1.0))
    sv.set_dt(None, cfl=0.7)
    sv.set_end_time(0.0)
    return sv


def run_bf16x3(mesh, args, stage_bytes, peak, dofs, fp32_ms):
    """The same workload with the basis contractions on the tensor cores
    (DGX_FP32_BF16X3): step time, roofline fraction of its stage kernel, and
    accuracy against the FP64 path after 100 steps from the same state."""
    import torch
    from dgcuda_gb300 import _ffi
    try:
        sv = density_wave_solver(mesh, _ffi.FP32_BF16X3)
    except Exception as exc:   # e.g. the tensor-core self-test refused the device
        return {"unavailable": str(exc)}
    stream = torch.cuda.Stream()
    ms, stage_ms, launches, _, _ = time_steps(sv, args.steps, args.warmup, stream, 1)
    achieved = stage_bytes / (stage_ms * 1e-3) / 1e9
    acc = run_accuracy(args.mesh_n, precision=_ffi.FP32_BF16X3)
    return {"value": dofs / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "speedup_vs_fp32": fp32_ms / ms,
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "kernel": "stage_kernel_tc<3,EULER> (fused RK4 stage, BF16x3 MMA)"},
            "accuracy": acc}


def run_fp64(mesh, args, dofs, steps: int = 10):
    """The same workload in FP64 (DGX_FP64, the reference's precision): step
    time, for a same-precision comparison with the reference's own CUDA solver
    rebuilt for sm_103a (the reference arm's `reference_gpu`, FP64)."""
    import torch
    from dgcuda_gb300 import _ffi
    sv = density_wave_solver(mesh, _ffi.FP64)
    stream = torch.cuda.Stream()
    ms, stage_ms, launches, _, _ = time_steps(sv, steps, 3, stream, 1)
    sv.close()
    return {"value": dofs / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "steps": steps, "dtype": "f64",
            "gpu_launches": launches,
            "what": "the FP64 path (scalar FP64 stage kernel, FP64 state) on the same workload; compare with "
                    "the reference arm's reference_gpu (the reference's CUDA solver, FP64)"}


def run_fp32_comp(mesh, args, dofs, fp32_ms, steps: int = 50):
    """The same workload in the compensated FP32 precision (DGX_FP32_COMP:
    the RK4 increments accumulated apart from the state, the state carried as
    c + lo): step time beside the plain FP32 path's."""
    import torch
    from dgcuda_gb300 import _ffi
    sv = density_wave_solver(mesh, _ffi.FP32_COMP)
    stream = torch.cuda.Stream()
    ms, stage_ms, launches, _, _ = time_steps(sv, steps, 3, stream, 1)
    sv.close()
    return {"value": dofs / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "steps": steps, "dtype": "f32",
            "gpu_launches": launches, "time_vs_fp32": ms / fp32_ms,
            "what": "FP32 state and arithmetic, RK4 increments accumulated apart from the state and the "
                    "state updated by an error-free two-sum (19 state passes per step instead of 13)"}


def run_ours(args, rank, world, local):
    import torch
    torch.cuda.set_device(local)
    from dgcuda_gb300 import _ffi, build
    build.build()
    n = args.mesh_n
    mesh = build_mesh(n)
    E = mesh.num_elem
    prec = {"bf16x3": _ffi.FP32_BF16X3, "fp32comp": _ffi.FP32_COMP}.get(args.precision, _ffi.FP32)
    sv = density_wave_solver(mesh, prec)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    dofs = 4 * 10 * E
    X = dofs * 4
    G = 20 * E + 24 * mesh.num_sides
    # algorithmic bytes per DOF-update: the reference's RK4 in its fused
    # two-register form moves 16X + 4G per step (stages 3X+G, 5X+G, 5X+G,
    # 3X+G: 69.6 B per DOF-update at this size).  The kernels run a 13-pass form
    # that moves 13X + 4G (stages 2X+G, 3X+G, 5X+G, 3X+G); the roofline line
    # reports both, the first as `achieved`/`frac`.
    step_bytes = 16 * X + 4 * G                   # algorithmic bytes per RK4 step
    stage_bytes = (13 * X + 3 * G) / 3.0          # per timed stage 2-4 launch (average; stage 1 is timed with the CFL kernel)
    moved_step_bytes = 13 * X + 4 * G
    moved_stage_bytes = (11 * X + 3 * G) / 3.0
    if prec == _ffi.FP32_COMP:   # the compensated form: stages 4X+G, 5X+G, 5X+G, 5X+G
        moved_step_bytes = 19 * X + 4 * G
        moved_stage_bytes = 5 * X + G

    clocks = ClockSampler(local)
    clocks.start()
    ms_step, stage_ms, launches, t_wall0, t_wall1 = time_steps(sv, args.steps, args.warmup, stream, world)
    value = dofs * world / (ms_step * 1e-3)

    e2e = run_e2e(sv, mesh, prec, dofs, X, args.steps, world)
    clocks.stop()
    ck = clocks.summary(t_wall0, t_wall1)
    if rank != 0:
        return None

    peak, peak_src = peaks()
    achieved = stage_bytes / (stage_ms * 1e-3) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", {_ffi.FP32: "stage_kernel_density_wave_p3.json",
                                           _ffi.FP32_BF16X3: "stage_kernel_tc_density_wave_p3.json",
                                           _ffi.FP32_COMP: "stage_kernel_comp_density_wave_p3.json"}[prec])
    if os.path.exists(prof) and n == 1024:
        try:
            traffic = json.load(open(prof)).get("dram_bytes_per_launch")
        except Exception:
            traffic = None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(workload(n), precision=args.precision, num_elem=E, num_sides=mesh.num_sides, dofs=dofs,
                       parallelism="replicas" if world > 1 else "single"),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": {_ffi.FP32_BF16X3: "stage_kernel_tc<3,EULER> (fused RK4 stage, BF16x3 MMA)",
                                _ffi.FP32_COMP: "stage_kernel<3,EULER> (fused RK4 stage, FP32, compensated)"}.get(
                                    prec, "stage_kernel<3,EULER> (fused RK4 stage, FP32)"),
                     "algorithmic_bytes_per_launch": stage_bytes,
                     "algorithmic_bytes_per_step": step_bytes,
                     "step_achieved": step_bytes / (ms_step * 1e-3) / 1e9,
                     "moved_bytes_per_launch": moved_stage_bytes,
                     "moved_bytes_per_step": moved_step_bytes,
                     "achieved_moved": moved_stage_bytes / (stage_ms * 1e-3) / 1e9,
                     "frac_moved": moved_stage_bytes / (stage_ms * 1e-3) / 1e9 / peak,
                     "bytes_note": "achieved/frac: the reference algorithm's bytes (16X+4G per step, fused "
                                   "two-register RK4); *_moved: the bytes the 13-pass kernels move (13X+4G)",
                     "peak_source": f"{peak_src} hbm_gbs"},
        "e2e": e2e,
        "clocks": ck,
        "gpu_launches": launches,
    }
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_sample()
    if not args.no_extra and prec == _ffi.FP32:
        out["bf16x3"] = run_bf16x3(mesh, args, stage_bytes, peak, dofs, ms_step)
        out["fp64"] = run_fp64(mesh, args, dofs)
        out["fp32_comp"] = run_fp32_comp(mesh, args, dofs, ms_step)
        out["accuracy"] = run_accuracy(args.mesh_n)
        out["batched"] = run_batched()
        out["served"] = run_served_stated()
        out["served_scaled"] = run_served()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--mesh-n", type=int, default=1024)
    ap.add_argument("--precision", choices=["fp32", "bf16x3", "fp32comp"], default="fp32",
                    help="arithmetic of the timed path: plain FP32, FP32 with the basis "
                         "contractions on the tensor cores (BF16x3), or FP32 with compensated "
                         "RK4 accumulation")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the batched and served sections")
    ap.add_argument("--only", choices=["batched", "served", "served_stated"], default=None,
                    help="run and print one section alone (for profiling it)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_init()
    if args.only:
        import torch
        torch.cuda.set_device(local)
        from dgcuda_gb300 import build
        build.build()
        fn = {"batched": run_batched, "served": run_served, "served_stated": run_served_stated}[args.only]
        print(json.dumps(fn()), flush=True)
        return
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        out = run_ours(args, rank, world, local)
    if out is not None:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
