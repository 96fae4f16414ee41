#!/usr/bin/env python3
"""Benchmark of the per-step finite-volume update on GB300.

Headline workload: 2D Euler shear layer, gamma = 1.4, 2048 x 2048 periodic
cells on [0,1]^2; rho = 2 and v_x = +0.5 for |y - 0.5| < 0.25, rho = 1 and
v_x = -0.5 elsewhere, p = 2.5, v_y = 0.01 sin(4 pi x) + seeded uniform noise of
amplitude 1e-3; PPM (McCorquodale-Colella limiter) + HLLC + SSPRK3 at CFL 0.8.
One step = one full SSPRK3 step (three stages) of the whole grid.  Seeded
synthetic data; no dataset is involved.

Legs of the default arm (all numbers in cell-updates/s):
  value        FP32 (FP64 pressure recovery), state resident in HBM
  fp64_plain   the plain all-FP64 path on the same workload
  l1_rho       L1(rho) of FP32 against FP64 at t=0.05 on the workload's grid
  accuracy_t_end_512  the same error measure to t_end=1.0 on a 512^2 grid, beside an
               FP64 twin started one ulp away (--accuracy: the 2048^2 and 1024^2 runs)
  batched_to_t_end / mhd_accuracy  configurations 4 and 3 against FP64 (to t=0.25, t=0.05)
  e2e          through the C ABI with the state copied host->device and
               device->host (pinned) every step
  batched      512 independent four-quadrant Riemann grids, 128^2..1024^2,
               PLM+LLF / PPM+HLLC 50/50, FP32, one persistent kernel per sweep
  serving      continuous batching of a seeded Poisson request stream
               (sizes scaled down 4x per axis from the full request mix so the
               leg takes seconds; see --serve-*)
  cpu_baseline the oracle (NumPy restatement of the reference) on one core,
               SSPRK3 steps of a 256^2 instance of the headline workload
--impl reference: the reference's algorithm (the oracle) on all host cores,
independent 256^2 instances, one process per core.

Multi-GPU (torchrun): independent replicas, no collective; value sums ranks.
"""

import argparse
import ctypes
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

SEED = 20261203
METRIC = "cell-updates/s FP32-batched vs FP64 plain (L1<=1e-5); serve p50/p99 ms"
WORKLOAD = "2D Euler shear layer 2048^2 periodic, PPM(mc) with flattening and artificial viscosity + HLLC + SSPRK3, CFL 0.8"
# Mean DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per sweep launch
# over the SSPRK3 steps of the headline FP32 workload at 2048^2, from one ncu
# launch list (profiles/sweep_kernel_f32_ppm_hllc_2d.md); scaled by cells for
# other sizes.  Slightly above the algorithmic bytes: the viscous strip reads
# the stage state once more besides its cell averages.
SWEEP_DRAM_BYTES = 223.1e6
SWEEP_DRAM_CELLS = 2048 * 2048
# Floating-point operations per cell-update of one SSPRK3 step (every kernel of the step),
# from ncu's SASS op counters (fadd + fmul + 2 x ffma + 2 x fadd2 + 2 x fmul2 + 4 x ffma2, and
# the FP64 counterparts) over one step of the workload at 512^2 (profiles/flops_step_2d_shear.md;
# FP32 with the 32 x 8 tile along axis 0 and 32 x 15 along axis 1, FP64 with 32 x 15 on both).
# FP64 division and square root are instruction sequences, which is why the FP64 step counts
# more operations.
FLOPS_FP32_PER_CELL_UPDATE = 4771.1
FLOPS_FP64_PER_CELL_UPDATE = 11544.4
# warp instructions per cell-update of the FP32 step (smsp__inst_executed.sum of every launch of a
# step, launch list at 2048^2, profiles/sweep_kernel_f32_ppm_hllc_2d.md): against the issue rate of
# one warp instruction per SM sub-partition per clock
WARP_INSTR_FP32_PER_CELL_UPDATE = 331.0
SMSP_PER_SM = 4
# per-SM, per-clock issue rates of the FP32 and FP64 fused multiply-add pipes on GB300
# (ncu: sm__sass_thread_inst_executed_op_{ffma,dfma}_pred_on.sum.peak_sustained / SMs)
FFMA_PER_SM_CLK, DFMA_PER_SM_CLK = 128, 2


def shear_layer(n, seed=SEED):
    """Point primitives of the shear-layer workload, shape (n, n, 8)."""
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + .5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    w = np.zeros((n, n, 8))
    inner = np.abs(Y - .5) < .25
    w[..., 0] = np.where(inner, 2.0, 1.0)
    w[..., 1] = np.where(inner, .5, -.5)
    w[..., 2] = .01 * np.sin(4 * np.pi * X) + rng.uniform(-1e-3, 1e-3, size=(n, n))
    w[..., 4] = 2.5
    return w


def run_config(n, precision):
    from astrea_gb300.solver import RunConfig
    # textbook HLLC (ASTREA_FLAG_PHYSICAL): the reference's 2D HLLC (normal velocity by
    # iteration position, star momentum always in component 1, f_plus for sL > 0) loses
    # positivity on this flow within a few steps; the arithmetic per cell is the same
    return RunConfig(dim=2, n0=n, n1=n, model=4, precision=precision, scheme="ppm", solver="hllc",
                     integrator="ssprk33", boundary="wrap", gamma=1.4, dx=1.0 / n, cfl=0.8, t_end=1.0, compat=False,
                     flatten=True, viscosity=True)


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.3)
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
        sm, mx, power, reasons = [], None, [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
                power.append(float(f[3]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(power) if power else None}


def alu_roofline(value32, value64, sm_max_mhz):
    """FP32 and FP64 ALU rooflines of the step: counted operations per cell-update x rate against
    the fused multiply-add peak at the maximum SM clock seen (2 operations per FMA)."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    clk = (sm_max_mhz or 2070.0) * 1e6
    out = {"source": "ncu SASS op counters of one step (fadd + fmul + 2 ffma; FP64 alike), peak = SMs x FMA/clk x 2 x "
                     "max SM clock", "sms": sms, "sm_max_mhz": clk / 1e6}
    for name, flops, value, rate in (("fp32", FLOPS_FP32_PER_CELL_UPDATE, value32, FFMA_PER_SM_CLK),
                                     ("fp64", FLOPS_FP64_PER_CELL_UPDATE, value64, DFMA_PER_SM_CLK)):
        if value is None:
            continue
        peak = sms * rate * 2 * clk / 1e12
        got = flops * value / 1e12
        out[name] = {"flops_per_cell_update": flops, "achieved_tflops": got, "peak_tflops": peak, "frac": got / peak}
    if value32 is not None:
        peak_issue = sms * SMSP_PER_SM * clk
        got_issue = WARP_INSTR_FP32_PER_CELL_UPDATE * value32
        out["issue_fp32"] = {"warp_instructions_per_cell_update": WARP_INSTR_FP32_PER_CELL_UPDATE,
                             "achieved_per_s": got_issue, "peak_per_s": peak_issue, "frac": got_issue / peak_issue,
                             "note": "instruction issue, the bound of this stencil"}
    return out


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def cpu_sample_worker(args):
    """One bounded CPU sample: ``steps`` SSPRK3 steps of an n x n shear layer with the oracle."""
    n, seed, steps = args
    import numpy as np_
    sys.path.insert(0, ROOT)
    from oracle import stepper
    # LAPACK eigenvalues of the interface Jacobians, as the reference computes its wave speeds
    cfg = stepper.OracleConfig(dim=2, scheme="ppm", solver="hllc", integrator="ssprk33", gamma=1.4, bc="wrap",
                               dx=1.0 / n, cfl=0.8, eig="lapack", t_end=1.0, compat=False, flatten=True,
                               viscosity=True)
    q = stepper.initialise(shear_layer(n, seed), cfg)
    t, idx, order = 0.0, 1, [0, 1]
    t0 = time.perf_counter()
    with np_.errstate(all="ignore"):
        for _ in range(steps):
            q, t, idx, order, _dt = stepper.step(q, cfg, t, idx, order)
    return time.perf_counter() - t0


def cpu_baseline(n=256, procs=1, steps=1):
    """Oracle (NumPy restatement of the reference) on host cores: cell-updates/s."""
    if procs <= 1:
        dt = cpu_sample_worker((n, SEED, steps))
        return n * n * steps / dt, 1
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        t0 = time.perf_counter()
        pool.map(cpu_sample_worker, [(n, SEED + i, steps) for i in range(procs)])
        wall = time.perf_counter() - t0
    return procs * n * n * steps / wall, procs


def dist_init():
    """Ranks of a torchrun launch (one replica per GPU); NCCL, or gloo for host-only runs (ASTREA_DIST_BACKEND)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(os.environ.get("ASTREA_DIST_BACKEND", "nccl"))
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, ws):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([x], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reference_arm(args):
    """The reference's CPU path (the oracle, bit-exact with it) on every host core: ``procs`` processes,
    each timed step one SSPRK3 step of an independent instance per process.  The instance side is sized
    so that the ``--steps`` timed steps take about two minutes in all."""
    ws, rank, _ = dist_init()
    if rank != 0:
        return 0
    import multiprocessing as mp
    procs = max(1, len(os.sched_getaffinity(0)))
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        pool.map(cpu_sample_worker, [(32, SEED, 1)] * procs)  # start the workers and their imports
        t0 = time.perf_counter()
        pool.map(cpu_sample_worker, [(64, SEED + i, 1) for i in range(procs)])
        t64 = time.perf_counter() - t0
        budget = 120.0 / max(1, args.steps)
        n = 32
        for cand in (256, 128, 64):
            if t64 * (cand / 64) ** 2 <= budget:
                n = cand
                break
        for _ in range(args.warmup):
            pool.map(cpu_sample_worker, [(n, SEED + i, 1) for i in range(procs)])
        vals = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            pool.map(cpu_sample_worker, [(n, SEED + i, 1) for i in range(procs)])
            vals.append(procs * n * n / (time.perf_counter() - t0))
    value = statistics.median(vals)
    sample = (f"{procs} processes, each timed step one SSPRK3 step of an independent {n}^2 instance per process, "
              f"oracle (NumPy restatement of the reference, LAPACK wave speeds as in the reference)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * n * n * procs / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": sample},
            "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": procs, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def batched_cfg(n, ppm, precision=32):
    """One grid of the batched workload: n^2 four-quadrant data, PPM+HLLC or PLM+LLF, to t=0.25."""
    from astrea_gb300.solver import RunConfig
    return RunConfig(dim=2, n0=n, n1=n, model=4, precision=precision, scheme="ppm" if ppm else "plm",
                     solver="hllc" if ppm else "llf", integrator="ssprk33", boundary="edge", gamma=1.4,
                     dx=1.0 / n, cfl=0.8, t_end=0.25, compat=False)


def batched_leg(steps, warmup, ngrids=512, seed=SEED):
    """512 four-quadrant Riemann grids, sides 2^k (k in 7..10), PLM+LLF / PPM+HLLC 50/50, FP32."""
    import torch
    from astrea_gb300.batch import Batch
    from astrea_gb300.serving import Request
    rng = np.random.default_rng(seed)
    cfgs, seeds = [], []
    for g in range(ngrids):
        n = 2 ** int(rng.integers(7, 11))
        ppm = bool(rng.uniform() < .5)
        cfgs.append(batched_cfg(n, ppm))
        seeds.append(int(rng.integers(1 << 31)))
    b = Batch(cfgs)
    for g, c in enumerate(cfgs):
        # four-quadrant point primitives, filled on the device from the grid's four seeded states
        r = Request(rid=g, arrival=0.0, dim=2, n=4, mhd=False, scheme="plm", solver="llf", t_end=.25, seed=seeds[g])
        q4 = torch.as_tensor(r.initial_state(), dtype=torch.float32, device="cuda")  # 4x4: one state per quadrant
        w = q4[[0, 2]][:, [0, 2]].repeat_interleave(c.n0 // 2, 0).repeat_interleave(c.n1 // 2, 1)
        b.initialise_one(g, w)
    torch.cuda.synchronize()
    cells = sum(c.n0 * c.n1 for c in cfgs)
    b.step(warmup, graph=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    c_before = b.clocks()["steps"].copy()
    e0.record()
    b.step(steps, graph=True)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clk = b.clocks()
    done_updates = float(sum((clk["steps"][g] - c_before[g]) * cfgs[g].n0 * cfgs[g].n1 for g in range(ngrids)))
    out = {"value": done_updates / (ms / 1e3), "unit": "cell-updates/s", "grids": ngrids, "cells": cells,
           "tiles": b.tiles(),
           "steps": steps, "ms_per_step": ms / steps, "non_finite_grids": int((clk["status"] != 0).sum()),
           "workload": "512 four-quadrant Riemann grids 128^2..1024^2, PLM+LLF/PPM+HLLC 50/50, FP32, edge, CFL 0.8",
           "graph": "one CUDA graph per step, persistent sweep kernels over a tile work list"}
    del b
    torch.cuda.empty_cache()
    out["fp64_check"] = batched_fp64_check(cfgs, seeds, warmup + steps)
    return out


def batched_cpu_worker(args):
    """One SSPRK3 step of one four-quadrant grid of the batched workload with the oracle (LAPACK
    wave speeds as the reference); returns the seconds it took."""
    n, ppm, seed = args
    import numpy as np_
    sys.path.insert(0, ROOT)
    from oracle import stepper
    from astrea_gb300.serving import Request
    r = Request(rid=0, arrival=0.0, dim=2, n=n, mhd=False, scheme="plm", solver="llf", t_end=.25, seed=seed)
    cfg = stepper.OracleConfig(dim=2, scheme="ppm" if ppm else "plm", solver="hllc" if ppm else "llf",
                               integrator="ssprk33", gamma=1.4, bc="edge", dx=1.0 / n, cfl=0.8, eig="lapack",
                               t_end=0.25, compat=False)
    q = stepper.initialise(r.initial_state(), cfg)
    t0 = time.perf_counter()
    with np_.errstate(all="ignore"):
        stepper.step(q, cfg, 0.0, 1, [0, 1])
    return time.perf_counter() - t0


def batched_cpu_baseline(n=128, seed=SEED):
    """The batched workload's methods on the host cores: one process per core, each one SSPRK3 step
    of an independent 128^2 four-quadrant grid (half PLM+LLF, half PPM+HLLC), oracle."""
    import multiprocessing as mp
    procs = max(1, len(os.sched_getaffinity(0)))
    rng = np.random.default_rng(seed)
    jobs = [(n, k % 2 == 1, int(rng.integers(1 << 31))) for k in range(procs)]
    with mp.get_context("spawn").Pool(procs) as pool:
        pool.map(batched_cpu_worker, [(16, False, 1)] * procs)  # start the workers and their imports
        t0 = time.perf_counter()
        pool.map(batched_cpu_worker, jobs)
        wall = time.perf_counter() - t0
    return {"value": procs * n * n / wall, "unit": "cell-updates/s", "cores": procs, "kind": "port",
            "sample": f"{procs} processes, each one SSPRK3 step of an independent {n}^2 four-quadrant grid of the "
                      f"workload (PLM+LLF or PPM+HLLC), oracle with LAPACK wave speeds as in the reference"}


def batched_fp64_check(cfgs, seeds, steps, count=32):
    """Per-instance FP32-vs-FP64 L1(rho) of the first ``count`` batched grids after ``steps`` steps."""
    import torch
    from dataclasses import replace
    from astrea_gb300.batch import Batch
    from astrea_gb300.serving import Request
    sub = cfgs[:count]
    out = {}
    for prec in (32, 64):
        b = Batch([replace(c, precision=prec) for c in sub])
        for g, c in enumerate(sub):
            r = Request(rid=g, arrival=0.0, dim=2, n=4, mhd=False, scheme="plm", solver="llf", t_end=.25,
                        seed=seeds[g])
            q4 = torch.as_tensor(r.initial_state(), dtype=torch.float64, device="cuda")
            w = q4[[0, 2]][:, [0, 2]].repeat_interleave(c.n0 // 2, 0).repeat_interleave(c.n1 // 2, 1)
            b.initialise_one(g, w)
        b.step(steps, graph=True)
        torch.cuda.synchronize()
        out[prec] = ([b.planes(g)[0].double().clone() for g in range(len(sub))], b.clocks()["status"])
        del b
    finite = [(a, d) for a, d, st32, st64 in zip(out[32][0], out[64][0], out[32][1], out[64][1])
              if st32 == 0 and st64 == 0 and torch.isfinite(a).all()]
    # a grid with a non-positive density in either precision is on its way to blowing up (the
    # unstable PLM+LLF instances at CFL 0.8): counted apart, not in the error statistics
    l1 = [float(torch.mean(torch.abs(a - d))) for a, d in finite if float(a.min()) > 0 and float(d.min()) > 0]
    return {"instances": len(sub), "finite_in_both": len(finite), "non_positive_density": len(finite) - len(l1),
            "steps": steps, "l1_rho_median": float(np.median(l1)) if l1 else None,
            "l1_rho_max": float(np.max(l1)) if l1 else None}


def orszag_tang(n):
    """Point primitives of the periodic Orszag-Tang vortex on [0,1]^2 (gamma = 5/3)."""
    x = (np.arange(n) + .5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    w = np.zeros((n, n, 8))
    w[..., 0] = 25.0 / (36.0 * np.pi)
    w[..., 4] = 5.0 / (12.0 * np.pi)
    w[..., 1] = -np.sin(2 * np.pi * Y)
    w[..., 2] = np.sin(2 * np.pi * X)
    w[..., 5] = -np.sin(2 * np.pi * Y) / np.sqrt(4 * np.pi)
    w[..., 6] = np.sin(4 * np.pi * X) / np.sqrt(4 * np.pi)
    return w


def div_b(state, dx):
    """Central-difference div B of the cell-averaged field (periodic), on the device: (mean |.|, max |.|)."""
    import torch
    bx, by = state[5].double(), state[6].double()
    d = (torch.roll(bx, -1, 0) - torch.roll(bx, 1, 0)) / (2 * dx) + (torch.roll(by, -1, 1) - torch.roll(by, 1, 1)) / (2 * dx)
    return float(d.abs().mean()), float(d.abs().max())


def mhd_leg(n, steps):
    """Orszag-Tang 1024^2, WENO5 + HLLD + SSPRK3, CFL 0.4: FP32 rate, L1(rho) vs FP64, div B."""
    import torch
    from astrea_gb300.solver import RunConfig, Solver
    w = orszag_tang(n)

    def cfg(prec):
        return RunConfig(dim=2, n0=n, n1=n, model=8, precision=prec, scheme="weno5", solver="hlld",
                         integrator="ssprk33", boundary="wrap", gamma=5.0 / 3.0, dx=1.0 / n, cfl=0.4, t_end=0.5,
                         compat=False)
    res = {}
    for prec in (32, 64):
        s = Solver(cfg(prec))
        s.initialise(w)
        s.reset_clock()
        if prec == 32:
            res["div_b_initial"] = div_b(s.state, 1.0 / n)[0]
        s.step(2, graph=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        s.step(steps, graph=True)
        e1.record()
        torch.cuda.synchronize()
        res[prec] = {"rate": n * n * steps / (e0.elapsed_time(e1) / 1e3), "rho": s.state[0].double().clone(),
                     "div_b": div_b(s.state, 1.0 / n), "clock": s.clock()}
        del s
        torch.cuda.empty_cache()
    l1 = float(torch.mean(torch.abs(res[32]["rho"] - res[64]["rho"])))
    return {"workload": f"Orszag-Tang {n}^2 periodic, WENO5 + HLLD (published form, flag PHYSICAL) + SSPRK3, CFL 0.4, "
                        f"cell-centred B (the reference's constrained transport with an HLL-type solver goes "
                        f"non-finite near t=0.19 on this vortex, in the oracle too)",
            "steps": steps + 2, "t": res[32]["clock"]["t"],
            "fp32": {"value": res[32]["rate"], "unit": "cell-updates/s"},
            "fp64": {"value": res[64]["rate"], "unit": "cell-updates/s"},
            "l1_rho_fp32_vs_fp64": l1,
            "div_b": {"initial_mean_abs": res["div_b_initial"], "fp32_mean_abs": res[32]["div_b"][0],
                      "fp32_max_abs": res[32]["div_b"][1], "fp64_mean_abs": res[64]["div_b"][0],
                      "fp64_max_abs": res[64]["div_b"][1],
                      "form": "central difference of cell-averaged B (the reference has no div B diagnostic)"},
            "status": [int(res[32]["clock"]["status"]), int(res[64]["clock"]["status"])]}


def advance_to(s, t_target, chunk=0.5):
    """Step solver ``s`` until its clock reaches ``t_target``, a checkpoint of its configuration
    (the step that would cross a checkpoint is clipped to land on it, astrea.py:74-78, so the
    clock stops exactly there).  Steps go in chunks of ``chunk`` x the steps estimated to remain
    at the mean dt of the previous chunk (the clock's own dt may be a clipped one), so that a
    chunk does not run past the target.  Returns the clock."""
    prev = None
    while True:
        c = s.clock()
        if c["status"]:
            raise RuntimeError(f"grid stopped (status {c['status']}) at t={c['t']}")
        if c["t"] >= t_target * (1 - 1e-12) or c["done"]:
            return c
        if prev is not None and c["steps"] > prev["steps"] and c["t"] > prev["t"]:
            dt = (c["t"] - prev["t"]) / (c["steps"] - prev["steps"])
            n = max(1, int((t_target - c["t"]) / dt * chunk))
        else:
            n = 1
        prev = c
        s.step(n, graph=True)


def l1_series(make, w, times, twin_ulps=False, t_end=None, checkpoints=None, extra=None):
    """L1 of density, FP32 against FP64, at each of ``times`` (checkpoints of the configurations).

    ``make(precision, t_end, checkpoints)`` gives the RunConfig.  With ``twin_ulps`` a second FP64
    run starts from the same state with every cell's density moved by one unit in the last place
    (up or down, seeded), which measures how far the flow itself separates two runs that differ
    only by round-off.  Returns per time: t, L1(rho) FP32-FP64, [L1(rho) FP64-FP64'], step counts,
    and the wall seconds of each leg."""
    import torch
    from astrea_gb300.solver import Solver
    runs = {"fp32": 32, "fp64": 64}
    if twin_ulps:
        runs["fp64_twin"] = 64
    solvers, wall = {}, {k: 0.0 for k in runs}
    for k, prec in runs.items():
        s = Solver(make(prec, t_end, checkpoints))
        s.initialise(w)
        if k == "fp64_twin":
            g = torch.Generator(device="cpu").manual_seed(SEED)
            up = (torch.rand(s.state[0].shape, generator=g) < .5).to(s.state.device)
            rho = s.state[0]
            s.state[0] = torch.where(up, torch.nextafter(rho, torch.full_like(rho, float("inf"))),
                                     torch.nextafter(rho, torch.full_like(rho, -float("inf"))))
        s.reset_clock()
        solvers[k] = s
    out = []
    for t in times:
        row = {"t": t}
        try:
            for k, s in solvers.items():
                t0 = time.perf_counter()
                c = advance_to(s, t)
                torch.cuda.synchronize()
                wall[k] += time.perf_counter() - t0
                row[f"steps_{k}"] = c["steps"]
                row[f"t_{k}"] = c["t"]
        except RuntimeError as e:  # a grid stopped (non-finite): keep the rows so far
            row["error"] = f"{k}: {e}"
            out.append(row)
            break
        rho64 = solvers["fp64"].state[0]
        row["l1_rho_fp32_vs_fp64"] = float(torch.mean(torch.abs(solvers["fp32"].state[0].double() - rho64)))
        if twin_ulps:
            row["l1_rho_fp64_vs_fp64_ulp_twin"] = float(torch.mean(torch.abs(solvers["fp64_twin"].state[0] - rho64)))
        row["finite"] = bool(all(torch.isfinite(s.state).all() for s in solvers.values()))
        if extra is not None:
            row.update(extra(solvers))
        out.append(row)
    del solvers
    torch.cuda.empty_cache()
    return {"series": out, "wall_s": wall}


def accuracy_shear(n, times, twin_ulps=False):
    """Configuration 2's error measure (L1(rho), FP32 against FP64) at checkpoints up to its end time."""
    w = shear_layer(n)

    def make(prec, t_end, checkpoints):
        from dataclasses import replace
        return replace(run_config(n, prec), t_end=t_end, checkpoints=checkpoints)
    res = l1_series(make, w, times, twin_ulps, t_end=1.0, checkpoints=20)
    res.update({"workload": f"shear layer {n}^2 (the headline method), checkpoints every 0.05 up to t_end=1.0",
                "twin": "FP64 from the same state with every cell's density moved by +-1 ulp (seeded)"
                        if twin_ulps else None})
    return res


def accuracy_mhd(n, times):
    """Configuration 3 (Orszag-Tang, WENO5 + HLLD, CFL 0.4): L1(rho) FP32 against FP64 and div B
    of both, at checkpoints up to t_end=0.5."""
    import torch
    from astrea_gb300.solver import RunConfig, Solver
    w = orszag_tang(n)

    def make(prec, t_end, checkpoints):
        return RunConfig(dim=2, n0=n, n1=n, model=8, precision=prec, scheme="weno5", solver="hlld",
                         integrator="ssprk33", boundary="wrap", gamma=5.0 / 3.0, dx=1.0 / n, cfl=0.4, t_end=t_end,
                         checkpoints=checkpoints, compat=False)
    def divs(solvers):
        # div B of both states, and of the FP64 state rounded to FP32: the floor that FP32 storage
        # alone puts under a central difference (its rounding of B, amplified by 1/(2 dx))
        s64 = solvers["fp64"].state
        return {"div_b_fp32": div_b(solvers["fp32"].state, 1.0 / n)[0], "div_b_fp64": div_b(s64, 1.0 / n)[0],
                "div_b_fp64_rounded_to_fp32": div_b(s64.float(), 1.0 / n)[0]}
    res = l1_series(make, w, times, t_end=0.5, checkpoints=10, extra=divs)
    res["workload"] = (f"Orszag-Tang {n}^2, WENO5 + HLLD (published form) + SSPRK3, CFL 0.4, cell-centred B, "
                       f"checkpoints every 0.05 up to t_end=0.5")
    return res


def accuracy_batched(ngrids=512, seed=SEED, fp64_small=256, fp64_large=(16, 8)):
    """Configuration 4 to its end time (t=0.25): the whole batch in FP32 until every grid is done
    (whole-job cell-updates/s), then per-instance L1(rho) against the batched FP64 engine for every
    instance of at most ``fp64_small``^2 cells and the first ``fp64_large`` (512^2, 1024^2) ones."""
    import torch
    from dataclasses import replace
    from astrea_gb300.batch import Batch
    from astrea_gb300.serving import Request
    rng = np.random.default_rng(seed)
    cfgs, seeds = [], []
    for g in range(ngrids):
        nn = 2 ** int(rng.integers(7, 11))
        ppm = bool(rng.uniform() < .5)
        cfgs.append(batched_cfg(nn, ppm))
        seeds.append(int(rng.integers(1 << 31)))

    def fill(b, sub, idx):
        for g, c in enumerate(sub):
            r = Request(rid=g, arrival=0.0, dim=2, n=4, mhd=False, scheme="plm", solver="llf", t_end=.25,
                        seed=seeds[idx[g]])
            q4 = torch.as_tensor(r.initial_state(), dtype=torch.float64, device="cuda")
            w = q4[[0, 2]][:, [0, 2]].repeat_interleave(c.n0 // 2, 0).repeat_interleave(c.n1 // 2, 1)
            b.initialise_one(g, w)
        torch.cuda.synchronize()

    b = Batch(cfgs)
    fill(b, cfgs, list(range(ngrids)))
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    clk = b.run(check_every=32)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    wall32 = time.perf_counter() - t0
    updates = float(sum(int(clk["steps"][g]) * cfgs[g].n0 * cfgs[g].n1 for g in range(ngrids)))
    rho32 = {g: b.planes(g)[0].double().clone() for g in range(ngrids)}
    st32 = clk["status"].copy()
    # the FP32 wave-speed maximum drops a NaN operand, so a grid can hold non-finite cells with a
    # clean status: such grids count as non-finite too (status bit 0 set here)
    for g in range(ngrids):
        if st32[g] == 0 and not bool(torch.isfinite(b.planes(g)).all()):
            st32[g] |= 1
    del b
    torch.cuda.empty_cache()
    # FP64 reference instances
    picked = [g for g in range(ngrids) if cfgs[g].n0 <= fp64_small]
    for side, count in zip((512, 1024), fp64_large):
        picked += [g for g in range(ngrids) if cfgs[g].n0 == side][:count]
    sub = [replace(cfgs[g], precision=64) for g in picked]
    b64 = Batch(sub)
    fill(b64, sub, picked)
    t1 = time.perf_counter()
    clk64 = b64.run(check_every=32)
    wall64 = time.perf_counter() - t1
    per = []
    for j, g in enumerate(picked):
        ok = st32[g] == 0 and clk64["status"][j] == 0
        l1 = float(torch.mean(torch.abs(rho32[g] - b64.planes(j)[0]))) if ok else None
        per.append({"grid": g, "n": cfgs[g].n0, "scheme": cfgs[g].scheme, "l1_rho": l1,
                    "status32": int(st32[g]), "status64": int(clk64["status"][j])})
    del b64
    torch.cuda.empty_cache()
    l1s = [p["l1_rho"] for p in per if p["l1_rho"] is not None]
    by_n = {}
    for p in per:
        if p["l1_rho"] is not None:
            by_n.setdefault(p["n"], []).append(p["l1_rho"])
    return {"workload": "512 four-quadrant Riemann grids 128^2..1024^2, PLM+LLF/PPM+HLLC 50/50, FP32, to t=0.25",
            "fp32": {"value": updates / (ms / 1e3), "unit": "cell-updates/s", "ms": ms, "wall_s": wall32,
                     "cell_updates": updates, "max_steps": int(clk["steps"].max()),
                     "non_finite_grids": int((st32 != 0).sum()), "t_min": float(clk["t"].min())},
            "fp64_check": {"instances": len(picked), "finite_in_both": len(l1s), "wall_s": wall64,
                           "l1_rho_median": float(np.median(l1s)) if l1s else None,
                           "l1_rho_p90": float(np.percentile(l1s, 90)) if l1s else None,
                           "l1_rho_max": float(np.max(l1s)) if l1s else None,
                           "l1_rho_median_by_side": {str(k): float(np.median(v)) for k, v in sorted(by_n.items())},
                           "non_finite_both": int(sum(1 for p in per if p["status32"] != 0 and p["status64"] != 0)),
                           "non_finite_fp64_only": int(sum(1 for p in per if p["status32"] == 0 and p["status64"] != 0)),
                           "non_finite_fp32_only": int(sum(1 for p in per if p["status32"] != 0 and p["status64"] == 0)),
                           "non_finite_by_scheme": {sch: [int(sum(1 for p in per if p["scheme"] == sch and p["status32"])),
                                                          int(sum(1 for p in per if p["scheme"] == sch and p["status64"])),
                                                          int(sum(1 for p in per if p["scheme"] == sch))]
                                                    for sch in ("plm", "ppm")}},
            "per_instance": per}


def sod_cfg(n):
    from astrea_gb300.solver import RunConfig
    return RunConfig(dim=1, n0=n, model=3, precision=64, scheme="plm", solver="llf", integrator="ssprk33",
                     boundary="edge", gamma=1.4, dx=1.0 / n, cfl=0.8, t_end=0.2)


def sod_point(n):
    w = np.zeros((n, 8))
    w[: n // 2, 0], w[: n // 2, 4] = 1.0, 1.0
    w[n // 2:, 0], w[n // 2:, 4] = .125, .1
    return w


def snapshot_leg(n=512, steps=240, every=20):
    """Cost of the reference's per-step snapshots (astrea.py:47-50) when they are written while the
    device keeps stepping: the headline method at n^2, FP32, with and without snapshots."""
    import shutil
    import tempfile
    import torch
    from astrea_gb300 import snapshots
    from astrea_gb300.solver import Solver
    cfg = run_config(n, 32)
    w0 = shear_layer(n)

    def fresh():
        s = Solver(cfg)
        s.initialise(w0)
        s.reset_clock()
        s.step(3, graph=True)
        s.reset_clock()
        torch.cuda.synchronize()
        return s

    s = fresh()
    t0 = time.perf_counter()
    s.step(steps, graph=True)
    torch.cuda.synchronize()
    plain = time.perf_counter() - t0
    s = fresh()  # (t_end = 1 is far off: the run is bounded by max_snapshots)
    d = tempfile.mkdtemp(prefix="astrea_snap_")
    try:
        store = snapshots.DirectoryStore(d, snapshots.new_file_attrs())
        t0 = time.perf_counter()
        written = snapshots.run_with_snapshots(s, store, "run", every=every, max_snapshots=steps // every)
        torch.cuda.synchronize()
        snap = time.perf_counter() - t0
        nbytes = sum(os.path.getsize(os.path.join(d, "run", f)) for f in os.listdir(os.path.join(d, "run"))
                     if f.endswith(".npy"))
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return {"workload": f"{n}^2 headline method, FP32, {steps} steps, a primitive snapshot every {every} steps "
                        f"(.npy store on the box's disk; the reference writes gzip HDF5 every step)",
            "steps_per_s_plain": steps / plain, "steps_per_s_with_snapshots": len(written) * every / snap,
            "snapshots": len(written), "snapshot_mb": nbytes / 1e6}


def sod_leg(n=4096):
    """The plain method (FP64, reference quirks kept) on the 1D Sod problem to t = 0.2 through Solver.run."""
    import torch
    from astrea_gb300.solver import Solver
    s = Solver(sod_cfg(n))
    s.initialise(sod_point(n))
    s.reset_clock()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    clk = s.run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    return {"workload": f"1D Sod N={n}, PLM-minmod + LLF + SSPRK3, CFL 0.8, to t=0.2, FP64 plain",
            "steps": int(clk["steps"]), "t": clk["t"], "ms": ms, "value": n * clk["steps"] / (ms / 1e3),
            "unit": "cell-updates/s"}, s.conservative().cpu().numpy()


def sod_oracle(n=4096):
    """CPU baseline of the Sod workload (the oracle to t = 0.2, one core) and its final state."""
    from oracle import stepper
    oc = stepper.OracleConfig(dim=1, scheme="plm", solver="llf", integrator="ssprk33", gamma=1.4, bc="edge",
                              dx=1.0 / n, cfl=0.8, eig="analytic", t_end=0.2)
    t0 = time.perf_counter()
    q, t, steps, _dts = stepper.run(stepper.initialise(sod_point(n), oc), oc)
    wall = time.perf_counter() - t0
    return q, t, steps, wall


def serving_leg(count, rates, seed=SEED, max_wall_s=30.0):
    """Seeded request streams at each arrival rate: p50/p99 latency and aggregate cell-updates/s."""
    from astrea_gb300.serving import Server, make_requests
    # the largest request of this mix needs ~2e4 steps; a request past 5e4 has a collapsed time step
    srv = Server(hbm_budget_bytes=150e9, precision=32, max_slots=256, steps_per_poll=8, max_steps=50000)
    sweep = []
    for i, rate in enumerate(rates):
        reqs = make_requests(count, rate, seed=seed + i, n1d=(64, 16384), n2d=(32, 512))
        stats = srv.serve(reqs, max_wall_s=max_wall_s)
        out = stats.summary()
        out["unfinished"] = count - out["requests"]
        out["rate_per_s"] = rate
        sweep.append(out)
    head = dict(sweep[0])
    head.update({"rates": sweep, "requests_per_rate": count,
                 "mix": "40% 1D N log-U[64,16384], 60% 2D side log-U[32,512] (the full mix / 4 per axis), "
                        "Euler|MHD 50/50, {PLM,PPM,WENO5}x{LLF,HLLC|HLLD}, t_end U[.05,.3], CFL 0.8 (1D) / 0.4 (2D), FP32",
                 "hbm_budget_gb": 150})
    return head


def run_alone(r, precision, max_steps=200000):
    """One request solved by the single-grid solver to its end time; returns (status, steps, seconds)."""
    import torch
    from astrea_gb300.solver import Solver
    s = Solver(r.config(precision))
    s.initialise(r.initial_state())
    s.reset_clock()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    status = 0
    try:
        clk = s.run(max_steps=max_steps, check_every=64)
        status = clk["status"] | (0 if clk["done"] else 4)
        steps = clk["steps"]
    except Exception:  # noqa: BLE001 - a non-finite grid raises; its status is what is wanted
        clk = s.clock()
        status, steps = clk["status"] or 1, clk["steps"]
    torch.cuda.synchronize()
    return int(status), int(steps), time.perf_counter() - t0


def serving_full(count, rates, seed=SEED, max_wall_s=1800.0, alone_sample=40, fp64_max_cells=512 * 512):
    """The serving workload at its configured size range (1D N log-U[256, 65536], 2D side log-U[128, 2048],
    150 GB budget): per arrival rate p50/p99 latency and cell-updates/s of the requests that finished cleanly;
    every request that ended non-finite is solved again alone in FP64 (2D ones of at most ``fp64_max_cells``
    cells, 1D ones of at most 16384) to see whether the method or FP32 fails it; and a sample of requests solved one at a time by the
    single-grid solver, for the rate of the same work without batching."""
    import torch
    from astrea_gb300.serving import Server, make_requests
    srv = Server(hbm_budget_bytes=150e9, precision=32, max_slots=256, steps_per_poll=8, max_steps=200000)
    out = {"mix": "40% 1D N log-U[256,65536], 60% 2D side log-U[128,2048], Euler|MHD 50/50, "
                  "{PLM,PPM,WENO5}x{LLF,HLLC|HLLD}, t_end U[.05,.3], CFL 0.8 (1D) / 0.4 (2D), FP32, HBM budget 150 GB",
           "requests_per_rate": count, "rates": []}
    for i, rate in enumerate(rates):
        reqs = make_requests(count, rate, seed=seed + i)
        stats = srv.serve(reqs, max_wall_s=max_wall_s)
        row = stats.summary()
        row["rate_per_s"] = rate
        row["unfinished"] = len(stats.unfinished)
        row["offered_cell_updates"] = float(sum(r.cells * r.steps for r in reqs))
        failed = [r for r in reqs if r.status & 1]
        rerun = []
        for r in failed:
            if (r.dim == 2 and r.cells <= fp64_max_cells) or (r.dim == 1 and r.n <= 16384):
                st, steps, _ = run_alone(r, 64)
                rerun.append({"rid": r.rid, "dim": r.dim, "n": r.n, "mhd": r.mhd, "scheme": r.scheme,
                              "solver": r.solver, "status32": r.status, "status64": st, "steps64": steps})
                torch.cuda.empty_cache()
        row["non_finite"] = len(failed)
        row["non_finite_rerun_fp64"] = len(rerun)
        row["non_finite_also_in_fp64"] = sum(1 for x in rerun if x["status64"] & 1)
        row["rerun"] = rerun
        out["rates"].append(row)
        print(json.dumps({"serving_rate": row}), flush=True)
    # the same kind of work one request at a time (no batching): a seeded sample of the stream
    reqs = make_requests(alone_sample, rates[0], seed=seed + 100)
    upd, secs = 0.0, 0.0
    for r in reqs:
        st, steps, sec = run_alone(r, 32)
        if st == 0:
            upd += r.cells * steps
            secs += sec
        torch.cuda.empty_cache()
    out["alone"] = {"requests": alone_sample, "cell_updates_per_s": upd / max(secs, 1e-9),
                    "note": "the requests that finished cleanly, solved one after another by the single-grid solver "
                            "(graph steps, clock read every 64 steps)"}
    return out


def accuracy_campaign(args):
    """Configurations 2-4 to their end times; one JSON line (not a bench line)."""
    import torch
    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    out = {"accuracy": True}

    def leg(name, fn, *a):
        t0 = time.perf_counter()
        try:
            out[name] = fn(*a)
        except Exception as e:  # noqa: BLE001 - reported in the line
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        out[name + "_s"] = time.perf_counter() - t0
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        print(json.dumps({name: out[name]}), flush=True)

    leg("shear_layer", accuracy_shear, args.n, [0.05, 0.1, 0.25, 0.5, 1.0])
    leg("shear_layer_twin", accuracy_shear, args.twin_n, [0.05, 0.1, 0.25, 0.5, 1.0], True)
    leg("orszag_tang", accuracy_mhd, args.mhd_n, [0.05, 0.1, 0.2, 0.3, 0.4, 0.5])
    leg("batched", accuracy_batched)
    if rank == 0:
        print(json.dumps(out), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--fp64-steps", type=int, default=5)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--batch-steps", type=int, default=10)
    ap.add_argument("--serve-requests", type=int, default=120)
    ap.add_argument("--serve-rates", default="50,500,2000", help="arrival rates (requests/s) of the serving sweep")
    ap.add_argument("--mhd-n", type=int, default=1024)
    ap.add_argument("--mhd-steps", type=int, default=20)
    ap.add_argument("--sod-n", type=int, default=4096)
    ap.add_argument("--cpu-n", type=int, default=256)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched and serving legs")
    ap.add_argument("--only-fp32", action="store_true",
                    help="time the FP32 path only (no FP64, e2e, batched, serving or CPU legs); for profiler captures")
    ap.add_argument("--accuracy", action="store_true",
                    help="only the accuracy campaign: configurations 2-4 run to their end times (FP32 against FP64 "
                         "at checkpoints; an FP64 ulp-twin of the shear layer; the batch against the FP64 batch); "
                         "prints one JSON line")
    ap.add_argument("--twin-n", type=int, default=1024, help="grid of the FP64 ulp-twin of the shear layer")
    ap.add_argument("--serving-full", action="store_true",
                    help="only the serving workload at its configured size range (see --serve-requests, "
                         "--serve-rates); prints one JSON line")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    if args.accuracy:
        return accuracy_campaign(args)
    if args.serving_full:
        import torch
        torch.cuda.set_device(0)
        res = serving_full(args.serve_requests, [float(r) for r in args.serve_rates.split(",")])
        print(json.dumps({"serving_full": res}), flush=True)
        return 0

    import torch
    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    from astrea_gb300 import _lib
    from astrea_gb300.solver import Solver
    n = args.n
    w0 = shear_layer(n)
    cells = n * n

    # ---- FP32 (headline), state resident in HBM: one captured CUDA graph per step
    s32 = Solver(run_config(n, 32))
    s32.initialise(w0)
    s32.reset_clock()
    s32.step(args.warmup, graph=True)
    torch.cuda.synchronize()
    barrier(ws)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as cs:
        torch.cuda.synchronize()
        e0.record(stream)
        s32.step(args.steps, graph=True)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = allmax(e0.elapsed_time(e1), ws)
    barrier(ws)
    value = ws * cells * args.steps / (ms / 1e3)
    clk32 = s32.clock()
    tiles32 = s32.sweep_tiles()
    # the same number of steps again with an event pair around every launch, for the per-kernel
    # times of the roofline (the events cost a few percent of step time, hence a second pass)
    kernel_ms = (ctypes.c_double * 4)()
    launches = (ctypes.c_int * 4)()
    torch.cuda.synchronize()
    _lib.check(s32.lib.astrea_step_timed(s32.handle, ctypes.c_void_p(s32.state.data_ptr()), args.steps,
                                         kernel_ms, launches, ctypes.c_void_p(stream.cuda_stream)))
    torch.cuda.synchronize()

    # roofline of the sweep kernel: algorithmic bytes per launch / mean launch time.  The
    # algorithmic bytes of a cell-update (one SSPRK3 step of one cell) are 8*C*s = 128 B (the
    # stage reads 1 + 2 + 2 and writes 3 state passes; C = 4 stored variables, s = 4 bytes); a
    # step is six sweep launches over every cell, so one launch carries 128 B x cells / 6.
    # (What a launch actually moves is more -- the cell averages in, a divergence or stage
    # result out, and the viscous strip -- and is reported as ``traffic``.)
    C, sz = 4, 4
    sweep_launches = max(launches[0], 1)
    alg_per_launch = 8 * C * sz * cells / 6.0
    achieved = alg_per_launch / (kernel_ms[0] / sweep_launches / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    step_alg = cells * 8 * C * sz  # 8 state passes per SSPRK3 step: the minimum traffic
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": SWEEP_DRAM_BYTES * cells / SWEEP_DRAM_CELLS,
                "kernel": "sweep_kernel (every sweep launch of the timed steps)", "peak_source": peak_kind,
                "alg_bytes_per_launch": alg_per_launch,
                "alg_bytes_per_cell_update": 8 * C * sz,
                "step_frac": step_alg * (value / ws) / cells / 1e9 / peak,
                "note": "issue-bound stencil: hundreds of warp instructions per cell-update against 128 B; "
                        "frac = (128 B x cells / 6) per sweep launch / mean launch time / measured HBM peak",
                "kernel_timing": "CUDA events around every launch, in a second pass of the same steps right after "
                                 "the timed graph replay"}
    if launches[3]:
        ca_bytes = cells * C * sz * 2  # FP32: the state in, one order of cell averages out
        roofline["cell_average_prepass"] = {"launches": launches[3], "ms": kernel_ms[3],
                                            "achieved_gbs": ca_bytes / (kernel_ms[3] / launches[3] / 1e3) / 1e9,
                                            "alg_bytes_per_launch": ca_bytes}

    if args.only_fp32:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                              "config": {"workload": WORKLOAD, "cells": cells}, "only_fp32": True,
                              "kernel_ms": {"sweep": kernel_ms[0], "combine0": kernel_ms[1],
                                            "bookkeeping": kernel_ms[2], "cell_average": kernel_ms[3]},
                              "roofline": roofline}), flush=True)
        return 0

    # ---- FP64 plain, same workload
    s64 = Solver(run_config(n, 64))
    s64.initialise(w0)
    s64.reset_clock()
    s64.step(1, graph=True)
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    s64.step(args.fp64_steps, graph=True)
    f1.record(stream)
    torch.cuda.synchronize()
    ms64 = f0.elapsed_time(f1)
    value64 = cells * args.fp64_steps / (ms64 / 1e3)
    del s64
    torch.cuda.empty_cache()

    # ---- end to end through the C ABI with host buffers (pinned): every step copies the state in
    # from page-locked host memory and leaves its result there (astrea_step_host: the last sweep of
    # the step writes the result to the host buffer while it computes); the result of one step is
    # the input of the next, as in a caller that keeps the grid on the host
    host = torch.empty_like(s32.state, device="cpu").pin_memory()
    host.copy_(s32.state.cpu())
    for _ in range(2):
        s32.step_host(host, host)
    torch.cuda.synchronize()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    for _ in range(args.e2e_steps):
        s32.step_host(host, host)
    g1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = allmax(g0.elapsed_time(g1), ws)
    e2e = ws * cells * args.e2e_steps / (e2e_ms / 1e3)
    # the same with the result copied out after the step (no fused host store), for comparison
    h2 = host.clone().pin_memory()
    for _ in range(2):
        s32.state.copy_(h2, non_blocking=True)
        s32.step(1, graph=True)
        h2.copy_(s32.state, non_blocking=True)
    torch.cuda.synchronize()
    g0.record(stream)
    for _ in range(args.e2e_steps):
        s32.state.copy_(h2, non_blocking=True)
        s32.step(1, graph=True)
        h2.copy_(s32.state, non_blocking=True)
    g1.record(stream)
    torch.cuda.synchronize()
    e2e_copy = ws * cells * args.e2e_steps / (allmax(g0.elapsed_time(g1), ws) / 1e3)
    state_bytes = s32.state.numel() * s32.state.element_size()
    del s32
    torch.cuda.empty_cache()

    def leg(fn, *a):
        """An auxiliary leg: its failure is reported in the line instead of ending the run."""
        try:
            return fn(*a)
        except Exception as e:  # noqa: BLE001 - reported, the headline line still prints
            return {"error": f"{type(e).__name__}: {e}"}
        finally:
            torch.cuda.synchronize()
            torch.cuda.empty_cache()

    # ---- accuracy: L1(rho) of FP32 against FP64 at checkpoints of the run (the workload's error
    # measure).  On the workload's grid at t=0.05; to t_end=1.0 on a 512^2 grid together with an
    # FP64 twin started one ulp away (the 2048^2 FP64 run to t=1.0 takes 11 minutes and the
    # 1024^2 pair 3: ``--accuracy`` runs them)
    accuracy = leg(accuracy_shear, n, [0.05])
    accuracy_t_end = leg(accuracy_shear, 512, [0.05, 0.25, 1.0], True) if not args.no_extras else None

    batched = serving = mhd = sod = sod_state = snaps = mhd_acc = batched_t_end = None
    if not args.no_extras:
        batched = leg(batched_leg, args.batch_steps, 2)
        batched_t_end = leg(accuracy_batched, 512, SEED, 128, (2, 1))
        if isinstance(batched_t_end, dict):
            batched_t_end.pop("per_instance", None)
        mhd_acc = leg(accuracy_mhd, args.mhd_n, [0.05])
        serving = leg(serving_leg, args.serve_requests, [float(r) for r in args.serve_rates.split(",")])
        mhd = leg(mhd_leg, args.mhd_n, args.mhd_steps)
        sod_out = leg(sod_leg, args.sod_n)
        if isinstance(sod_out, tuple):
            sod, sod_state = sod_out
        else:
            sod = sod_out
        snaps = leg(snapshot_leg)
        if rank == 0 and not args.no_cpu and isinstance(batched, dict) and "value" in batched:
            batched["cpu_baseline"] = leg(batched_cpu_baseline)

    cpu = None
    if rank == 0 and not args.no_cpu and sod_state is not None:
        try:
            q, t_o, steps_o, wall = sod_oracle(args.sod_n)
            sod["cpu_baseline"] = {"value": args.sod_n * steps_o / wall, "unit": "cell-updates/s", "cores": 1,
                                   "kind": "port",
                                   "sample": f"the whole run ({steps_o} steps), oracle with closed-form wave speeds "
                                             f"(the reference's LAPACK path is slower), 1 core"}
            sod["steps_oracle"] = steps_o
            sod["rel_err_vs_oracle"] = float(np.max(np.abs(sod_state - q)) / np.max(np.abs(q)))
            sod["l1_rho_vs_oracle"] = float(np.mean(np.abs(sod_state[:, 0] - q[:, 0])))
        except Exception as e:  # noqa: BLE001 - reported in the line
            sod["oracle_error"] = f"{type(e).__name__}: {e}"
    if rank == 0 and not args.no_cpu:
        try:
            v, cores = cpu_baseline(args.cpu_n, 1, args.cpu_steps)
            cpu = {"value": v, "unit": "cell-updates/s", "cores": cores, "kind": "port",
                   "sample": f"{args.cpu_steps} SSPRK3 steps of a {args.cpu_n}^2 instance of the workload, oracle "
                             f"(NumPy restatement of the reference, LAPACK wave speeds as in the reference), 1 core"}
        except Exception as e:  # noqa: BLE001 - reported in the line
            cpu = {"error": f"{type(e).__name__}: {e}"}

    if rank == 0:
        clocks = cs.summary()
        line = {
            "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "cells": cells, "precision": "fp32 (FP64 pressure recovery)",
                       "hllc": "textbook (flag PHYSICAL)",
                       "flattening_viscosity": "flags FLATTEN|VISCOSITY; the reference's code for both fails when "
                                               "called, formulas per the cited papers (parity unpinned)",
                       "parallelism": f"replicas x{ws}",
                       "l2": "working set 5 x 67 MB > L2: inputs larger than L2",
                       "sweep_tiles": tiles32, "tiles_from": "autotuner (timed on the grid at the first step)"},
            "fp64_plain": {"value": value64, "unit": "cell-updates/s", "steps": args.fp64_steps,
                           "ms_per_step": ms64 / args.fp64_steps},
            "fp32_over_fp64": value / ws / value64,
            # same precision against the reference's algorithm on the host: the FP64 plain GPU path over
            # the oracle on one core (FP64, LAPACK wave speeds); the reference arm runs it on every core
            "fp64_over_cpu_baseline_per_core": (value64 / cpu["value"]) if isinstance(cpu, dict) and cpu.get("value")
                                               else None,
            "l1_rho_fp32_vs_fp64": (accuracy.get("series") or [{}])[0].get("l1_rho_fp32_vs_fp64")
                                   if isinstance(accuracy, dict) else None,
            "l1_at_t": 0.05,
            "accuracy": accuracy, "accuracy_t_end_512": accuracy_t_end,
            "roofline": roofline,
            "alu_roofline": alu_roofline(value / ws, value64, (clocks or {}).get("sm_max_mhz")),
            "kernel_ms": {"sweep": kernel_ms[0], "combine0": kernel_ms[1], "bookkeeping": kernel_ms[2],
                          "cell_average": kernel_ms[3]},
            "gpu_launches": sum(launches),
            "launches_per_step": sum(launches) / args.steps,
            "e2e": {"value": e2e, "unit": "cell-updates/s", "h2d_bytes_per_step": state_bytes,
                    "d2h_bytes_per_step": state_bytes, "steps": args.e2e_steps,
                    "path": "astrea_step_host: H2D copy of the state, the step, the result stored to the pinned host "
                            "buffer by the last sweep",
                    "with_copy_after_step": e2e_copy},
            "batched": batched,
            "serving": serving,
            "mhd_orszag_tang": mhd,
            "mhd_accuracy": mhd_acc,
            "batched_to_t_end": batched_t_end,
            "sod_1d": sod,
            "snapshots": snaps,
            "clocks": clocks,
            "cpu_baseline": cpu,
            "t_simulated": clk32["t"],
        }
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
