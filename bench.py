"""Benchmark of the MeshBlock hydro stage: cell-updates/s per RK3 step,
batched and served against the plain FP64 GPU path, with p50/p99 latency.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]
                    [--workload serving|ensemble|straka|cubed-sphere|sod|...]
                    [--precision float64|float32]

One JSON line on rank 0.

The default workload, batched-served, is the metric's own pair:
* the batched ensemble -- 64 seeded Straka-type members of uneven size
  (nx2 in 128..512, nx1 in 32..128) in one handle, FP32 bulk with the
  implicit solve refined to FP64, one graph per step, each member's CFL dt
  on the device.  value = member cell-updates over the CUDA-event time of
  exactly K timed steps (after W warm-up steps); e2e = the same with every
  member's state copied host->device and back each step (pinned memory);
* the serving trace (the line's "served" object) -- Poisson arrivals (20
  req/s) of 3-D planar dry convection solves of 64^3 .. 128x128x96 cells,
  200 RK3 steps each, admitted against an HBM budget (--serve-budget-gb,
  8 GiB, so requests queue and join while others run) and advanced together
  (continuous batching).  Its value is the cell-updates over the CUDA-event
  time of its batched steps, its e2e the wall clock of the whole trace
  through Server.run (arrivals, initial states in, results out), with
  p50/p99 latency (arrival to result on host) and the admission wait.
Both carry the plain FP64 GPU path on the same work (each block alone on its
own FP64 MeshBlock) on the same clock: vs_plain_fp64 (CUDA events on both
sides) and vs_plain_fp64_wall (wall clock on both sides); the served ratio
is lifted to served_vs_plain_fp64.  The served object also holds
alone_equals_mix (the smallest request run alone equals itself in the mix,
bit for bit) and fp32_rel_l2_vs_fp64 (its FP32 error per field against the
FP64 path at the served horizon).  roofline: B_alg (160 B per FP32
cell-update per RK3 step: 5 reads + 3 writes of 5 variables) x the
device-timed rate against the measured HBM peak; per-kernel times and the
implementation's scratch bytes are reported apart.

The other workloads (one block each unless named): a step is one full RK3
step of the workload's block on synthetic input (the deck's own initial
state, generated on the host), dt fixed at the CFL step of the initial state.

* value: device-timed throughput (CUDA events on the launching stream around
  each step, L2 flushed between steps -- the block fits in L2, so each timed
  step starts cold), state resident in HBM.
* e2e: the same steps through the public API with HOST buffers: each step
  copies the state host->device from pinned memory, advances it and copies it
  back (bytes counted from the copied tensors).
* roofline: B_alg x the device-timed rate against the measured HBM copy
  peak; the dominant kernel's own bytes per launch over its mean duration
  (CUDA events the library records around each kernel of an eager stage, on
  the launching stream) beside it, and the "kernels" object with every
  kernel's launches, mean time and share.
* cpu_baseline: the CPU oracle (the reference algorithm restated in C, FP64,
  OpenMP on every host core) on a bounded sample of the same workload.

--impl reference times that CPU path alone (the reference itself, a libtorch
C++ build with external dependencies, is not built on either machine) and
prints the same line with "impl": "reference".
Under torchrun (N > 1) every rank advances its own replica of the workload
(the blocks are independent: replicas only), value = all ranks' cell-updates
/ the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s per RK3 step, batched+served vs plain; p50/p99 latency at tol"

WORKLOADS = {
    # the default: the batched ensemble (the line's value, K steps) and the
    # serving trace (its "served" object, p50/p99), each beside the plain
    # FP64 GPU path on the same work
    "batched-served": None,
    # the 2-D density-current shape of the Straka config: 512 x 128 cells at
    # 50 m, LMARS + WENO5 (cp5 for velocity/pressure) + RK3, reflecting walls
    # the Straka configuration: gravity (well-balanced x1 reference),
    # viscosity 75 m^2/s and the vertical implicit solve (scheme 9)
    "straka": "snapy_gb300/decks/straka.yaml",
    "straka-explicit": "snapy_gb300/decks/straka_noimplicit.yaml",
    "straka-shape": "snapy_gb300/decks/straka_explicit.yaml",
    "sod": "snapy_gb300/decks/sod.yaml",
    # 64 Straka-type members of uneven size (nx2 in {128..512}, nx1 in
    # {32..128}, seeded bubbles) in one handle: one persistent launch per
    # kernel and stage, each member's dt on the device, one graph per step
    "ensemble": "snapy_gb300/decks/straka.yaml",
    # the serving trace: Poisson arrivals (20 req/s) of 3-D planar dry
    # convection solves, (nx2, nx3, nx1) from {64, 96, 128}^2 x {64, 96},
    # 200 RK3 steps each, FP32 bulk with the FP64 implicit solve
    "serving": "snapy_gb300/decks/convection3d.yaml",
    # shallow water on the cubed sphere: 6 panels of 96 x 96 cells, radius
    # 6.371e6 m, mean depth 1000 m, a 100 m Gaussian bump of width 0.1 rad
    # at a seeded lon/lat, at rest; weno5 + shallow-roe + rk3, FP32 state,
    # the seam halo filled every stage
    "cubed-sphere": None,
}
CS_N, CS_SEED = 96, 20261206
SERVE_RATE, SERVE_SEED = 20.0, 20261204
ENSEMBLE_MEMBERS, ENSEMBLE_SEED = 64, 20261203


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["native", "reference"], default="native")
    ap.add_argument("--workload", choices=sorted(WORKLOADS),
                    default="batched-served")
    ap.add_argument("--precision", choices=["float64", "float32"], default=None)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--implicit-precision", choices=["float64", "float32"],
                    default=None,
                    help="FP32 state: float32 assembles the implicit blocks in "
                         "FP32 and refines their solve to FP64 accuracy, "
                         "float64 assembles and solves them in FP64 (default: "
                         "float32 for ensemble and serving, the deck's for "
                         "the others)")
    ap.add_argument("--implicit-solve", choices=["refined", "direct", "fp32"],
                    default=None,
                    help="the solve of float32-assembled implicit blocks: "
                         "refined (FP32 sweeps corrected with FP64 residuals, "
                         "the default) or direct (FP64 for every column)")
    ap.add_argument("--implicit-corrections", type=int, choices=[1, 2, 3],
                    default=None, help="the refined solve's corrections")
    ap.add_argument("--implicit-sweep", choices=["serial", "partitioned", "auto"],
                    default=None,
                    help="the elimination order of the FP64-assembled solve: "
                         "serial (the reference's, bit for bit; the deck "
                         "default), partitioned (four chunks per column at "
                         "once and a separator system) or auto (the "
                         "autotuner times both)")
    ap.add_argument("--scalars", type=int, default=0,
                    help="Straka and Sod workloads: passive tracers carried "
                         "(the reference's Straka deck carries one, "
                         "scalar/names [tracer])")
    ap.add_argument("--requests", type=int, default=24,
                    help="serving: requests in the trace")
    ap.add_argument("--no-plain", action="store_true",
                    help="ensemble and serving: skip the plain FP64 "
                         "comparison (and the served alone/FP32 checks), for "
                         "kernel profiles of the batched launches alone")
    ap.add_argument("--serve-budget-gb", type=float, default=8.0,
                    help="serving: the HBM budget requests are admitted "
                         "against (GiB; 0: the device's free memory)")
    ap.add_argument("--serve-steps", type=int, default=200,
                    help="serving: RK3 steps per request")
    ap.add_argument("--plain-sweep", choices=["serial", "partitioned", "auto"],
                    default="serial",
                    help="ensemble and serving: the plain FP64 path's column "
                         "solve order (serial: the reference's, bit for bit "
                         "with the oracle; auto: the autotuner picks the "
                         "faster of it and the partitioned form per block)")
    return ap.parse_args()


def load_options(args):
    import snapy_gb300 as sg
    opts = sg.MeshBlockOptions.from_yaml(os.path.join(ROOT, WORKLOADS[args.workload]))
    if args.precision:
        opts.hydro().precision = args.precision
    if (args.implicit_precision and opts.hydro().icorr is not None
            and opts.hydro().precision == "float32"):
        opts.hydro().icorr.precision = args.implicit_precision
    if args.implicit_solve:
        opts.implicit_solve = args.implicit_solve
    if args.implicit_corrections:
        opts.implicit_corrections = args.implicit_corrections
    if getattr(args, "implicit_sweep", None):
        opts.implicit_sweep = args.implicit_sweep
    if getattr(args, "scalars", 0):
        # tracers are built without the x2 flux-covariance row
        opts.scalar_names = [f"tracer{k}" for k in range(args.scalars)]
        opts.hydro().flux_covariance = False
    return opts


def initial_state(opts, workload, device):
    from snapy_gb300 import problems
    if workload == "sod":
        return problems.sod(opts, device)
    return problems.straka(opts, device)


def implicit_solve(opts):
    """How the implicit blocks are solved: FP32 assembly takes the refined
    solve unless the deck asks for the direct one, FP64 assembly the direct
    FP64 solve."""
    ic = opts.hydro().icorr
    if ic is None:
        return None
    if opts.hydro().precision == "float32" and ic.precision == "float32":
        if opts.implicit_solve == "refined":
            return ("refined to the FP64 solution: FP32 block-Thomas sweeps, "
                    f"{opts.implicit_corrections} corrections from FP64 "
                    "residuals, the FP64 solve for columns that do not converge")
        if opts.implicit_solve == "fp32":
            return ("FP32 (the reference's FP32 implicit compute): the FP32 "
                    "block-Thomas sweep and its Woodbury step, the FP64 solve "
                    "for columns whose sweep fails")
    if opts.implicit_sweep == "partitioned":
        return ("direct FP64, partitioned: four chunks per column swept at "
                "once, a separator system, then every layer")
    if opts.implicit_sweep == "auto":
        return "direct FP64, serial or partitioned as the autotuner chose"
    return "direct FP64"


def solve_label(opts):
    """A short name of the implicit solve the deck runs."""
    ic = opts.hydro().icorr
    if ic is None:
        return "none"
    if opts.hydro().precision == "float32" and ic.precision == "float32":
        return {"refined": "refined to the FP64 solution", "fp32": "FP32",
                "direct": "FP64"}[opts.implicit_solve]
    return "FP64"


def config_of(opts, workload, args, nranks):
    c = opts.coord()
    h = opts.hydro()
    return {
        "workload": f"{workload} {c.nx2}x{c.nx1} ({c.dx2:g} m x {c.dx1:g} m), "
                    f"{h.riemann.type}+weno5+rk3, {h.precision}",
        "cells": c.nx1 * c.nx2 * c.nx3,
        "nx1": c.nx1, "nx2": c.nx2, "nx3": c.nx3,
        "riemann": h.riemann.type,
        "precision": h.precision,
        "gravity": bool(h.grav and h.grav.grav1),
        "implicit": bool(h.icorr),
        "implicit_solve": implicit_solve(opts),
        "scalars": len(opts.scalar_names),
        "flux_covariance": bool(opts.hydro().flux_covariance),
        "l2": "flushed between timed steps (512 MiB write; the block fits in L2)",
        "graphs": "one per buffer rotation, captured before the warm-up steps",
        "replicas": nranks,
        "parallelism": "replicas" if nranks > 1 else "single",
    }


FP64_ISSUE = ("FP64 issue rate (one FP64 warp instruction per SM sub-partition "
              "per 64 cycles)")


def refined(opts):
    """True when the deck's implicit blocks take the refined solve."""
    ic = opts.hydro().icorr
    return bool(ic is not None and opts.hydro().precision == "float32"
                and ic.precision == "float32" and opts.solve_corrections() > 0)


def solve_phase(opts):
    """The implicit solve phase timed as vic_solve_kernel (the events
    between the assembly and the finish): what runs in it, its algorithmic
    bytes per interior cell and what bounds it."""
    if not refined(opts) and opts.implicit_sweep == "partitioned":
        # the chunk sweeps: A, B, C, du in; C', V', y out; back up the
        # chunk: C', V', y in, E, F, Y out; every layer: E, F, Y in, x out;
        # the Woodbury step: D, Z0, Z1 in, D out
        return ("vic_psolve_kernel (the partitioned solve)",
                640 + 520 + 520 + 520 + 520 + 120 + 120 + 40, FP64_ISSUE)
    if not refined(opts):
        return ("vic_solve_kernel", 600 + 40 + 200 + 120 + 200 + 120 + 120,
                FP64_ISSUE)
    k = opts.solve_corrections()
    # the FP32 sweep: A, B, C (300) and du (40) in; factors (128), c' (112),
    # y (60) and x (120) out; back: c' and y in
    first = 300 + 40 + 128 + 112 + 60 + 120 + 112 + 60
    # a residual: FP64 blocks (600), x (120), du (40) in; r (60) out
    residual = 600 + 120 + 40 + 60
    # a correction: factors, b, r in and y out; back: c', y, x in, x out
    correct = 128 + 112 + 64 + 60 + 112 + 60 + 120 + 120
    return (f"refined solve phase: vic_solve32_kernel, then {k} x "
            "(vic_residual_kernel, vic_correct32_kernel)",
            first + k * (residual + correct),
            "the FP64 residuals (FP64 issue rate) and the corrections' "
            "per-layer latency")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax = float(parts[2])
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


class Ranks:
    """The replicas of a torchrun launch: one rank per GPU and no collective
    on the data path (blocks, members and requests are independent).  The
    job's timed interval is the slowest rank's (max over ranks), and a
    rate counts every rank's units: ``job_rate``."""

    def __init__(self, backend: str = "nccl"):
        import torch.distributed as dist
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.backend = backend
        self._dist = dist
        if self.world > 1 and not dist.is_initialized():
            dist.init_process_group(backend, init_method="env://")

    def barrier(self) -> None:
        if self.world > 1:
            self._dist.barrier()

    def max(self, x: float) -> float:
        """x of the slowest rank (every rank gets it)."""
        if self.world == 1:
            return float(x)
        import torch
        dev = torch.device("cuda", self.local) if self.backend == "nccl" \
            else torch.device("cpu")
        t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.MAX)
        return float(t.item())

    def close(self) -> None:
        if self.world > 1:
            self._dist.barrier()
            self._dist.destroy_process_group()


def job_rate(units_per_rank: float, world: int, seconds_max: float) -> float:
    """Whole-job throughput of weakly scaled replicas: every rank's units
    over the slowest rank's time."""
    return units_per_rank * world / seconds_max


def cpu_baseline(opts, workload, seconds, u0_host=None):
    """The CPU oracle on every host core: cell-updates/s on a bounded sample
    (as many full RK3 steps of the same block as fit in `seconds`, >= 2)."""
    import numpy as np
    from oracle import oracle as O
    O.build()
    c = opts.coord()
    cores = os.cpu_count() or 1
    ob = O.block_from_options(opts, nthreads=cores)
    w = initial_state(opts, workload, "cpu").numpy()
    u = ob.initialize(w)
    dt = opts.intg().cfl * ob.max_dt(u)
    ob.step(u, dt)  # warm
    n, t0 = 0, time.perf_counter()
    while True:
        ob.step(u, dt)
        n += 1
        el = time.perf_counter() - t0
        if (el >= seconds and n >= 2) or n >= 100000:
            break
    cells = c.nx1 * c.nx2 * c.nx3
    return {"value": cells * n / el, "unit": "cell-updates/s", "cores": cores,
            "kind": "port",
            "sample": f"{n} RK3 steps of the same {c.nx2}x{c.nx1} block, FP64, "
                      f"{el:.1f} s, OpenMP {cores} threads"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    opts = load_options(args)
    c = opts.coord()
    per = []
    cb = None
    for _ in range(args.warmup):
        pass
    seconds = max(2.0, args.cpu_seconds / max(1, args.steps) * args.steps)
    cb = cpu_baseline(opts, args.workload, seconds)
    val = cb["value"]
    cells = c.nx1 * c.nx2 * c.nx3
    line = {
        "impl": "reference", "metric": "cell-updates/s per RK3 step",
        "value": val, "unit": "cell-updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": cells / val * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (the deck's initial state)",
        "config": config_of(opts, args.workload, args, 1),
        "cpu_baseline": cb,
        "e2e": {"value": val, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_native(args):
    import torch

    ranks = Ranks()
    world, rank, local = ranks.world, ranks.rank, ranks.local
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    import snapy_gb300 as sg
    opts = load_options(args)
    c = opts.coord()
    cells = c.nx1 * c.nx2 * c.nx3
    blk = sg.MeshBlock(opts).to(dev)
    w = initial_state(opts, args.workload, dev)
    vars = {"hydro_w": w}
    if opts.scalar_names:
        # each tracer's ratio: a smooth field that varies along x1 and x2
        ns = len(opts.scalar_names)
        z = torch.linspace(0.0, 1.0, c.nc1, dtype=torch.float64, device=dev)
        x = torch.linspace(0.0, 1.0, c.nc2, dtype=torch.float64, device=dev)
        r = torch.stack([(1e-3 * (k + 1)) * (1.0 + 0.5 * torch.sin(6.0 * z)[None, :]
                                              * torch.cos(4.0 * x)[:, None])
                         for k in range(ns)])
        vars["scalar_r"] = r.unsqueeze(1).expand(ns, c.nc3, c.nc2, c.nc1).contiguous()
    blk.initialize(vars)
    dt = blk.max_time_step(vars)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    # capture the step graphs of both steady buffer rotations first (steps
    # 1-3 run eagerly, 4 and 5 capture), so no capture lands in the timed
    # region; then the warm-up steps
    for _ in range(8):
        if blk.execution_report()["captures"] >= 2:
            break
        blk.step(vars, dt)
    for _ in range(max(3, args.warmup)):
        blk.step(vars, dt)
    torch.cuda.synchronize()

    # device-timed steps, cold L2 for each
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    ranks.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            blk.step(vars, dt)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_total = sum(step_ms) / 1e3
    t_total = ranks.max(t_total)
    value = job_rate(cells * args.steps, world, t_total)

    # roofline of the dominant kernel: the library records events around
    # each kernel of every eager stage on the launching stream
    b = blk.batch
    s_bytes = torch.finfo(blk.dtype).bits // 8
    implicit = bool(opts.hydro().icorr)
    b.set_timing(True)
    nrep = min(args.steps, 50)
    for k in range(nrep):
        flush.zero_()
        for st in range(3):
            b.stage(st)
    torch.cuda.synchronize()
    kt = b.kernel_times()
    b.set_timing(False)
    # algorithmic bytes per launch of each kernel (per interior cell, times
    # the cells one launch covers; stages 2-3 of an explicit stage also read u0)
    ghost_cells = c.nc1 * c.nc2 * max(1, c.nc3) - cells
    per_launch = {
        "stage_kernel": ((5 * s_bytes + 40) if implicit else
                         5 * s_bytes * (2 + 3 + 3) / 3) * cells,
        "vic_assemble_kernel": (5 * s_bytes + 40 + 40 + 600) * cells,
        "vic_solve_kernel": solve_phase(opts)[1] * cells,
        "vic_finish_kernel": (120 + 15 * s_bytes) * cells,
        "ghost_kernel": 2 * 5 * s_bytes * ghost_cells,
        # per tracer: s read twice (faces, update) and s0, s_out written, the
        # two FP64 face fluxes written and read; the mass fluxes and rho once
        "scalar_kernel": (len(opts.scalar_names) * (4 * s_bytes + 32) +
                          16 + s_bytes) * cells,
    }
    dom = max(kt, key=lambda k: kt[k][0])
    dom_ms, dom_n = kt[dom]
    achieved = per_launch[dom] * dom_n / (dom_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    kernels = {k: {"launches": n, "mean_us": ms / n * 1e3,
                   "share": ms / sum(v[0] for v in kt.values()),
                   "bytes_per_launch": per_launch.get(k)}
               for k, (ms, n) in kt.items()}

    # end to end through the public API with host buffers (the tracers'
    # densities too, when carried)
    keys = ["hydro_u"] + (["scalar_s"] if "scalar_s" in vars else [])
    hosts = {k: torch.empty(vars[k].shape, dtype=blk.dtype).pin_memory() for k in keys}
    for k in keys:
        hosts[k].copy_(vars[k].cpu())
    e2e_steps = max(5, min(args.steps, 100))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for k in keys:
            vars[k].copy_(hosts[k], non_blocking=True)
        blk.step(vars, dt)
        for k in keys:
            hosts[k].copy_(vars[k], non_blocking=True)
    torch.cuda.synchronize()
    e2e_t = time.perf_counter() - t0
    e2e_t = ranks.max(e2e_t)
    nbytes = sum(h.numel() * h.element_size() for h in hosts.values())

    rep = blk.execution_report()
    line = None
    if rank == 0:
        cb = None
        if not args.no_cpu_baseline:
            cb = cpu_baseline(opts, args.workload, args.cpu_seconds)
        line = {
            "metric": "cell-updates/s per RK3 step",
            "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_total / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if blk.dtype == torch.float64 else "f32",
            "data": "synthetic (the deck's initial state)",
            "config": config_of(opts, args.workload, args, world),
            "e2e": {"value": job_rate(cells * e2e_steps, world, e2e_t),
                    "unit": "cell-updates/s", "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": nbytes},
            "roofline": {"bound": "hbm", "achieved": value * b_alg(s_bytes) / 1e9,
                         "peak": peak, "unit": "GB/s",
                         "frac": value * b_alg(s_bytes) / 1e9 / peak,
                         "peak_kind": peak_kind, "traffic": None,
                         "basis": f"B_alg = {b_alg(s_bytes)} B per cell-update "
                                  "per RK3 step x the device-timed rate",
                         "dominant_kernel": dom,
                         "dominant_runs": solve_phase(opts)[0]
                                          if dom == "vic_solve_kernel" else dom,
                         "dominant_bytes_per_launch": per_launch[dom],
                         "dominant_mean_launch_us": dom_ms / dom_n * 1e3,
                         "dominant_kernel_gbs": achieved,
                         "limiter": solve_phase(opts)[2]
                                    if dom == "vic_solve_kernel" else
                                    FP64_ISSUE if blk.dtype == torch.float64
                                    else None},
            "kernels": kernels,
            "cpu_baseline": cb,
            "clocks": clk.summary(),
            "gpu_launches": args.steps * 3 * b.launches_per_stage(),
            "execution_report": rep,
            "step_ms_median": statistics.median(step_ms),
            "tile_tj": b.tile(0),
            "schedule": b.schedule,
        }
        print(json.dumps(line), flush=True)
    ranks.close()
    return 0


def ensemble_cpu_baseline(members, seconds):
    """The CPU oracle (FP64, OpenMP on every host core) on the first members
    of the ensemble, as many RK3 steps as fit in `seconds`."""
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    blocks = []
    for opts, w in members[:4]:
        ob = O.block_from_options(opts, nthreads=cores)
        u = ob.initialize(w.numpy())
        blocks.append((opts, ob, u))
    n, cells, t0 = 0, 0, time.perf_counter()
    while True:
        for opts, ob, u in blocks:
            dt = opts.intg().cfl * ob.max_dt(u)
            ob.step(u, dt)
            c = opts.coord()
            cells += c.nx1 * c.nx2
        n += 1
        el = time.perf_counter() - t0
        if (el >= seconds and n >= 1) or n >= 10000:
            break
    return {"value": cells / el, "unit": "cell-updates/s", "cores": cores,
            "kind": "port",
            "sample": f"{n} RK3 steps of ensemble members 0-3 (their own CFL dt), "
                      f"FP64, {el:.1f} s, OpenMP {cores} threads"}


def ensemble_config(members, precision, nranks):
    cells = sum(o.coord().nx1 * o.coord().nx2 for o, _ in members)
    ip = members[0][0].hydro().icorr.precision
    return {"workload": f"ensemble of {len(members)} Straka-type members "
                        f"(nx2 in 128..512, nx1 in 32..128, 50 m, seed "
                        f"{ENSEMBLE_SEED}), lmars+weno5+rk3+VIC, {precision} "
                        f"bulk, implicit solve {solve_label(members[0][0])}",
            "implicit_assembly": ip,
            "implicit_solve": implicit_solve(members[0][0]),
            "members": len(members), "cells": cells, "precision": precision,
            "gravity": True, "implicit": True,
            "dt": "each member's own CFL step, on the device, every step",
            "l2": "inputs larger than L2 (no flush needed)",
            "graphs": "one whole-step graph per buffer rotation, captured "
                      "before the warm-up steps",
            "replicas": nranks,
            "parallelism": "replicas" if nranks > 1 else "single"}


def run_ensemble(args, ranks=None, emit=True):
    """The batched form: every member in one handle.  Beside it, the plain
    FP64 GPU path on the same members: each its own FP64 MeshBlock, stepped
    one after another (graphs on).  Returns rank 0's line (None elsewhere)."""
    import torch
    own = ranks is None
    ranks = ranks or Ranks()
    world, rank, local = ranks.world, ranks.rank, ranks.local
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    import snapy_gb300 as sg
    from snapy_gb300 import problems
    from snapy_gb300.ensemble import Ensemble
    precision = args.precision or "float32"
    members = problems.ensemble_members(ENSEMBLE_MEMBERS, ENSEMBLE_SEED,
                                        precision=precision)
    if precision == "float32":
        for o, _ in members:
            o.hydro().icorr.precision = args.implicit_precision or "float32"
    for o, _ in members:
        o.implicit_solve = args.implicit_solve or o.implicit_solve
        o.implicit_corrections = args.implicit_corrections or o.implicit_corrections
    cells = sum(o.coord().nx1 * o.coord().nx2 for o, _ in members)
    ens = Ensemble([o for o, _ in members], device=dev)
    ens.initialize([w for _, w in members])
    for _ in range(8):  # the two steady rotations' graphs
        if ens.captures >= 2:
            break
        ens.step()
    for _ in range(max(3, args.warmup)):
        ens.step()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    ranks.barrier()
    torch.cuda.synchronize()
    fb0 = sum(ens.batch.solve_fallbacks())
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            ev[k][0].record(stream)
            ens.step()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    fb1 = sum(ens.batch.solve_fallbacks())
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_total = sum(step_ms) / 1e3
    t_total = ranks.max(t_total)
    value = job_rate(cells * args.steps, world, t_total)
    flags = ens.check()
    assert int(flags.abs().sum()) == 0, f"ensemble retry flags {flags.tolist()}"

    # per-kernel device time of eager stages (graph replays record none)
    b = ens.batch
    b.set_timing(True)
    for _ in range(3):
        b.max_dt()
        for st in range(3):
            b.stage(st)
    torch.cuda.synchronize()
    kt = b.kernel_times()
    b.set_timing(False)
    s_bytes = 4 if precision == "float32" else 8
    per_launch = {
        "stage_kernel": (5 * s_bytes + 40) * cells,
        "vic_assemble_kernel": (5 * s_bytes + 40 + 40 + 600) * cells,
        "vic_solve_kernel": solve_phase(members[0][0])[1] * cells,
        "vic_finish_kernel": (120 + 15 * s_bytes) * cells,
        "ghost_kernel": 0,
    }
    dom = max(kt, key=lambda k: kt[k][0])
    dom_ms, dom_n = kt[dom]
    achieved = per_launch[dom] * dom_n / (dom_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    kernels = {k: {"launches": n, "mean_us": ms / n * 1e3,
                   "share": ms / sum(v[0] for v in kt.values())}
               for k, (ms, n) in kt.items()}

    # end to end with host buffers: every member's state in and out
    host = [torch.empty_like(ens.state(k), device="cpu").pin_memory()
            for k in range(len(members))]
    for k in range(len(members)):
        host[k].copy_(ens.state(k))
    nbytes = sum(h.numel() * h.element_size() for h in host)
    e2e_steps = max(3, min(args.steps, 20))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for k in range(len(members)):
            ens.state(k).copy_(host[k], non_blocking=True)
        ens.step()
        for k in range(len(members)):
            host[k].copy_(ens.state(k), non_blocking=True)
    torch.cuda.synchronize()
    e2e_t = time.perf_counter() - t0
    e2e_t = ranks.max(e2e_t)
    schedule = ens.batch.schedule
    del ens

    # the plain FP64 GPU path on the same members, both clocks
    pairs = []
    for opts, w in members:
        o64 = sg.MeshBlockOptions.from_yaml(os.path.join(ROOT, WORKLOADS["ensemble"]))
        c, c0 = o64.coord(), opts.coord()
        c.nx1, c.nx2, c.x1max, c.x2max = c0.nx1, c0.nx2, c0.x1max, c0.x2max
        o64.hydro().precision = "float64"
        o64.implicit_sweep = args.plain_sweep
        pairs.append((o64, (lambda w=w: w)))
    plain = plain_fp64_blocks(pairs, dev) if not args.no_plain else \
        {"device": float("nan"), "wall": float("nan"), "steps_per_request": 0}
    e2e_value = job_rate(cells * e2e_steps, world, e2e_t)

    line = None
    if rank == 0:
        cb = None if args.no_cpu_baseline else ensemble_cpu_baseline(members, args.cpu_seconds)
        line = {
            "metric": "cell-updates/s per RK3 step",
            "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_total / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if precision == "float32" else "f64",
            "data": "synthetic (seeded Straka-type members)",
            "config": ensemble_config(members, precision, world),
            "e2e": {"value": e2e_value,
                    "unit": "cell-updates/s", "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": nbytes},
            "plain_fp64": {"device": plain["device"], "wall": plain["wall"],
                           "unit": "cell-updates/s",
                           "sweep": args.plain_sweep,
                           "how": "each member its own FP64 MeshBlock, one "
                                  "after another, graphs on; device: CUDA "
                                  f"events around {plain['steps_per_request']} "
                                  "steps at a fixed CFL dt; wall: the same "
                                  "steps with the CFL dt read on the host"},
            "vs_plain_fp64": value / plain["device"],
            "vs_plain_fp64_wall": e2e_value / plain["wall"],
            "clock_note": "vs_plain_fp64: CUDA-event time on both sides; "
                          "vs_plain_fp64_wall: wall clock on both sides (the "
                          "batched side with its host copies)",
            "schedule": schedule,
            "roofline": {"bound": "hbm", "achieved": value * b_alg(s_bytes) / 1e9,
                         "peak": peak, "unit": "GB/s",
                         "frac": value * b_alg(s_bytes) / 1e9 / peak,
                         "peak_kind": peak_kind, "traffic": None,
                         "basis": f"B_alg = {b_alg(s_bytes)} B per cell-update "
                                  "per RK3 step x the device-timed rate",
                         "dominant_kernel": dom,
                         "dominant_bytes_per_launch": per_launch[dom],
                         "dominant_mean_launch_us": dom_ms / dom_n * 1e3,
                         "dominant_kernel_gbs": achieved,
                         "limiter": solve_phase(members[0][0])[2]
                                    if dom == "vic_solve_kernel" else
                                    FP64_ISSUE},
            "kernels": kernels,
            "cpu_baseline": cb,
            "clocks": clk.summary(),
            "gpu_launches": args.steps * (2 + 3 * b.launches_per_stage()),
            "step_ms_median": statistics.median(step_ms),
            "step_ms_range": [min(step_ms), max(step_ms)],
            # the reference's implicit.fp64_columns monitor over the timed
            # steps: columns the refined solve left to the direct FP64 solve
            "implicit_fp64_columns": {
                "timed_steps": fb1 - fb0,
                "columns": sum(o.coord().nx2 for o, _ in members)},
        }
        if emit:
            print(json.dumps(line), flush=True)
    if own:
        ranks.close()
    return line


def run_reference_ensemble(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from snapy_gb300 import problems
    precision = args.precision or "float32"
    members = problems.ensemble_members(ENSEMBLE_MEMBERS, ENSEMBLE_SEED,
                                        precision=precision)
    cb = ensemble_cpu_baseline(members, max(2.0, args.cpu_seconds))
    val = cb["value"]
    cells = sum(o.coord().nx1 * o.coord().nx2 for o, _ in members)
    print(json.dumps({
        "impl": "reference", "metric": "cell-updates/s per RK3 step",
        "value": val, "unit": "cell-updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": cells / val * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Straka-type members)",
        "config": ensemble_config(members, precision, 1),
        "cpu_baseline": cb,
        "e2e": {"value": val, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}), flush=True)
    return 0


def serving_trace(n, steps, precision=None, implicit_precision=None,
                  implicit_solve=None, implicit_corrections=None):
    """The serving trace: n requests with seeded sizes and seeds, exponential
    inter-arrival times of mean 1 / SERVE_RATE."""
    import torch
    import snapy_gb300 as sg
    from snapy_gb300 import problems
    from snapy_gb300.serving import Request
    g = torch.Generator().manual_seed(SERVE_SEED)
    t, reqs = 0.0, []
    for i in range(n):
        t += float(-torch.log(torch.rand(1, generator=g, dtype=torch.float64)) / SERVE_RATE)
        pick = lambda seq: seq[int(torch.randint(len(seq), (1,), generator=g))]
        nx2, nx3, nx1 = pick((64, 96, 128)), pick((64, 96, 128)), pick((64, 96))
        opts = sg.MeshBlockOptions.from_yaml(os.path.join(ROOT, WORKLOADS["serving"]))
        c = opts.coord()
        c.nx1, c.nx2, c.nx3 = nx1, nx2, nx3
        c.x1max, c.x2max, c.x3max = nx1 * 50.0, nx2 * 50.0, nx3 * 50.0
        if precision:
            opts.hydro().precision = precision
        if opts.hydro().precision == "float32" and implicit_precision:
            opts.hydro().icorr.precision = implicit_precision
        if implicit_solve:
            opts.implicit_solve = implicit_solve
        if implicit_corrections:
            opts.implicit_corrections = implicit_corrections
        seed = SERVE_SEED + 1 + i
        reqs.append(Request(i, opts, (lambda o=opts, s=seed: problems.convection3d(o, "cpu", seed=s)),
                            steps, t))
    return reqs


def serving_config(reqs, nranks, budget=None):
    return {"workload": f"serving trace: {len(reqs)} 3-D planar dry convection "
                        f"solves, Poisson arrivals {SERVE_RATE:g}/s (seed "
                        f"{SERVE_SEED}), (nx2, nx3, nx1) in {{64,96,128}}^2 x "
                        f"{{64,96}} at 50 m, {reqs[0].steps} RK3 steps each, "
                        f"lmars+weno5+rk3+VIC, {reqs[0].options.hydro().precision} "
                        f"bulk, implicit solve {solve_label(reqs[0].options)}",
            "requests": len(reqs), "steps_per_request": reqs[0].steps,
            "implicit_assembly": reqs[0].options.hydro().icorr.precision,
            "implicit_solve": implicit_solve(reqs[0].options),
            "cells": [r.cells for r in reqs],
            "hbm_budget_bytes": budget,
            "admission": "first come first served against the HBM budget",
            "batching": "continuous: every running request in the same "
                        "launches, handle rebuilt on admission/completion",
            "l2": "inputs larger than L2 (no flush needed)",
            "replicas": nranks,
            "parallelism": "replicas" if nranks > 1 else "single"}


# algorithmic bytes per cell-update per RK3 step of a fused three-stage
# SSP-RK3 that keeps u0: 5 reads + 3 writes of nvar = 5 values
def b_alg(s_bytes: int, nvar: int = 5) -> int:
    return 8 * nvar * s_bytes


def as_fp64(opts):
    """A copy of a deck on the plain FP64 path: FP64 state, FP64 implicit
    assembly and the direct solve."""
    import copy
    o = copy.deepcopy(opts)
    o.hydro().precision = "float64"
    if o.hydro().icorr is not None:
        o.hydro().icorr.precision = "float64"
    return o


def plain_fp64(reqs, dev, steps=3, sweep="serial"):
    """plain_fp64_blocks over serving requests: each grid shape of the trace
    is measured once (on its first request), and the trace's plain time is
    every request's cell-steps at its shape's rate."""
    first = {}
    for r in reqs:
        c = r.options.coord()
        first.setdefault((c.nx1, c.nx2, c.nx3), r)
    rate = {}
    for shape, r in first.items():
        o64 = as_fp64(r.options)
        o64.implicit_sweep = sweep
        rate[shape] = plain_fp64_blocks([(o64, r.initial)], dev, steps)
    out = {"steps_per_request": steps, "shapes": len(rate)}
    for clock in ("device", "wall"):
        t = 0.0
        for r in reqs:
            c = r.options.coord()
            t += r.cells * r.steps / rate[(c.nx1, c.nx2, c.nx3)][clock]
        out[clock] = sum(r.cells * r.steps for r in reqs) / t
    return out


def plain_fp64_blocks(pairs, dev, steps=3):
    """The plain FP64 GPU path on the same blocks: each alone, its own
    FP64 MeshBlock (graphs on), one after another.

    device: cell-updates over the CUDA-event time of `steps` steps per
    request at that request's fixed CFL dt (no host read inside the timed
    steps: the plain path at its fastest).
    wall: the same requests stepped as a user drives MeshBlock -- the CFL dt
    read on the host every step -- over host wall-clock time."""
    import torch
    import snapy_gb300 as sg
    stream = torch.cuda.current_stream()
    dev_s, wall_s, n = 0.0, 0.0, 0
    for o64, initial in pairs:
        c = o64.coord()
        cells = c.nx1 * c.nx2 * c.nx3
        blk = sg.MeshBlock(o64).to(dev)
        vars = {"hydro_w": initial().to(dev)}
        blk.initialize(vars)
        for _ in range(6):  # eager steps and both rotations' graphs
            blk.step(vars, blk.max_time_step(vars))
        dt = blk.max_time_step(vars)
        torch.cuda.synchronize()
        evs = []
        for _ in range(steps):
            e0, e1 = (torch.cuda.Event(enable_timing=True),
                      torch.cuda.Event(enable_timing=True))
            e0.record(stream)
            blk.step(vars, dt)
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        dev_s += sum(a.elapsed_time(b) for a, b in evs) / 1e3
        t1 = time.perf_counter()
        for _ in range(steps):
            blk.step(vars, blk.max_time_step(vars))
        torch.cuda.synchronize()
        wall_s += time.perf_counter() - t1
        n += cells * steps
        del blk, vars
    return {"device": n / dev_s, "wall": n / wall_s, "steps_per_request": steps}


def fp64_reference_state(req, dev):
    """The request's FP64 state after its steps: the plain FP64 path
    (bitwise the CPU oracle's FP64 path), each step at its own CFL dt."""
    import torch
    import snapy_gb300 as sg
    blk = sg.MeshBlock(as_fp64(req.options)).to(dev)
    vars = {"hydro_w": req.initial().to(dev)}
    blk.initialize(vars)
    for _ in range(req.steps):
        blk.step(vars, blk.max_time_step(vars))
        assert blk.check_redo(vars) == 0
    torch.cuda.synchronize()
    return vars["hydro_u"].detach().cpu()


def rel_l2_fields(got, want):
    """Relative L2 of each of the five fields over the interior."""
    sl = (slice(3, -3),) * (got.dim() - 1)
    out = []
    for v in range(5):
        a, b = got[v][sl].double(), want[v][sl].double()
        den = float(b.norm())
        if den == 0.0:  # momenta at rest: scale by the density's momentum unit
            den = float(want[0][sl].double().norm())
        out.append(float((a - b).norm()) / den)
    return out


def run_serving(args, ranks=None, emit=True):
    """The serving trace through Server.run, beside the plain FP64 path on
    the same requests.  Returns rank 0's line (None elsewhere)."""
    import copy
    import torch
    own = ranks is None
    ranks = ranks or Ranks()
    world, rank, local = ranks.world, ranks.rank, ranks.local
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    from snapy_gb300.serving import Server
    budget = int(args.serve_budget_gb * (1 << 30)) if args.serve_budget_gb else None
    # warm-up: a short trace compiles nothing but touches every code path
    warm = serving_trace(2, max(3, args.warmup), args.precision,
                         args.implicit_precision or "float32",
                         args.implicit_solve, args.implicit_corrections)
    for r in warm:
        r.arrival = 0.0
    Server(dev).run(warm)
    reqs = serving_trace(args.requests, args.serve_steps, args.precision,
                         args.implicit_precision or "float32",
                         args.implicit_solve, args.implicit_corrections)
    torch.cuda.synchronize()
    ranks.barrier()
    srv = Server(dev, hbm_budget=budget, timing=True)
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        srv.run(reqs)
        wall = time.perf_counter() - t0
    bad = [r.rid for r in reqs if r.flags]
    assert not bad, f"retry flags on requests {bad}"
    total = sum(r.cells * r.steps for r in reqs)
    gpu_s = sum(srv.gpu_step_ms) / 1e3
    gpu_s, wall = ranks.max(gpu_s), ranks.max(wall)
    lat = sorted(r.latency for r in reqs)
    wait = sorted(r.admitted - r.arrival for r in reqs)
    q = lambda xs, f: xs[min(len(xs) - 1, int(round(f * (len(xs) - 1))))]
    kms = srv.kernel_ms
    dom = max(kms, key=lambda k: kms[k][0])
    prec = reqs[0].options.hydro().precision
    s_bytes = 4 if prec == "float32" else 8
    value = job_rate(total, world, gpu_s)
    peak, peak_kind = peaks()
    achieved = value * b_alg(s_bytes) / 1e9
    ktot = sum(v[0] for v in kms.values())
    # the same requests on the plain FP64 GPU path, both clocks
    plain = plain_fp64(reqs, dev, sweep=args.plain_sweep) if not args.no_plain else \
        {"device": float("nan"), "wall": float("nan"), "steps_per_request": 0}
    # the smallest request alone (a fresh server) equals itself in the mix,
    # and its FP32 result against the FP64 path at the served horizon
    small = min(reqs, key=lambda r: (r.cells, r.rid))
    same, err = None, None
    if not args.no_plain:
        alone = copy.copy(small)
        alone.arrival, alone.result, alone.done, alone.admitted = 0.0, None, None, None
        Server(dev).run([alone])
        same = bool(torch.equal(alone.result, small.result))
    if prec == "float32" and not args.no_plain:
        want = fp64_reference_state(small, dev)
        # the FP32 state holds anomalies about the FP64 hydrostatic base
        # (the serving slot's, from the same initial state): add it back
        from snapy_gb300.batch import fill_base
        from snapy_gb300.meshblock import block_of
        d = block_of(small.options)
        nc1 = d["nc1"]
        t = torch.zeros(5 * nc1 + 1, dtype=torch.float64, device=dev)
        fill_base(t, small.initial().to(dev), d)
        tot = small.result.double().clone()
        tot[0] += t[0:nc1].cpu()
        tot[4] += t[2 * nc1:3 * nc1].cpu()
        err = rel_l2_fields(tot, want)
    line = None
    if rank == 0:
        cb = None
        if not args.no_cpu_baseline:
            cb = serving_cpu_baseline(small, args.cpu_seconds)
        line = {
            "metric": "cell-updates/s per RK3 step",
            "value": value, "unit": "cell-updates/s",
            "n_gpus": world, "steps": len(srv.gpu_step_ms), "warmup": args.warmup,
            "ms_per_step": gpu_s / len(srv.gpu_step_ms) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if prec == "float32" else "f64",
            "data": "synthetic (seeded convection requests, seeded arrivals)",
            "config": serving_config(reqs, world, srv.budget),
            "latency": {"p50_s": q(lat, 0.5), "p99_s": q(lat, 0.99),
                        "min_s": lat[0], "max_s": lat[-1],
                        "admission_wait_p50_s": q(wait, 0.5),
                        "admission_wait_p99_s": q(wait, 0.99),
                        "unit": "s, arrival to result on host"},
            "e2e": {"value": job_rate(total, world, wall), "unit": "cell-updates/s",
                    "h2d_bytes_per_step": srv.h2d_bytes / len(srv.gpu_step_ms),
                    "d2h_bytes_per_step": srv.d2h_bytes / len(srv.gpu_step_ms),
                    "wall_s": wall,
                    "note": "wall clock of the whole trace through Server.run: "
                            "arrivals, initial states host->device, results "
                            "device->host"},
            "plain_fp64": {"device": plain["device"], "wall": plain["wall"],
                           "unit": "cell-updates/s",
                           "sweep": args.plain_sweep,
                           "how": "each request alone, its own FP64 MeshBlock, "
                                  "graphs on; device: CUDA events around "
                                  f"{plain['steps_per_request']} steps at a fixed "
                                  "CFL dt; wall: the same steps with the CFL dt "
                                  "read on the host each step"},
            "vs_plain_fp64": value / plain["device"],
            "vs_plain_fp64_wall": job_rate(total, world, wall) / plain["wall"],
            "clock_note": "vs_plain_fp64: CUDA-event time on both sides; "
                          "vs_plain_fp64_wall: wall clock on both sides",
            "alone_equals_mix": same,
            "fp32_rel_l2_vs_fp64": err,
            "fp32_check": (f"request {small.rid} ({small.cells} cells) after "
                           f"{small.steps} steps, relative L2 per field "
                           "(rho, m1, m2, m3, E) against the FP64 path"),
            "max_running": srv.max_running, "handle_rebuilds": srv.rebuilds,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "traffic": None,
                         "basis": f"B_alg = {b_alg(s_bytes)} B per cell-update "
                                  "per RK3 step (5 reads + 3 writes x 5 "
                                  f"variables x {s_bytes} B) x the device-timed "
                                  "cell-updates/s of the whole step",
                         "dominant_kernel": dom,
                         "dominant_share": kms[dom][0] / ktot,
                         "scratch_bytes_per_cell_step": serving_scratch(reqs[0].options),
                         "limiter": solve_phase(reqs[0].options)[2]
                                    if dom == "vic_solve_kernel" else FP64_ISSUE},
            "kernels": {k: {"launches": n, "mean_us": ms / n * 1e3,
                            "share": ms / ktot}
                        for k, (ms, n) in kms.items()},
            "cpu_baseline": cb,
            "clocks": clk.summary(),
            "gpu_launches": srv.launches,
        }
        if emit:
            print(json.dumps(line), flush=True)
    if own:
        ranks.close()
    return line


def serving_scratch(opts):
    """Bytes of implementation scratch (the implicit solve's and the x3
    sweep's) moved per interior cell per RK3 step: not algorithmic."""
    c = opts.coord()
    per_stage = solve_phase(opts)[1] + (40 + 600 + 40)  # solve phase, assembly
    per_stage += 120  # the finish's D, du, du0
    if c.nx3 > 1:
        per_stage += 2 * 5 * 4  # a3 dF3 written and read
    return 3 * per_stage


def serving_cpu_baseline(req, seconds):
    """The CPU oracle (FP64, OpenMP on every host core) on the smallest
    request of the trace, as many RK3 steps as fit in `seconds`."""
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    ob = O.block_from_options(req.options, nthreads=cores)
    u = ob.initialize(req.initial().numpy())
    n, t0 = 0, time.perf_counter()
    while True:
        ob.step(u, req.options.intg().cfl * ob.max_dt(u))
        n += 1
        el = time.perf_counter() - t0
        if (el >= seconds and n >= 1) or n >= 10000:
            break
    c = req.options.coord()
    return {"value": req.cells * n / el, "unit": "cell-updates/s", "cores": cores,
            "kind": "port",
            "sample": f"{n} RK3 steps of the smallest request ({c.nx2}x{c.nx3}x"
                      f"{c.nx1}), FP64, {el:.1f} s, OpenMP {cores} threads"}


def run_reference_serving(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    reqs = serving_trace(args.requests, args.serve_steps, args.precision)
    cb = serving_cpu_baseline(min(reqs, key=lambda r: r.cells),
                              max(2.0, args.cpu_seconds))
    val = cb["value"]
    print(json.dumps({
        "impl": "reference", "metric": "cell-updates/s per RK3 step",
        "value": val, "unit": "cell-updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": reqs[0].cells / val * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded convection requests, seeded arrivals)",
        "config": serving_config(reqs, 1, int(args.serve_budget_gb * (1 << 30))
                                 if args.serve_budget_gb else None),
        "cpu_baseline": cb,
        "e2e": {"value": val, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}), flush=True)
    return 0


def cs_config(n, precision, nranks):
    return {"workload": f"cubed sphere shallow water: 6 panels x {n}x{n}, "
                        "radius 6.371e6 m, depth 1000 m, 100 m Gaussian bump "
                        f"(0.1 rad, seed {CS_SEED}), weno5+shallow-roe+rk3, "
                        f"{precision}, seam halo every stage",
            "cells": 6 * n * n, "panels": 6, "n": n, "precision": precision,
            "dt": "the CFL step on the device, every step",
            "l2": "flushed between timed steps (512 MiB write; the state fits in L2)",
            "graphs": "one step graph per buffer rotation, captured before the warm-up",
            "replicas": nranks, "parallelism": "replicas" if nranks > 1 else "single"}


def cs_cpu_baseline(n, seconds):
    """The cubed-sphere oracle (numpy plumbing over the C oracle's face
    functions, FP64, OpenMP) on the same grid, as many RK3 steps as fit."""
    import numpy as np
    from oracle import oracle as O
    from oracle.cubed_sphere import CubedSphere
    from snapy_gb300 import cubed_sphere as cs
    O.build()
    o = CubedSphere(n, cs.RK3, 0.9)
    u = cs.bump(n, seed=CS_SEED)
    o.fill(u)
    u0 = np.zeros_like(u)
    k, t0 = 0, time.perf_counter()
    while True:
        dt = o.max_dt(u)
        for st in range(3):
            o.stage(u, u0, dt, st)
        k += 1
        el = time.perf_counter() - t0
        if (el >= seconds and k >= 1) or k >= 10000:
            break
    return {"value": 6 * n * n * k / el, "unit": "cell-updates/s",
            "cores": os.cpu_count() or 1, "kind": "port",
            "sample": f"{k} RK3 steps of the same 6 x {n}x{n} sphere, FP64, "
                      f"{el:.1f} s (numpy over the C oracle, OpenMP)"}


def run_cubed_sphere(args):
    import torch
    from snapy_gb300 import cubed_sphere as cs
    ranks = Ranks()
    world, rank, local = ranks.world, ranks.rank, ranks.local
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    precision = args.precision or "float32"
    dtype = torch.float32 if precision == "float32" else torch.float64
    n = CS_N
    sp = cs.SphereSW(n, dtype=dtype, device=dev)
    u_init = cs.bump(n, seed=CS_SEED)
    sp.initialize(u_init)
    for _ in range(8):
        if sp.captures >= 2:
            break
        sp.step()
    for _ in range(max(3, args.warmup)):
        sp.step()
    torch.cuda.synchronize()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    ranks.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            sp.step()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_total = sum(step_ms) / 1e3
    t_total = ranks.max(t_total)
    cells = 6 * n * n
    value = job_rate(cells * args.steps, world, t_total)
    assert torch.isfinite(sp.state()).all()
    # one stage (flux, seam flux, update, seam halo) timed alone, L2 flushed
    s_bytes = 4 if dtype == torch.float32 else 8
    stage_ms, stage_bytes = [], []
    for k in range(min(args.steps, 20)):
        for st in range(3):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sp._chk(sp.L.sg_cs_stage(sp.h, st, sp.dt.data_ptr(), stream.cuda_stream), "sg_cs_stage")
            e1.record(stream)
            stage_ms.append((e0, e1))
            stage_bytes.append((2 if st == 0 else 3) * 4 * s_bytes * cells)
    torch.cuda.synchronize()
    durs = [a.elapsed_time(b) / 1e3 for a, b in stage_ms]
    achieved = sum(stage_bytes) / sum(durs) / 1e9
    peak, peak_kind = peaks()
    # end to end with host buffers
    host = torch.empty(sp.state().shape, dtype=dtype).pin_memory()
    host.copy_(sp.state())
    nbytes = host.numel() * host.element_size()
    e2e_steps = max(5, min(args.steps, 50))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sp.state().copy_(host, non_blocking=True)
        sp.step()
        host.copy_(sp.state(), non_blocking=True)
    torch.cuda.synchronize()
    e2e_t = time.perf_counter() - t0
    if rank == 0:
        cb = None if args.no_cpu_baseline else cs_cpu_baseline(n, args.cpu_seconds)
        print(json.dumps({
            "metric": "cell-updates/s per RK3 step",
            "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_total / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if dtype == torch.float32 else "f64",
            "data": "synthetic (seeded Gaussian bump)",
            "config": cs_config(n, precision, world),
            "e2e": {"value": job_rate(cells * e2e_steps, world, e2e_t), "unit": "cell-updates/s",
                    "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "traffic": None,
                         "kernel": "one stage: cs_flux + cs_seam_flux + cs_update + cs_ghost",
                         "bytes_per_launch": statistics.mean(stage_bytes),
                         "mean_launch_us": statistics.mean(durs) * 1e6},
            "cpu_baseline": cb, "clocks": clk.summary(),
            "gpu_launches": args.steps * (2 + 3 * 5),
            "step_ms_median": statistics.median(step_ms)}), flush=True)
    ranks.close()
    return 0


def run_reference_cubed_sphere(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cb = cs_cpu_baseline(CS_N, max(2.0, args.cpu_seconds))
    val = cb["value"]
    print(json.dumps({
        "impl": "reference", "metric": "cell-updates/s per RK3 step",
        "value": val, "unit": "cell-updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 6 * CS_N * CS_N / val * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Gaussian bump)",
        "config": cs_config(CS_N, args.precision or "float32", 1), "cpu_baseline": cb,
        "e2e": {"value": val, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}), flush=True)
    return 0


def run_batched_served(args):
    """The default line: the batched ensemble (value, e2e, K steps timed)
    with the serving trace as its "served" object; the headline latency and
    the served-vs-plain ratio are lifted to the top level."""
    ranks = Ranks()
    line = run_ensemble(args, ranks, emit=False)
    served = run_serving(args, ranks, emit=False)
    if ranks.rank == 0:
        line["metric"] = METRIC
        line["config"]["workload"] = ("batched + served: " +
                                      line["config"]["workload"] + "; " +
                                      served["config"]["workload"])
        line["latency"] = served["latency"]
        line["served_vs_plain_fp64"] = served["vs_plain_fp64"]
        line["served_vs_plain_fp64_wall"] = served["vs_plain_fp64_wall"]
        line["served"] = served
        line["gpu_launches"] += served["gpu_launches"]
        print(json.dumps(line), flush=True)
    ranks.close()
    return 0


def run_reference_batched_served(args):
    """The reference arm of the default line: the CPU oracle on the
    ensemble's members (value), with the served trace's CPU sample beside."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import io
    import contextlib
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        run_reference_ensemble(args)
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    line["metric"] = METRIC
    reqs = serving_trace(args.requests, args.serve_steps, args.precision)
    line["config"]["workload"] = ("batched + served: " + line["config"]["workload"]
                                  + "; " + serving_config(reqs, 1)["workload"])
    line["served_cpu_baseline"] = serving_cpu_baseline(
        min(reqs, key=lambda r: r.cells), max(2.0, args.cpu_seconds / 2))
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.workload == "batched-served":
        if args.impl == "reference":
            return run_reference_batched_served(args)
        return run_batched_served(args)
    if args.workload == "cubed-sphere":
        if args.impl == "reference":
            return run_reference_cubed_sphere(args)
        return run_cubed_sphere(args)
    if args.workload == "serving":
        if args.impl == "reference":
            return run_reference_serving(args)
        run_serving(args)
        return 0
    if args.workload == "ensemble":
        if args.impl == "reference":
            return run_reference_ensemble(args)
        run_ensemble(args)
        return 0
    if args.impl == "reference":
        return run_reference(args)
    return run_native(args)


if __name__ == "__main__":
    sys.exit(main())
