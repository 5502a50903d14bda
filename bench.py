#!/usr/bin/env python
"""Benchmark of the forward-solver hot path (seis3d_wave time loop) on GB300.

Workload (default, --config c2): 400x400x200 interior grid, 1 km horizontal spacing,
0.5-2 km stretched vertical spacing, layered medium with a seeded +/-5% Gaussian-
correlated (10 km) Vp/Vs perturbation, 12-cell CFS-PML on five faces, free surface,
64 surface receivers, and three simulations (vertical/horizontal point forces Fx, Fy,
Fz; Ricker 0.2 Hz) that together produce the strain Green's tensors.  One bench step =
one LDDRK4 time step of the three simulations stepped as a batch: four fused stage
launches, each covering all three, plus each simulation's step-end kernel.  Inputs are
synthetic and seeded.  The register sets (9 components x 4 x 32M points x 4 B per
simulation) are far larger than L2, so no L2 flush is used.

Metric: grid-point updates per second (interior points x steps / device time).

--impl reference times the reference's algorithm on the host cores instead: the
oracle (a restatement of the Fortran solver, which cannot be compiled here) with all
available threads, one time step of one simulation per bench step.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic DRAM bytes of the fused scheme per interior point per time step (FP32):
# W ping-pong, RK registers m and t, medium (lambda, mu, rho):
#   stage 1: read W 9 + medium 3, write W' 9 + t 9                = 30 floats
#   stage 2, 3: read W 9 + medium 3 + m 9 + t 9, write W' 9 + t 9  = 48 floats each
#   stage 4: read W 9 + medium 3 + t 9, write W 9                  = 30 floats
# Of the 156 values, 12 are the medium (always FP32) and 144 are wavefield registers,
# which --storage bf16/fp16 holds in 2 bytes.  That is RK form 0 (fwant_set_rk_scheme), the
# reference's registers.  Form 1, the default of the fast FP32 form, runs stages 1-3
# without the accumulator t and forms it at stage 3:
#   stage 1: read W 9 + medium 3, write W' 9                        = 21 floats
#   stage 2: read W 9 + medium 3 + m 9, write W' 9                  = 30 floats
#   stage 3: read W 9 + medium 3 + m 9 + W2 9, write W' 9 + t 9     = 48 floats
#   stage 4: read W 9 + medium 3 + t 9, write W 9                   = 30 floats
# 129 values, 117 of them wavefield registers.
FIELD_VALUES_PT_STEP = {0: 144, 1: 117}
MEDIUM_VALUES_PT_STEP = 12
STORAGE_BYTES = {"fp32": 4, "bf16": 2, "fp16": 2}


def bytes_pt_step(storage, scheme=0):
    return FIELD_VALUES_PT_STEP[scheme] * STORAGE_BYTES[storage] + MEDIUM_VALUES_PT_STEP * 4


# CFS-PML memory variables, per slab point per step: 6 variables x (3+5+5+3) floats (form 0)
# or x (2+3+5+3) floats (form 1)
def bytes_pml_pt_step(scheme=0):
    return 6 * (16 if scheme == 0 else 13) * 4


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=32)
    p.add_argument("--warmup", type=int, default=8)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--config", choices=["c2", "c1", "c3", "c5", "lsqr", "media", "ker", "assm"], default="c2",
                   help="c5: train the waveform surrogate on 512 FD solves and screen 64 held-out models; "
                        "lsqr: LSQR iterations of the damped, smoothed inversion (inv.LSQR) on a synthetic system; "
                        "media: the effective-medium preprocessor (seis3d_media) on the C2 grid; "
                        "ker: the sensitivity-kernel accumulation (SI_ker_sta sgt2scatter3) of one SGT block; "
                        "assm: the kernel assembly onto inversion blocks (SI_ker2assm) of two kernel volumes")
    p.add_argument("--ker-points", type=int, default=16384, help="kernel points of the --config ker block")
    p.add_argument("--assm-shuffle", action="store_true",
                   help="--config assm: list each block's pixels in a random order instead of i fastest")
    p.add_argument("--lsqr-scale", type=float, default=1.0,
                   help="fraction of the LSQR system's measurements and blocks (profiling)")
    p.add_argument("--cpu-steps", type=int, default=2, help="steps of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--e2e-steps", type=int, default=None,
                   help="time steps of the C2 end-to-end leg (default 1000, a quarter of the 4000-step C2 job, so "
                        "that its one upload of the medium is spread over steps as in the job; --steps with --grid)")
    p.add_argument("--no-c3", action="store_true",
                   help="skip the C3 batched-vs-single comparison of the default (C2) line")
    p.add_argument("--c3-steps", type=int, default=16, help="timed steps of each C3 leg (multiple of 8)")
    p.add_argument("--hill", action="store_true",
                   help="--config c1: the seeded 2 km Gaussian hill on top (terrain-following grid, one solver)")
    p.add_argument("--no-companions", action="store_true",
                   help="skip the short runs of the other hot-path rows (C1, media, ker, assm, LSQR) that the "
                        "default (C2) line carries under 'companions'")
    p.add_argument("--grid", default=None, help="override the C2 interior size, e.g. 200x200x100 (profiling)")
    p.add_argument("--sims", type=int, default=3, help="number of force components simulated (C2)")
    p.add_argument("--autotune", action="store_true",
                   help="run the project's autotuner (tile shape and planes per CTA of every member, the batch's CTA "
                        "schedule) before timing; the end-to-end leg applies the tuned settings")
    p.add_argument("--tile-rows", type=int, choices=[8, 16], default=None,
                   help="rows of the stage kernel's 32-column tile (default 8; 16 for FP32 storage)")
    p.add_argument("--storage", choices=["fp32", "bf16", "fp16"], default="fp32",
                   help="storage of the wavefield registers (arithmetic stays FP32)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_value(world, npts, steps, dev_ms_max):
    """Whole-job rate of N replicas: every rank processed npts x steps points, the job took
    the slowest rank's time (G points / s)."""
    return world * npts * steps / (dev_ms_max * 1e-3) / 1e9


class Dist:
    """Barrier and max-reduction over ranks (gloo on CPU tensors; replicas only)."""

    def __init__(self, world):
        self.world = world
        if world > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, v):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device, period_ms=200):
        self.device = device
        self.period_ms = int(period_ms)
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic_ratio(scheme=1, storage="fp32"):
    """Measured DRAM bytes over algorithmic bytes of the stage kernel in RK form `scheme`,
    from the committed ncu summary (captured on a smaller grid of the same kernel), or None.
    BF16 storage has its own capture (form 1); FP16 shares its layout and halo."""
    if storage == "fp32":
        path = os.path.join(ROOT, "profiles", "stage_batch_kernel_c2.md")
    elif scheme == 1:
        path = os.path.join(ROOT, "profiles", "stage_batch_kernel_bf16_c2.md")
    else:
        return None
    if not os.path.exists(path):
        return None
    key = "dram_traffic_over_algorithmic" if scheme == 1 else "dram_traffic_over_algorithmic_form0"
    m = re.search(key + r":\s*([0-9.eE+-]+)", open(path).read())
    return float(m.group(1)) if m else None


def make_models(config, seed, grid=None, sims=3):
    from fwant_gb300 import inputs
    if config == "c1":
        m = inputs.config_c1(seed=seed)
        return [m], "C1: 100x100x60, FP32, 12-cell CFS-PML x5, free surface, Fz Ricker 0.2 Hz, 16 receivers"
    if config == "c3":
        ms = inputs.config_c3(seed=seed)
        return ms, (f"C3: {len(ms)} virtual sources of seeded sizes (horizontal 160-320, depth 80-160 cells), "
                    "C2 physics, one vertical surface force and 16 receivers each, stepped as one batch")
    if grid:
        ni, nj, nk = (int(v) for v in grid.lower().split("x"))
        base = inputs.make_model(ni, nj, nk, seed=seed, nrecv=64, perturb=0.05, name=f"C2-physics {grid}")
    else:
        base = inputs.config_c2(seed=seed, component=0)
    models = []
    for c in range(sims):
        m = inputs.Model(**{k: getattr(base, k) for k in base.__dataclass_fields__})
        f = np.zeros((1, 1), np.float32)
        m.fx, m.fy, m.fz = f.copy(), f.copy(), f.copy()
        (m.fx, m.fy, m.fz)[c][0, 0] = np.float32(1.0e15)
        models.append(m)
    size = grid or "400x400x200"
    return models, (f"C2: {size}, FP32, +/-5% Gaussian-correlated Vp/Vs (10 km), 12-cell CFS-PML x5, "
                    f"free surface, {sims} force component(s) of (Fx,Fy,Fz) x 64 surface receivers")


def slab_points(m):
    n = [int(v) for v in m.pml_number]
    tot = 0
    tot += (n[0] + 1) * m.nj * m.nk if n[0] > 0 else 0
    tot += (n[1] + 1) * m.nj * m.nk if n[1] > 0 else 0
    tot += (n[2] + 1) * m.ni * m.nk if n[2] > 0 else 0
    tot += (n[3] + 1) * m.ni * m.nk if n[3] > 0 else 0
    tot += (n[4] + 1) * m.ni * m.nj if n[4] > 0 else 0
    tot += (n[5] + 1) * m.ni * m.nj if n[5] > 0 else 0
    return tot


def cpu_sample(models, steps):
    """The oracle on all host threads: `steps` time steps of the first simulation."""
    from fwant_gb300 import inputs
    from oracle import oracle as O
    O.build()
    threads = O.set_threads(os.cpu_count() or 1, timing=True)
    m = models[0]
    o = O.Oracle(m.ni, m.nj, m.nk, m.stept, timing=True)
    inputs.attach(o, m, metric=O.metric(m.x, m.y, m.z))
    o.run(1)  # first touch of every array
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    o.close()
    return m.npoints * steps / dt / 1e9, threads, dt


def _timing_flags():
    from oracle import oracle as O
    return O.build_flags(timing=True)


def _checker_flags():
    from oracle import oracle as O
    return O.build_flags()


def _reference_line(args, metric, unit, v, dt, desc, sample, threads, dtype):
    out = {
        "impl": "reference", "metric": metric, "value": v, "unit": unit,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "replicas only",
        "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded)",
        "config": {"workload": desc, "sample": sample},
        "cpu_baseline": {"value": v, "unit": unit, "cores": threads, "kind": "port", "sample": sample,
                         "build": _timing_flags()},
        "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    return 0


def run_reference_media(args):
    """the oracle's effmedia_eval + media_extend with all host threads, each step the top
    planes of the bench's grid"""
    from oracle import oracle as O
    O.build()
    threads = O.set_threads(os.cpu_count() or 1, timing=True)
    ni, nj, nk, x, y, z, zt, calls, desc = media_workload(args.grid)
    kk = min(nk, 8)
    o = O.MediaOracle(ni, nj, kk, x, y, z[nk - kk:], zt, (1, 1, 1), timing=True)
    for name, a in calls:
        getattr(o, name)(*a)
    for _ in range(max(args.warmup, 1)):
        o.eval()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.eval()
    dt = time.perf_counter() - t0
    sample = f"the top {kk} planes of the grid ({ni}x{nj}x{kk} points) per step, {threads} threads"
    return _reference_line(args, "effective-medium grid points per second", "GPts/s", ni * nj * kk * args.steps / dt / 1e9,
                           dt, desc, sample, threads, "f32")


def run_reference_lsqr(args):
    """the oracle's sequential LSQR on the bench's system, one iteration per step"""
    from oracle import oracle as O
    O.build()
    rp, col, val, rhs, ncol = lsqr_system(args.lsqr_scale)
    nnz = int(rp[-1])
    t0 = time.perf_counter()
    O.lsqr(rp, col, val, rhs, ncol, atol=0.0, btol=0.0, maxit=args.steps, timing=True)
    dt = time.perf_counter() - t0
    sample = f"{args.steps} iterations of the sequential restatement (setup and |A|_F included), 1 thread"
    return _reference_line(args, "LSQR matrix entries per second", "Gentries/s", nnz * args.steps / dt / 1e9, dt,
                           f"inversion system, {nnz} stored entries", sample, 1, "f64")


def run_reference_ker(args):
    """the oracle's FP64-accumulation sgt2scatter3 with all host threads, each step a
    sample of the block's points"""
    from oracle import oracle as O
    O.build()
    threads = O.set_threads(os.cpu_count() or 1, timing=True)
    npts, knt = args.ker_points, 500
    lam, mu, sgt = ker_block(npts, knt)
    ns = min(npts, 1024)
    sub = [a[:, :, :ns].copy() for a in sgt]
    for _ in range(max(args.warmup, 1)):
        O.sgt2scatter3(lam[:ns], mu[:ns], sub[:3], sub[3], 0.1, mode=1, timing=True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.sgt2scatter3(lam[:ns], mu[:ns], sub[:3], sub[3], 0.1, mode=1, timing=True)
    dt = time.perf_counter() - t0
    dfma = ns * 3 * 7 * knt * (knt - 1) / 2
    sample = f"{ns} of the {npts} kernel points per step, {threads} threads"
    return _reference_line(args, "sensitivity-kernel accumulation FP64 throughput", "TFLOP/s",
                           2 * dfma * args.steps / dt / 1e12, dt, f"sgt2scatter3 of one SGT block ({npts} points)",
                           sample, threads, "f64")


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    if args.config == "media":
        return run_reference_media(args)
    if args.config == "lsqr":
        return run_reference_lsqr(args)
    if args.config == "ker":
        return run_reference_ker(args)
    if args.config == "assm":
        return run_reference_assm(args)
    models, desc = make_models(args.config, seed=0, grid=args.grid, sims=args.sims)
    from fwant_gb300 import inputs
    from oracle import oracle as O
    O.build()
    threads = O.set_threads(os.cpu_count() or 1, timing=True)
    m = models[0]
    o = O.Oracle(m.ni, m.nj, m.nk, m.stept, timing=True)
    inputs.attach(o, m, metric=O.metric(m.x, m.y, m.z))
    o.run(max(args.warmup, 1))
    t0 = time.perf_counter()
    o.run(args.steps)
    dt = time.perf_counter() - t0
    v = m.npoints * args.steps / dt / 1e9
    sample = (f"one time step of one of the three simulations ({m.ni}x{m.nj}x{m.nk}) per bench step, "
              f"{args.steps} steps after {max(args.warmup, 1)} warm-up")
    out = {
        "impl": "reference", "metric": "grid-point updates per second", "value": v, "unit": "GPts/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": desc, "sample": sample, "l2": "inputs larger than L2 (no flush)"},
        "cpu_baseline": {"value": v, "unit": "GPts/s", "cores": threads, "kind": "port", "sample": sample,
                         "build": _timing_flags(), "checker_build": _checker_flags()},
        "e2e": {"value": v, "unit": "GPts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    return 0


def lsqr_system(scale=1.0, seed=0):
    """A synthetic inversion system shaped like the reference's: 1.5M unknowns (3
    components x 500k blocks + station and event terms), 25,000 measurements whose kernel
    rows are 64 runs of 250 consecutive blocks (a localised sensitivity kernel in block
    order), one damping row per unknown and first-difference smoothing rows along the block
    order of each component.  scale < 1 shrinks the measurements and the blocks together,
    so rows and columns keep their lengths (profiling a smaller system of the same shape).
    Returns (row_ptr, col, val, rhs, ncol)."""
    rng = np.random.default_rng(seed)
    nblk, ncmp, nsta, nevt = max(2_000, int(500_000 * scale)), 3, 400, 2_000
    nm = nblk * ncmp
    ncol = nm + nsta + nevt
    ndata = max(1, int(25_000 * scale))
    runs, runlen = 64, 250
    starts = rng.integers(0, nm - runlen, size=(ndata, runs))
    starts.sort(axis=1)
    kcols = (starts[:, :, None] + np.arange(runlen)[None, None, :]).reshape(ndata, -1)
    sta = nm + rng.integers(0, nsta, size=ndata)
    evt = nm + nsta + rng.integers(0, nevt, size=ndata)
    dcols = np.concatenate([kcols, sta[:, None], evt[:, None]], axis=1)
    nper = dcols.shape[1]
    dvals = rng.normal(size=(ndata, nper)) * 1e-3
    dvals[:, -2:] = rng.choice([-1.0, 1.0], size=(ndata, 2))
    smo = np.arange(nm)
    smo = smo[(smo + 1) % nblk != 0]  # first differences within each component
    rp = np.concatenate([np.arange(ndata + 1, dtype=np.int64) * nper,
                         ndata * nper + np.arange(1, ncol + 1, dtype=np.int64),
                         ndata * nper + ncol + 2 * np.arange(1, smo.size + 1, dtype=np.int64)])
    col = np.concatenate([dcols.reshape(-1), np.arange(ncol), np.stack([smo, smo + 1], axis=1).reshape(-1)])
    val = np.concatenate([dvals.reshape(-1), np.full(ncol, 0.05), np.tile([-0.5, 0.5], smo.size)])
    rhs = np.concatenate([rng.normal(size=ndata), np.zeros(ncol + smo.size)])
    return rp, col.astype(np.int32), val.astype(np.float64), rhs, ncol


def lsqr_bytes_per_iteration(nnz, nrow, ncol):
    """Algorithmic bytes of one LSQR iteration: both products read every stored entry once
    (8 B value + 4 B index, compressed rows and compressed columns) and their offsets; the
    vector passes read and write u twice (product, normalisation), v twice, and x, w, sig
    with v once more in the update.  Gathered vector reads are not counted (L2)."""
    return 24 * nnz + 8 * (nrow + ncol) + 32 * nrow + 88 * ncol


def run_lsqr(args, rank):
    """The inversion's LSQR (fwant_lsqr_*) on the synthetic system: K iterations timed on
    the device, the roofline of the iteration, the oracle's sequential LSQR on the host for
    a bounded sample, and the end-to-end job through the public API (upload, solve,
    solution read back)."""
    import fwant_gb300 as fw
    if rank != 0:
        return 0
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    rp, col, val, rhs, ncol = lsqr_system(args.lsqr_scale)
    nrow, nnz = rp.size - 1, int(rp[-1])
    t0 = time.perf_counter()
    L = fw.Lsqr(rp, col, val, rhs, ncol, device=dev)
    create_s = time.perf_counter() - t0
    warm = max(args.warmup, 3)
    L.solve(0.0, 0.0, warm)
    clocks = Clocks(dev)
    clocks.start()
    it = L.solve(0.0, 0.0, args.steps)
    dev_ms = L.last_solve_ms()
    clk = clocks.stop()
    x, _ = L.solution()
    finite = bool(np.all(np.isfinite(x)))
    value = nnz * it / (dev_ms * 1e-3) / 1e9
    per_it = lsqr_bytes_per_iteration(nnz, nrow, ncol)
    achieved = per_it * it / (dev_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    out = {
        "metric": "LSQR matrix entries per second", "value": value, "unit": "Gentries/s", "n_gpus": 1,
        "steps": it, "warmup": warm, "ms_per_step": dev_ms / it, "higher_is_better": True, "scaling": "replicas only",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"inversion system: {nrow} rows x {ncol} unknowns, {nnz} stored entries "
                               f"({int(25_000 * args.lsqr_scale)} measurements x 16,002 entries, damping, smoothing)",
                   "l2": "matrix larger than L2 (no flush)", "solution_finite": finite,
                   "iteration": "one LSQR iteration (A v, A^T u, two normalisations, update, test) per step"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": None,
                     "algorithmic_bytes_per_iteration": per_it},
        "clocks": clk, "create_s": create_s,
        # per 32 iterations one graph of 7 kernels each, plus 5 start kernels
        "gpu_launches": 5 + 7 * 32 * ((it + 31) // 32),
    }
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        k = 2
        t1 = time.perf_counter()
        O.lsqr(rp, col, val, rhs, ncol, atol=0.0, btol=0.0, maxit=k, timing=True)
        dt = time.perf_counter() - t1
        out["cpu_baseline"] = {"value": nnz * k / dt / 1e9, "unit": "Gentries/s", "cores": 1, "kind": "port",
                               "build": O.build_flags(timing=True),
                               "sample": f"{k} iterations of the sequential restatement on the same system, "
                                         f"{dt:.1f} s (setup and |A|_F included)"}
    if not args.no_e2e:
        t1 = time.perf_counter()
        L2 = fw.Lsqr(rp, col, val, rhs, ncol, device=dev)
        it2 = L2.solve(0.0, 0.0, args.steps)
        x2, e2 = L2.solution()
        wall = time.perf_counter() - t1
        L2.close()
        out["e2e"] = {"value": nnz * it2 / wall / 1e9, "unit": "Gentries/s",
                      "h2d_bytes_per_step": (rp.nbytes + col.nbytes + val.nbytes + rhs.nbytes) / it2,
                      "d2h_bytes_per_step": (x2.nbytes + e2.nbytes) / it2, "wall_s": wall,
                      "includes": "transpose on the host, upload, |A|_F, K iterations, solution and errors read back"}
    L.close()
    print(json.dumps(out), flush=True)
    return 0


def media_workload(grid=None):
    from fwant_gb300 import inputs
    ni, nj, nk = (int(v) for v in (grid or "400x400x200").lower().split("x"))
    x, y, z = inputs.grid_c2(ni, nj, nk)
    calls = inputs.media_models(x, y, z, seed=0)
    desc = (f"effective medium of a {ni}x{nj}x{nk} grid (C2 spacing) from a 4-layer cart1d background and a "
            f"+/-5% Gaussian-correlated (10 km) volume perturbation sampled every 2 km; half_sample_point 1 1 1 "
            f"(8 sub-cell samples per point)")
    return ni, nj, nk, x, y, z, float(z[-4]), calls, desc


# Algorithmic DRAM bytes of one evaluation per grid point: lambda, mu, rho written once at
# every point (ghosts included) plus the ghost extension's reads; model data stays in cache
MEDIA_BYTES_PT = 12


def run_media(args, rank):
    """The medium preprocessor (fwant_media_*): K evaluations of the effective medium on
    the device, the oracle's evaluation of a slab of the same grid on the host, and the
    end-to-end job through the public API (upload grid and models, evaluate, read the
    three arrays back)."""
    import fwant_gb300 as fw
    if rank != 0:
        return 0
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    ni, nj, nk, x, y, z, zt, calls, desc = media_workload(args.grid)
    npts = ni * nj * nk
    nx3 = (ni + 6) * (nj + 6) * (nk + 6)
    M = fw.Media(ni, nj, nk, x, y, z, zt, (1, 1, 1), device=dev)
    for name, a in calls:
        getattr(M, name)(*a)
    warm = max(args.warmup, 3)
    for _ in range(warm):
        M.eval(copy=False)
    clocks = Clocks(dev)
    clocks.start()
    ms = []
    for _ in range(args.steps):
        M.eval(copy=False)
        ms.append(M.last_eval_ms())
    clk = clocks.stop()
    dt_info = M.stept_check()
    dev_ms = float(np.sum(ms))
    value = npts * args.steps / (dev_ms * 1e-3) / 1e9
    achieved = MEDIA_BYTES_PT * nx3 * args.steps / (dev_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    out = {
        "metric": "effective-medium grid points per second", "value": value, "unit": "GPts/s", "n_gpus": 1,
        "steps": args.steps, "warmup": warm, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "replicas only", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": desc, "l2": "outputs (408 MB) larger than L2 (no flush)",
                   "step": "one effmedia_eval + media_extend pass over the grid",
                   "dtmax": dt_info[0], "dtmax_at": dt_info[1]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": None,
                     "note": "issue-bound, not memory-bound: 12 B written per point against 8 sub-cell samples "
                             "of bisections, interpolation weights and IEEE divisions"},
        "clocks": clk, "gpu_launches": 2 * args.steps,
    }
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        threads = O.set_threads(os.cpu_count() or 1, timing=True)
        kk = min(nk, 20)
        zs = z[nk - kk:]  # the top kk planes of the same grid (with their ghosts)
        o = O.MediaOracle(ni, nj, kk, x, y, zs, zt, (1, 1, 1), timing=True)
        for name, a in calls:
            getattr(o, name)(*a)
        t1 = time.perf_counter()
        o.eval()
        dt = time.perf_counter() - t1
        out["cpu_baseline"] = {"value": ni * nj * kk / dt / 1e9, "unit": "GPts/s", "cores": threads, "kind": "port",
                               "build": O.build_flags(timing=True),
                               "sample": f"the top {kk} planes of the same grid ({ni}x{nj}x{kk} points, "
                                         f"same models), {dt:.1f} s"}
    if not args.no_e2e:
        t1 = time.perf_counter()
        M2 = fw.Media(ni, nj, nk, x, y, z, zt, (1, 1, 1), device=dev)
        h2d = x.nbytes + y.nbytes + z.nbytes
        for name, a in calls:
            getattr(M2, name)(*a)
            h2d += sum(v.nbytes for v in a if isinstance(v, np.ndarray))
        lam, mu, rho = M2.eval()
        wall = time.perf_counter() - t1
        M2.close()
        out["e2e"] = {"value": npts / wall / 1e9, "unit": "GPts/s", "h2d_bytes_per_step": h2d,
                      "d2h_bytes_per_step": lam.nbytes + mu.nbytes + rho.nbytes, "wall_s": wall,
                      "includes": "handle creation, grid and model upload, one evaluation, lambda/mu/rho read back"}
    M.close()
    print(json.dumps(out), flush=True)
    return 0


def assm_workload(grid=None, brick=4, seed=0, shuffle=False):
    """Inversion blocks of brick^3 kernel points tiling a kernel volume of the C2 grid's size,
    random cell volumes, and two kernel volumes (phase Vp and Vs) in Fortran order.  Each
    block lists its pixels i fastest, the order a generator looping over k, j, i writes
    (shuffle: one random order, the worst case for cache reuse)."""
    ki, kj, kk = (int(v) for v in (grid or "400x400x200").lower().split("x"))
    if ki % brick or kj % brick or kk % brick:
        raise SystemExit(f"the kernel volume must be a multiple of {brick} in every direction")
    rng = np.random.default_rng(seed)
    nb = (ki // brick, kj // brick, kk // brick)
    nblk, max_pix = nb[0] * nb[1] * nb[2], brick ** 3
    order = rng.permutation(max_pix) if shuffle else np.arange(max_pix)
    loc = np.array(np.unravel_index(order, (brick,) * 3, order="F"), np.int32)
    bidx = np.array(np.unravel_index(np.arange(nblk), nb, order="F"), np.int32)
    pixs = np.empty((3, max_pix, nblk), np.int32)
    for d in range(3):
        pixs[d] = loc[d][:, None] + brick * bidx[d][None, :] + 1
    npix = np.full(nblk, max_pix, np.int32)
    volume = (rng.uniform(0.5, 2.0, (max_pix, nblk)) * 1.0e6).astype(np.float32)
    kernels = [np.asfortranarray(rng.standard_normal((ki, kj, kk), np.float32) * np.float32(1e-10)) for _ in range(2)]
    desc = (f"projection of two {ki}x{kj}x{kk} kernel volumes (phase Vp, Vs) onto {nblk} inversion blocks of "
            f"{brick}x{brick}x{brick} points (pixels {'in a shuffled order' if shuffle else 'i fastest'})")
    return (ki, kj, kk), volume, npix, pixs, kernels, desc


# Algorithmic DRAM bytes of one projection: per pixel its offset and volume (8 B) and the
# kernel values (4 B per volume); per block its pixel count, B written and S read and written
def assm_bytes(nvol, nblk, nq):
    return nvol * (8 + 4 * nq) + nblk * (4 + 12 * nq)


def run_assm(args, rank):
    """The kernel assembly (fwant_assm_*): K projections of two kernel volumes on the device
    (kernel time from CUDA events around the projection launch), the restatement's projection
    on the host, and the end-to-end call with host kernels (upload, projection, blocks back)."""
    import fwant_gb300 as fw
    if rank != 0:
        return 0
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    shape, volume, npix, pixs, ks, desc = assm_workload(args.grid, shuffle=args.assm_shuffle)
    nvol, nblk = int(np.prod(shape)), volume.shape[1]
    A = fw.Assm(shape, volume, npix, pixs, device=dev)
    warm = max(args.warmup, 3)
    for _ in range(warm):
        A.project(ks)
    clocks = Clocks(dev)
    clocks.start()
    ms, walls = [], []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        B = A.project(ks)
        walls.append(time.perf_counter() - t1)
        ms.append(A.last_ms())
    clk = clocks.stop()
    dev_ms = float(np.sum(ms))
    value = 2 * nvol * args.steps / (dev_ms * 1e-3) / 1e9
    achieved = assm_bytes(nvol, nblk, 2) * args.steps / (dev_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    out = {
        "metric": "kernel points assembled per second", "value": value, "unit": "GPts/s", "n_gpus": 1,
        "steps": args.steps, "warmup": warm, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "replicas only", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": desc, "l2": f"kernels and pixel lists ({(8 + 8) * nvol / 1e6:.0f} MB) larger than L2 "
                                            f"(no flush)", "step": "one pick: both volumes onto every block"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": None,
                     "algorithmic_bytes_per_launch": assm_bytes(nvol, nblk, 2)},
        "clocks": clk, "gpu_launches": args.steps,
        "e2e": {"value": 2 * nvol * args.steps / float(np.sum(walls)) / 1e9, "unit": "GPts/s",
                "h2d_bytes_per_step": 2 * 4 * nvol, "d2h_bytes_per_step": 2 * 4 * nblk,
                "includes": "kernel upload from host arrays, projection, block values read back"},
    }
    if not args.no_cpu_baseline:
        from oracle import assm_oracle as AO
        t1 = time.perf_counter()
        want = AO.project(ks[0], volume, npix, pixs)
        dt = time.perf_counter() - t1
        out["config"]["matches_restatement"] = bool(np.array_equal(B[0], want))
        out["cpu_baseline"] = {"value": nvol / dt / 1e9, "unit": "GPts/s", "cores": 1, "kind": "port",
                               "sample": f"one volume's projection by the numpy restatement, {dt:.1f} s"}
    A.close()
    print(json.dumps(out), flush=True)
    return 0


def run_reference_assm(args):
    """the restatement's projection (numpy, one thread), each step one kernel volume"""
    from oracle import assm_oracle as AO
    shape, volume, npix, pixs, ks, desc = assm_workload(args.grid, shuffle=args.assm_shuffle)
    nvol = int(np.prod(shape))
    steps = max(1, min(args.steps, 4))
    for _ in range(1):
        AO.project(ks[0], volume, npix, pixs)
    t0 = time.perf_counter()
    for s in range(steps):
        AO.project(ks[s % 2], volume, npix, pixs)
    dt = time.perf_counter() - t0
    sample = f"{steps} single-volume projections of the restatement (numpy, 1 thread)"
    return _reference_line(args, "kernel points assembled per second", "GPts/s", nvol * steps / dt / 1e9, dt, desc,
                           sample, 1, "f32")


# GB300's FP64 FMA rate: no measured figure is available to the benchmark, so the nominal
# dense FP64 rate stands as the denominator of the kernel-accumulation roofline
FP64_NOMINAL_TFLOPS = 1.25


def ker_block(npts, knt=500, seed=0):
    rng = np.random.default_rng(seed)
    lam = np.full(npts, 3.0e10, np.float32) * (1 + 0.05 * rng.random(npts, dtype=np.float32))
    mu = np.full(npts, 2.5e10, np.float32) * (1 + 0.05 * rng.random(npts, dtype=np.float32))
    sgt = [rng.standard_normal((6, knt, npts), dtype=np.float32) for _ in range(4)]
    return lam, mu, sgt


def run_ker(args, rank):
    """The sensitivity-kernel accumulation (fwant_sgtker_*): sgt2scatter3 of the three
    receiver force components against the source SGT for every point of one block (FP64
    sums on the GPU), timed on the device; the oracle's FP64-accumulation form on a sample
    of the points on the host; and the end-to-end job (upload the media and four SGT series,
    scatter, window integrals of the three components, kernels read back)."""
    import fwant_gb300 as fw
    if rank != 0:
        return 0
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    npts, knt, kdt = args.ker_points, 500, 0.1
    lam, mu, sgt = ker_block(npts, knt)
    # 7 FMA per lag for each of the 3 components, knt (knt - 1) / 2 lags per point
    dfma = npts * 3 * 7 * knt * (knt - 1) / 2
    K = fw.SgtKernel(npts, knt, kdt, device=dev)
    K.set_media(lam, mu)
    for w in range(4):
        K.set_sgt(w, sgt[w])
    warm = max(args.warmup, 3)
    for _ in range(warm):
        K.scatter(7)
    clocks = Clocks(dev)
    clocks.start()
    ms = []
    for _ in range(args.steps):
        K.scatter(7)
        ms.append(K.last_scatter_ms())
    clk = clocks.stop()
    K.close()
    dev_ms = float(np.sum(ms))
    tflops = 2 * dfma * args.steps / (dev_ms * 1e-3) / 1e12
    out = {
        "metric": "sensitivity-kernel accumulation FP64 throughput", "value": tflops, "unit": "TFLOP/s",
        "n_gpus": 1, "steps": args.steps, "warmup": warm, "ms_per_step": dev_ms / args.steps,
        "higher_is_better": True, "scaling": "replicas only", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": f"sgt2scatter3 of one SGT block: {npts} kernel points x {knt} frames, receiver "
                               f"X, Y, Z force SGTs against the source SGT (flags 7), FP64 sums",
                   "step": "one fwant_sgtker_scatter over the block", "l2": "SGT series (786 MB) larger than L2"},
        "roofline": {"bound": "fp64", "achieved": tflops, "peak": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                     "frac": tflops / FP64_NOMINAL_TFLOPS, "peak_source": "nominal GB300 dense FP64 rate",
                     "traffic": None},
        "clocks": clk, "gpu_launches": args.steps,
    }
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        threads = O.set_threads(os.cpu_count() or 1, timing=True)
        ns = min(npts, 2048)
        sub = [a[:, :, :ns].copy() for a in sgt]
        t1 = time.perf_counter()
        O.sgt2scatter3(lam[:ns], mu[:ns], sub[:3], sub[3], kdt, mode=1, timing=True)
        dt = time.perf_counter() - t1
        out["cpu_baseline"] = {"value": 2 * dfma * ns / npts / dt / 1e12, "unit": "TFLOP/s", "cores": threads,
                               "kind": "port", "sample": f"{ns} of the {npts} points, same series, {dt:.1f} s",
                               "build": O.build_flags(timing=True)}
    if not args.no_e2e:
        v = np.sin(np.arange(knt, dtype=np.float32) * np.float32(0.05))
        u = np.cos(np.arange(knt, dtype=np.float32) * np.float32(0.05))
        t1 = time.perf_counter()
        K2 = fw.SgtKernel(npts, knt, kdt, device=dev)
        K2.set_media(lam, mu)
        for w in range(4):
            K2.set_sgt(w, sgt[w])
        K2.scatter(7)
        outs = K2.kernel(3, v, u, 50, 450, 1.0e15)
        wall = time.perf_counter() - t1
        K2.close()
        out["e2e"] = {"value": 2 * dfma / wall / 1e12, "unit": "TFLOP/s",
                      "h2d_bytes_per_step": lam.nbytes + mu.nbytes + sum(a.nbytes for a in sgt) + v.nbytes + u.nbytes,
                      "d2h_bytes_per_step": sum(o.nbytes for o in outs), "wall_s": wall,
                      "includes": "handle creation, media and SGT upload, one scatter, window integrals, kernels read back"}
    print(json.dumps(out), flush=True)
    return 0


def c3_batched_vs_single(dev, steps):
    """C3's 32 seeded virtual sources of uneven sizes (160-320 x 160-320 x 80-160, C2
    physics, one surface force each): device time per source and step when the members
    are stepped as one batch (one launch per RK stage and group of up to 16 members, the
    interior-only and full forms where a stage has both) against each member stepped
    alone (its own launches).  Both legs replay 8-step CUDA graphs; CUDA events."""
    import fwant_gb300 as fw
    from fwant_gb300 import inputs
    t0 = time.perf_counter()
    models = inputs.config_c3(seed=0)
    sims = [inputs.attach(fw.Solver(m.ni, m.nj, m.nk, m.stept, device=dev), m) for m in models]
    npts = sum(m.npoints for m in models)
    n = len(models)
    b = fw.Batch(sims)
    b.run(8)  # warm-up block (graph capture)
    b.run(steps)
    batched_ms = b.last_run_ms()
    launches = b.launches_per_step()
    b.close()
    single_ms = 0.0
    for s in sims:
        s.run(8)
        s.run(steps)
        single_ms += s.last_run_ms()
    for s in sims:
        s.close()
    return {
        "workload": f"C3: {n} virtual sources, {npts / 1e6:.1f} M interior points in all, {steps} steps per leg",
        "batched_ms_per_source_step": batched_ms / steps / n,
        "single_ms_per_source_step": single_ms / steps / n,
        "batched_value": npts * steps / (batched_ms * 1e-3) / 1e9,
        "single_value": npts * steps / (single_ms * 1e-3) / 1e9,
        "unit": "GPts/s",
        "speedup": single_ms / batched_ms,
        "batched_launches_per_step": launches,
        "wall_s": time.perf_counter() - t0,
    }


# The other rows of the hot path, each run briefly as its own process (own device memory,
# own CUDA context) with the same flags a user would give it; the default C2 line carries
# their measured figures so that every row has a number from the same run.
COMPANIONS = (("c1", "c1", ["--steps", "2008", "--warmup", "8"]),
              ("c1_hill", "c1", ["--steps", "2008", "--warmup", "8", "--hill"]),
              ("media", "media", ["--steps", "3", "--warmup", "3"]),
              ("ker", "ker", ["--steps", "3", "--warmup", "3"]),
              ("assm", "assm", ["--steps", "5", "--warmup", "3"]),
              ("lsqr", "lsqr", ["--steps", "20", "--warmup", "3"]))


def companions():
    import subprocess
    out = {}
    for name, cfg, extra in COMPANIONS:
        t0 = time.perf_counter()
        cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--config", cfg, "--no-cpu-baseline", "--no-e2e",
               *extra]
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=600,
                               env={k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE")})
        except subprocess.TimeoutExpired:
            out[name] = {"failed": "timed out after 600 s"}
            continue
        line = next((x for x in reversed(r.stdout.splitlines()) if x.startswith("{")), None)
        if r.returncode != 0 or line is None:
            out[name] = {"failed": (r.stderr or r.stdout)[-300:]}
            continue
        d = json.loads(line)
        roof = d.get("roofline") or {}
        out[name] = {"metric": d.get("metric"), "value": d.get("value"), "unit": d.get("unit"),
                    "ms_per_step": d.get("ms_per_step"), "roofline_frac": roof.get("frac"),
                    "roofline_bound": roof.get("bound"), "workload": (d.get("config") or {}).get("workload"),
                    "flags": " ".join(extra), "wall_s": time.perf_counter() - t0}
    return out


def run_c1_hill(args, rank):
    """C1 as specified: the 100x100x60 model with the seeded 2 km Gaussian hill on top (the
    terrain-following extension, which steps one solver alone), 2008 steps by default.  Device
    time of the time loop (8-step CUDA graphs), per-stage CUDA events."""
    import fwant_gb300 as fw
    from fwant_gb300 import inputs
    if rank != 0:
        return 0
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    m = inputs.config_c1(seed=0)
    h = inputs.gaussian_hill(m, 2000.0, seed=0)
    s = inputs.attach(fw.Solver(m.ni, m.nj, m.nk, m.stept, device=dev), m)
    s.set_topography(h)
    stage_ms, end_ms = s.profile_stages(8)
    warm = max(args.warmup, 3)
    s.run(warm)
    clocks = Clocks(dev)
    clocks.start()
    s.run(args.steps)
    dev_ms = s.last_run_ms()
    clk = clocks.stop()
    scheme = s.rk_scheme
    s.check()
    s.close()
    npts = int(m.npoints)
    # the terrain form also reads the plane's four metric values per point and stage
    algo = (bytes_pt_step("fp32", scheme) + 4 * 4 * 4) * npts + bytes_pml_pt_step(scheme) * slab_points(m)
    launch_ms = float(np.mean(stage_ms))
    peak, peak_kind = peaks()
    achieved = algo / 4.0 / (launch_ms * 1e-3) / 1e9
    out = {
        "metric": "grid-point updates per second", "value": npts * args.steps / (dev_ms * 1e-3) / 1e9,
        "unit": "GPts/s", "n_gpus": 1, "steps": args.steps, "warmup": warm, "ms_per_step": dev_ms / args.steps,
        "higher_is_better": True, "scaling": "replicas only", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": "C1: 100x100x60 with a seeded 2 km Gaussian hill (terrain-following grid), FP32, "
                               "12-cell CFS-PML x5, free surface, Fz Ricker 0.2 Hz, 16 receivers",
                   "l2": "inputs smaller than L2 (the C1 size)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": None, "stage_ms": stage_ms, "step_end_ms": end_ms,
                     "rk_scheme": scheme},
        "clocks": clk, "gpu_launches": (4 + 1) * args.steps,
    }
    print(json.dumps(out), flush=True)
    return 0


def run_surrogate(args, rank):
    """C5 workload: the surrogate's screening speedup over FD solves at 1% waveform error."""
    from fwant_gb300 import surrogate
    if rank != 0:
        return 0
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    t0 = time.perf_counter()
    r = surrogate.run_c5(device=dev)
    wall = time.perf_counter() - t0
    out = {
        "metric": "surrogate screening speedup over FD solves at 1% waveform error", "value": r["speedup"],
        "unit": "x", "n_gpus": 1, "steps": r["n_test"], "warmup": 0, "higher_is_better": True,
        "scaling": "replicas only", "vs_baseline": None, "dtype": "bf16 weights, f32 accumulation",
        "data": "synthetic (seeded)",
        "config": {"workload": f"C5: {r['n_train'] + r['n_val']} FD solves at {r['grid']} with +/-5% Vs "
                               f"perturbations ({r['corr_km']} km correlation) train an ensemble of {r['ensemble']} "
                               f"networks; {r['n_test']} held-out models screened"},
        "surrogate": r, "wall_s": wall,
    }
    print(json.dumps(out), flush=True)
    return 0


def run_ours(args, rank, world):
    import fwant_gb300 as fw
    from fwant_gb300 import inputs
    if args.config == "c1" and args.hill:
        return run_c1_hill(args, rank)
    if args.config == "c5":
        return run_surrogate(args, rank)
    if args.config == "lsqr":
        return run_lsqr(args, rank)
    if args.config == "media":
        return run_media(args, rank)
    if args.config == "ker":
        return run_ker(args, rank)
    if args.config == "assm":
        return run_assm(args, rank)
    dist = Dist(world)
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    fw.load_library()
    models, desc = make_models(args.config, seed=rank, grid=args.grid, sims=args.sims)
    storage = {"fp32": fw.STORAGE_FP32, "bf16": fw.STORAGE_BF16, "fp16": fw.STORAGE_FP16}[args.storage]

    def make_solver(m):
        s = fw.Solver(m.ni, m.nj, m.nk, m.stept, device=dev, storage=storage)
        if args.storage == "fp16":
            # a 1e15 N surface force on 1 km cells peaks near 50 m/s and 1.2e9 Pa at the source
            s.set_storage_scale(2.0 ** 9, 2.0 ** -15)
        if args.tile_rows:
            s.tile_rows = args.tile_rows
        return s

    sims = [inputs.attach(make_solver(m), m) for m in models]
    npts = sum(m.npoints for m in models)
    # per-launch timing of the stage kernel (CUDA events around each launch, eager)
    # the simulations step together: each RK stage of all of them is one launch
    batch = fw.Batch(sims)
    tuned = None
    if args.autotune:
        t_tune = time.perf_counter()
        ctas = batch.autotune(4)
        tuned = {"planes_per_cta": [s.planes_per_cta for s in sims], "tile_rows": sims[0].tile_rows,
                 "tile": f"32x{sims[0].tile_rows}", "ctas": ctas, "lean_stages": sims[0].lean_stages,
                 "tune_s": time.perf_counter() - t_tune}
    # per-launch timing of the stage kernel (CUDA events around each launch, eager)
    stage_ms, end_ms = batch.profile_stages(8)
    launches = batch.launches_per_step()
    warm = max(args.warmup, 3)
    batch.run(warm)
    clocks = Clocks(dev, period_ms=50)  # the timed region of C2 lasts a few hundred ms
    dist.barrier()
    clocks.start()
    t_host = time.perf_counter()
    batch.run(args.steps)  # whole 8-step blocks replay a CUDA graph; returns after device completion
    dev_ms = batch.last_run_ms()
    t_host = time.perf_counter() - t_host
    clk = clocks.stop()
    finite = True
    for s in sims:
        try:
            s.check()
        except fw.FwantError:
            finite = False
    dist.barrier()
    dev_ms = dist.max(dev_ms)
    value = replica_value(world, npts, args.steps, dev_ms)

    # roofline of the stage kernel: one launch covers one stage of every simulation
    m0 = models[0]
    scheme = sims[0].rk_scheme
    algo_bytes_step = sum(bytes_pt_step(args.storage, scheme) * int(m.npoints) + bytes_pml_pt_step(scheme) *
                          slab_points(m) for m in models)
    launch_ms = float(np.mean(stage_ms))
    achieved = algo_bytes_step / 4.0 / (launch_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    tr = ncu_traffic_ratio(scheme, args.storage)
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": peak_kind, "traffic": (tr * algo_bytes_step / 4.0) if tr else None,
            "traffic_note": "bytes per stage (its interior-only and full launches): ncu DRAM/algorithmic "
                            "ratio (profiles/stage_batch_kernel_" + ("c2" if args.storage == "fp32" else "bf16_c2")
                            + ".md) x algorithmic bytes of the stage",
            "stage_ms": stage_ms, "step_end_ms": end_ms,
            "algorithmic_bytes_per_stage": algo_bytes_step / 4.0, "rk_scheme": scheme}
    if scheme == 1:
        # the same time against the bytes of RK form 0 (t carried, the reference's registers):
        # how close the step comes to what the carried-t scheme could reach at the copy peak
        ref_bytes_step = sum(bytes_pt_step(args.storage, 0) * int(m.npoints) + bytes_pml_pt_step(0) *
                             slab_points(m) for m in models)
        ach0 = ref_bytes_step / 4.0 / (launch_ms * 1e-3) / 1e9
        roof["form0_equivalent"] = {"achieved": ach0, "frac": ach0 / peak, "unit": "GB/s",
                                    "algorithmic_bytes_per_stage": ref_bytes_step / 4.0}

    out = {
        "metric": "grid-point updates per second", "value": value, "unit": "GPts/s", "n_gpus": world,
        "steps": args.steps, "warmup": warm, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": desc, "points_per_step": npts, "l2": "inputs larger than L2 (no flush)",
                   "storage": args.storage, "tile": f"32x{sims[0].tile_rows}", "fields_finite_after_run": finite,
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
        "host_wall_s": t_host, "roofline": roof, "clocks": clk, "autotune": tuned,
        # per step, as the batch counts them: per group of up to 16 simulations and per stage
        # the interior-only launch (where that stage has one) and the full launch, and the
        # step-end (receivers + step counter) kernel of every simulation
        "gpu_launches": args.steps * launches,
    }
    if args.config == "c3":
        # the same simulations launched one at a time (one simulation per stage launch)
        single_ms = 0.0
        for s in sims:
            s.run(8)
            s.run(args.steps)
            single_ms += s.last_run_ms()
        out["config"]["single_launch_value"] = npts * args.steps / (single_ms * 1e-3) / 1e9
        out["config"]["single_launch_ms_per_step"] = single_ms / args.steps
    batch.close()
    for s in sims:
        s.close()

    if not args.no_e2e:
        # The whole job through the public API: create, upload the model from host arrays,
        # run, read the seismograms back; host wall clock.  C2 is a 4000-step job with one
        # upload of the medium; the leg runs a quarter of it (or --e2e-steps).
        esteps = args.e2e_steps or (1000 if args.config == "c2" and not args.grid else args.steps)
        eclocks = Clocks(dev)
        eclocks.start()
        t0 = time.perf_counter()
        h2d = d2h = 0
        esims = []
        for m in models:
            s = make_solver(m)
            inputs.attach(s, m)
            if tuned:
                s.planes_per_cta = tuned["planes_per_cta"][len(esims)]
                s.lean_stages = tuned["lean_stages"]
                s.tile_rows = tuned["tile_rows"]
            esims.append(s)
            h2d += 3 * m.lam.nbytes + m.x.nbytes + m.y.nbytes + m.z.nbytes
        eb = fw.Batch(esims)
        if tuned:
            eb.set_ctas(tuned["ctas"])
        eb.run(esteps)
        for s in esims:
            sg = s.get_seismo()
            d2h += sg.nbytes
        eb.close()
        for s in esims:
            s.close()
        t_e2e = dist.max(time.perf_counter() - t0)
        eclk = eclocks.stop()
        out["e2e"] = {"value": world * npts * esteps / t_e2e / 1e9, "unit": "GPts/s",
                      "h2d_bytes_per_step": h2d // esteps, "d2h_bytes_per_step": d2h // esteps,
                      "steps": esteps, "wall_s": t_e2e, "clocks": eclk,
                      "includes": "solver creation, model upload, run, seismogram download"}
    if args.config == "c2" and not args.grid and not args.no_c3 and world == 1:
        out["batched_vs_single"] = c3_batched_vs_single(dev, max(8, args.c3_steps // 8 * 8))
    if args.config == "c2" and not args.grid and not args.no_companions and world == 1:
        out["companions"] = companions()
    if rank == 0 and not args.no_cpu_baseline:
        v, thr, dt = cpu_sample(models, args.cpu_steps)
        out["cpu_baseline"] = {"value": v, "unit": "GPts/s", "cores": thr, "kind": "port",
                               "build": _timing_flags(), "checker_build": _checker_flags(),
                               "sample": f"{args.cpu_steps} time steps of one simulation "
                                         f"({m0.ni}x{m0.nj}x{m0.nk}), {dt:.1f} s"}
    if rank == 0:
        print(json.dumps(out), flush=True)
    dist.close()
    return 0


def main():
    args = parse_args()
    rank, world, _ = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world)


if __name__ == "__main__":
    sys.exit(main())
