#!/usr/bin/env python3
"""Benchmark of the GB300 RK4 substep library on the 256^3 + 8M-particle
heated, two-way-coupled workload (the headline configuration).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One JSON line on stdout (rank 0).  `value` is whole-job Mcell-steps/s with the
state resident in HBM; `e2e` is the same metric through the C ABI with the
step-boundary state round-tripped every step between pinned host buffers and
the device in one tpm_step_state call (its transfers overlapping the step;
`three_calls` times tpm_load_state / tpm_step / tpm_save_state instead).  At
one GPU the default run adds `ensemble48` and `adjoint64`: summaries of the
48-box batched ensemble and of the 200-step discrete adjoint (each also runs
alone with --workload; --no-extras skips them).  With
--gpus N > 1 every rank runs an independent replica box (the path does not
shard), and `value` sums the cells of all ranks over the slowest rank's time.
`--impl reference` times the reference's CPU implementation of the path on
this host instead (the reference build when it exists here, else the C
restatement of it), on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "triplyperiodic-modified_gb300"))

METRIC = "Mcell-steps/s at 256³+8M particles, mixed vs FP64 on 1 GB300; % HBM roofline"
UNIT = "Mcell-steps/s"
WORKLOAD = "box256_p8e6_heated"
FALLBACK_HBM_GBS = 6800.0

# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of a
# kernel on a workload, the mean over the launches of one single-pass ncu
# capture of every kernel of this bench's two profiled steps (the command is
# in the summary of the capture)
NCU_TRAFFIC = {
    ("box256_p8e6_heated", True, "fft_x_fwd_resid"): 8.644e8,
    ("box256_p8e6_heated", True, "particle_push"): 3.849e9,
    ("box256_p8e6_heated", True, "rhs_momentum"): 2.007e9,
    ("box256_p8e6_heated", True, "poisson_rhs"): 1.279e9,
    ("box256_p8e6_heated", True, "rho_update"): 1.347e9,
    ("box256_p8e6_heated", False, "rhs_momentum"): 2.595e9,
    ("box256_p8e6_heated", False, "fft_x_fwd_resid"): 9.36e8,
}

# FP64 path: FP64 operations per cell per launch of a kernel, from one ncu
# capture of two eager FP64 steps of the 128^3 box with 1e6 particles
# (0.48 particles per cell, the headline workload's density):
# (flops = 2 DFMA + DADD + DMUL thread instructions, FP64-pipe thread
# instructions of any kind), both divided by the cells of a launch.  The FP64
# kernels keep the reference's unfused multiply-adds (parity), so a flop
# costs about one pipe instruction; the FMA peak counts two per instruction.
FP64_OPS = {
    "rhs_momentum": (203.0, 222.1),
    "fft_x_fwd_resid": (47.6, 44.8),
    "fft_y": (15.2, 13.1),
    "fft_z_solve": (28.6, 27.6),
    "fft_x_inv_update": (19.5, 20.8),
}
FP64_FLOP_PER_CELL_STEP = 4090.7  # all kernels of a step, same capture

# Algorithmic bytes per launch of each kernel, (bytes per cell, bytes per
# particle), for FP64 storage: each value a kernel must read or write once.
# `value` is the headline (mixed-precision) path; the FP64 path is reported
# beside it under "fp64".
KERNEL_BYTES = {
    # U, RU_int, F_p, RU, RU_np1 in; RU_np1, RU_new out (3 each)
    "rhs_momentum": (21 * 8, 0),
    # RU_new 3, Rho_new, Q, face coefficients 3 in; RHS, divergence, cc out
    "poisson_rhs": (11 * 8, 0),
    "poisson_faces": (10 * 8, 0),
    # P, C 3, cc, RHS in; the half spectrum (one complex per two cells) out
    "fft_x_fwd_resid": (6 * 8 + 8, 0),
    # the half spectrum in and out
    "fft_y": (16, 0),
    "fft_z_solve": (16, 0),
    # the half spectrum in; P in and out
    "fft_x_inv_update": (24, 0),
    "deposit_heat": (4 + 8, 32),
    "deposit_conc": (4 + 8, 24),
    "deposit_momentum": (4 + 24, 48),
    # base, int and np1 sets in, np1 and new out (7 values each), heat rate in
    # and out, the cell keys and deposit payloads out
    "particle_push": (0, 488),
    # RU_int 3, Rho_int in; U 3 out
    "face_velocity": (7 * 8, 0),
    # RU_int 3, Rho, Rho_np1 in; Rho_new, Rho_np1, 1/Rho_new, T out
    "rho_update": (9 * 8, 0),
    # P, RU_new 3, RU_np1 3 in; RU_new 3, RU_np1 3 out
    "project": (13 * 8, 0),
}


def peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        for k in ("hbm_gbs", "hbm_GBs", "copy_gbs"):
            if k in d:
                return float(d[k]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- GPU arm
def make_workload(name=WORKLOAD, precision=0, N=None, npart=None, grid=None):
    """The workload's parameters and seeded state; `grid` (nx, ny, nz) replaces
    its cubic box by one of equal cells (a small case of the same kernels)."""
    from tpm import inputs, params as P

    w = dict(P.WORKLOADS[name])
    N = N or w["N"]
    npart = npart if npart is not None else w["npart"]
    p = P.physical(N, npart, nu=w["nu"], A=w["A"], tau_p=w["tau_p"],
                   mass_loading=w["mass_loading"], heating_Q=w["heating_Q"], iterations=20,
                   epsilon=1e-13, precision=precision)
    if grid:
        nx, ny, nz = grid
        d = p.Lx / p.Nx
        p = p.replace(Nx=nx, Ny=ny, Nz=nz, Lx=d * nx, Ly=d * ny, Lz=d * nz)
    s = inputs.make_state(p, npart, seed=w["seed"])
    p = p.replace(dt=inputs.cfl_dt(p, s.RU))
    return p, s


def time_gpu(p, s, steps, warmup, dist, device, tiles=None):
    import torch
    from tpm import capi

    ctx = capi.Context(p, s.npart)
    ctx.load(s)
    if tiles:  # fixed FFT tiles (reproducible launch shapes, e.g. under a profiler)
        ctx.set_fft_tiles(tiles)
        pens = list(tiles)
    else:
        pens = ctx.autotune()  # FFT pencils per block for this grid (results do not change)
    ctx.initialize()
    ctx.set_graph(True)  # each step one CUDA graph launch (bit-identical to eager steps)
    for _ in range(warmup):
        ctx.step()
    ctx.sync()
    stream = torch.cuda.ExternalStream(ctx.stream(), device=device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    it0 = ctx.scalars()["total_poisson_iterations"]
    l0 = ctx.launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(device) as clk:
        e0.record(stream)
        ctx.run(steps)
        e1.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    sc = ctx.scalars()
    iters = sc["total_poisson_iterations"] - it0
    n_it = iters / (4.0 * steps)
    # the launch counter counts a graph's Poisson loop body (6 kernels) once per
    # solve; the device repeats it once per further iteration
    launches = ctx.launch_count() - l0 + 6 * max(0, iters - 4 * steps)
    # per-kernel durations (CUDA events around each launch on the same stream;
    # profiled steps run eagerly).  The NVTX range lets an ncu launch list
    # take exactly these two steps (ncu --nvtx --nvtx-include profiled_steps/).
    import torch

    ctx.profile(True)
    torch.cuda.nvtx.range_push("profiled_steps")
    ctx.run(2)
    ctx.sync()
    torch.cuda.nvtx.range_pop()
    prof = ctx.profile_report()
    ctx.profile(False)
    ctx.fft_pens = pens
    return ctx, ms, n_it, launches, prof, clk.summary()


def time_e2e(ctx, steps, warmup=3):
    """Same metric through the C ABI with host buffers: every step takes the
    step-boundary state from pinned host memory and returns it there.  Timed
    through tpm_step_state (load, step and save in one call, the transfers
    overlapping the step: the headline), and through the three calls
    tpm_load_state, tpm_step and tpm_save_state (their host-clock split
    reported beside it).  `warmup` untimed rounds of each first: the device
    buffers alternate between two layouts from step to step, and the first
    step in each captures its CUDA graphs."""
    import numpy as np
    import torch

    st = ctx.download_state()

    def pinned_like(a):
        t = torch.empty(a.shape, dtype=torch.float64 if a.dtype == np.float64 else torch.int32,
                        pin_memory=True)
        v = t.numpy()
        v[...] = a
        return v

    host = {k: pinned_like(st[k]) for k in ctx.STATE_FIELDS}
    if ctx.npart:
        host["part"] = {q: pinned_like(v) for q, v in st["part"].items()}
        host["RHS_T"] = pinned_like(st["RHS_T"])
    host["scalars"] = st["scalars"]
    h2d = sum(host[k].nbytes for k in ctx.STATE_FIELDS)
    if ctx.npart:
        h2d += sum(v.nbytes for v in host["part"].values()) + host["RHS_T"].nbytes
    # one call per step
    for _ in range(warmup):
        host = ctx.step_state(host, out=host)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        host = ctx.step_state(host, out=host)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / steps
    # three calls per step
    for _ in range(warmup):
        ctx.upload_state(host)
        ctx.step()
        host = ctx.download_state(out=host)
    torch.cuda.synchronize()
    parts = [0.0, 0.0, 0.0]  # upload and resume, step, download (host clock)
    t1 = time.perf_counter()
    for _ in range(steps):
        ta = time.perf_counter()
        ctx.upload_state(host)
        tb = time.perf_counter()
        ctx.step()
        ctx.sync()
        tc = time.perf_counter()
        host = ctx.download_state(out=host)
        td = time.perf_counter()
        parts[0] += tb - ta
        parts[1] += tc - tb
        parts[2] += td - tc
    torch.cuda.synchronize()
    ms3 = (time.perf_counter() - t1) * 1e3 / steps
    split = {"ms_per_step": round(ms, 3),
             "three_calls": {"ms_per_step": round(ms3, 3),
                             "upload_and_resume_ms": round(parts[0] * 1e3 / steps, 3),
                             "step_ms": round(parts[1] * 1e3 / steps, 3),
                             "download_ms": round(parts[2] * 1e3 / steps, 3)}}
    return ms, h2d, h2d, split


def cpu_sample(workload):
    """The bounded CPU sample of a workload: a 128^3 box (the workload's own
    box if smaller) at the workload's particle density and physics."""
    from tpm import params as P

    w = P.WORKLOADS[workload]
    Ns = min(128, w["N"])
    nps = int(round(w["npart"] * (Ns / w["N"]) ** 3))
    p, s = make_workload(workload, 0, N=Ns, npart=nps)
    return Ns, nps, p, s


def host_info():
    """Core count and CPU model of this host."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"cores": os.cpu_count(), "model": model or platform.machine()}


def cpu_rate(workload, warmup, steps):
    """The reference's CPU implementation of the step on one host core, on the
    bounded sample of the workload: the reference's own build where it was
    compiled on this host (its step loop timed by its own clock), else the C
    restatement of it (warm-up steps, then the timed steps).  Returns the
    rate, the Poisson iterations per solve of the timed steps (the C
    restatement's count; the reference's FFT solver does not record it,
    poisson.cpp:391-411) and a description of the sample."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import pyoracle

    pyoracle.build()
    Ns, nps, p, s = cpu_sample(workload)
    n_it = None
    if pyoracle.have_reference():
        kind = "reference"
        secs = pyoracle.run_reference(p, s, steps)["seconds"]
        what = "the reference's own sources built on this host"
    else:
        kind = "port"
        o = pyoracle.Oracle(p, s.npart)
        o.load(s)
        o.initialize()
        for _ in range(warmup):
            o.step()
        it0 = o.scalars()["total_poisson_iterations"]
        t0 = time.perf_counter()
        for _ in range(steps):
            o.step()
        secs = time.perf_counter() - t0
        n_it = (o.scalars()["total_poisson_iterations"] - it0) / (4.0 * steps)
        o.close()
        what = f"the C restatement of the reference, after {warmup} warm-up step(s)"
    host = host_info()
    return {"value": round(p.ncell * steps / secs / 1e6, 4), "unit": UNIT, "cores": 1,
            "kind": kind, "n_it": n_it, "seconds_per_step": round(secs / steps, 3),
            "host": host,
            "sample": f"{steps} RK4 step(s) of a {Ns}^3 box with {nps} particles (the workload's "
                      f"particle density and physics), {secs / steps:.1f} s per step on one core "
                      f"of a {host['cores']}-core {host['model']} host, {what}"}


def cpu_baseline_port(workload):
    """The reported CPU baseline of the GPU arm: the same sample and step
    count as the reference arm (2 timed steps after 1 warm-up step)."""
    return cpu_rate(workload, 1, 2)


def max_over_ranks(x, dist, device="cpu"):
    """Max of a per-rank float over the job (the slowest rank sets the time)."""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, ncell, steps, max_ms):
    """Replicas: every rank advances its own box of `ncell` cells `steps` times;
    the job's rate is all ranks' cell-steps over the slowest rank's time."""
    return world * ncell * steps / (max_ms * 1e-3) / 1e6


def kernel_bytes(name, ncell, npart, mixed):
    bc, bp = KERNEL_BYTES.get(name, (0, 0))
    if not mixed and name == "poisson_rhs":  # FP64: face values precomputed by poisson_faces
        bc = 10 * 8
    if mixed:  # complex64 spectrum on the mixed path; its fused TMA passes
        # (on grids of whole 32 x 8 tiles): the density update with the face
        # velocity (RU_int 3, Rho_int, Rho, Rho_np1 in; Rho_np1, Rho_new, T and
        # U 3 in FP32 out) and the Poisson right-hand side with the face
        # coefficients (Rho_new, RU_new 3, Q in; RHS, divergence, cc in FP32,
        # C/d^2 3 as FP32 pairs out)
        bc = {"fft_y": 8, "fft_z_solve": 8, "fft_x_fwd_resid": 6 * 8 + 4,
              "fft_x_inv_update": 4 + 16, "rho_update": 6 * 8 + 3 * 8 + 12,
              "poisson_rhs": 5 * 8 + 2 * 8 + 4 + 3 * 8}.get(name, bc)
    return bc * ncell + bp * npart


def step_bytes(ncell, npart, n_it, mixed):
    """Algorithmic bytes per RK4 step (the fixed count per cell-step: 61
    stored values per cell and stage plus 15 per further Poisson iteration,
    and the mean reset), with the FFT traffic at the spectrum's width: N^3 [4 ((50 + 4 (n_it-1)) w + 11 n_it w_fft) + 9 w] + Np 4 (37 w_p + 16);
    w = w_p = 8 (FP64 state on both paths), w_fft = 8 (FP64) or 4 (mixed)."""
    w, wf = 8, (4 if mixed else 8)
    per_cell = 4 * ((50 + 4 * (n_it - 1)) * w + 11 * n_it * wf) + 9 * w
    return ncell * per_cell + npart * 4 * (37 * 8 + 16)


def path_result(p, s, ms, steps, world, n_it, launches, prof, clocks, mixed, peak,
                workload=None):
    ms_per_step = ms / steps
    dom_name, (nl, tot_ms) = max(prof.items(), key=lambda kv: kv[1][1])
    per_launch = kernel_bytes(dom_name, p.ncell, s.npart, mixed)
    achieved = per_launch / (tot_ms / nl * 1e-3) / 1e9
    sb = step_bytes(p.ncell, s.npart, n_it, mixed)
    sgbs = sb / (ms_per_step * 1e-3) / 1e9
    total_prof = sum(v[1] for v in prof.values())
    return {
        "value": whole_job_rate(world, p.ncell, steps, ms),
        "ms_per_step": ms_per_step, "n_it": n_it, "launches": launches, "clocks": clocks,
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": NCU_TRAFFIC.get((workload, mixed, dom_name)),
                     "algorithmic_bytes": int(per_launch),
                     "kernel_share": round(tot_ms / total_prof, 4)},
        "step_roofline": {"achieved_gbs": round(sgbs, 1), "frac": round(sgbs / peak, 4),
                          "algorithmic_bytes_per_step": int(sb)},
        "kernels_ms_per_step": {k: round(v[1] / 2, 3) for k, v in
                                sorted(prof.items(), key=lambda kv: -kv[1][1])},
        "kernel_launches_per_step": {k: v[0] / 2 for k, v in prof.items()},
        "mparticle_steps_per_s": world * s.npart * steps / (ms * 1e-3) / 1e6,
    }


def compare_paths(a, b, idx):
    """Per-field relative differences of context a (mixed) against b (FP64) at
    the same step: max|a - b| / max|b| per field and particle quantity, plus
    the particles whose interpolation cell differs between the two - by
    truncation, the gas-velocity cell (particle.cpp:340-360), or by rounding,
    the temperature and concentration cell (particle.cpp:430-456,522-555) -
    and the particles whose velocity differs by more than 1e-6 of the largest
    speed (the mark of a particle that took another cell's velocity)."""
    import numpy as np

    out = {}
    for g in ("RU", "RHO", "P", "C", "Q"):
        x, y = a.download_field(g), b.download_field(g)
        ymax = float(np.abs(y).max())
        if ymax < 1e-9:  # a field at roundoff level (Q of an unheated run): absolute
            out[g] = {"abs_diff": float(np.abs(x - y).max()), "fp64_max": ymax}
        else:
            out[g] = float(np.abs(x - y).max() / ymax)
    pa, pb = a.download_particles("base"), b.download_particles("base")
    out["particles"] = max(float(np.abs(pa[q] - pb[q]).max() / max(np.abs(pb[q]).max(), 1e-300))
                           for q in ("x", "y", "z", "u", "v", "w", "T"))
    trunc_diff = np.zeros(len(pa["x"]), bool)
    round_diff = np.zeros(len(pa["x"]), bool)
    for q, i in zip(("x", "y", "z"), idx):
        ua, ub = pa[q] * i, pb[q] * i
        trunc_diff |= np.trunc(ua) != np.trunc(ub)
        round_diff |= np.floor(ua + 0.5) != np.floor(ub + 0.5)
    vmax = max(float(np.abs(pb[q]).max()) for q in ("u", "v", "w"))
    vdiff = np.zeros(len(pa["x"]), bool)
    for q in ("u", "v", "w"):
        vdiff |= np.abs(pa[q] - pb[q]) > 1e-6 * vmax
    out["particles_other_cell_trunc"] = int(trunc_diff.sum())
    out["particles_other_cell_round"] = int(round_diff.sum())
    out["particles_velocity_off_1e-6"] = int(vdiff.sum())
    return out


def mixed_accuracy_fresh(p64, s, checkpoints=(1, 10)):
    """Mixed against FP64 from the same seeded state on fresh contexts,
    compared after exactly `checkpoints` RK4 steps (eager stepping; graph
    replay is bit-identical)."""
    from tpm import capi, params as P

    ctx = {}
    for name, prec in (("mixed", P.PREC_MIXED), ("fp64", P.PREC_FP64)):
        c = capi.Context(p64.replace(precision=prec), s.npart)
        c.load(s)
        c.initialize()
        ctx[name] = c
    idx = (p64.Nx / p64.Lx, p64.Ny / p64.Ly, p64.Nz / p64.Lz)
    out, done = {}, 0
    for n in checkpoints:
        for c in ctx.values():
            c.run(n - done)
            c.sync()
        done = n
        r = compare_paths(ctx["mixed"], ctx["fp64"], idx)
        r["max_abs_div_after_projection"] = ctx["mixed"].scalars()["max_abs_div"]
        out[f"after_{n}_step" + ("s" if n > 1 else "")] = r
    for c in ctx.values():
        c.close()
    return out


def fp64_peaks():
    """The FP64 roof: the library's FMA-chain probe (tpm_measure_fp64_peak)
    and, for comparison, cuBLAS DGEMM 4096^3 through torch (best of 5)."""
    import ctypes

    import torch
    from tpm import capi

    t = ctypes.c_double(0)
    probe = None
    if capi.load_library().tpm_measure_fp64_peak(ctypes.byref(t)) == 0 and t.value > 0:
        probe = t.value
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        a @ b
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ b
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return {"fma_probe_tflops": round(probe, 4) if probe else None,
            "dgemm_tflops": round(best, 4),
            "how": "FMA probe: 8 independent DFMA chains per thread, 8 blocks of 256 per SM, "
                   "best of 3 CUDA-event-timed launches; DGEMM: torch.matmul float64 4096^3"}


def fp64_roofline(r, ncell, peaks):
    """The FP64 path against the FP64 pipe (its bound), for its dominant kernel
    and for the whole step."""
    peak = peaks["fma_probe_tflops"] or peaks["dgemm_tflops"]
    name = r["roofline"]["kernel"]
    out = {"bound": "fp64", "peak_tflops": peak,
           "peak_source": "measured FMA probe" if peaks["fma_probe_tflops"] else "measured DGEMM"}
    if name in FP64_OPS:
        flops, inst = FP64_OPS[name]
        ms = r["kernels_ms_per_step"][name] / r["kernel_launches_per_step"][name]
        ach = flops * ncell / (ms * 1e-3) / 1e12
        inst_rate = inst * ncell / (ms * 1e-3) / 1e12
        out.update({"kernel": name, "flop_per_cell": flops, "fp64_inst_per_cell": inst,
                    "achieved_tflops": round(ach, 4), "frac": round(ach / peak, 4),
                    "achieved_tinst_s": round(inst_rate, 4),
                    "inst_frac": round(inst_rate / (peak / 2), 4)})
    step = FP64_FLOP_PER_CELL_STEP * ncell / (r["ms_per_step"] * 1e-3) / 1e12
    out["step"] = {"flop_per_cell_step": FP64_FLOP_PER_CELL_STEP,
                   "achieved_tflops": round(step, 4), "frac": round(step / peak, 4)}
    return out


def cufft_solve_ms(shape, lengths, dtype, reps=10):
    """A constant-coefficient Poisson solve through cuFFT (torch.fft: 3-D R2C,
    divide by the modified wave number, C2R), CUDA-event timed: the library
    comparison for the hand-written pencil FFTs (no residual, no update)."""
    import torch

    dev = torch.device("cuda")
    nz, ny, nx = shape
    x = torch.randn(shape, dtype=dtype, device=dev)
    ks = []
    for n, L in ((nz, lengths[2]), (ny, lengths[1])):
        k = torch.fft.fftfreq(n, d=1.0 / n, device=dev).to(dtype) * (2 * 3.141592653589793 / L)
        h = L / n
        ks.append((2.0 / h ** 2) * (1 - torch.cos(k * h)))
    kx = torch.arange(nx // 2 + 1, device=dev).to(dtype) * (2 * 3.141592653589793 / lengths[0])
    hx = lengths[0] / nx
    mwn = ks[0][:, None, None] + ks[1][None, :, None] + ((2.0 / hx ** 2) * (1 - torch.cos(kx * hx)))[None, None, :]
    mwn[0, 0, 0] = 1.0
    inv = 1.0 / mwn
    inv[0, 0, 0] = 0.0

    def solve():
        return torch.fft.irfftn(torch.fft.rfftn(x) * inv, s=shape)

    for _ in range(3):
        solve()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        solve()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


FFT_KERNELS = ("fft_x_fwd_resid", "fft_y", "fft_z_solve", "fft_x_inv_update", "finish_max")


def gpu_main(args):
    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as td

        td.init_process_group("nccl", device_id=torch.device("cuda", local))
        dist = td
    from tpm import params as P

    p64, s = make_workload(args.workload, 0, npart=args.particles, grid=args.grid)
    peak, peak_kind = peaks()
    paths = ["fp64", "mixed"] if args.precision == "both" else [args.precision]
    res, ctxs = {}, {}
    for name in paths:
        p = p64.replace(precision=P.PREC_MIXED if name == "mixed" else P.PREC_FP64)
        ctx, ms, n_it, launches, prof, clocks = time_gpu(p, s, args.steps, args.warmup, dist,
                                                         local, args.fft_tiles)
        ms = max_over_ranks(ms, dist, "cuda")
        res[name] = path_result(p, s, ms, args.steps, world, n_it, launches, prof, clocks,
                                name == "mixed", peak, workload=args.workload)
        res[name]["fft_pencils_per_block"] = ctx.fft_pens
        ctxs[name] = ctx
    head = "mixed" if "mixed" in res else "fp64"
    accuracy = None
    if "mixed" in ctxs and "fp64" in ctxs:
        # both timed paths ran the same steps from the same state
        a, b = ctxs["mixed"], ctxs["fp64"]
        idx = (p64.Nx / p64.Lx, p64.Ny / p64.Ly, p64.Nz / p64.Lz)
        after = compare_paths(a, b, idx)
        after["steps"] = a.scalars()["num_timestep"]
        after["max_abs_div_after_projection"] = a.scalars()["max_abs_div"]
        ctxs["fp64"].close()
        accuracy = mixed_accuracy_fresh(p64, s, (1, 10))
        accuracy["after_timed_run"] = after
    hctx = ctxs[head]
    e2e_ms, h2d, d2h, e2e_split = time_e2e(hctx, 2 * max(1, min(args.steps // 2, 3)))
    e2e_ms = max_over_ranks(e2e_ms, dist, "cuda")
    e2e_value = whole_job_rate(world, p64.ncell, 1, e2e_ms)
    r = res[head]
    box = (f"{p64.Nx}^3" if p64.Nx == p64.Ny == p64.Nz else f"{p64.Nx}x{p64.Ny}x{p64.Nz}")
    line = {
        "metric": METRIC, "value": round(r["value"], 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(r["ms_per_step"], 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if head == "fp64" else "mixed (f32 compute, f64 state and residuals)",
        "data": "synthetic (seeded solenoidal E(k)~k^4 exp(-2(k/4)^2) velocity, uniform particles)",
        "config": {"workload": f"{args.workload}: {box} cells, {s.npart} particles, heated, "
                               f"two-way coupled, Poisson eps=1e-13 (mean {r['n_it']:.2f} "
                               f"iterations)",
                   "precision": head, "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (working set ~8 GB per path)"},
        "roofline": dict(r["roofline"], peak_source=f"{peak_kind} HBM copy bandwidth"),
        "step_roofline": r["step_roofline"],
        "e2e": dict({"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                     "d2h_bytes_per_step": int(d2h)}, **e2e_split),
        "gpu_launches": int(r["launches"]),
        "clocks": r["clocks"],
        "kernels_ms_per_step": r["kernels_ms_per_step"],
        "mparticle_steps_per_s": round(r["mparticle_steps_per_s"], 3),
        "fft_pencils_per_block": r["fft_pencils_per_block"],
    }
    if "fp64" in res and head != "fp64":
        f = res["fp64"]
        line["fp64"] = {"value": round(f["value"], 3), "ms_per_step": round(f["ms_per_step"], 3),
                        "fft_pencils_per_block": f["fft_pencils_per_block"],
                        "n_it": f["n_it"], "roofline": f["roofline"],
                        "fp64_roofline": fp64_roofline(f, p64.ncell, fp64_peaks()),
                        "step_roofline": f["step_roofline"], "clocks": f["clocks"],
                        "kernels_ms_per_step": f["kernels_ms_per_step"]}
        line["mixed_vs_fp64_speedup"] = round(r["value"] / f["value"], 3)
    if head == "fp64":
        line["fp64_roofline"] = fp64_roofline(r, p64.ncell, fp64_peaks())
    if accuracy:
        line["mixed_accuracy"] = accuracy
    # the pencil-FFT pressure iteration against cuFFT doing only the spectral solve
    import torch

    cmp = {}
    for name, r_ in res.items():
        per_it = sum(r_["kernels_ms_per_step"].get(k, 0.0) for k in FFT_KERNELS) / (4 * r_["n_it"])
        dtype = torch.float32 if name == "mixed" else torch.float64
        cmp[name] = {"own_iteration_ms": round(per_it, 4),
                     "cufft_solve_ms": round(cufft_solve_ms((p64.Nz, p64.Ny, p64.Nx),
                                                            (p64.Lx, p64.Ly, p64.Lz), dtype), 4),
                     "note": "own = residual + R2C/C2R pencil FFTs + divide + P update "
                             "(5 kernels); cuFFT = rfftn, divide, irfftn only"}
    line["fft_vs_cufft"] = cmp
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_port(args.workload)
    hctx.close()
    if world == 1 and args.workload == WORKLOAD and args.grid is None and args.particles is None \
            and not args.no_extras:
        # the batched-ensemble and adjoint workloads at their default sizes,
        # summarised in the same line (each also runs alone with --workload)
        line["ensemble48"] = summary(ensemble_main(argparse.Namespace(steps=10, warmup=3)))
        line["adjoint64"] = summary(adjoint_main(argparse.Namespace(steps=10, warmup=3)))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def summary(line):
    keep = ("metric", "value", "unit", "steps", "warmup", "ms_per_step", "dtype", "config",
            "vs_sequential", "sequential_value", "adjoint_over_forward", "forward_ms_per_step",
            "e2e", "gpu_launches", "clocks")
    return {k: line[k] for k in keep if k in line}


# ------------------------------------------------------ batched ensemble
ENSEMBLE = "ensemble48"


def ensemble_main(args):
    """48 independent boxes (32^3..96^3, 1e4..5e5 particles, mixed precision)
    stepped as one CUDA graph per step with concurrent per-box streams and
    autotuned FFT tiles, against the same boxes stepped one after another."""
    import torch
    from tpm import capi, inputs, params as P

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    boxes = P.ensemble_boxes(48, P.PREC_MIXED)
    params, states = [], []
    for p, npart, seed in boxes:
        st = inputs.make_state(p, npart, seed=seed)
        params.append(p.replace(dt=inputs.cfl_dt(p, st.RU)))
        states.append(st)
    ncell = sum(p.ncell for p in params)
    npart = sum(st.npart for st in states)

    def fresh():
        b = capi.Batch(params, [st.npart for st in states])
        for box, st in zip(b.boxes, states):
            box.load(st)
        b.autotune()
        for box in b.boxes:
            box.initialize()
        return b

    out = {}
    for mode, graph in (("graph", True), ("sequential", False)):
        b = fresh()
        b.run(args.warmup, graph=graph)
        b.sync()
        l0 = sum(box.launch_count() for box in b.boxes)
        it0 = [box.scalars()["total_poisson_iterations"] for box in b.boxes]
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            t0 = time.perf_counter()
            b.run(args.steps, graph=graph)
            b.sync()
            secs = time.perf_counter() - t0
        launches = sum(box.launch_count() for box in b.boxes) - l0
        if graph:  # loop bodies repeated on the device (6 kernels per extra iteration)
            launches += sum(6 * max(0, box.scalars()["total_poisson_iterations"] - i0 - 4 * args.steps)
                            for box, i0 in zip(b.boxes, it0))
        out[mode] = {"secs": secs, "launches": launches, "clocks": clk.summary()}
        if mode == "graph":  # end to end: each step's statistics read back to the host
            t0 = time.perf_counter()
            for _ in range(args.steps):
                b.run(1, graph=True)
                stats = [box.statistics() for box in b.boxes]
            e2e_secs = time.perf_counter() - t0
            d2h = len(stats) * ctypes_sizeof_stats()
        b.close()
    g, q = out["graph"], out["sequential"]
    value = world * ncell * args.steps / g["secs"] / 1e6
    line = {
        "metric": "aggregate Mcell-steps/s, 48-box ensemble (32^3..96^3), 1 GB300",
        "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(g["secs"] * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "mixed (f32 compute, f64 state and residuals)",
        "data": "synthetic (seeds 0-47, solenoidal E(k)~k^4 exp(-2(k/4)^2), uniform particles)",
        "config": {"workload": f"{ENSEMBLE}: 48 boxes, {ncell} cells, {npart} particles, "
                               f"nu for kmax*eta=1.5", "parallelism": f"replicas x{world}",
                   "l2": "working set ~4 GB, larger than L2"},
        "vs_sequential": round(q["secs"] / g["secs"], 3),
        "sequential_value": round(world * ncell * args.steps / q["secs"] / 1e6, 3),
        "mparticle_steps_per_s": round(world * npart * args.steps / g["secs"] / 1e6, 3),
        "e2e": {"value": round(world * ncell * args.steps / e2e_secs / 1e6, 3), "unit": UNIT,
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(g["launches"]),
        "clocks": g["clocks"],
    }
    return line


ADJOINT = "adjoint64"


def adjoint_main(args):
    """Gradient of J = TKE + var(C) after a 200-step horizon (64^3 cells, 2e5
    two-way-coupled particles, checkpoints every 20 steps) by the discrete
    adjoint, timed against the same forward steps alone."""
    import numpy as np
    import torch
    from tpm import capi, params as P

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    horizon = args.steps if args.steps != 10 else 200
    p, s = make_workload("box64_p2e5", P.PREC_FP64)

    def fresh():
        c = capi.Context(p, s.npart)
        c.load(s)
        c.initialize()
        return c

    c = fresh()
    c.run(args.warmup)
    c.sync()
    c = fresh()
    t0 = time.perf_counter()
    c.run(horizon)
    c.sync()
    fwd = time.perf_counter() - t0
    c = fresh()
    torch.cuda.synchronize()
    l0 = c.launch_count()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        J, g, gA, gt = c.adjoint(horizon, checkpoint_every=20, w_tke=1.0, w_cvar=1.0)
        adj = time.perf_counter() - t0
    launches = c.launch_count() - l0
    value = world * p.ncell * horizon / adj / 1e6
    line = {
        "metric": "adjoint Mcell-steps/s (forward + checkpointed recomputation + backward), "
                  "64^3 + 2e5 particles, 200-step horizon",
        "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": horizon,
        "warmup": args.warmup, "ms_per_step": round(adj * 1e3 / horizon, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seed 3, solenoidal E(k)~k^4 exp(-2(k/4)^2), uniform particles)",
        "config": {"workload": f"{ADJOINT}: {p.Nx}^3, {s.npart} particles, nu={p.Mu0:g}, "
                               f"tau_p=0.1, mass loading 0.3, checkpoints every 20 steps",
                   "parallelism": f"replicas x{world}"},
        "adjoint_over_forward": round(adj / fwd, 3),
        "forward_ms_per_step": round(fwd * 1e3 / horizon, 3),
        "J": J, "grad_norms": {"dJ_dRU0_l2": float(np.sqrt(np.sum(g * g))), "dJ_dA": gA,
                               "dJ_dtau": gt},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(g.nbytes / horizon)},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    return line


LONGRUN = "longrun256"


def longrun_main(args):
    """Config 2's long check: the mixed and FP64 paths run the 256^3 + 8M
    workload for 1000 steps (--steps) from the same state and are compared on
    TKE, dissipation, rms velocity, concentration variance, the energy spectrum
    and the particle RDF (the flow is chaotic, so fields are not compared)."""
    import numpy as np
    import torch
    from tpm import capi, params as P

    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    nsteps = args.steps if args.steps != 10 else 1000
    p64, s = make_workload(WORKLOAD, P.PREC_FP64)
    out, times = {}, {}
    for name, prec in (("mixed", P.PREC_MIXED), ("fp64", P.PREC_FP64)):
        c = capi.Context(p64.replace(precision=prec), s.npart)
        c.load(s)
        c.initialize()
        c.set_graph(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c.run(nsteps)
        c.sync()
        times[name] = time.perf_counter() - t0
        st = c.statistics()
        E, _ = c.spectrum()
        pairs, g = c.rdf(0.3, 30)
        out[name] = {"stats": st, "E": E, "pairs": pairs.astype(float)}
        c.close()
    a, b = out["mixed"], out["fp64"]
    rel = {k: abs(a["stats"][k] - b["stats"][k]) / abs(b["stats"][k])
           for k in ("TKE", "dissipation", "u_rms", "C_var", "Tg_mean", "Tp_mean", "P0")}
    sig = b["E"] > 1e-3 * b["E"].max()
    rel["spectrum_max_shell"] = float(np.max(np.abs(a["E"][sig] - b["E"][sig]) / b["E"][sig]))
    ca, cb = np.cumsum(a["pairs"]), np.cumsum(b["pairs"])
    rel["rdf_cumulative_pairs"] = float(np.max(np.abs(ca[5:] - cb[5:]) / cb[5:]))
    line = {
        "metric": "mixed vs FP64 statistics after a long run, 256^3 + 8M particles",
        "value": max(rel.values()), "unit": "max relative difference", "n_gpus": 1,
        "steps": nsteps, "warmup": 0, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "mixed vs f64", "data": "synthetic (seed 2)",
        "config": {"workload": f"{WORKLOAD}, {nsteps} steps each path, graph-replayed"},
        "relative_differences": rel,
        "statistics": {k: {q: a["stats"][q] if k == "mixed" else b["stats"][q]
                           for q in ("TKE", "dissipation", "u_rms", "C_var", "T_cur")}
                       for k in ("mixed", "fp64")},
        "seconds": times,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def ctypes_sizeof_stats():
    import ctypes

    from tpm.params import TpmStats

    return ctypes.sizeof(TpmStats)


# ---------------------------------------------------------- reference arm
def reference_main(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    if args.workload in (ENSEMBLE, ADJOINT, LONGRUN):
        print(json.dumps({"impl": "reference", "unavailable":
                          "the reference runs one box per MPI job and has no adjoint"}), flush=True)
        return
    # bounded sample: the 128^3 box at the workload's particle density and
    # physics; at most 1 warm-up and 2 timed steps whatever --steps/--warmup ask
    # (one step of the sample takes several seconds on one core)
    steps_run, warm_run = max(1, min(args.steps, 2)), min(args.warmup, 1)
    cb = cpu_rate(args.workload, warm_run, steps_run)
    value = cb["value"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(cb["seconds_per_step"] * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload} (sampled: {cb['sample']})",
                   "precision": "fp64", "parallelism": "1 host core",
                   "timed_steps": steps_run, "warmup_steps": warm_run},
        "n_it": cb["n_it"],
        "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample", "n_it",
                                             "host")},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="both", choices=["both", "fp64", "mixed"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the ensemble and adjoint summaries of the default run")
    ap.add_argument("--fft-tiles", type=lambda v: [int(t) for t in v.split(",")], default=None,
                    help="pencils x,y,z and threads x,y,z of the FFT passes instead of "
                         "autotuning them (one precision at a time)")
    ap.add_argument("--grid", type=lambda v: tuple(int(t) for t in v.split(",")), default=None,
                    help="nx,ny,nz: the workload's physics on this box of the same cell size "
                         "(small cases for profilers)")
    ap.add_argument("--particles", type=int, default=None,
                    help="particle count instead of the workload's")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.impl == "reference":
        reference_main(args)
    elif args.workload in (ENSEMBLE, ADJOINT):
        line = (ensemble_main if args.workload == ENSEMBLE else adjoint_main)(args)
        if int(os.environ.get("RANK", "0")) == 0:
            print(json.dumps(line), flush=True)
    elif args.workload == LONGRUN:
        longrun_main(args)
    else:
        gpu_main(args)


if __name__ == "__main__":
    main()
