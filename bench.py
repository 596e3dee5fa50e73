"""Benchmark of the hot path: one JSON line per run (rank 0).

Default workload (the configuration the headline metric is quoted on): 3D
compressible Euler, CWENO4 reconstruction + Rusanov flux + SSPRK(4,3), FP64,
256^3 cells, periodic, Gaussian acoustic pulse, CFL 0.4.  One "step" is one
SSPRK(4,3) time step (4 RHS stages) of the whole grid; the metric is
cell-updates/s (cells x steps / s).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl reference]

Other workloads (--workload): euler256_fp32 (FP32 reconstruction/flux, FP64
state), euler256_df64 (double-float reconstruction on the FP32 pipe, FP64 state and
flux, held to the FP64 error bars), euler256_linear (optimal-weight linear reconstruction), euler256_weno3,
euler256_hllc, ns256_tgv (viscous Taylor-Green), acoustic256 (3D acoustic FV),
sw2d4096 (2D standing wave, RK104), mp3d256 (3D primitive multiphase), pc2d2048 (2d/HyPE-2D path-conservative
Kapila, order 3), kapila1024[_fp32|_learned], blast256/512,
ctcs512 (2D CTCS 512^2), batch256 (256 batched monopole CTCS instances).
--grid N sets the cells per axis of the 3D Euler / Navier-Stokes and 2D acoustic
workloads (small cases for profiling).

N > 1 (torchrun): replicas only -- each rank runs the same workload on its own
GPU, no data exchange; value = all ranks' cell-updates / max time.
``--impl reference`` times the CPU implementation of the path on the host
cores (the reference compiled in place when present, else its C restatement)
on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

# algorithmic HBM bytes per unit (FP64 state): Euler SSPRK(4,3), 5 variables:
# per stage read 40 + write 40 B, plus one extra read of u^n in the stage-3
# combination -> 4*80 + 40 = 360 B per cell-update, 90 B per cell-stage.
EULER_BYTES_PER_CELL_STAGE = 90.0
EULER_BYTES_PER_CELL_UPDATE = 360.0
# Navier-Stokes: the R4 coefficients (5 x 20 doubles) written by the reconstruction and
# read back by the face kernels, 1600 B more per cell-stage
NS_COEF_BYTES_PER_CELL_STAGE = 1600.0
# CTCS: read p^n, p^{n-1}, write p^{n+1}: 24 B per cell-update
CTCS_BYTES_PER_CELL_UPDATE = 24.0


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _profile_figure(name: str, key: str):
    """a number from a committed ncu summary under profiles/ (line 'key = value')"""
    path = os.path.join(ROOT, "profiles", name)
    try:
        with open(path) as f:
            for line in f:
                if line.strip().startswith(key) and "=" in line:
                    return float(line.split("=", 1)[1].split()[0])
    except Exception:
        pass
    return None


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return ws, rank, local


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def _max_over_ranks(ws, x: float) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _gpu_index(local: int) -> int:
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        try:
            return int(vis.split(",")[local])
        except Exception:
            return local
    return local


# ------------------------------------------------------------------ CPU side
def cpu_euler_rate(n: int, steps: int, use_ref: bool = True):
    """cell-updates/s of the CPU implementation on an n^3 sample of the pulse workload."""
    from acoustic_petsc_gb300 import workloads
    from oracle import pyoracle as O

    O.build(O.ref_dir())
    U = workloads.euler_pulse(n)
    cfg = O.euler_cfg(n, 1.0 / n, cfl=0.4, nthreads=os.cpu_count() or 1)
    kind = "port"
    if use_ref and O.ref_available():
        kind = "reference"
        t0 = time.perf_counter()
        _, _, _, rc = O.ref_euler_run(cfg, U, steps)
        dt = time.perf_counter() - t0
        cores = 1
    else:
        O.euler_run(cfg, U, 1)  # warm
        t0 = time.perf_counter()
        _, _, _, rc = O.euler_run(cfg, U, steps)
        dt = time.perf_counter() - t0
        cores = O.threads()
    assert rc == 0
    return n**3 * steps / dt, cores, kind, dt


def cpu_ctcs_rate(n: int, steps: int):
    from acoustic_petsc_gb300 import workloads
    from oracle import pyoracle as O

    O.build(None)
    p0, p1, h, dt, alpha = workloads.ctcs_gaussian(n)
    t0 = time.perf_counter()
    O.ctcs2d_plane(p0, p1, alpha, 3, steps)
    d = time.perf_counter() - t0
    return n * n * steps / d, O.threads(), "port", d


# ------------------------------------------------------------------ GPU workloads
RECON_TAG = {0: "cweno4", 1: "cweno4_linear", 3: "weno3"}
RECON_NAME = {0: "CWENO4 (gamma 0.85)", 1: "linear R4", 3: "WENO3 (3d/weno3/Euler, central weight 100)"}
FLUX_TAG = {0: "rusanov", 1: "hllc", 2: "rothllc"}
FLUX_NAME = {0: "Rusanov", 1: "HLLC", 2: "rotated HLLC"}


EULER_DTYPE = {0: "f64", 1: "f64 state / f32 recon+flux",
               2: "f64 state and stage accumulation / df64 recon+Rusanov flux (FP32 pairs, 48-bit significand, "
                  "on deviations from a reference state)"}


def run_euler(args, ws, rank, local, precision=0, recon=0, n=256, flux=0, viscous=False):
    import torch

    import acoustic_petsc_gb300 as H
    from acoustic_petsc_gb300 import workloads

    L = H.lib()
    H._lib.check(L.hype_set_device(local), "hype_set_device")
    torch.cuda.set_device(local)
    n = args.grid or n
    if viscous:  # the Taylor-Green run of 3d/weno4/Navier-Stokes-3D (hype.c:33-55) at n^3
        U0 = workloads.taylor_green(n)
        ctx = H.AppCtx(N_x=n, N_y=n, N_z=n, h=2.0 * math.pi / n, x_min=-math.pi, y_min=-math.pi, z_min=-math.pi,
                       CFL=0.6, precision=precision, recon=recon, flux=flux, mu=0.01, prandtl=1.0, cv=2.5)
    else:
        U0 = workloads.euler_pulse(n)
        ctx = H.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, precision=precision, recon=recon, flux=flux)
    s = H.EulerSolver(ctx)
    s.set_state(U0)
    s.step(max(args.warmup, 3))
    stream = torch.cuda.ExternalStream(L.hype_euler_stream(s._h))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    H._lib.check(L.hype_euler_profile(s._h, 1), "profile")
    l0 = H.launches()
    _barrier(ws)
    torch.cuda.synchronize()
    with Clocks(_gpu_index(local)) as clk:
        e0.record(stream)
        s.step(args.steps)
        e1.record(stream)
        e1.synchronize()
    torch.cuda.synchronize()
    _barrier(ws)
    launches = H.launches() - l0
    ms = e0.elapsed_time(e1)
    ms_max = _max_over_ranks(ws, ms)
    # the state after the timed steps, for the double-float form beside this one (default workload)
    with_alt = precision == 0 and recon == 0 and flux == 0 and not viscous and not args.no_alt_forms
    U_fp64 = s.get_state() if with_alt else None
    prof_ms = (C.c_double * 3)()
    prof_n = (C.c_longlong * 3)()
    H._lib.check(L.hype_euler_profile_read(s._h, prof_ms, prof_n), "profile_read")
    H._lib.check(L.hype_euler_profile(s._h, 0), "profile")
    cells = n**3
    value = ws * cells * args.steps / (ms_max * 1e-3)
    # ---- the stage (recon + faces + update) as the dominant unit of work
    stages = max(prof_n[0], 1)
    t_stage = (prof_ms[0] + prof_ms[1] + prof_ms[2]) / stages * 1e-3
    # the viscous path also writes and reads the 100 R4 coefficients of each cell
    bytes_stage = EULER_BYTES_PER_CELL_STAGE + (NS_COEF_BYTES_PER_CELL_STAGE if viscous else 0.0)
    achieved_gbs = bytes_stage * cells / t_stage / 1e9
    peak, peak_kind = _peaks()
    tag = {0: "fp64", 1: "fp32", 2: "df64"}[precision] + ("_linear" if recon else "") + ("_ns" if viscous else "")
    prof_file = ("ns3d_tgv_stage_fp64.txt" if precision == 0 else f"ns3d_tgv_stage_{tag}.txt") if viscous else \
        f"euler_stage_{tag}.txt"
    traffic = _profile_figure(prof_file, "dram_bytes_per_cell_stage")
    flops_cell = _profile_figure(prof_file, "fp_flops_per_cell_stage")
    fpeak = C.c_double()
    # the double-float form runs its reconstruction on the FP32 pipe
    H._lib.check(H._lib.probes().hype_probe_fma_peak(1 if precision == 2 else precision, C.byref(fpeak)), "probe")
    # the FP32 Rusanov form runs the fused stage kernel (ghost fill + one pass per stage)
    fused = precision == 1 and flux == 0 and not viscous
    per_kernel = ({"ghost": prof_ms[0] / stages, "stage_fused": prof_ms[1] / stages,
                   "first_stage_combine": prof_ms[2] / stages} if fused else
                  {"recon": prof_ms[0] / stages, "faces": prof_ms[1] / stages, "update": prof_ms[2] / stages})
    roof = {"kernel": ("RK stage = k_ghost + k_stage_f32 (per-stage average)" if fused else
                       "RK stage = k_ghost + k_recon + k_faces x3 + k_update (per-stage average)"), "bound": "hbm",
            "achieved": achieved_gbs, "peak": peak, "unit": "GB/s", "frac": achieved_gbs / peak,
            "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
            "traffic": traffic * cells if traffic else None, "algorithmic_bytes": bytes_stage * cells,
            "per_kernel_ms": per_kernel}
    alu = None
    instr32 = _profile_figure(prof_file, "issued_thread_instructions_per_cell_stage") if precision == 1 else None
    if instr32:
        # the fused FP32 stage: every issued thread instruction against the FP32 pipe's issue ceiling
        # (the FMA probe's rate / 2: an FMA is two flops, one instruction)
        ach_i = instr32 * cells / t_stage
        alu = {"bound": "fp32 issue", "issued_thread_instructions_per_cell_stage": instr32,
               "achieved_instr_per_s": ach_i, "peak_instr_per_s": fpeak.value * 1e12 / 2,
               "frac": ach_i / (fpeak.value * 1e12 / 2),
               "peak_kind": "measured FMA issue ceiling (hype_probe_fma_peak)"}
        alg = _profile_figure("flops_euler_cweno4_rusanov.txt", "algorithmic_flops_per_cell_stage") \
            if recon == 0 and flux == 0 and not viscous else None
        if alg:
            alu["algorithmic_flops_per_cell_stage"] = alg
            alu["algorithmic_achieved_tflops"] = alg * cells / t_stage / 1e12
            alu["algorithmic_frac"] = alu["algorithmic_achieved_tflops"] / fpeak.value
    elif flops_cell:
        ach = flops_cell * cells / t_stage / 1e12
        alu = {"bound": "fp64" if precision == 0 else "fp32", "achieved": ach, "peak": fpeak.value, "unit": "TFLOP/s",
               "frac": ach / fpeak.value, "flops_per_cell_stage": flops_cell,
               "peak_kind": "measured FMA issue ceiling (hype_probe_fma_peak)"}
        # the reference algorithm's own operation count (oracle/flopcount.py on its expression trees):
        # the work the GPU form does with fewer operations, as a rate against the same peak
        alg = (_profile_figure("flops_euler_cweno4_rusanov.txt", "algorithmic_flops_per_cell_stage")
               if recon == 0 and flux == 0 and not viscous else None)
        if alg:
            alu["algorithmic_flops_per_cell_stage"] = alg
            alu["algorithmic_achieved"] = alg * cells / t_stage / 1e12
            alu["algorithmic_frac"] = alu["algorithmic_achieved"] / fpeak.value
            alu["algorithmic_source"] = "profiles/flops_euler_cweno4_rusanov.txt (reference expression trees)"
        instr_cell = _profile_figure(prof_file, "fp64_instructions_per_cell_stage") if precision == 0 else None
        if instr_cell:
            # an FMA counts two flops, an add or multiply one: against the issue ceiling
            # (peak / 2 instructions per second) the FP64 pipe's occupancy shows directly
            alu["fp64_instructions_per_cell_stage"] = instr_cell
            alu["instruction_issue_frac"] = instr_cell * cells / t_stage / (fpeak.value * 1e12 / 2)
    # ---- end to end through the public API with host buffers (pinned)
    e2e = None
    if rank == 0 or ws > 1:
        host = torch.empty((n, n, n, 5), dtype=torch.float64, pin_memory=True)
        host.numpy()[...] = U0
        hv = host.numpy()
        ke = max(1, min(3, args.steps))
        for _ in range(2):  # warm-up of both copy directions through the same buffer
            s.set_state(hv)
            s.step(1)
            H._lib.check(L.hype_euler_download(s._h, hv.ctypes.data_as(H._lib.D)), "download")
        hv[...] = U0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(ke):
            s.set_state(hv)  # H2D of the step's input from pinned host memory
            s.step(1)
            H._lib.check(L.hype_euler_download(s._h, hv.ctypes.data_as(H._lib.D)), "download")  # D2H, pinned
        e1.record(stream)
        e1.synchronize()
        wall = time.perf_counter() - t0
        ms_e2e = _max_over_ranks(ws, max(e0.elapsed_time(e1), wall * 1e3))
        nb = cells * 5 * 8
        e2e = {"value": ws * cells * ke / (ms_e2e * 1e-3), "unit": "cell-updates/s", "h2d_bytes_per_step": nb,
               "d2h_bytes_per_step": nb, "steps": ke,
               "path": "EulerSolver.set_state -> step(1) -> get_state (hype_euler_upload/step/download)"}
    # the double-float form (same initial state and steps), timed after the FP64 form's legs
    alt = None
    if with_alt:
        so = lambda h: torch.cuda.ExternalStream(L.hype_euler_stream(h))  # noqa: E731
        alt = _euler_df64_beside(args, ws, n, U0, U_fp64, stream_of=so)
        alt.update(_euler_df64_beside(args, ws, n, U0, U_fp64, stream_of=so, precision=1))
    del U_fp64
    clocks = clk.summary()
    s.close()
    out = {
        "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": EULER_DTYPE[precision],
        "data": ("synthetic: Taylor-Green vortex of initial_condition.c at the cell centres" if viscous else
                 "synthetic: Gaussian acoustic pulse dp = 1e-3 exp(-r^2/(2*0.04^2)), 5^3-Gauss cell averages"),
        "config": {"workload": (f"ns3d_tgv_{RECON_TAG[recon]}_{FLUX_TAG[flux]}_ssprk43_{n}" if viscous else
                                f"euler3d_{RECON_TAG[recon]}_{FLUX_TAG[flux]}_ssprk43_{n}"),
                   "cells": cells, "grid": [n, n, n], "domain": "[-pi,pi]^3 periodic" if viscous else "[0,1]^3 periodic",
                   "cfl": 0.6 if viscous else 0.4, "gamma": 1.4,
                   "viscosity": {"mu": 0.01, "prandtl": 1.0, "cv": 2.5} if viscous else None,
                   "reconstruction": RECON_NAME[recon], "flux": FLUX_NAME[flux],
                   "time": "SSPRK(4,3) (PETSc TSSSP RKS3, 4 stages), dt from the last stage (monitor semantics)",
                   "parallelism": "replicas" if ws > 1 else "single GPU",
                   "l2": f"inputs larger than L2 (state 5*8*{n}^3 B = {5 * 8 * n**3 / 1e6:.0f} MB vs 129 MB); no flush"},
        "roofline": roof, "gpu_launches": launches, "clocks": clocks, "e2e": e2e,
    }
    if alu:
        out["roofline_alu"] = alu
    if alt:
        out["alt_forms"] = alt
    return out


def _euler_df64_beside(args, ws, n, U0, U_fp64, stream_of, precision=2):
    """another precision form of the same workload (default: HYPE_PREC_DF64, state, face fluxes and
    stage accumulation in FP64, reconstruction and Rusanov flux in FP32 pairs on deviations; 1: the
    fused FP32 stage), the same warm-up and timed steps from the same state, and its largest state
    difference from the FP64 run"""
    import torch

    import acoustic_petsc_gb300 as H

    L = H.lib()
    ctx = H.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, precision=precision)
    d = H.EulerSolver(ctx)
    d.set_state(U0)
    d.step(max(args.warmup, 3))
    stream = stream_of(d._h)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    H._lib.check(L.hype_euler_profile(d._h, 1), "profile")
    _barrier(ws)
    torch.cuda.synchronize()
    e0.record(stream)
    d.step(args.steps)
    e1.record(stream)
    e1.synchronize()
    ms = _max_over_ranks(ws, e0.elapsed_time(e1))
    prof_ms = (C.c_double * 3)()
    prof_n = (C.c_longlong * 3)()
    H._lib.check(L.hype_euler_profile_read(d._h, prof_ms, prof_n), "profile_read")
    H._lib.check(L.hype_euler_profile(d._h, 0), "profile")
    stages = max(prof_n[0], 1)
    diff = float(np.abs(d.get_state() - U_fp64).max() / np.abs(U_fp64).max())
    d.close()
    tag = "df64" if precision == 2 else "fp32"
    per = ({"recon": prof_ms[0] / stages, "faces": prof_ms[1] / stages, "update": prof_ms[2] / stages}
           if precision == 2 else {"ghost": prof_ms[0] / stages, "stage_fused": prof_ms[1] / stages})
    return {tag: {"value": ws * n**3 * args.steps / (ms * 1e-3), "unit": "cell-updates/s",
                  "ms_per_step": ms / args.steps,
                  "dtype": EULER_DTYPE[precision],
                  "per_kernel_ms": per,
                  "state_rel_linf_diff_vs_fp64": diff,
                  "steps_compared": max(args.warmup, 3) + args.steps,
                  "profile": f"profiles/euler_stage_{tag}.txt"}}


def run_ctcs(args, ws, rank, local, n=512):
    import torch

    import acoustic_petsc_gb300 as H
    from acoustic_petsc_gb300 import workloads

    L = H.lib()
    H._lib.check(L.hype_set_device(local), "hype_set_device")
    torch.cuda.set_device(local)
    p0, p1, h, dt, alpha = workloads.ctcs_gaussian(n)
    lf = H.Leapfrog(p0.shape, dx=h, dt=dt, c0=1.0, form=0, bc=H._lib.BC_ZERO)
    lf.set(p0, p1)
    steps_per = 1000  # one "step" of this workload = the 1000-step run
    lf.UpdatePressure(steps_per * max(args.warmup, 3) // 10)
    lf.sync()
    l0 = H.launches()
    _barrier(ws)
    torch.cuda.synchronize()
    with Clocks(_gpu_index(local)) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            lf.UpdatePressure(steps_per)
        lf.sync()
        sec = time.perf_counter() - t0
    launches = H.launches() - l0
    sec = _max_over_ranks(ws, sec)
    value = ws * n * n * steps_per * args.steps / sec
    peak, kind = _peaks()
    achieved = CTCS_BYTES_PER_CELL_UPDATE * n * n * steps_per * args.steps / sec / 1e9
    return {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": sec * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic Gaussian pulse",
            "config": {"workload": "ctcs2d_512_1000steps", "grid": [n, n], "bc": "zero-Dirichlet", "cfl": 0.5,
                       "l2": "L2-resident working set (2 MB per level): HBM roofline does not bind"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None},
            "gpu_launches": launches, "clocks": clk.summary()}


def run_batch(args, ws, rank, local, ninst=256, steps_per=2000):
    """Batched 2D acoustics: 256 seeded instances (sides log-uniform 64..1024), one bench step =
    the workload's 2000 CTCS steps of every instance; per-instance wall time = from the start of
    the 2000-step call to the instance's completion (device events of its size class)."""
    import torch

    import acoustic_petsc_gb300 as H
    from acoustic_petsc_gb300 import workloads

    L = H.lib()
    H._lib.check(L.hype_set_device(local), "hype_set_device")
    torch.cuda.set_device(local)
    inst = workloads.monopole_batch(ninst)
    b = H.BatchLeapfrog([H.Monopole(**m) for m in inst], tile=(0, 0))
    tile = b.tile()
    ncls, cls = b.classes()
    nodes = sum(m["nx"] * m["ny"] for m in inst)
    for _ in range(max(args.warmup, 3)):
        b.step(steps_per)
    b.sync()
    l0 = H.launches()
    _barrier(ws)
    times = []
    with Clocks(_gpu_index(local)) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            b.step(steps_per)
            times.append(b.instance_times())  # waits for the call
        b.sync()
        sec = time.perf_counter() - t0
    launches = H.launches() - l0
    sec = _max_over_ranks(ws, sec)
    value = ws * nodes * steps_per * args.steps / sec
    T = np.median(np.array(times), axis=0)  # per instance, median over the timed calls
    # the same calls with every instance in one class (all advance together): the aggregate
    # rate the size classes must not lose, and the per-instance time they replace
    b.set_classes(1)
    b.step(steps_per)
    b.sync()
    t1 = time.perf_counter()
    b.step(steps_per)
    b.sync()
    sec1 = time.perf_counter() - t1
    T1 = b.instance_times()
    b.close()
    peak, kind = _peaks()
    achieved = CTCS_BYTES_PER_CELL_UPDATE * nodes * steps_per * args.steps / sec / 1e9
    fpeak = C.c_double()
    H._lib.check(H._lib.probes().hype_probe_fma_peak(0, C.byref(fpeak)), "probe")
    rate = nodes * steps_per * args.steps / sec
    return {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": sec * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic seeded monopole instances",
            "config": {"workload": "batch_ctcs_256_instances_2000_steps", "instances": ninst, "nodes": nodes,
                       "steps_per_bench_step": steps_per, "sizes": "log-uniform 64^2..1024^2 (seed 7)",
                       "tile": list(tile), "size_classes": ncls,
                       "l2": "levels 3 x 8 B x nodes > L2: streamed from HBM"},
            "per_instance_wall_s": {
                "p50": float(np.percentile(T, 50)), "p99": float(np.percentile(T, 99)), "max": float(T.max()),
                "by_class": [float(T[cls == c][0]) for c in range(ncls)],
                "note": "seconds from the start of a 2000-step call to each instance's completion (device events "
                        "of its size class), median over the timed calls",
                "single_class": {"p50": float(np.percentile(T1, 50)), "p99": float(np.percentile(T1, 99)),
                                 "value": nodes * steps_per / sec1}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None},
            "roofline_alu": {"bound": "fp64 issue", "fp64_instructions_per_node_update": 6,
                             "achieved_instr_per_s": 6 * rate, "peak_instr_per_s": fpeak.value * 1e12 / 2,
                             "frac": 6 * rate / (fpeak.value * 1e12 / 2),
                             "peak_kind": "measured FMA issue ceiling (hype_probe_fma_peak), an FMA = 2 flops"},
            "gpu_launches": launches, "clocks": clk.summary()}


def run_mp2d(args, ws, rank, local, n=1024, precision=0, model=1):
    import torch

    import acoustic_petsc_gb300 as H
    from acoustic_petsc_gb300 import workloads

    L = H.lib()
    H._lib.check(L.hype_set_device(local), "hype_set_device")
    torch.cuda.set_device(local)
    U0, h = workloads.kapila_bubble(n, model=model)
    m = H.Multiphase2D(n, n, h, CFL=0.4, boundaries=(2, 2, 2, 2), model=model, eos=workloads.KAPILA_EOS,
                       stepper=H._lib.STEP_SSPRK43, precision=precision)
    m.set_state(U0)
    m.step(max(args.warmup, 3))
    stream = torch.cuda.ExternalStream(L.hype_mp2d_stream(m._h))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = H.launches()
    _barrier(ws)
    torch.cuda.synchronize()
    with Clocks(_gpu_index(local)) as clk:
        e0.record(stream)
        m.step(args.steps)
        e1.record(stream)
        e1.synchronize()
    launches = H.launches() - l0
    ms = _max_over_ranks(ws, e0.elapsed_time(e1))
    nv = 6 if model == 1 else 5
    bytes_cu = 4 * (2 * 8 * nv) + 8 * nv  # SSPRK(4,3): 4 stages read+write the state, one extra read of u^n
    cells = n * n
    value = ws * cells * args.steps / (ms * 1e-3)
    peak, kind = _peaks()
    ach = bytes_cu * cells * args.steps / (ms * 1e-3) / 1e9
    fb = m.fallback_cells
    m.close()
    return {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if precision == 0 else "f64 state / f32 recon+flux",
            "data": "synthetic: shock-driven air bubble in water (1e8 Pa step at x<0.2)",
            "config": {"workload": f"kapila5_2d_{n}" if model == 1 else f"diffuse_interface_2d_{n}", "grid": [n, n],
                       "eos": "water gamma 4.4 p_inf 6e8 Pa / air gamma 1.4", "flux": "rotated HLLC",
                       "time": "SSPRK(4,3)", "cfl": 0.4, "fallback_cells_in_run": fb},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "traffic": None, "algorithmic_bytes_per_cell_update": bytes_cu},
            "gpu_launches": launches, "clocks": clk.summary()}


def run_blast(args, ws, rank, local, n=512, ntrain=64, tau=0.01, prob=0.2):
    """3D Euler blast at scale: learned troubled-cell indicator + FP32 reconstruction/flux
    vs the plain full-CWENO4 forms (FP32 and FP64) on the same GPU."""
    import torch

    import acoustic_petsc_gb300 as H
    from acoustic_petsc_gb300 import indicator, workloads

    L = H.lib()
    H._lib.check(L.hype_set_device(local), "hype_set_device")
    torch.cuda.set_device(local)
    # 1. labels from the solver itself on a small run of the same problem, trained on the GPU
    tr = H.EulerSolver(H.AppCtx(N_x=ntrain, N_y=ntrain, N_z=ntrain, h=1.0 / ntrain, CFL=0.4, positivity=1,
                                precision=H._lib.PREC_FP32))
    tr.set_state(workloads.euler_blast(ntrain))
    Xs, Ds = [], []
    for _ in range(6):
        tr.step(4)
        X, D = indicator.sample(tr)
        Xs.append(X)
        Ds.append(D)
    tr.close()
    X, D = np.concatenate(Xs), np.concatenate(Ds)
    y = indicator.labels(D, tau)
    t0 = time.perf_counter()
    params, loss = indicator.train(X, y, epochs=10, batch=4096, lr=3e-3, seed=0)
    t_train = time.perf_counter() - t0
    recall, precision, flagged_train = indicator.recall_precision(indicator.score(X, params), y, prob)
    # 2. the 512^3 runs (one context, reconstruction switched between the forms)
    U0 = workloads.euler_blast(n)
    cells = n**3
    res = {}
    ctx = H.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, positivity=1, precision=H._lib.PREC_FP32,
                   recon=H._lib.RECON_CWENO4)
    s = H.EulerSolver(ctx)
    s.set_mlp(params, prob)
    stream = torch.cuda.ExternalStream(L.hype_euler_stream(s._h))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rho = {}
    clocks = None
    launches = 0
    # the learned FP32 form twice: the gate scored on every stage's input (what the unfused kernels
    # do), and scored once per step with its flags widened by a cell for the step's four stages
    for form, recon, per_step in (("plain_fp32", H._lib.RECON_CWENO4, False),
                                  ("learned_fp32", H._lib.RECON_LEARNED, False),
                                  ("learned_fp32_per_step", H._lib.RECON_LEARNED, True)):
        s.set_recon(recon)
        s.set_gate_per_step(per_step)
        s.set_state(U0)
        s.t, s.next_dt = 0.0, 0.0
        s.step(max(args.warmup, 3))
        s.indicator_stats(reset=True)
        l0 = H.launches()
        torch.cuda.synchronize()
        with Clocks(_gpu_index(local)) as clk:
            e0.record(stream)
            s.step(args.steps)
            e1.record(stream)
            e1.synchronize()
        ms = _max_over_ranks(ws, e0.elapsed_time(e1))
        flagged, fb = s.indicator_stats(reset=True)
        res[form] = {"value": ws * cells * args.steps / (ms * 1e-3), "ms_per_step": ms / args.steps,
                     "flagged_per_cell_stage": flagged / (4.0 * cells * args.steps),
                     "positivity_fallback_rate": fb / (4.0 * cells * args.steps)}
        rho[form] = s.get_state()[..., 0]
        if form == "learned_fp32_per_step":
            clocks = clk.summary()
            launches = H.launches() - l0
    l1 = float(np.abs(rho["learned_fp32"] - rho["plain_fp32"]).mean() / np.abs(rho["plain_fp32"]).mean())
    l1_step = float(np.abs(rho["learned_fp32_per_step"] - rho["plain_fp32"]).mean() / np.abs(rho["plain_fp32"]).mean())
    s.close()
    del rho
    # 3. the plain and the indicator-gated FP64 forms (FP64 traces: 130 GB of scratch at 512^3), two steps
    #    each from the same state, the second one timed; the gate pays where the nonlinear weights are
    #    expensive, i.e. in FP64
    s64 = H.EulerSolver(H.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, positivity=1))
    s64.set_mlp(params, prob)
    stream = torch.cuda.ExternalStream(L.hype_euler_stream(s64._h))
    rho64 = {}
    for form, recon in (("plain_fp64", H._lib.RECON_CWENO4), ("learned_fp64", H._lib.RECON_LEARNED)):
        s64.set_recon(recon)
        s64.set_state(U0)
        s64.t, s64.next_dt = 0.0, 0.0
        s64.step(1)
        s64.indicator_stats(reset=True)
        e0.record(stream)
        s64.step(1)
        e1.record(stream)
        e1.synchronize()
        ms64 = _max_over_ranks(ws, e0.elapsed_time(e1))
        flagged, fb = s64.indicator_stats(reset=True)
        res[form] = {"value": ws * cells / (ms64 * 1e-3), "ms_per_step": ms64,
                     "flagged_per_cell_stage": flagged / (4.0 * cells) if form == "learned_fp64" else None}
        rho64[form] = s64.get_state()[..., 0]
    s64.close()
    # 4. the same two forms with the double-float reconstruction and flux (FP64 error bars)
    sdf = H.EulerSolver(H.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, positivity=1,
                                 precision=H._lib.PREC_DF64))
    sdf.set_mlp(params, prob)
    stream = torch.cuda.ExternalStream(L.hype_euler_stream(sdf._h))
    for form, recon in (("plain_df64", H._lib.RECON_CWENO4), ("learned_df64", H._lib.RECON_LEARNED)):
        sdf.set_recon(recon)
        sdf.set_state(U0)
        sdf.t, sdf.next_dt = 0.0, 0.0
        sdf.step(1)
        sdf.indicator_stats(reset=True)
        e0.record(stream)
        sdf.step(1)
        e1.record(stream)
        e1.synchronize()
        msdf = _max_over_ranks(ws, e0.elapsed_time(e1))
        flagged, fb = sdf.indicator_stats(reset=True)
        res[form] = {"value": ws * cells / (msdf * 1e-3), "ms_per_step": msdf,
                     "flagged_per_cell_stage": flagged / (4.0 * cells) if form == "learned_df64" else None}
        rho64[form] = sdf.get_state()[..., 0]
    sdf.close()
    ref64 = rho64["plain_fp64"]
    l1_64 = float(np.abs(rho64["learned_fp64"] - ref64).mean() / np.abs(ref64).mean())
    l1_df = {f: float(np.abs(rho64[f] - ref64).mean() / np.abs(ref64).mean()) for f in ("plain_df64", "learned_df64")}
    del rho64, ref64
    v = res["learned_fp32_per_step"]["value"]
    peak, kind = _peaks()
    ach = EULER_BYTES_PER_CELL_UPDATE * v / ws / 1e9
    return {"metric": "cell-updates/s", "value": v, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": res["learned_fp32_per_step"]["ms_per_step"],
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 state / f32 recon+flux, bf16 indicator",
            "data": "synthetic: spherical blast p ratio 10, rho ratio 8, r0 0.1, seeded 1e-3 pressure noise",
            "config": {"workload": f"euler3d_blast_{n}_learned_indicator", "grid": [n, n, n], "cfl": 0.4,
                       "positivity_fallback": "first order at inadmissible face traces",
                       "indicator": {"train_grid": ntrain, "samples": int(X.shape[0]), "tau": tau,
                                     "prob_threshold": prob, "train_s": t_train, "final_loss": loss,
                                     "recall": recall, "precision": precision, "flagged_train": flagged_train}},
            "forms": res,
            "value_form": "learned_fp32_per_step",
            "speedup_vs_plain_fp32": v / res["plain_fp32"]["value"],
            "speedup_per_stage_gate_vs_plain_fp32": res["learned_fp32"]["value"] / res["plain_fp32"]["value"],
            "speedup_vs_plain_fp64": v / res["plain_fp64"]["value"],
            "l1_rho_learned_vs_plain_fp32": l1,
            "l1_rho_learned_per_step_vs_plain_fp32": l1_step,
            "speedup_learned_fp64_vs_plain_fp64": res["learned_fp64"]["value"] / res["plain_fp64"]["value"],
            "l1_rho_learned_fp64_vs_plain_fp64_after_2_steps": l1_64,
            "speedup_learned_df64_vs_plain_fp64": res["learned_df64"]["value"] / res["plain_fp64"]["value"],
            "l1_rho_vs_plain_fp64_after_2_steps": {"plain_df64": l1_df["plain_df64"],
                                                   "learned_df64": l1_df["learned_df64"],
                                                   "learned_fp64": l1_64},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "traffic": None},
            "gpu_launches": launches, "clocks": clocks}


def _train_blast_indicator(H, ntrain=64, tau=0.01, prob=0.2):
    """the troubled-cell network trained on the GPU from solver labels of a small blast run"""
    from acoustic_petsc_gb300 import indicator, workloads

    tr = H.EulerSolver(H.AppCtx(N_x=ntrain, N_y=ntrain, N_z=ntrain, h=1.0 / ntrain, CFL=0.4, positivity=1,
                                precision=H._lib.PREC_FP32))
    tr.set_state(workloads.euler_blast(ntrain))
    Xs, Ds = [], []
    for _ in range(6):
        tr.step(4)
        X, D = indicator.sample(tr)
        Xs.append(X)
        Ds.append(D)
    tr.close()
    X, D = np.concatenate(Xs), np.concatenate(Ds)
    y = indicator.labels(D, tau)
    t0 = time.perf_counter()
    params, loss = indicator.train(X, y, epochs=10, batch=4096, lr=3e-3, seed=0)
    t_train = time.perf_counter() - t0
    recall, precision, flagged = indicator.recall_precision(indicator.score(X, params), y, prob)
    meta = {"train_grid": ntrain, "samples": int(X.shape[0]), "tau": tau, "prob_threshold": prob,
            "train_s": t_train, "final_loss": loss, "recall": recall, "precision": precision,
            "flagged_train": flagged}
    return params, meta


def _blast_form(H, n, U0, precision, recon, params, prob, dt, nsteps, per_step=False):
    """one form of the blast run with a fixed dt; returns its density and timing / counts
    (per_step: the fused FP32 stage's gate scored once per step)"""
    import torch

    L = H.lib()
    ctx = H.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, positivity=1, precision=precision, recon=recon,
                   dt_mode=H._lib.DT_FIXED)
    s = H.EulerSolver(ctx)
    if recon == H._lib.RECON_LEARNED:
        s.set_mlp(params, prob)
        if per_step:
            s.set_gate_per_step(True)
    s.set_state(U0)
    s.indicator_stats(reset=True)
    stream = torch.cuda.ExternalStream(L.hype_euler_stream(s._h))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    s.step(nsteps, dt=dt)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    flagged, fb = s.indicator_stats()
    rho = np.ascontiguousarray(s.get_state()[..., 0])
    t = s.t
    s.close()
    cells = n**3
    return rho, {"value": cells * nsteps / (ms * 1e-3), "ms_per_step": ms / nsteps, "steps": nsteps, "t_final": t,
                 "flagged_per_cell_stage": flagged / (4.0 * cells * nsteps) if recon == H._lib.RECON_LEARNED else None,
                 "positivity_fallback_rate": fb / (4.0 * cells * nsteps)}


def run_blast_stage_kernels(args, ws, rank, local, n=256, prob=0.2):
    """Per-stage kernel times of the fused FP32 forms on the blast (positivity fallback on): plain
    CWENO4, plain R4 (the floor any gate can reach), the learned gate scored on every stage's input
    and scored once per step; from the context's per-kernel CUDA events ([0] ghost fill plus the
    gate's scoring / widening passes, [1] the fused stage kernel), averaged over the timed stages."""
    import ctypes as C

    import torch

    import acoustic_petsc_gb300 as H
    from acoustic_petsc_gb300 import workloads

    L = H.lib()
    H._lib.check(L.hype_set_device(local), "hype_set_device")
    torch.cuda.set_device(local)
    P = H._lib
    params, meta = _train_blast_indicator(H, prob=prob)
    U0 = workloads.euler_blast(n)
    out = {}
    with Clocks(_gpu_index(local)) as clk:
        for name, recon, per_step in (("plain_cweno4", P.RECON_CWENO4, False), ("plain_r4", P.RECON_LINEAR4, False),
                                      ("learned", P.RECON_LEARNED, False),
                                      ("learned_per_step", P.RECON_LEARNED, True)):
            s = H.EulerSolver(H.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, positivity=1,
                                       precision=P.PREC_FP32, recon=recon))
            if recon == P.RECON_LEARNED:
                s.set_mlp(params, prob)
                s.set_gate_per_step(per_step)
            s.set_state(U0)
            s.step(max(args.warmup, 3))
            s.indicator_stats(reset=True)
            H._lib.check(L.hype_euler_profile(s._h, 1), "profile")
            s.step(args.steps)
            ms = (C.c_double * 3)()
            cnt = (C.c_longlong * 3)()
            H._lib.check(L.hype_euler_profile_read(s._h, ms, cnt), "profile_read")
            H._lib.check(L.hype_euler_profile(s._h, 0), "profile")
            flagged, fb = s.indicator_stats()
            stages = max(cnt[1], 1)
            out[name] = {"ghost_and_gate_ms": ms[0] / stages, "stage_fused_ms": ms[1] / stages,
                         "total_ms": (ms[0] + ms[1] + ms[2]) / stages,
                         "flagged_per_cell_stage": flagged / (stages * n**3), "positivity_fallbacks": fb}
            s.close()
    base = out["plain_cweno4"]["total_ms"]
    for v in out.values():
        v["speedup_vs_plain_cweno4"] = base / v["total_ms"]
    v = n**3 / (out["learned_per_step"]["total_ms"] * 4e-3)
    return {"metric": "cell-updates/s", "value": v, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": 4 * out["learned_per_step"]["total_ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 state / f32 recon+flux, bf16 indicator",
            "data": "synthetic: spherical blast p ratio 10, rho ratio 8, r0 0.1, seeded 1e-3 pressure noise",
            "config": {"workload": f"euler3d_blast_{n}_fp32_stage_kernels", "grid": [n, n, n], "indicator": meta,
                       "timing": "per-kernel CUDA events (hype_euler_profile), per RK stage"},
            "stage_kernels": out, "gpu_launches": None, "clocks": clk.summary()}


def run_blast_horizon(args, ws, rank, local, n=512, nsteps=500, prob=0.2, smax_bound=3.0, fp32_only=False):
    """The blast workload to its full length: 512^3, 500 SSPRK(4,3) steps at a fixed dt
    (CFL 0.4 against a wave-speed bound of 3), every form timed and compared.
    (a) distance from the FP64-bar reference at 512^3: L1(rho) of each form against the plain
        double-float run (the plain FP64 run is too slow to take 500 steps here; the two agree to
        round-off, shown over the first 50 steps);
    (b) accuracy: the same problem at 256^3 (initial state = the 512^3 one averaged over 2^3 cells,
        250 steps of twice the dt) in every form, L1(rho) against the 512^3 reference averaged to
        256^3, and each form's error over plain CWENO4's in the same arithmetic (the 1.05 bar).
    fp32_only: the FP32 forms alone, against the plain FP32 run at 512^3 as the reference (1.2e-8 in
    L1(rho) from the double-float one after the 500 steps; a few minutes instead of half an hour)."""
    import torch

    import acoustic_petsc_gb300 as H
    from acoustic_petsc_gb300 import workloads

    L = H.lib()
    H._lib.check(L.hype_set_device(local), "hype_set_device")
    torch.cuda.set_device(local)
    P = H._lib
    params, meta = _train_blast_indicator(H, prob=prob)
    U0 = workloads.euler_blast(n)
    dt = 0.4 * (1.0 / n) / (3.0 * smax_bound)
    l1 = lambda a, b: float(np.abs(a - b).sum() / np.abs(b).sum())  # noqa: E731
    forms512 = {}
    if fp32_only:
        return _blast_horizon_fp32(H, n, nsteps, prob, dt, params, meta, U0, l1, ws, local)
    with Clocks(_gpu_index(local)) as clk:
        ref, forms512["plain_df64"] = _blast_form(H, n, U0, P.PREC_DF64, P.RECON_CWENO4, params, prob, dt, nsteps)
        for name, prec, recon in (("plain_fp32", P.PREC_FP32, P.RECON_CWENO4),
                                  ("learned_fp32", P.PREC_FP32, P.RECON_LEARNED),
                                  ("learned_fp32_per_step", P.PREC_FP32, P.RECON_LEARNED),
                                  ("learned_df64", P.PREC_DF64, P.RECON_LEARNED)):
            rho, forms512[name] = _blast_form(H, n, U0, prec, recon, params, prob, dt, nsteps,
                                              per_step=name.endswith("per_step"))
            forms512[name]["l1_rho_vs_plain_df64"] = l1(rho, ref)
            del rho
        # the double-float reference against plain FP64 over the first 50 steps
        r64, f64 = _blast_form(H, n, U0, P.PREC_FP64, P.RECON_CWENO4, params, prob, dt, 50)
        rdf, _ = _blast_form(H, n, U0, P.PREC_DF64, P.RECON_CWENO4, params, prob, dt, 50)
        f64["l1_rho_vs_plain_df64_after_50_steps"] = l1(rdf, r64)
        forms512["plain_fp64_50_steps"] = f64
        del r64, rdf
        # (b) 256^3 from the averaged initial state, against the averaged 512^3 reference
        m = n // 2
        U1 = U0.reshape(m, 2, m, 2, m, 2, 5).mean(axis=(1, 3, 5))
        del U0
        ref_c = ref.reshape(m, 2, m, 2, m, 2).mean(axis=(1, 3, 5))
        del ref
        forms256 = {}
        for name, prec, recon in (("plain_fp64", P.PREC_FP64, P.RECON_CWENO4),
                                  ("learned_fp64", P.PREC_FP64, P.RECON_LEARNED),
                                  ("plain_fp32", P.PREC_FP32, P.RECON_CWENO4),
                                  ("learned_fp32", P.PREC_FP32, P.RECON_LEARNED),
                                  ("learned_fp32_per_step", P.PREC_FP32, P.RECON_LEARNED),
                                  ("plain_df64", P.PREC_DF64, P.RECON_CWENO4),
                                  ("learned_df64", P.PREC_DF64, P.RECON_LEARNED)):
            rho, forms256[name] = _blast_form(H, m, U1, prec, recon, params, prob, 2.0 * dt, nsteps // 2,
                                              per_step=name.endswith("per_step"))
            forms256[name]["l1_rho_error_vs_512_reference"] = l1(rho, ref_c)
            del rho
    for name in forms256:
        base = "plain_" + name.split("_")[1]
        forms256[name]["error_over_plain_same_arithmetic"] = (forms256[name]["l1_rho_error_vs_512_reference"] /
                                                              forms256[base]["l1_rho_error_vs_512_reference"])
        forms256[name]["error_over_plain_fp64"] = (forms256[name]["l1_rho_error_vs_512_reference"] /
                                                   forms256["plain_fp64"]["l1_rho_error_vs_512_reference"])
    v = forms512["learned_fp32"]["value"]
    return {"metric": "cell-updates/s", "value": v, "unit": "cell-updates/s", "n_gpus": ws, "steps": nsteps,
            "warmup": 0, "ms_per_step": forms512["learned_fp32"]["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 state / f32 recon+flux, bf16 indicator",
            "data": "synthetic: spherical blast p ratio 10, rho ratio 8, r0 0.1, seeded 1e-3 pressure noise",
            "config": {"workload": f"euler3d_blast_{n}_{nsteps}_steps", "grid": [n, n, n], "dt": dt,
                       "dt_rule": f"fixed: CFL 0.4 h / (3 x {smax_bound})", "positivity_fallback": "first order",
                       "indicator": meta},
            "forms_512": forms512, "forms_256_vs_512_reference": forms256,
            "speedup_learned_fp32_vs_plain_fp32": v / forms512["plain_fp32"]["value"],
            "speedup_learned_fp32_per_step_vs_plain_fp32": (forms512["learned_fp32_per_step"]["value"] /
                                                            forms512["plain_fp32"]["value"]),
            "speedup_learned_fp32_vs_plain_fp64": v / forms512["plain_fp64_50_steps"]["value"],
            "gpu_launches": None, "clocks": clk.summary()}


def _blast_horizon_fp32(H, n, nsteps, prob, dt, params, meta, U0, l1, ws, local):
    """run_blast_horizon's FP32 forms: the plain FP32 run at n^3 is the reference"""
    P = H._lib
    forms512 = {}
    with Clocks(_gpu_index(local)) as clk:
        ref, forms512["plain_fp32"] = _blast_form(H, n, U0, P.PREC_FP32, P.RECON_CWENO4, params, prob, dt, nsteps)
        for name in ("learned_fp32", "learned_fp32_per_step"):
            rho, forms512[name] = _blast_form(H, n, U0, P.PREC_FP32, P.RECON_LEARNED, params, prob, dt, nsteps,
                                              per_step=name.endswith("per_step"))
            forms512[name]["l1_rho_vs_plain_fp32"] = l1(rho, ref)
            del rho
        m = n // 2
        U1 = U0.reshape(m, 2, m, 2, m, 2, 5).mean(axis=(1, 3, 5))
        ref_c = ref.reshape(m, 2, m, 2, m, 2).mean(axis=(1, 3, 5))
        del ref
        forms256 = {}
        for name, recon in (("plain_fp32", P.RECON_CWENO4), ("learned_fp32", P.RECON_LEARNED),
                            ("learned_fp32_per_step", P.RECON_LEARNED)):
            rho, forms256[name] = _blast_form(H, m, U1, P.PREC_FP32, recon, params, prob, 2.0 * dt, nsteps // 2,
                                              per_step=name.endswith("per_step"))
            forms256[name]["l1_rho_error_vs_512_reference"] = l1(rho, ref_c)
            del rho
    for name in forms256:
        forms256[name]["error_over_plain_same_arithmetic"] = (forms256[name]["l1_rho_error_vs_512_reference"] /
                                                              forms256["plain_fp32"]["l1_rho_error_vs_512_reference"])
    v = forms512["learned_fp32_per_step"]["value"]
    return {"metric": "cell-updates/s", "value": v, "unit": "cell-updates/s", "n_gpus": ws, "steps": nsteps,
            "warmup": 0, "ms_per_step": forms512["learned_fp32_per_step"]["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 state / f32 recon+flux, bf16 indicator",
            "data": "synthetic: spherical blast p ratio 10, rho ratio 8, r0 0.1, seeded 1e-3 pressure noise",
            "config": {"workload": f"euler3d_blast_{n}_{nsteps}_steps_fp32_forms", "grid": [n, n, n], "dt": dt,
                       "reference": f"plain FP32 CWENO4 at {n}^3", "positivity_fallback": "first order",
                       "indicator": meta},
            "forms_512": forms512, "forms_256_vs_512_reference": forms256,
            "speedup_learned_fp32_per_step_vs_plain_fp32": v / forms512["plain_fp32"]["value"],
            "speedup_learned_fp32_vs_plain_fp32": forms512["learned_fp32"]["value"] / forms512["plain_fp32"]["value"],
            "gpu_launches": None, "clocks": clk.summary()}


def run_mp2d_learned(args, ws, rank, local, n=1024, ntrain=256, tau=1e-4, prob=0.2):
    """Config 3 with the learned indicator: Kapila 1024^2 shock-bubble, FP64 state, FP32
    reconstruction/flux; plain CWENO4 vs the indicator-gated form (network trained on the
    GPU on labels from a 256^2 run of the same problem) vs plain FP64, on the same GPU."""
    import torch

    import acoustic_petsc_gb300 as H
    from acoustic_petsc_gb300 import indicator, workloads

    L = H.lib()
    H._lib.check(L.hype_set_device(local), "hype_set_device")
    torch.cuda.set_device(local)
    Lc = H._lib

    def solver(nn, precision, recon=Lc.RECON_CWENO4):
        U, h = workloads.kapila_bubble(nn, model=1)
        m = H.Multiphase2D(nn, nn, h, CFL=0.4, boundaries=(2, 2, 2, 2), model=Lc.MP_KAPILA5, eos=workloads.KAPILA_EOS,
                           stepper=Lc.STEP_SSPRK43, precision=precision, recon=recon)
        m.set_state(U)
        return m, U

    tr, _ = solver(ntrain, Lc.PREC_FP64)
    Xs, Ds = [], []
    for _ in range(6):
        tr.step(40)
        X, D = indicator.sample(tr)
        Xs.append(X)
        Ds.append(D)
    tr.close()
    X, D = np.concatenate(Xs), np.concatenate(Ds)
    y = indicator.labels(D, tau)
    t0 = time.perf_counter()
    params, loss = indicator.train(X, y, epochs=10, batch=4096, lr=3e-3, seed=0)
    t_train = time.perf_counter() - t0
    recall, precision, flagged_train = indicator.recall_precision(indicator.score(X, params), y, prob)
    res = {}
    clocks, launches = None, 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rho = {}
    # the learned forms with the gate scored in every stage's reconstruction, and scored once per step
    for form, prec, recon in (("plain_fp32", Lc.PREC_FP32, Lc.RECON_CWENO4), ("learned_fp32", Lc.PREC_FP32, Lc.RECON_LEARNED),
                              ("learned_fp32_per_step", Lc.PREC_FP32, Lc.RECON_LEARNED),
                              ("plain_fp64", Lc.PREC_FP64, Lc.RECON_CWENO4),
                              ("learned_fp64", Lc.PREC_FP64, Lc.RECON_LEARNED),
                              ("learned_fp64_per_step", Lc.PREC_FP64, Lc.RECON_LEARNED)):
        m, _ = solver(n, prec, recon)
        if recon == Lc.RECON_LEARNED:
            m.set_mlp(params, prob)
            m.set_gate_per_step(form.endswith("per_step"))
        m.step(max(args.warmup, 3))
        m.indicator_stats(reset=True)
        stream = torch.cuda.ExternalStream(L.hype_mp2d_stream(m._h))
        l0 = H.launches()
        torch.cuda.synchronize()
        with Clocks(_gpu_index(local)) as clk:
            e0.record(stream)
            m.step(args.steps)
            e1.record(stream)
            e1.synchronize()
        ms = _max_over_ranks(ws, e0.elapsed_time(e1))
        res[form] = {"value": ws * n * n * args.steps / (ms * 1e-3), "ms_per_step": ms / args.steps,
                     "flagged_per_cell_stage": m.indicator_stats() / (4.0 * n * n * args.steps),
                     "minmod_fallback_cells": m.fallback_cells}
        if form == "learned_fp32_per_step":
            clocks, launches = clk.summary(), H.launches() - l0
        if "fp64" in form:
            q = m.get_state()
            rho[form] = q[..., 0] + q[..., 1]  # alpha1 rho1 + alpha2 rho2
        m.close()
    l1_64 = float(np.abs(rho["learned_fp64"] - rho["plain_fp64"]).mean() / np.abs(rho["plain_fp64"]).mean())
    l1_64s = float(np.abs(rho["learned_fp64_per_step"] - rho["plain_fp64"]).mean() / np.abs(rho["plain_fp64"]).mean())
    v = res["learned_fp32_per_step"]["value"]
    peak, kind = _peaks()
    return {"metric": "cell-updates/s", "value": v, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": res["learned_fp32_per_step"]["ms_per_step"],
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 state / f32 recon+flux, bf16 indicator",
            "data": "synthetic: shock-driven air bubble in water (stiffened gases), 1e8 Pa step at x < 0.2",
            "config": {"workload": f"kapila2d_{n}_learned_indicator", "grid": [n, n], "cfl": 0.4,
                       "scheme": "primitive CWENO4 + 8-node PAD/minmod + rotated HLLC + SSPRK(4,3)",
                       "indicator": {"train_grid": ntrain, "samples": int(X.shape[0]), "tau": tau,
                                     "prob_threshold": prob, "train_s": t_train, "final_loss": loss,
                                     "recall": recall, "precision": precision, "flagged_train": flagged_train}},
            "forms": res, "value_form": "learned_fp32_per_step", "speedup_vs_plain_fp32": v / res["plain_fp32"]["value"],
            "speedup_per_stage_gate_vs_plain_fp32": res["learned_fp32"]["value"] / res["plain_fp32"]["value"],
            "speedup_vs_plain_fp64": v / res["plain_fp64"]["value"],
            "speedup_learned_fp64_vs_plain_fp64": res["learned_fp64"]["value"] / res["plain_fp64"]["value"],
            "speedup_learned_fp64_per_step_vs_plain_fp64": (res["learned_fp64_per_step"]["value"] /
                                                            res["plain_fp64"]["value"]),
            "l1_rho_learned_fp64_vs_plain_fp64": l1_64,
            "l1_rho_learned_fp64_per_step_vs_plain_fp64": l1_64s,
            "roofline": {"bound": "hbm", "achieved": None, "peak": peak, "unit": "GB/s", "frac": None, "traffic": None},
            "gpu_launches": launches, "clocks": clocks}


def run_acoustic(args, ws, rank, local, n=256, precision=0):
    """acoustic FV path of 3d/weno4/plane_wave: the plane wave k = (1,1,1) on [0, 2 pi]^3,
    periodic, R4 face gradients + central flux, SSPRK(4,3) with dt = h CFL / 3, CFL 0.5"""
    import math

    import torch

    import acoustic_petsc_gb300 as H

    L = H.lib()
    H._lib.check(L.hype_set_device(local), "hype_set_device")
    torch.cuda.set_device(local)
    h = 2 * math.pi / n
    s = H.AcousticFV3D(n, n, n, h, h * 0.5 / 3.0, precision=precision)
    x = (np.arange(n) + 0.5) * h
    ph = x[:, None, None] + x[None, :, None] + x[None, None, :]
    U0 = np.stack([np.sin(ph), -math.sqrt(3.0) * np.cos(ph)], -1)
    s.set_state(U0)
    s.step(max(args.warmup, 3))
    stream = torch.cuda.ExternalStream(L.hype_acoustic_stream(s._h))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = H.launches()
    _barrier(ws)
    torch.cuda.synchronize()
    with Clocks(_gpu_index(local)) as clk:
        e0.record(stream)
        s.step(args.steps)
        e1.record(stream)
        e1.synchronize()
    launches = H.launches() - l0
    ms = _max_over_ranks(ws, e0.elapsed_time(e1))
    cells = n**3
    value = ws * cells * args.steps / (ms * 1e-3)
    peak, kind = _peaks()
    bytes_cu = 4 * 32 + 16  # per stage read + write (u, v), one extra read of u^n per step
    ach = bytes_cu * cells * args.steps / (ms * 1e-3) / 1e9
    s.close()
    return {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64" if precision == 0 else "f64 state / df64 (FP32 pairs) gradients and fluxes",
            "data": "synthetic plane wave sin(x+y+z), exact cell-centre values",
            "config": {"workload": f"acoustic_fv_plane_wave_{n}" + ("_df64" if precision else ""), "grid": [n, n, n],
                       "cfl": 0.5,
                       "scheme": "R4 face gradients + central flux + SSPRK(4,3), 3d/weno4/plane_wave"},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "traffic": None},
            "gpu_launches": launches, "clocks": clk.summary()}


def run_sw2d(args, ws, rank, local, n=4096):
    """2D acoustic FV program of 2d/weno4/standing_wave at n^2: sin(2 pi x) sin(2 pi y) on
    [-1,1]^2, adiabatic walls, R4 edge gradients + averaged flux, SSP RK104 with
    dt = h CFL / 2, CFL 0.5"""
    import torch

    import acoustic_petsc_gb300 as H

    L = H.lib()
    H._lib.check(L.hype_set_device(local), "hype_set_device")
    torch.cuda.set_device(local)
    n = args.grid or n
    h = 2.0 / n
    s = H.AcousticFV2D(n, n, h, 0.5 * h * 0.5, x_min=-1.0, y_min=-1.0)
    x = -1.0 + (np.arange(n) + 0.5) * h
    U0 = np.zeros((n, n, 2))
    U0[..., 0] = np.sin(2 * math.pi * x)[None, :] * np.sin(2 * math.pi * x)[:, None]
    s.set_state(U0)
    s.step(max(args.warmup, 3))
    stream = torch.cuda.ExternalStream(L.hype_acoustic2d_stream(s._h))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = H.launches()
    _barrier(ws)
    torch.cuda.synchronize()
    with Clocks(_gpu_index(local)) as clk:
        e0.record(stream)
        s.step(args.steps)
        e1.record(stream)
        e1.synchronize()
    launches = H.launches() - l0
    ms = _max_over_ranks(ws, e0.elapsed_time(e1))
    cells = n * n
    value = ws * cells * args.steps / (ms * 1e-3)
    peak, kind = _peaks()
    # per RK104 step and cell: 10 stages of read + write (u, v), the two combinations
    # (read 2 states, write 1) and the final read of the second register
    bytes_cu = 10 * 32 + 2 * 48 + 16
    ach = bytes_cu * cells * args.steps / (ms * 1e-3) / 1e9
    # end to end: host state in, one step, host state out (pinned buffers)
    host = torch.empty((n, n, 2), dtype=torch.float64, pin_memory=True)
    hv = host.numpy()
    hv[...] = U0
    ke = max(1, min(3, args.steps))
    t0 = time.perf_counter()
    for _ in range(ke):
        s.set_state(hv)
        s.step(1)
        H._lib.check(L.hype_acoustic2d_download(s._h, hv.ctypes.data_as(H._lib.D)), "download")
    wall = time.perf_counter() - t0
    ms_e2e = _max_over_ranks(ws, wall * 1e3)
    s.close()
    nb = cells * 2 * 8
    return {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic standing wave sin(2 pi x) sin(2 pi y), cell centres",
            "config": {"workload": f"acoustic_fv_standing_wave_{n}", "grid": [n, n], "cfl": 0.5,
                       "scheme": "2D R4 edge gradients + averaged flux + SSP RK104, 2d/weno4/standing_wave",
                       "l2": f"state 2*8*{n}^2 B = {16 * cells / 1e6:.0f} MB vs 129 MB; no flush"},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "algorithmic_bytes_per_cell_update": bytes_cu, "traffic": None},
            "e2e": {"value": ws * cells * ke / (ms_e2e * 1e-3), "unit": "cell-updates/s", "h2d_bytes_per_step": nb,
                    "d2h_bytes_per_step": nb, "steps": ke,
                    "path": "AcousticFV2D.set_state -> step(1) -> get_state"},
            "gpu_launches": launches, "clocks": clk.summary()}


def run_mp3d(args, ws, rank, local, n=256):
    """3D primitive multiphase (3d/weno4/Viscous-Multiphase-Fourth-Order) at n^3: the program's
    layered shock / gas-layer set-up along z, transmissive, CFL 0.9, its EOS and viscous dt limit"""
    import torch

    import acoustic_petsc_gb300 as H
    from acoustic_petsc_gb300 import workloads

    L = H.lib()
    H._lib.check(L.hype_set_device(local), "hype_set_device")
    torch.cuda.set_device(local)
    n = args.grid or n
    h = 1.0 / n
    U0 = workloads.mp3d_layers(n, n, n)
    s = H.Multiphase3D(n, n, n, h, CFL=0.9, x_min=-0.5, y_min=-0.5, z_min=-0.5)
    s.set_state(U0)
    s.step(max(args.warmup, 3))
    stream = torch.cuda.ExternalStream(L.hype_mp3d_stream(s._h))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = H.launches()
    _barrier(ws)
    torch.cuda.synchronize()
    with Clocks(_gpu_index(local)) as clk:
        e0.record(stream)
        s.step(args.steps)
        e1.record(stream)
        e1.synchronize()
    launches = H.launches() - l0
    ms = _max_over_ranks(ws, e0.elapsed_time(e1))
    cells = n**3
    value = ws * cells * args.steps / (ms * 1e-3)
    peak, kind = _peaks()
    bytes_cu = 4 * 96 + 48  # per stage read + write of 6 doubles, one extra read of u^n per step
    ach = bytes_cu * cells * args.steps / (ms * 1e-3) / 1e9
    host = torch.empty((n, n, n, 6), dtype=torch.float64, pin_memory=True)
    hv = host.numpy()
    hv[...] = U0
    ke = max(1, min(2, args.steps))
    t0 = time.perf_counter()
    for _ in range(ke):
        s.set_state(hv)
        s.step(1)
        H._lib.check(L.hype_mp3d_download(s._h, hv.ctypes.data_as(H._lib.D)), "download")
    wall = time.perf_counter() - t0
    ms_e2e = _max_over_ranks(ws, wall * 1e3)
    s.close()
    nb = cells * 6 * 8
    return {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: the program's z-layered shock / light-gas set-up, interfaces smoothed over 0.02",
            "config": {"workload": f"mphase3d_layers_{n}", "grid": [n, n, n], "cfl": 0.9,
                       "scheme": "primitive CWENO4 + 33-node PAD + rotated HLLC + SSPRK(4,3), "
                                 "3d/weno4/Viscous-Multiphase-Fourth-Order",
                       "l2": f"state 6*8*{n}^3 B = {48 * cells / 1e6:.0f} MB vs 129 MB; no flush"},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "algorithmic_bytes_per_cell_update": bytes_cu, "traffic": None},
            "e2e": {"value": ws * cells * ke / (ms_e2e * 1e-3), "unit": "cell-updates/s", "h2d_bytes_per_step": nb,
                    "d2h_bytes_per_step": nb, "steps": ke, "path": "Multiphase3D.set_state -> step(1) -> get_state"},
            "gpu_launches": launches, "clocks": clk.summary()}


def run_pc2d(args, ws, rank, local, n=2048, order=3):
    """the path-conservative scheme of 2d/HyPE-2D (Kapila model, order N, Rusanov + Roe-path
    fluctuation, the program's stepper for N) on an n^2 drop, transmissive, CFL 0.9"""
    import torch

    import acoustic_petsc_gb300 as H
    from acoustic_petsc_gb300 import workloads

    L = H.lib()
    H._lib.check(L.hype_set_device(local), "hype_set_device")
    torch.cuda.set_device(local)
    n = args.grid or n
    U0 = workloads.kapila_drop(n)
    s = H.PathConservative2D(n, n, 1.0 / n, order=order, CFL=0.9)
    s.set_state(U0)
    s.step(max(args.warmup, 3))
    stream = torch.cuda.ExternalStream(L.hype_pc2d_stream(s._h))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = H.launches()
    _barrier(ws)
    torch.cuda.synchronize()
    with Clocks(_gpu_index(local)) as clk:
        e0.record(stream)
        s.step(args.steps)
        e1.record(stream)
        e1.synchronize()
    launches = H.launches() - l0
    ms = _max_over_ranks(ws, e0.elapsed_time(e1))
    cells = n * n
    value = ws * cells * args.steps / (ms * 1e-3)
    peak, kind = _peaks()
    stages = {0: 1, 1: 2, 2: 4, 3: 10}[order]
    bytes_cu = stages * 96 + (2 * 144 + 48 if order == 3 else 48)
    ach = bytes_cu * cells * args.steps / (ms * 1e-3) / 1e9
    host = torch.empty((n, n, 6), dtype=torch.float64, pin_memory=True)
    hv = host.numpy()
    hv[...] = U0
    ke = max(1, min(3, args.steps))
    t0 = time.perf_counter()
    for _ in range(ke):
        s.set_state(hv)
        s.step(1)
        H._lib.check(L.hype_pc2d_download(s._h, hv.ctypes.data_as(H._lib.D)), "download")
    wall = time.perf_counter() - t0
    ms_e2e = _max_over_ranks(ws, wall * 1e3)
    fb = s.fallback_cells
    s.close()
    nb = cells * 6 * 8
    return {"metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: Kapila drop (phase 1 in phase 2, gamma 1.4 both), seeded 1 % velocity noise",
            "config": {"workload": f"pathcons2d_kapila_n{order}_{n}", "grid": [n, n], "cfl": 0.9, "order": order,
                       "scheme": "2d/HyPE-2D RHSFunction: conservative WENO of order N + node PAD + Rusanov + "
                                 "Roe-path fluctuation + volume NCP, SSP stepper of N (bit-identical to the reference)",
                       "fallback_cells_last_step": fb,
                       "l2": f"state 6*8*{n}^2 B = {48 * cells / 1e6:.0f} MB vs 129 MB; no flush"},
            "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                         "algorithmic_bytes_per_cell_update": bytes_cu, "traffic": None},
            "e2e": {"value": ws * cells * ke / (ms_e2e * 1e-3), "unit": "cell-updates/s", "h2d_bytes_per_step": nb,
                    "d2h_bytes_per_step": nb, "steps": ke, "path": "PathConservative2D.set_state -> step(1) -> get_state"},
            "gpu_launches": launches, "clocks": clk.summary()}


WORKLOADS = {
    "blast512": run_blast,
    "blast256": lambda a, *r: run_blast(a, *r, n=256),
    "blast512_horizon": run_blast_horizon,
    "blast128_horizon": lambda a, *r: run_blast_horizon(a, *r, n=128, nsteps=40),
    "blast512_horizon_fp32": lambda a, *r: run_blast_horizon(a, *r, fp32_only=True),
    "blast256_stage_kernels": run_blast_stage_kernels,
    "blast128_stage_kernels": lambda a, *r: run_blast_stage_kernels(a, *r, n=128),
    "kapila1024": lambda a, *r: run_mp2d(a, *r, precision=0),
    "kapila1024_learned": run_mp2d_learned,
    "acoustic256": run_acoustic,
    "acoustic256_df64": lambda a, *r: run_acoustic(a, *r, precision=2),
    "acoustic128": lambda a, *r: run_acoustic(a, *r, n=128),
    "acoustic128_df64": lambda a, *r: run_acoustic(a, *r, n=128, precision=2),
    "kapila1024_fp32": lambda a, *r: run_mp2d(a, *r, precision=1),
    "euler256_hllc": lambda a, *r: run_euler(a, *r, precision=0, recon=0, flux=1),
    "euler256_rothllc": lambda a, *r: run_euler(a, *r, precision=0, recon=0, flux=2),
    "euler256": lambda a, *r: run_euler(a, *r, precision=0, recon=0),
    "euler256_fp32": lambda a, *r: run_euler(a, *r, precision=1, recon=0),
    "euler256_df64": lambda a, *r: run_euler(a, *r, precision=2, recon=0),
    "euler256_df64_linear": lambda a, *r: run_euler(a, *r, precision=2, recon=1),
    "euler128_df64": lambda a, *r: run_euler(a, *r, precision=2, recon=0, n=128),
    "euler256_linear": lambda a, *r: run_euler(a, *r, precision=0, recon=1),
    "euler256_fp32_linear": lambda a, *r: run_euler(a, *r, precision=1, recon=1),
    "euler256_weno3": lambda a, *r: run_euler(a, *r, precision=0, recon=3),
    "ns256_tgv": lambda a, *r: run_euler(a, *r, precision=0, recon=1, viscous=True),
    "ns256_tgv_df64": lambda a, *r: run_euler(a, *r, precision=2, recon=1, viscous=True),
    "euler64": lambda a, *r: run_euler(a, *r, precision=0, recon=0, n=64),
    "euler128": lambda a, *r: run_euler(a, *r, precision=0, recon=0, n=128),
    "euler128_fp32": lambda a, *r: run_euler(a, *r, precision=1, recon=0, n=128),
    "sw2d4096": run_sw2d,
    "mp3d256": run_mp3d,
    "pc2d2048": run_pc2d,
    "ctcs512": run_ctcs,
    "batch256": run_batch,
}


# one CPU sample of the 3D Euler workload for the reference arm and the GPU line's cpu_baseline:
# the 256^3 pulse's physics on 128^3 cells (the per-cell rate of the restatement grows with the
# grid up to about this size; the whole 256^3 grid would take minutes per step)
EULER_CPU_SAMPLE_N = 128


def _reference_program_figures():
    """the reference program's own per-core rate, measured where its sources are (the GPU machine has
    none): profiles/cpu_reference_euler.txt"""
    if not os.path.exists(os.path.join(ROOT, "profiles", "cpu_reference_euler.txt")):
        return None
    keys = ("reference_cweno4_per_core_cell_updates_per_s", "restatement_over_reference_per_core_cweno4",
            "reference_weno3_per_core_cell_updates_per_s", "restatement_over_reference_per_core_weno3")
    out = {k: _profile_figure("cpu_reference_euler.txt", k) for k in keys}
    out["source"] = "profiles/cpu_reference_euler.txt (python oracle/time_reference.py 32, x86_64 host, 1 core)"
    return out


def reference_arm(args, ws, rank):
    """CPU implementation of the path on all host cores, bounded sample per step."""
    if rank != 0:
        return None
    n = int(os.environ.get("HYPE_REF_SAMPLE_N", str(EULER_CPU_SAMPLE_N)))
    if args.workload.startswith("euler"):
        rates = []
        for _ in range(max(args.warmup, 0)):
            cpu_euler_rate(n, 1, use_ref=False)
        t_all = 0.0
        for _ in range(args.steps):
            r, cores, kind, d = cpu_euler_rate(n, 1, use_ref=False)
            rates.append(r)
            t_all += d
        value = n**3 * args.steps / t_all
        sample = (f"1 SSPRK(4,3) step of a {n}^3 periodic pulse grid per bench step (same physics as 256^3); "
                  "the C restatement of the reference's RHS (bit-identical to the reference compiled in place), "
                  "all host threads")
        cfg_w = "euler3d_cweno4_rusanov_ssprk43_256"
    else:
        r, cores, kind, d = cpu_ctcs_rate(512, 200)
        value, sample, cfg_w = r, "200 steps of the 512^2 CTCS run", "ctcs2d_512_1000steps"
    return {"impl": "reference", "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s",
            "higher_is_better": True, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "config": {"workload": cfg_w},
            "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": cores, "kind": kind,
                             "sample": sample},
            "reference_program": _reference_program_figures() if args.workload.startswith("euler") else None,
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="euler256", choices=sorted(WORKLOADS))
    ap.add_argument("--no-alt-forms", action="store_true",
                    help="skip the double-float form measured beside the default FP64 Euler workload")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--grid", type=int, default=0,
                    help="cells per axis of the 3D Euler / Navier-Stokes workloads (default 256; smaller for profiling)")
    args = ap.parse_args()
    ws, rank, local = _dist()
    if args.impl == "reference":
        out = reference_arm(args, ws, rank)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    out = WORKLOADS[args.workload](args, ws, rank, local)
    if rank == 0 and not args.no_cpu_baseline:
        if args.workload.startswith("kapila"):
            from acoustic_petsc_gb300 import workloads
            from oracle import pyoracle as O

            O.build(None)
            n = 256
            U0, h = workloads.kapila_bubble(n)
            cfg = O.mp2d_cfg(n, n, h, cfl=0.4, bc=(2, 2, 2, 2), model=1, eos=workloads.KAPILA_EOS,
                             nthreads=os.cpu_count() or 1)
            O.mp2d_run(cfg, U0, 1)
            t0 = time.perf_counter()
            O.mp2d_run(cfg, U0, 4)
            d = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": n * n * 4 / d, "unit": "cell-updates/s", "cores": O.threads(),
                                   "kind": "port", "sample": f"4 SSPRK(4,3) steps of the {n}^2 version ({d:.1f} s)"}
        elif args.workload.startswith("pc2d"):
            from acoustic_petsc_gb300 import workloads
            from oracle import pyoracle as O

            O.build(None)
            n = 512
            cfg = O.h2d_cfg(3, n, n, 1.0 / n, cfl=0.9, bc=(2,) * 4, nthreads=os.cpu_count() or 1)
            U0 = workloads.kapila_drop(n)
            O.h2d_run(cfg, U0, 1)
            t0 = time.perf_counter()
            O.h2d_run(cfg, U0, 2)
            d = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": n * n * 2 / d, "unit": "cell-updates/s", "cores": O.threads(),
                                   "kind": "port", "sample": f"2 RK104 steps of the order-3 {n}^2 drop ({d:.1f} s)"}
        elif args.workload.startswith("mp3d"):
            from acoustic_petsc_gb300 import workloads
            from oracle import pyoracle as O

            O.build(None)
            n = 48
            cfg = O.mp3d_cfg(n, 1.0 / n, cfl=0.9, bc=(2,) * 6, nthreads=os.cpu_count() or 1)
            U0 = workloads.mp3d_layers(n, n, n)
            O.mp3d_run(cfg, U0, 1)
            t0 = time.perf_counter()
            O.mp3d_run(cfg, U0, 2)
            d = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": n**3 * 2 / d, "unit": "cell-updates/s", "cores": O.threads(),
                                   "kind": "port", "sample": f"2 SSPRK(4,3) steps of the {n}^3 layered set-up ({d:.1f} s)"}
        elif args.workload.startswith("sw2d"):
            from oracle import pyoracle as O

            O.build(None)
            n = 1024
            cfg = O.sw2d_cfg(n, n, 2.0 / n, -1.0, -1.0, (4,) * 4, 1.0, 1.0, 1.0)
            U0 = O.sw2d_ic(cfg)
            O.sw2d_run(cfg, U0, 1, 0.5 * cfg.h * 0.5)
            t0 = time.perf_counter()
            O.sw2d_run(cfg, U0, 10, 0.5 * cfg.h * 0.5)
            d = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": n * n * 10 / d, "unit": "cell-updates/s", "cores": O.threads(),
                                   "kind": "port", "sample": f"10 RK104 steps of the {n}^2 standing wave ({d:.1f} s)"}
        elif args.workload.startswith("ns"):
            from acoustic_petsc_gb300 import workloads
            from oracle import pyoracle as O

            O.build(None)
            n = 96
            cfg = O.euler_cfg(n, 2.0 * math.pi / n, cfl=0.6, origin=(-math.pi,) * 3, recon=1, mu=0.01,
                              nthreads=os.cpu_count() or 1)
            U0 = workloads.taylor_green(n)
            O.euler_run(cfg, U0, 1)
            t0 = time.perf_counter()
            O.euler_run(cfg, U0, 2)
            d = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": n**3 * 2 / d, "unit": "cell-updates/s", "cores": O.threads(),
                                   "kind": "port", "sample": f"2 SSPRK(4,3) steps of the {n}^3 Taylor-Green run ({d:.1f} s)"}
        elif args.workload.startswith("euler") or args.workload.startswith("blast"):
            n = EULER_CPU_SAMPLE_N if args.workload != "euler64" else 48
            r, cores, kind, d = cpu_euler_rate(n, 2, use_ref=False)
            out["cpu_baseline"] = {"value": r, "unit": "cell-updates/s", "cores": cores, "kind": kind,
                                   "sample": f"2 SSPRK(4,3) steps of a {n}^3 periodic pulse grid ({d:.1f} s wall), "
                                             "the same sample as the reference arm"}
            ref = _reference_program_figures()
            if ref:
                out["cpu_baseline"]["reference_program"] = ref
        else:
            r, cores, kind, d = cpu_ctcs_rate(512, 300)
            out["cpu_baseline"] = {"value": r, "unit": "cell-updates/s", "cores": cores, "kind": kind,
                                   "sample": f"300 steps of the 512^2 CTCS run ({d:.1f} s wall)"}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
