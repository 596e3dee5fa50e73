"""Host-side mirror of the reference's operator interface for the hot path.

The reference registers ``RHSFunction(TS ts, PetscReal t, Vec U, Vec RHS, void *ctx)``
with ``TSSetRHSFunction`` (3d/weno4/Navier-Stokes-3D/hype.c:176) and advances with
TSSSP RKS3/4 stages; its acoustic codes call ``CTCS(da, Pold, Pcurr, Pnew, &user)``
(2d/ctcs/plane_wave/wave.c:161) and ``UpdatePressure(...)``
(3d/ctcs/point_source/wave.c:138).  The classes here keep those names, argument
meanings and the error behaviour of the C ABI (an inadmissible state raises
``HypeError`` with code HYPE_ERR_STATE where the reference would MPI_Abort).
Arrays use the DMDA layout: AoS ``[k][j][i][c]`` for HyPE states, ``[j][i]`` or
``[k][j][i]`` for CTCS levels.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from ._lib import check

_D = C.POINTER(C.c_double)


def _dp(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise ValueError("arrays must be C-contiguous float64")
    return a.ctypes.data_as(_D)


def write_petsc_vec(path, v, block_size=1):
    """PETSc binary Vec record of v (what VecView on a binary viewer writes)"""
    v = np.ascontiguousarray(v, dtype=np.float64).ravel()
    check(L.lib().hype_write_petsc_vec(os.fsencode(path), _dp(v), v.size, int(block_size)), "hype_write_petsc_vec")


def read_petsc_vec(path, n):
    """n values of a PETSc binary Vec record (what VecLoad reads)"""
    v = np.empty(int(n))
    check(L.lib().hype_read_petsc_vec(os.fsencode(path), _dp(v), v.size), "hype_read_petsc_vec")
    return v


def write_vtk(path, aos, h, origin=(0.0, 0.0, 0.0), names=None, title="HyPE solution"):
    """legacy VTK 2.0 ASCII file of a cell-centred [k][j][i][c] (or [j][i][c]) array"""
    aos = np.ascontiguousarray(aos, dtype=np.float64)
    shp = aos.shape[:-1]
    nz, ny, nx = (1,) + shp if len(shp) == 2 else shp
    nc = aos.shape[-1]
    names = names or [f"c{q}" for q in range(nc)]
    arr = (C.c_char_p * nc)(*[n.encode() for n in names])
    check(L.lib().hype_write_vtk(os.fsencode(path), title.encode(), nx, ny, nz, origin[0], origin[1], origin[2], h, nc, arr,
                                 _dp(aos)), "hype_write_vtk")


@dataclass
class AppCtx:
    """The fields of the reference's AppCtx (3d/weno4/Navier-Stokes-3D/hype.h:245-276)
    that the RHS reads, plus the GPU-side options."""
    N_x: int
    N_y: int
    N_z: int
    h: float
    x_min: float = 0.0
    y_min: float = 0.0
    z_min: float = 0.0
    CFL: float = 0.4
    gamma: float = 1.4
    boundaries: tuple = (L.BC_PERIODIC,) * 6  # left,right,bottom,top,back,front
    recon: int = L.RECON_CWENO4
    # PREC_FP64 (the reference's arithmetic), PREC_FP32 (reconstruction and flux in FP32), or
    # PREC_DF64 (reconstruction and Rusanov / viscous fluxes in FP32 pairs on deviations from a
    # reference state, state and stages in FP64: the FP64 form's error bars at about 4x its speed)
    precision: int = L.PREC_FP64
    dt_mode: int = L.DT_MONITOR
    flux: int = L.FLUX_RUSANOV
    positivity: int = 0  # 1: first-order fallback on inadmissible face traces
    # Navier-Stokes constants (3d/weno4/Navier-Stokes-3D/hype.h:38-41: C_V 2.5, PR 1.0, MU_0 0.01);
    # mu = 0 is the Euler system
    mu: float = 0.0
    prandtl: float = 1.0
    cv: float = 2.5
    dt: float = 0.0  # the reference's Ctx->dt output of RHSFunction

    def params(self) -> L.EulerParams:
        p = L.EulerParams()
        p.nx, p.ny, p.nz = self.N_x, self.N_y, self.N_z
        p.x_min, p.y_min, p.z_min, p.h = self.x_min, self.y_min, self.z_min, self.h
        p.cfl, p.gamma = self.CFL, self.gamma
        for q in range(6):
            p.bc[q] = int(self.boundaries[q])
        p.recon, p.precision, p.dt_mode, p.flux = self.recon, self.precision, self.dt_mode, self.flux
        p.positivity = self.positivity
        p.mu, p.prandtl, p.cv = self.mu, self.prandtl, self.cv
        return p


class EulerSolver:
    """3D Euler CWENO4 + Rusanov RHS and SSPRK(4,3) stepper on one GPU."""

    def __init__(self, ctx: AppCtx):
        self.ctx = ctx
        self._h = C.c_void_p()
        check(L.lib().hype_euler_create(C.byref(ctx.params()), C.byref(self._h)), "hype_euler_create")
        self.shape = (ctx.N_z, ctx.N_y, ctx.N_x, 5)
        self.t = 0.0
        self.next_dt = 0.0

    def close(self):
        if self._h:
            L.lib().hype_euler_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def RHSFunction(self, t: float, U: np.ndarray, RHS: np.ndarray | None = None) -> np.ndarray:
        """Drop-in for RHSFunction(ts, t, U, RHS, &Ctx): fills RHS and sets ctx.dt."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.shape != self.shape:
            raise ValueError(f"U must have shape {self.shape}")
        if RHS is None:
            RHS = np.empty_like(U)
        dt = C.c_double(0.0)
        rc = L.lib().hype_euler_rhs(self._h, t, _dp(U), _dp(RHS), C.byref(dt))
        self.ctx.dt = dt.value
        check(rc, "RHSFunction")
        return RHS

    def set_state(self, U: np.ndarray) -> None:
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.shape != self.shape:
            raise ValueError(f"U must have shape {self.shape}")
        check(L.lib().hype_euler_upload(self._h, _dp(U)), "hype_euler_upload")

    def get_state(self) -> np.ndarray:
        U = np.empty(self.shape)
        check(L.lib().hype_euler_download(self._h, _dp(U)), "hype_euler_download")
        return U


    def write_restart(self, path):
        """the resident state as a PETSc binary Vec (restart1.bin of the reference's monitor)"""
        check(L.lib().hype_euler_write_restart(self._h, os.fsencode(path)), "hype_euler_write_restart")

    def read_restart(self, path):
        check(L.lib().hype_euler_read_restart(self._h, os.fsencode(path)), "hype_euler_read_restart")

    def write_vtk(self, path):
        check(L.lib().hype_euler_write_vtk(self._h, os.fsencode(path)), "hype_euler_write_vtk")
    def step(self, nsteps: int, dt: float | None = None) -> L.Status:
        """nsteps of SSPRK(4,3) on the resident state (TSSolve with TSSSP RKS3, 4 stages)."""
        t = C.c_double(self.t)
        d = C.c_double(self.next_dt if dt is None else dt)
        st = L.Status()
        rc = L.lib().hype_euler_step(self._h, int(nsteps), C.byref(t), C.byref(d), C.byref(st))
        self.t, self.next_dt = t.value, d.value
        check(rc, "hype_euler_step")
        return st

    def device_state_ptr(self) -> int:
        return int(L.lib().hype_euler_state_device(self._h))

    def monitor(self) -> tuple[float, float]:
        """(KineticEnergy, Dissipation) of the resident state: the two numbers the
        reference's MonitorFunction writes to ke.csv every 10 steps
        (3d/weno4/Navier-Stokes-3D/monitor_function.c:77-85)."""
        ke, dr = C.c_double(), C.c_double()
        check(L.lib().hype_euler_monitor(self._h, C.byref(ke), C.byref(dr)), "hype_euler_monitor")
        return ke.value, dr.value

    # ---- learned troubled-cell indicator (no counterpart in the reference) ----
    def set_mlp(self, params: np.ndarray, prob_threshold: float = 0.2) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        check(L.lib().hype_euler_set_mlp(self._h, p.ctypes.data_as(L.F), float(prob_threshold)), "hype_euler_set_mlp")

    def set_recon(self, recon: int) -> None:
        check(L.lib().hype_euler_set_recon(self._h, int(recon)), "hype_euler_set_recon")
        self.ctx.recon = recon

    def set_stage_kernel(self, mode: int) -> None:
        """L.STAGE_AUTO: the fused FP32 stage where it applies; L.STAGE_UNFUSED: separate kernels"""
        check(L.lib().hype_euler_set_stage_kernel(self._h, int(mode)), "hype_euler_set_stage_kernel")

    def set_gate_per_step(self, per_step: bool) -> None:
        """fused FP32 stage: score the gate once per step (flags widened by a cell, read by the
        step's four stages) instead of on every stage's input"""
        check(L.lib().hype_euler_set_gate_per_step(self._h, int(bool(per_step))), "hype_euler_set_gate_per_step")

    def gate_flags(self, widened: bool = False) -> np.ndarray:
        """the fused FP32 stage's gate flags of the last scoring, shape (nz+2, ny+2, nx+2), frame included"""
        c = self.ctx
        out = np.zeros((c.N_z + 2, c.N_y + 2, c.N_x + 2), dtype=np.uint8)
        check(L.lib().hype_euler_gate_flags(self._h, out.ctypes.data_as(C.c_void_p), int(bool(widened))),
              "hype_euler_gate_flags")
        return out

    def indicator_stats(self, reset: bool = True):
        f, b = C.c_longlong(), C.c_longlong()
        check(L.lib().hype_euler_indicator_stats(self._h, C.byref(f), C.byref(b), int(reset)), "indicator_stats")
        return f.value, b.value

    def shadow_step(self) -> float:
        """One step with the current reconstruction (the learned indicator) and, from the
        same state, one full-CWENO4 step (the shadow); the learned result is kept.
        Returns the relative L1 difference of the densities of the two."""
        t = C.c_double(self.t)
        d = C.c_double(self.next_dt)
        l1 = C.c_double()
        check(L.lib().hype_euler_shadow_step(self._h, C.byref(t), C.byref(d), C.byref(l1)), "hype_euler_shadow_step")
        self.t, self.next_dt = t.value, d.value
        return l1.value

    def sync(self):
        check(L.lib().hype_euler_sync(self._h), "hype_euler_sync")


def CTCS(p_old: np.ndarray, p: np.ndarray, alpha: float, bc: int = L.BC_PERIODIC) -> np.ndarray:
    """One leapfrog update of 2d/ctcs/plane_wave/wave.c:161-203 on host arrays; returns p_new."""
    p_old = np.ascontiguousarray(p_old, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    ny, nx = p.shape
    out = np.empty_like(p)
    check(L.lib().hype_ctcs2d_update(nx, ny, float(alpha), int(bc), _dp(p_old), _dp(p), _dp(out)), "CTCS")
    return out


class Leapfrog:
    """Resident CTCS solver (plane-wave form or point-source form, 2D/3D)."""

    def __init__(self, shape, dx, dt, c0=1.0, form=0, order=2, bc=L.BC_ZERO, f0=0.0, src=None, rec=None,
                 dy=None, dz=None):
        p = L.CtcsParams()
        p.dim = len(shape)
        if p.dim == 2:
            p.ny, p.nx = shape
            p.nz = 1
        else:
            p.nz, p.ny, p.nx = shape
        p.form, p.order, p.bc = form, order, bc
        p.dx = dx
        p.dy = dy if dy is not None else dx
        p.dz = dz if dz is not None else dx
        p.dt, p.c0, p.f0 = dt, c0, f0
        for q in range(3):
            p.src[q] = src[q] if src is not None and q < len(src) else (-1 if src is None else 0)
            p.rec[q] = rec[q] if rec is not None and q < len(rec) else (-1 if rec is None else 0)
        self.shape = tuple(shape)
        self.has_rec = rec is not None
        self._h = C.c_void_p()
        check(L.lib().hype_ctcs_create(C.byref(p), C.byref(self._h)), "hype_ctcs_create")
        self.it = 0

    def close(self):
        if self._h:
            L.lib().hype_ctcs_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set(self, p_old, p):
        a = np.ascontiguousarray(p_old, dtype=np.float64)
        b = np.ascontiguousarray(p, dtype=np.float64)
        check(L.lib().hype_ctcs_set(self._h, _dp(a), _dp(b)), "hype_ctcs_set")

    def get(self):
        a = np.empty(self.shape)
        b = np.empty(self.shape)
        check(L.lib().hype_ctcs_get(self._h, _dp(a), _dp(b)), "hype_ctcs_get")
        return a, b

    def UpdatePressure(self, nsteps: int = 1):
        """nsteps updates; returns the receiver samples (p before each update) when a receiver is set."""
        rec = np.zeros(nsteps) if self.has_rec else None
        check(L.lib().hype_ctcs_step(self._h, int(nsteps), self.it, _dp(rec) if rec is not None else None),
              "hype_ctcs_step")
        self.it += nsteps
        return rec

    def sync(self):
        check(L.lib().hype_ctcs_sync(self._h), "hype_ctcs_sync")


@dataclass
class Monopole:
    nx: int
    ny: int
    xmin: float
    ymin: float
    h: float
    c0: float
    dt: float
    xs: float
    ys: float
    sigma: float
    freq: float


class BatchLeapfrog:
    """Many independent 2D monopole-forced CTCS instances in one persistent launch per step."""

    def __init__(self, instances: list[Monopole], tile=(0, 0)):
        arr = (L.MonoInstance * len(instances))()
        for q, m in enumerate(instances):
            for f, _ in L.MonoInstance._fields_:
                setattr(arr[q], f, getattr(m, f))
        self.instances = list(instances)
        self._h = C.c_void_p()
        check(L.lib().hype_batch_create(len(instances), arr, C.byref(self._h)), "hype_batch_create")
        self.set_tile(*tile)

    def set_tile(self, tx=0, ty=0):
        check(L.lib().hype_batch_set_tile(self._h, int(tx), int(ty)), "hype_batch_set_tile")

    def tile(self):
        """the tile shape in use (width, height in nodes)"""
        tx, ty = C.c_int(), C.c_int()
        check(L.lib().hype_batch_get_tile(self._h, C.byref(tx), C.byref(ty)), "hype_batch_get_tile")
        return tx.value, ty.value

    def close(self):
        if self._h:
            L.lib().hype_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set(self, q, p_old, p):
        a = np.ascontiguousarray(p_old, dtype=np.float64)
        b = np.ascontiguousarray(p, dtype=np.float64)
        check(L.lib().hype_batch_set(self._h, int(q), _dp(a), _dp(b)), "hype_batch_set")

    def get(self, q):
        m = self.instances[q]
        a = np.empty((m.ny, m.nx))
        b = np.empty((m.ny, m.nx))
        check(L.lib().hype_batch_get(self._h, int(q), _dp(a), _dp(b)), "hype_batch_get")
        return a, b

    def step(self, nsteps: int, graph: bool = True):
        check(L.lib().hype_batch_step(self._h, int(nsteps), int(bool(graph))), "hype_batch_step")

    def set_classes(self, nclasses: int = 0):
        """size classes on prioritised streams (0: one per device priority level; 1: none)"""
        check(L.lib().hype_batch_set_classes(self._h, int(nclasses)), "hype_batch_set_classes")

    def classes(self):
        """(number of classes, each instance's class)"""
        n = C.c_int()
        cls = (C.c_int * len(self.instances))()
        check(L.lib().hype_batch_get_classes(self._h, C.byref(n), cls), "hype_batch_get_classes")
        return n.value, np.array(cls[:], dtype=np.int64)

    def instance_times(self):
        """seconds from the start of the last step() call to each instance's completion (device events)"""
        t = np.empty(len(self.instances))
        check(L.lib().hype_batch_instance_times(self._h, _dp(t)), "hype_batch_instance_times")
        return t

    def sync(self):
        check(L.lib().hype_batch_sync(self._h), "hype_batch_sync")


class Multiphase2D:
    """2D multiphase RHS + SSP stepper: the 4-equation diffuse-interface model of
    2d/weno4/bubble (model=MP_DI4) or the Kapila five-equation model (MP_KAPILA5)."""

    def __init__(self, nx, ny, h, x_min=0.0, y_min=0.0, CFL=0.9, boundaries=(L.BC_TRANSMISSIVE,) * 4,
                 model=L.MP_DI4, eos=(4.4, 6000.0, 1.4, 0.0), stepper=L.STEP_SSPRK43, precision=L.PREC_FP64,
                 dt_mode=L.DT_MONITOR, recon=L.RECON_CWENO4):
        p = L.Mp2dParams()
        p.nx, p.ny, p.x_min, p.y_min, p.h, p.cfl = nx, ny, x_min, y_min, h, CFL
        for q in range(4):
            p.bc[q] = int(boundaries[q])
        p.model = model
        p.g1, p.p1, p.g2, p.p2 = eos
        p.stepper, p.precision, p.dt_mode, p.recon = stepper, precision, dt_mode, recon
        self.nx, self.ny = nx, ny
        self.nv = 5 if model == L.MP_DI4 else 6
        self.shape = (ny, nx, self.nv)
        self.dt = 0.0
        self.t = 0.0
        self.next_dt = 0.0
        self.fallback_cells = 0
        self._h = C.c_void_p()
        check(L.lib().hype_mp2d_create(C.byref(p), C.byref(self._h)), "hype_mp2d_create")

    def close(self):
        if self._h:
            L.lib().hype_mp2d_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def RHSFunction(self, t, U, RHS=None):
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.shape != self.shape:
            raise ValueError(f"U must have shape {self.shape}")
        if RHS is None:
            RHS = np.empty_like(U)
        dt = C.c_double()
        rc = L.lib().hype_mp2d_rhs(self._h, t, _dp(U), _dp(RHS), C.byref(dt))
        self.dt = dt.value
        check(rc, "RHSFunction")
        return RHS

    def set_state(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        check(L.lib().hype_mp2d_upload(self._h, _dp(U)), "hype_mp2d_upload")

    def get_state(self):
        U = np.empty(self.shape)
        check(L.lib().hype_mp2d_download(self._h, _dp(U)), "hype_mp2d_download")
        return U


    def write_restart(self, path):
        """the resident state as a PETSc binary Vec"""
        check(L.lib().hype_mp2d_write_restart(self._h, os.fsencode(path)), "hype_mp2d_write_restart")

    def read_restart(self, path):
        check(L.lib().hype_mp2d_read_restart(self._h, os.fsencode(path)), "hype_mp2d_read_restart")

    def write_vtk(self, path):
        check(L.lib().hype_mp2d_write_vtk(self._h, os.fsencode(path)), "hype_mp2d_write_vtk")
    def step(self, nsteps, dt=None):
        t = C.c_double(self.t)
        d = C.c_double(self.next_dt if dt is None else dt)
        fb = C.c_longlong(0)
        rc = L.lib().hype_mp2d_step(self._h, int(nsteps), C.byref(t), C.byref(d), C.byref(fb))
        self.t, self.next_dt, self.fallback_cells = t.value, d.value, fb.value
        check(rc, "hype_mp2d_step")

    def sync(self):
        check(L.lib().hype_mp2d_sync(self._h), "hype_mp2d_sync")

    # learned troubled-cell indicator (no counterpart in the reference)
    def set_mlp(self, params, prob_threshold=0.5):
        params = np.ascontiguousarray(params, dtype=np.float32)
        check(L.lib().hype_mp2d_set_mlp(self._h, params.ctypes.data_as(L.F), float(prob_threshold)), "hype_mp2d_set_mlp")

    def set_recon(self, recon):
        check(L.lib().hype_mp2d_set_recon(self._h, int(recon)), "hype_mp2d_set_recon")

    def set_gate_per_step(self, per_step):
        """score the gate once per step (flags widened by a cell, read by the step's stages)"""
        check(L.lib().hype_mp2d_set_gate_per_step(self._h, int(bool(per_step))), "hype_mp2d_set_gate_per_step")

    def gate_flags(self, widened=False):
        """the per-step gate's last flags, shape (ny+2, nx+2), frame included"""
        out = np.zeros((self.ny + 2, self.nx + 2), dtype=np.uint8)
        check(L.lib().hype_mp2d_gate_flags(self._h, out.ctypes.data_as(C.c_void_p), int(bool(widened))),
              "hype_mp2d_gate_flags")
        return out

    def indicator_stats(self, reset=False):
        """owned-cell reconstructions flagged by the network since the last reset"""
        f = C.c_longlong()
        check(L.lib().hype_mp2d_indicator_stats(self._h, C.byref(f), int(reset)), "hype_mp2d_indicator_stats")
        return f.value

    def sample_features(self, stride=1):
        """(X[n][3][25], D[n]) of every stride-th owned cell of the resident state"""
        n = (self.nx * self.ny + stride - 1) // stride
        X = np.empty((n, 3, 25), dtype=np.float32)
        Dv = np.empty(n, dtype=np.float32)
        ns = C.c_longlong()
        check(L.lib().hype_mp2d_sample_features(self._h, int(stride), X.ctypes.data_as(L.F), Dv.ctypes.data_as(L.F),
                                                C.byref(ns)), "hype_mp2d_sample_features")
        return X, Dv


def _trace(fn, handle, capacity):
    """the stored receiver samples (the first ``capacity`` RHS evaluations) and the count"""
    count = C.c_longlong(0)
    check(fn(handle, None, None, 0, C.byref(count)), "receiver_trace")
    m = min(int(count.value), int(capacity))
    t = np.empty(m)
    u = np.empty(m)
    check(fn(handle, _dp(t), _dp(u), m, C.byref(count)), "receiver_trace")
    return t, u, int(count.value)


class AcousticFV3D:
    """The acoustic finite-volume path of 3d/weno4/plane_wave: u_tt = c^2 lap u as
    (u, v = u_t) with CWENO4 (default: its R4 limit, as the reference runs it)
    face-normal gradients, a central flux and SSPRK(4,3) with a fixed dt."""

    def __init__(self, N_x, N_y, N_z, h, dt, c=1.0, x_min=0.0, y_min=0.0, z_min=0.0,
                 boundaries=(L.BC_PERIODIC,) * 6, recon=L.RECON_LINEAR4, precision=L.PREC_FP64):
        p = L.AcousticParams()
        p.precision = precision
        p.nx, p.ny, p.nz = N_x, N_y, N_z
        p.x_min, p.y_min, p.z_min, p.h, p.c, p.dt = x_min, y_min, z_min, h, c, dt
        for q in range(6):
            p.bc[q] = int(boundaries[q])
        p.recon = recon
        self.shape = (N_z, N_y, N_x, 2)
        self.t = 0.0
        self._h = C.c_void_p()
        check(L.lib().hype_acoustic_create(C.byref(p), C.byref(self._h)), "hype_acoustic_create")
        self._trace_capacity = 0

    def close(self):
        if self._h:
            L.lib().hype_acoustic_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def RHSFunction(self, t, U, RHS=None):
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.shape != self.shape:
            raise ValueError(f"U must have shape {self.shape}")
        if RHS is None:
            RHS = np.empty_like(U)
        check(L.lib().hype_acoustic_rhs_t(self._h, float(t), _dp(U), _dp(RHS)), "RHSFunction")
        return RHS

    def set_point_source(self, source=None, f0=100.0, receiver=None, capacity=0):
        """the point source and receiver of 3d/weno4/point_source (hype.c:59-64): every RHS
        evaluation at time t adds Source(t)/h^3 (source.c:11-17, f0 the wavelet's dominant
        frequency) to the u_t equation of cell ``source`` = (isx, isy, isz) and records u of
        cell ``receiver`` = (irx, iry, irz) in a trace of up to ``capacity`` samples
        (rhs_function.c:337-346).  None turns either off."""
        sx, sy, sz = source if source is not None else (-1, 0, 0)
        rx, ry, rz = receiver if receiver is not None else (-1, 0, 0)
        check(L.lib().hype_acoustic_set_point_source(self._h, int(sx), int(sy), int(sz), float(f0), int(rx), int(ry),
                                                     int(rz), int(capacity)), "set_point_source")
        self._trace_capacity = int(capacity) if receiver is not None else 0

    def receiver_trace(self):
        """(t, u) of every recorded RHS evaluation (the columns of results/p.dat) and the
        number of evaluations seen"""
        return _trace(L.lib().hype_acoustic_trace, self._h, self._trace_capacity)

    def set_state(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        check(L.lib().hype_acoustic_upload(self._h, _dp(U)), "hype_acoustic_upload")

    def get_state(self):
        U = np.empty(self.shape)
        check(L.lib().hype_acoustic_download(self._h, _dp(U)), "hype_acoustic_download")
        return U

    def step(self, nsteps, t_final=0.0):
        """up to nsteps steps; t_final > 0 ends the run exactly on t_final
        (TS_EXACTFINALTIME_MATCHSTEP). Returns the steps taken."""
        t = C.c_double(self.t)
        n = C.c_int(0)
        check(L.lib().hype_acoustic_step(self._h, int(nsteps), float(t_final), C.byref(t), C.byref(n)),
              "hype_acoustic_step")
        self.t = t.value
        return n.value



class AcousticFV2D:
    """The 2D acoustic finite-volume program of 2d/weno4/standing_wave: (u, v = u_t) with
    the 2D R4 polynomial's edge-normal gradients, the averaged flux and SSP RK104 (the
    program's) or RKS3/4 stages with a fixed dt; bit-identical to the reference."""

    def __init__(self, N_x, N_y, h, dt, c=1.0, x_min=0.0, y_min=0.0, boundaries=(L.BC_ADIABATIC,) * 4,
                 stepper=L.STEP_SSPRK104):
        p = L.Acoustic2dParams()
        p.nx, p.ny, p.x_min, p.y_min, p.h, p.c, p.dt = N_x, N_y, x_min, y_min, h, c, dt
        for q in range(4):
            p.bc[q] = int(boundaries[q])
        p.stepper = stepper
        self.shape = (N_y, N_x, 2)
        self.t = 0.0
        self._h = C.c_void_p()
        check(L.lib().hype_acoustic2d_create(C.byref(p), C.byref(self._h)), "hype_acoustic2d_create")
        self._trace_capacity = 0

    def close(self):
        if self._h:
            L.lib().hype_acoustic2d_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def RHSFunction(self, t, U, RHS=None):
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.shape != self.shape:
            raise ValueError(f"U must have shape {self.shape}")
        if RHS is None:
            RHS = np.empty_like(U)
        check(L.lib().hype_acoustic2d_rhs_t(self._h, float(t), _dp(U), _dp(RHS)), "RHSFunction")
        return RHS

    def set_point_source(self, source=None, f0=65.0, receiver=None, capacity=0):
        """the line source and receiver of 2d/weno4/line_source (hype.c:52-55): Source(t)/h^2
        (source.c:12-18) added to the u_t equation of cell ``source`` = (isx, isy) at every RHS
        evaluation, u of cell ``receiver`` = (irx, iry) recorded (rhs_function.c:244-253)"""
        sx, sy = source if source is not None else (-1, 0)
        rx, ry = receiver if receiver is not None else (-1, 0)
        check(L.lib().hype_acoustic2d_set_point_source(self._h, int(sx), int(sy), float(f0), int(rx), int(ry),
                                                       int(capacity)), "set_point_source")
        self._trace_capacity = int(capacity) if receiver is not None else 0

    def receiver_trace(self):
        """(t, u) of every recorded RHS evaluation and the number of evaluations seen"""
        return _trace(L.lib().hype_acoustic2d_trace, self._h, self._trace_capacity)

    def set_state(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.shape != self.shape:
            raise ValueError(f"U must have shape {self.shape}")
        check(L.lib().hype_acoustic2d_upload(self._h, _dp(U)), "hype_acoustic2d_upload")

    def get_state(self):
        U = np.empty(self.shape)
        check(L.lib().hype_acoustic2d_download(self._h, _dp(U)), "hype_acoustic2d_download")
        return U

    def step(self, nsteps, t_final=0.0):
        """up to nsteps steps; t_final > 0 ends the run exactly on t_final
        (TS_EXACTFINALTIME_MATCHSTEP). Returns the steps taken."""
        t = C.c_double(self.t)
        n = C.c_int(0)
        check(L.lib().hype_acoustic2d_step(self._h, int(nsteps), float(t_final), C.byref(t), C.byref(n)),
              "hype_acoustic2d_step")
        self.t = t.value
        return n.value


class Multiphase3D:
    """The 3D primitive-variable multiphase RHS of 3d/weno4/Viscous-Multiphase-Fourth-Order
    (RHSFunctionPrimitive) and SSP RKS3/4 stages on one GPU: (rho, rho u, rho v, rho w, E, phi)
    with two stiffened gases mixed by phi, primitive CWENO4 with the 33-node admissibility
    fallback, rotated HLLC and the non-conservative phi equation.  The defaults are the
    program's compiled-in constants (hype.h:37-42): EOS (1.4, 0, 1.6, 0), viscosities 1.4 / 1.6
    in the dt limit."""

    def __init__(self, N_x, N_y, N_z, h, CFL=0.9, x_min=0.0, y_min=0.0, z_min=0.0,
                 boundaries=(L.BC_TRANSMISSIVE,) * 6, eos=(1.4, 0.0, 1.6, 0.0), mu=(1.4, 1.6), dt_mode=L.DT_MONITOR):
        p = L.Mp3dParams()
        p.nx, p.ny, p.nz, p.x_min, p.y_min, p.z_min, p.h, p.cfl = N_x, N_y, N_z, x_min, y_min, z_min, h, CFL
        for q in range(6):
            p.bc[q] = int(boundaries[q])
        p.g1, p.p1, p.g2, p.p2 = eos
        p.mu1, p.mu2 = mu
        p.dt_mode = dt_mode
        self.shape = (N_z, N_y, N_x, 6)
        self.t = 0.0
        self.next_dt = 0.0
        self.dt = 0.0
        self.fallback_cells = 0
        self._h = C.c_void_p()
        check(L.lib().hype_mp3d_create(C.byref(p), C.byref(self._h)), "hype_mp3d_create")

    def close(self):
        if self._h:
            L.lib().hype_mp3d_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def RHSFunctionPrimitive(self, t, U, RHS=None):
        """drop-in for RHSFunctionPrimitive(ts, t, U, RHS, &Ctx): fills RHS and sets self.dt"""
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.shape != self.shape:
            raise ValueError(f"U must have shape {self.shape}")
        if RHS is None:
            RHS = np.empty_like(U)
        dt = C.c_double(0.0)
        rc = L.lib().hype_mp3d_rhs(self._h, float(t), _dp(U), _dp(RHS), C.byref(dt))
        self.dt = dt.value
        check(rc, "RHSFunctionPrimitive")
        return RHS

    def set_state(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.shape != self.shape:
            raise ValueError(f"U must have shape {self.shape}")
        check(L.lib().hype_mp3d_upload(self._h, _dp(U)), "hype_mp3d_upload")

    def get_state(self):
        U = np.empty(self.shape)
        check(L.lib().hype_mp3d_download(self._h, _dp(U)), "hype_mp3d_download")
        return U

    def step(self, nsteps, dt=None):
        t = C.c_double(self.t)
        d = C.c_double(self.next_dt if dt is None else dt)
        fb = C.c_longlong(0)
        rc = L.lib().hype_mp3d_step(self._h, int(nsteps), C.byref(t), C.byref(d), C.byref(fb))
        self.t, self.next_dt, self.fallback_cells = t.value, d.value, fb.value
        check(rc, "hype_mp3d_step")


class PathConservative2D:
    """The path-conservative 2D scheme of 2d/HyPE-2D (RHSFunction) with its Kapila
    five-equation model on one GPU: Q = (a1 rho1, a2 rho2, rho u, rho v, E, a1), conservative
    reconstruction of order N = 0..3, node admissibility with first-order fallback, Rusanov
    flux + Roe-path fluctuation, the non-conservative volume term and the program's stepper
    for N; bit-identical to the reference.  The default EOS is the program's compiled-in one
    (hype.h:41-44: both phases gamma 1.4, pi 0)."""

    def __init__(self, N_x, N_y, h, order=1, CFL=0.9, x_min=0.0, y_min=0.0, boundaries=(L.BC_TRANSMISSIVE,) * 4,
                 eos=(1.4, 0.0, 1.4, 0.0)):
        p = L.Pc2dParams()
        p.nx, p.ny, p.x_min, p.y_min, p.h, p.cfl = N_x, N_y, x_min, y_min, h, CFL
        for q in range(4):
            p.bc[q] = int(boundaries[q])
        p.order = order
        p.g1, p.p1, p.g2, p.p2 = eos
        self.shape = (N_y, N_x, 6)
        self.t = 0.0
        self.next_dt = 0.0
        self.dt = 0.0
        self.fallback_cells = 0
        self._h = C.c_void_p()
        check(L.lib().hype_pc2d_create(C.byref(p), C.byref(self._h)), "hype_pc2d_create")

    def close(self):
        if self._h:
            L.lib().hype_pc2d_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def RHSFunction(self, t, U, RHS=None):
        """drop-in for RHSFunction(ts, t, U, RHS, &Ctx): fills RHS and sets self.dt"""
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.shape != self.shape:
            raise ValueError(f"U must have shape {self.shape}")
        if RHS is None:
            RHS = np.empty_like(U)
        dt = C.c_double(0.0)
        rc = L.lib().hype_pc2d_rhs(self._h, float(t), _dp(U), _dp(RHS), C.byref(dt))
        self.dt = dt.value
        check(rc, "RHSFunction")
        return RHS

    def set_state(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.shape != self.shape:
            raise ValueError(f"U must have shape {self.shape}")
        check(L.lib().hype_pc2d_upload(self._h, _dp(U)), "hype_pc2d_upload")

    def get_state(self):
        U = np.empty(self.shape)
        check(L.lib().hype_pc2d_download(self._h, _dp(U)), "hype_pc2d_download")
        return U

    def step(self, nsteps, dt=None):
        t = C.c_double(self.t)
        d = C.c_double(self.next_dt if dt is None else dt)
        fb = C.c_longlong(0)
        rc = L.lib().hype_pc2d_step(self._h, int(nsteps), C.byref(t), C.byref(d), C.byref(fb))
        self.t, self.next_dt, self.fallback_cells = t.value, d.value, fb.value
        check(rc, "hype_pc2d_step")

