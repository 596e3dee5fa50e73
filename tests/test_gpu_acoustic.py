"""Acoustic finite-volume path (3d/weno4/plane_wave) on the GPU: the reference's RHS
and steps (golden fixtures), the CPU checker, and the published convergence table."""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _solver(hype, shape, h, dt, bc=(0,) * 6):
    nx, ny, nz = shape
    return hype.AcousticFV3D(nx, ny, nz, h, dt, boundaries=bc)


@pytest.mark.parametrize("name", ["periodic", "adiabatic", "mixed"])
def test_rhs_and_steps_vs_reference(hype, name):
    z = np.load(os.path.join(GOLDEN, f"ref_acoustic_{name}.npz"))
    s = _solver(hype, tuple(int(v) for v in z["shape"]), float(z["h"]), float(z["dt"]), tuple(int(b) for b in z["bc"]))
    assert rel(s.RHSFunction(0.0, z["U"]), z["RHS"]) <= 1e-12
    s.set_state(z["U"])
    assert s.step(3) == 3
    assert rel(s.get_state(), z["U3"]) <= 1e-12
    assert abs(s.t - float(z["t3"])) <= 1e-15


def test_run_vs_oracle_with_matched_final_step(hype, oracle):
    n, h = 12, 2 * math.pi / 12
    cfg = oracle.acoustic_cfg(n, h, bc=(4, 4, 0, 0, 4, 4))
    U0 = oracle.plane_wave_ic(cfg)
    dt = h * 0.5 / 3.0
    s = _solver(hype, (n, n, n), h, dt, (4, 4, 0, 0, 4, 4))
    s.set_state(U0)
    taken = s.step(10**6, t_final=0.7)
    U, t, steps = oracle.acoustic_run(cfg, U0, 10**6, dt, t_final=0.7)
    assert taken == steps and s.t == t == 0.7
    assert rel(s.get_state(), U) <= 1e-10


def test_published_convergence_table(hype, oracle):
    """3d/weno4/plane_wave/results/main.tex:39-42 at final time 1.0, N = 16, 32, 64 (the
    GPU run, the oracle's projection and error norms), within 0.2 % of every entry"""
    with open(os.path.join(GOLDEN, "accuracy_tables.json")) as f:
        table = {int(r[0]): (r[1], r[2]) for r in json.load(f)["plane_wave_3d_main_tex"]}
    for n in (16, 32, 64):
        h = 2 * math.pi / n
        cfg = oracle.acoustic_cfg(n, h)
        s = _solver(hype, (n, n, n), h, h * 0.5 / 3.0)
        s.set_state(oracle.plane_wave_ic(cfg))
        s.step(10**6, t_final=1.0)
        l2, linf = oracle.plane_wave_errors(cfg, s.get_state(), s.t)
        print(f"plane wave N={n}: L2 {l2:.4e} (table {table[n][0]:.2e}), Linf {linf:.4e} (table {table[n][1]:.2e})")
        assert abs(l2 - table[n][0]) <= 2e-3 * table[n][0] and abs(linf - table[n][1]) <= 2e-3 * table[n][1]


# ---------------------------------------------------------------- 3d/weno4/point_source
@pytest.mark.parametrize("name", ["periodic", "mixed"])
def test_point_source_vs_reference(hype, oracle, name):
    """the RHS with Source(t)/h^3 at the source cell, and the program's run from rest (its
    RHSFunction call at t = 0, hype.c:160, then TSSolve): state against the reference's,
    receiver trace against its p.dat lines and, sample by sample, the CPU checker's"""
    z = np.load(os.path.join(GOLDEN, f"ref_psrc3d_{name}.npz"))
    n, h, dt, f0 = int(z["n"]), float(z["h"]), float(z["dt"]), float(z["f0"])
    src, rec = tuple(int(v) for v in z["src"]), tuple(int(v) for v in z["rec"])
    bc = tuple(int(b) for b in z["bc"])
    s = hype.AcousticFV3D(n, n, n, h, dt, c=float(z["c"]), boundaries=bc)
    s.set_point_source(src, f0, rec, capacity=1000)
    assert rel(s.RHSFunction(float(z["t_rhs"]), z["U"]), z["RHS"]) <= 1e-12
    t, u, cnt = s.receiver_trace()
    assert cnt == 1 and t[0] == float(z["t_rhs"]) and u[0] == z["U"][rec[2], rec[1], rec[0], 0]
    s.set_point_source(src, f0, rec, capacity=1000)
    U0 = np.zeros_like(z["U"])
    s.RHSFunction(0.0, U0)
    s.set_state(U0)
    assert s.step(int(z["steps"])) == int(z["steps"])
    assert rel(s.get_state(), z["Un"]) <= 1e-12 and s.t == float(z["tn"])
    t, u, cnt = s.receiver_trace()
    pdat = z["pdat"]
    assert cnt == len(pdat) == 1 + 4 * int(z["steps"])
    assert np.all(np.abs(pdat[:, 0] - t) <= 1e-5 * np.abs(t) + 1e-300)
    assert np.abs(pdat[:, 1] - u).max() <= 1e-11 * np.abs(u).max()
    cfg = oracle.acoustic_cfg(n, h, bc=bc, c=float(z["c"]))
    with oracle.point_source(src, f0, rec) as S:
        oracle.acoustic_rhs_at(cfg, 0.0, U0)
        oracle.acoustic_run(cfg, U0, int(z["steps"]), dt)
    to, uo, co = S.trace()
    assert co == cnt and np.array_equal(to, t) and rel(u, uo) <= 1e-12


def test_point_source_program_matches_greens_function(hype):
    """the whole 3d/weno4/point_source program (100^3 cells of h = 0.5, c = 250, dt = 5e-4,
    251 steps, source at (50,50,50), receiver at (57,57,57)) against the analytic receiver
    signal S(t - r/c) / (4 pi c^2 r): relative L2 misfit below 0.5 % (0.29 % measured with
    the CPU checker)"""
    from acoustic_petsc_gb300 import analytic

    n, h, dt, c, f0 = 100, 0.5, 0.0005, 250.0, 100.0
    s = hype.AcousticFV3D(n, n, n, h, dt, c=c)
    s.set_point_source((50, 50, 50), f0, (57, 57, 57), capacity=4 * 251 + 1)
    U0 = np.zeros((n, n, n, 2))
    s.RHSFunction(0.0, U0)
    s.set_state(U0)
    assert s.step(10**6, t_final=251 * dt) == 251
    t, u, cnt = s.receiver_trace()
    assert cnt == 1 + 4 * 251
    ts, us = t[1::4], u[1::4]  # the first stage of every step: t = step * dt
    ua = analytic.point_source_receiver_3d(ts, 7 * math.sqrt(3.0) * h, c, f0)
    misfit = analytic.relative_l2_misfit(us, ua)
    print(f"point source 100^3: receiver misfit {misfit:.3e}")
    assert misfit < 5e-3


# ---------------------------------------------------------------- the double-float form
@pytest.mark.parametrize("name", ["periodic", "adiabatic", "mixed"])
def test_df64_rhs_and_steps_vs_reference(hype, name):
    """HYPE_PREC_DF64 (R4, gradients and face fluxes in FP32 pairs, FP64 state and stages)
    at the FP64 form's bars against the reference fixtures"""
    from acoustic_petsc_gb300 import _lib as L

    z = np.load(os.path.join(GOLDEN, f"ref_acoustic_{name}.npz"))
    nx, ny, nz = (int(v) for v in z["shape"])
    mk = lambda: hype.AcousticFV3D(nx, ny, nz, float(z["h"]), float(z["dt"]), boundaries=tuple(int(b) for b in z["bc"]),
                                   precision=L.PREC_DF64)
    s = mk()
    e_rhs = rel(s.RHSFunction(0.0, z["U"]), z["RHS"])
    s.set_state(z["U"])
    assert s.step(3) == 3
    e3 = rel(s.get_state(), z["U3"])
    print(f"acoustic df64 {name}: RHS {e_rhs:.2e}, 3 steps {e3:.2e}")
    assert e_rhs <= 1e-12 and e3 <= 1e-12


def test_df64_convergence_table_and_point_source(hype, oracle):
    """the published convergence table (N = 16, 32, 64) and the 100^3 point-source receiver with
    the double-float form, as the FP64 form reproduces them"""
    from acoustic_petsc_gb300 import _lib as L
    from acoustic_petsc_gb300 import analytic

    with open(os.path.join(GOLDEN, "accuracy_tables.json")) as f:
        table = {int(r[0]): (r[1], r[2]) for r in json.load(f)["plane_wave_3d_main_tex"]}
    for n in (16, 32, 64):
        h = 2 * math.pi / n
        cfg = oracle.acoustic_cfg(n, h)
        s = hype.AcousticFV3D(n, n, n, h, h * 0.5 / 3.0, precision=L.PREC_DF64)
        s.set_state(oracle.plane_wave_ic(cfg))
        s.step(10**6, t_final=1.0)
        l2, linf = oracle.plane_wave_errors(cfg, s.get_state(), s.t)
        assert abs(l2 - table[n][0]) <= 2e-3 * table[n][0] and abs(linf - table[n][1]) <= 2e-3 * table[n][1]
    n, h, dt = 100, 0.5, 0.0005
    s = hype.AcousticFV3D(n, n, n, h, dt, c=250.0, precision=L.PREC_DF64)
    s.set_point_source((50, 50, 50), 100.0, (57, 57, 57), capacity=4 * 251 + 1)
    U0 = np.zeros((n, n, n, 2))
    s.RHSFunction(0.0, U0)
    s.set_state(U0)
    s.step(251)
    t, u, cnt = s.receiver_trace()
    misfit = analytic.relative_l2_misfit(u[1::4], analytic.point_source_receiver_3d(t[1::4], 7 * math.sqrt(3.0) * h,
                                                                                      250.0, 100.0))
    print(f"acoustic df64 point source 100^3: receiver misfit {misfit:.3e}")
    assert misfit < 5e-3
