"""The 2D acoustic FV program (2d/weno4/standing_wave) on the GPU: bit-identical to the
reference's RHS and RK104 / RKS3 steps (golden fixtures), bit-identical to the CPU
checker on whole runs, and the reference's published errors (results/Error.dat)
reproduced digit for digit."""
import json
import os

import numpy as np
import pytest

from acoustic_petsc_gb300 import _lib as L
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _solver(hype, z, stepper):
    return hype.AcousticFV2D(int(z["nx"]), int(z["ny"]), float(z["h"]), float(z["dt"]), x_min=float(z["xmin"]),
                             y_min=float(z["ymin"]), boundaries=tuple(int(b) for b in z["bc"]), stepper=stepper)


@pytest.mark.parametrize("name", ["periodic", "adiabatic", "mixed"])
def test_sw2d_rhs_and_steps_bitwise(hype, name):
    z = np.load(os.path.join(GOLDEN, f"ref_sw2d_{name}.npz"))
    for stepper, key in ((L.STEP_SSPRK104, "104"), (L.STEP_SSPRK43, "43")):
        s = _solver(hype, z, stepper)
        assert np.array_equal(s.RHSFunction(0.0, z["U"]), z["RHS"])
        s.set_state(z["U"])
        assert s.step(3) == 3
        assert np.array_equal(s.get_state(), z["U" + key])
        assert s.t == float(z["t" + key])


@pytest.mark.parametrize("N", [16, 32, 64, 128])
def test_sw2d_program_reproduces_error_dat(hype, oracle, N):
    """hype.c's run: the checker's projected initial condition, RK104 with dt = h CFL / 2
    to t = 1 (last step matched); the final state equals the checker's bit for bit and its
    errors print as results/Error.dat prints them"""
    with open(os.path.join(GOLDEN, "accuracy_tables.json")) as f:
        rows = {int(r[0]): r for r in json.load(f)["standing_wave_2d_Error_dat"]}
    cfg = oracle.standing_wave_cfg(N)
    U0 = oracle.sw2d_ic(cfg)
    dt = 0.5 * cfg.h * 0.5 / 1.0
    s = hype.AcousticFV2D(N, N, cfg.h, dt, x_min=-1.0, y_min=-1.0)
    s.set_state(U0)
    n = s.step(1 << 30, t_final=1.0)
    assert s.t == 1.0
    U = s.get_state()
    if N <= 64:
        Uo, t, no = oracle.sw2d_run(cfg, U0, 1 << 30, dt, t_final=1.0, stepper=1)
        assert n == no and np.array_equal(U, Uo)
    l2, linf = oracle.sw2d_errors(cfg, U, 1.0)
    assert "%.7e %.7e" % (l2, linf) == "%.7e %.7e" % (rows[N][1], rows[N][2])


def test_sw2d_rejects_bad_parameters(hype):
    for kw in (dict(boundaries=(0, 4, 4, 4)), dict(stepper=5), dict(boundaries=(1,) * 4)):
        with pytest.raises(hype.HypeError):
            hype.AcousticFV2D(8, 8, 0.1, 0.01, **kw)


# ---------------------------------------------------------------- 2d/weno4/line_source
@pytest.mark.parametrize("name", ["periodic", "mixed"])
def test_line_source_bitwise(hype, oracle, name):
    """Source(t)/h^2 at the source cell at every stage time; the state after the run from
    rest equals the reference's bit for bit, the receiver trace the CPU checker's"""
    z = np.load(os.path.join(GOLDEN, f"ref_lsrc2d_{name}.npz"))
    n, h, dt, f0, c = int(z["n"]), float(z["h"]), float(z["dt"]), float(z["f0"]), float(z["c"])
    src, rec = tuple(int(v) for v in z["src"]), tuple(int(v) for v in z["rec"])
    bc = tuple(int(b) for b in z["bc"])
    stepper = L.STEP_SSPRK104 if int(z["stepper"]) == 1 else L.STEP_SSPRK43
    s = hype.AcousticFV2D(n, n, h, dt, c=c, boundaries=bc, stepper=stepper)
    s.set_point_source(src, f0, rec, capacity=1000)
    assert np.array_equal(s.RHSFunction(float(z["t_rhs"]), z["U"]), z["RHS"])
    s.set_point_source(src, f0, rec, capacity=1000)
    U0 = np.zeros_like(z["U"])
    s.set_state(U0)
    assert s.step(int(z["steps"])) == int(z["steps"])
    assert np.array_equal(s.get_state(), z["Un"]) and s.t == float(z["tn"])
    t, u, cnt = s.receiver_trace()
    pdat = z["pdat"]
    assert cnt == len(pdat) == (10 if int(z["stepper"]) == 1 else 4) * int(z["steps"])
    assert np.abs(pdat[:, 1] - u).max() <= 1e-11 * np.abs(u).max()
    cfg = oracle.sw2d_cfg(n, n, h, bc=bc, c=c)
    with oracle.point_source(src, f0, rec) as S:
        oracle.sw2d_run(cfg, U0, int(z["steps"]), dt, stepper=int(z["stepper"]))
    to, uo, co = S.trace()
    assert co == cnt and np.array_equal(to, t) and np.array_equal(uo, u)


def test_line_source_trace_capacity(hype):
    """samples past the trace's capacity are counted, not stored"""
    s = hype.AcousticFV2D(16, 16, 1.0, 0.001, c=580.0, boundaries=(0,) * 4)
    s.set_point_source((8, 8), 65.0, (9, 9), capacity=7)
    s.set_state(np.zeros((16, 16, 2)))
    s.step(2)
    t, u, cnt = s.receiver_trace()
    assert cnt == 20 and len(t) == len(u) == 7
    s.set_point_source(None, 65.0, None)
    assert s.receiver_trace()[2] == 0


def test_line_source_program_matches_greens_function(hype):
    """the whole 2d/weno4/line_source program (500^2 cells of h = 1, c = 580, dt = 1e-3,
    RK104, 502 steps, source (250,250), receiver (330,330)) against results/green.py's
    comparison, the 2D Green's function convolved with the wavelet: relative L2 misfit
    below 0.2 % (0.054 % measured with the CPU checker)"""
    from acoustic_petsc_gb300 import analytic

    n, dt = 500, 0.001
    s = hype.AcousticFV2D(n, n, 1.0, dt, c=580.0, boundaries=(0,) * 4)
    s.set_point_source((250, 250), 65.0, (330, 330), capacity=10 * 502)
    s.set_state(np.zeros((n, n, 2)))
    assert s.step(10**6, t_final=502 * dt) == 502
    t, u, cnt = s.receiver_trace()
    assert cnt == 10 * 502
    ts, us = t[::10], u[::10]
    ua = analytic.line_source_receiver_2d(ts, 80 * np.sqrt(2.0), 580.0, 65.0)
    misfit = analytic.relative_l2_misfit(us, ua)
    print(f"line source 500^2: receiver misfit {misfit:.3e}")
    assert misfit < 2e-3
