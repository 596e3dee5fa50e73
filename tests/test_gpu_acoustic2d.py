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
