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
