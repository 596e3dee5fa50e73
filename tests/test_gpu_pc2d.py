"""The path-conservative 2D scheme of 2d/HyPE-2D with its Kapila model on the GPU:
bit-identical to the reference's RHS, dt and steps (golden fixtures, orders N = 1 and
3, incl. the first-order fallback) and to the CPU checker for every order N = 0..3 on
longer runs, reflective walls included."""
import os

import numpy as np
import pytest

from acoustic_petsc_gb300 import _lib as L
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["n1_mixed", "n1_sharp", "n3_mixed", "n3_sharp"])
def test_pc2d_vs_reference_bitwise(hype, name):
    z = np.load(os.path.join(GOLDEN, f"ref_h2d_{name}.npz"))
    mk = lambda: hype.PathConservative2D(int(z["nx"]), int(z["ny"]), float(z["h"]), order=int(z["N"]),
                                         CFL=float(z["cfl"]), boundaries=tuple(int(b) for b in z["bc"]),
                                         eos=tuple(float(v) for v in z["eos"]))
    s = mk()
    assert np.array_equal(s.RHSFunction(0.0, z["U"]), z["RHS"])
    assert s.dt == float(z["dt"])
    s = mk()
    s.set_state(z["U"])
    s.step(3)
    assert np.array_equal(s.get_state(), z["U3"])
    assert s.t == float(z["t3"])
    if name == "n3_sharp":  # the fourth-order polynomials overshoot the volume-fraction bounds
        assert s.fallback_cells > 0


@pytest.mark.parametrize("N", [0, 1, 2, 3])
@pytest.mark.parametrize("bc", [(2, 2, 1, 1), (1, 1, 0, 0)])
def test_pc2d_runs_vs_oracle_bitwise(hype, oracle, N, bc):
    """40 x 32 cells, 8 steps of the order-N stepper, reflective walls on two sides"""
    nx, ny, h = 40, 32, 1.0 / 40
    U0 = oracle.kp5_state(nx, ny, 90 + N, False)
    cfg = oracle.h2d_cfg(N, nx, ny, h, cfl=0.9, bc=bc)
    Uo, t, dt, rc = oracle.h2d_run(cfg, U0, 8)
    assert rc == 0
    s = hype.PathConservative2D(nx, ny, h, order=N, CFL=0.9, boundaries=bc)
    s.set_state(U0)
    s.step(8)
    assert np.array_equal(s.get_state(), Uo)
    assert s.t == t and s.next_dt == dt


def test_pc2d_rejects_bad_parameters(hype):
    for kw in (dict(order=4), dict(boundaries=(0, 2, 2, 2)), dict(eos=(1.0, 0.0, 1.4, 0.0))):
        with pytest.raises(hype.HypeError):
            hype.PathConservative2D(8, 8, 0.1, **kw)
