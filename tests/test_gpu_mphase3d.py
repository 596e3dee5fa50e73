"""3D primitive-variable multiphase RHS (3d/weno4/Viscous-Multiphase-Fourth-Order,
RHSFunctionPrimitive) on the GPU against the reference's outputs (golden fixtures:
RHS, dt and 3 SSP RKS3/4 steps, incl. the 33-node admissibility fallback) and the CPU
checker on longer runs.  Tolerance: relative L-inf <= 1e-12 after one RHS or step
(the reconstruction's operation order differs from the reference's; the first-order
fallback decisions are identical on these states)."""
import os

import numpy as np
import pytest

from acoustic_petsc_gb300 import _lib as L
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _solver(hype, z, **kw):
    nx, ny, nz = (int(v) for v in z["n"])
    return hype.Multiphase3D(nx, ny, nz, float(z["h"]), CFL=float(z["cfl"]), boundaries=tuple(int(b) for b in z["bc"]),
                             eos=tuple(float(v) for v in z["eos"]), mu=tuple(float(v) for v in z["mu"]), **kw)


NAMES = ["transmissive", "periodic", "walls", "sharp"]


def _off_walls(z):
    """cells not adjacent to a reflective face: at a mirror wall the rotated HLLC flux
    (pde.c:383-440) selects its star state by the sign of S_star, which is zero up to the
    rounding noise of the two mirrored reconstructions, and the tangential momentum
    flux changes sign with it; two correct implementations differ there by O(1)"""
    nx, ny, nz = (int(v) for v in z["n"])
    bc = [int(b) for b in z["bc"]]
    m = np.ones((nz, ny, nx), dtype=bool)
    if bc[0] == 1:
        m[:, :, 0] = m[:, :, -1] = False
    if bc[2] == 1:
        m[:, 0, :] = m[:, -1, :] = False
    if bc[4] == 1:
        m[0, :, :] = m[-1, :, :] = False
    return m


@pytest.mark.parametrize("name", NAMES)
def test_mp3d_rhs_vs_reference(hype, name):
    z = np.load(os.path.join(GOLDEN, f"ref_mp3d_{name}.npz"))
    s = _solver(hype, z)
    R = s.RHSFunctionPrimitive(0.0, z["U"])
    m = _off_walls(z)
    assert float(np.abs(R - z["RHS"])[m].max() / np.abs(z["RHS"]).max()) <= TOL
    assert abs(s.dt - float(z["dt"])) <= 1e-13 * float(z["dt"])


@pytest.mark.parametrize("name", ["transmissive", "periodic", "sharp"])
def test_mp3d_three_steps_vs_reference(hype, name):
    z = np.load(os.path.join(GOLDEN, f"ref_mp3d_{name}.npz"))
    s = _solver(hype, z)
    s.set_state(z["U"])
    s.step(1)
    fb = s.fallback_cells
    s.step(2)
    fb += s.fallback_cells
    assert rel(s.get_state(), z["U3"]) <= TOL
    assert abs(s.t - float(z["t3"])) <= 1e-13 * float(z["t3"])
    assert abs(s.next_dt - float(z["dt3"])) <= 1e-13 * float(z["dt3"])
    assert (fb > 0) == (name == "sharp")


def _layers(oracle, cfg, n):
    """the program's initial condition (initial_condition.c): z-layers of a shocked phase,
    the same phase at rest, a light gas layer and the phase at rest again, smoothed over a
    few cells so that a short run stays away from the admissibility floors"""
    nx, ny, nz = n
    z = -0.5 + (np.arange(nz) + 0.5) / nz
    V = np.zeros((nz, ny, nx, 6))
    s = lambda a: 0.5 * (1.0 + np.tanh(a / 0.02))
    w_shock = 1.0 - s(z + 0.25)
    w_gas = s(z + 0.1) * (1.0 - s(z - 0.1))
    V[..., 0] = (1.0 + 0.3765 * w_shock - 0.862 * w_gas)[:, None, None]
    V[..., 3] = (0.3948 * w_shock)[:, None, None]
    V[..., 4] = (1.0 + 0.57 * w_shock)[:, None, None]
    V[..., 5] = (1.0 - w_gas)[:, None, None]
    return oracle.mp3d_prim2cons(cfg, V)


@pytest.mark.parametrize("mu", [(1.4, 1.6), (0.0, 0.0)])
def test_mp3d_layer_run_vs_oracle(hype, oracle, mu):
    """8 x 8 x 64 cells of the program's layered set-up (transmissive, CFL 0.9), 6 steps,
    with the program's viscous dt limit and with the inviscid one"""
    n = (8, 8, 64)
    h = 1.0 / 64
    cfg = oracle.mp3d_cfg(n, h, cfl=0.9, bc=(2,) * 6, mu=mu)
    U0 = _layers(oracle, cfg, n)
    Uo, t, dt, rc = oracle.mp3d_run(cfg, U0, 6)
    assert rc == 0
    s = hype.Multiphase3D(*n, h, CFL=0.9, mu=mu)
    s.set_state(U0)
    s.step(6)
    assert rel(s.get_state(), Uo) <= 1e-11
    assert abs(s.t - t) <= 1e-12 * t


def test_mp3d_rejects_bad_parameters(hype):
    for kw in (dict(boundaries=(0, 2, 2, 2, 2, 2)), dict(eos=(1.0, 0.0, 1.6, 0.0)), dict(mu=(-1.0, 0.0))):
        with pytest.raises(hype.HypeError):
            hype.Multiphase3D(8, 8, 8, 0.1, **kw)
