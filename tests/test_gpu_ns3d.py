"""Viscous Navier-Stokes (3d/weno4/Navier-Stokes-3D) on the GPU against the
reference's outputs: the RHS and 3 steps on seeded states (relative L-inf
<= 1e-12, dt to 1e-13), and the reference's checked-in Taylor-Green history
ke.csv (KE and dissipation every 10 steps, printed to 9 digits)."""
import os

import numpy as np
import pytest

from acoustic_petsc_gb300 import _lib as L
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-12


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _solver(hype, z):
    n = int(z["n"])
    ctx = hype.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=float(z["cfl"]), boundaries=tuple(int(b) for b in z["bc"]),
                      recon=int(z["recon"]), mu=float(z["mu"]), prandtl=float(z["prandtl"]), cv=float(z["cv"]))
    return hype.EulerSolver(ctx)


@pytest.mark.parametrize("name", ["periodic", "walls", "mixed"])
def test_ns3d_rhs_vs_reference(hype, name):
    z = np.load(os.path.join(GOLDEN, f"ref_ns3d_{name}.npz"))
    s = _solver(hype, z)
    R = s.RHSFunction(0.0, z["U"])
    assert rel(R, z["RHS"]) <= TOL_STEP
    assert abs(s.ctx.dt - float(z["dt"])) <= 1e-13 * float(z["dt"])


@pytest.mark.parametrize("name", ["periodic", "walls", "mixed"])
def test_ns3d_three_steps_vs_reference(hype, name):
    z = np.load(os.path.join(GOLDEN, f"ref_ns3d_{name}.npz"))
    s = _solver(hype, z)
    s.set_state(z["U"])
    s.step(1)
    s.step(2)
    assert rel(s.get_state(), z["U3"]) <= TOL_STEP
    assert abs(s.t - float(z["t3"])) <= 1e-13 * float(z["t3"])
    assert abs(s.next_dt - float(z["dt3"])) <= 1e-13 * float(z["dt3"])


def test_ns3d_viscous_terms_are_not_negligible(hype):
    """the fixtures' viscous part is far above the tolerance: the same state without
    viscosity gives a different RHS"""
    z = np.load(os.path.join(GOLDEN, "ref_ns3d_periodic.npz"))
    n = int(z["n"])
    s = hype.EulerSolver(hype.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, recon=1))
    assert rel(s.RHSFunction(0.0, z["U"]), z["RHS"]) > 1e-4


def test_taylor_green_matches_ke_csv(hype, oracle):
    """32^3 Taylor-Green (Navier-Stokes-3D/hype.c:33-55, CFL 0.6, mu 0.01) from the
    checker's initial condition: t, KE and dissipation of the device monitor every 10
    steps against the reference's ke.csv rows 0-20, and the monitor's sums against
    the checker's on the same state"""
    ke = np.loadtxt(os.path.join(GOLDEN, "ns3d_tgv_ke.csv"), delimiter=",")
    n = 32
    h = 2.0 * np.pi / n
    cfg = oracle.euler_cfg(n, h, cfl=0.6, origin=(-np.pi,) * 3, recon=1, mu=0.01)
    U0 = oracle.tgv_ic(cfg)
    ctx = hype.AppCtx(N_x=n, N_y=n, N_z=n, h=h, x_min=-np.pi, y_min=-np.pi, z_min=-np.pi, CFL=0.6,
                      recon=L.RECON_LINEAR4, mu=0.01, prandtl=1.0, cv=2.5)
    s = hype.EulerSolver(ctx)
    s.set_state(U0)
    for r in range(0, 21):
        if r:
            s.step(10)
            assert abs(s.t - ke[r, 0]) <= 1e-8 * ke[r, 0]
        k, d = s.monitor()
        assert abs(k - ke[r, 1]) <= 1e-8 * ke[r, 1], (r, k, ke[r, 1])
        assert abs(d - ke[r, 2]) <= 1e-8 * ke[r, 2], (r, d, ke[r, 2])
        if r in (0, 20):
            U = s.get_state()
            assert abs(k - oracle.kinetic_energy(cfg, U)) <= 1e-13 * k
            assert abs(d - oracle.dissipation(cfg, U)) <= 1e-12 * d


def test_ns3d_rejects_unsupported_combinations(hype):
    base = dict(N_x=8, N_y=8, N_z=8, h=1.0 / 8, mu=0.01)
    for kw in (dict(precision=L.PREC_FP32), dict(recon=L.RECON_LEARNED), dict(prandtl=0.0), dict(cv=-1.0)):
        with pytest.raises(hype.HypeError):
            hype.EulerSolver(hype.AppCtx(**base, **kw))
    s = hype.EulerSolver(hype.AppCtx(**base, recon=L.RECON_LINEAR4))
    with pytest.raises(hype.HypeError):
        s.set_recon(L.RECON_LEARNED)


# ---------------------------------------------------------------- the double-float form
def _solver_df(hype, z):
    n = int(z["n"])
    ctx = hype.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=float(z["cfl"]), boundaries=tuple(int(b) for b in z["bc"]),
                      recon=int(z["recon"]), mu=float(z["mu"]), prandtl=float(z["prandtl"]), cv=float(z["cv"]),
                      precision=L.PREC_DF64)
    return hype.EulerSolver(ctx)


@pytest.mark.parametrize("name", ["periodic", "walls", "mixed"])
def test_ns3d_df64_rhs_and_steps_vs_reference(hype, name):
    """HYPE_PREC_DF64 with viscosity: R4 coefficients, face gradients, viscous and Rusanov fluxes
    in FP32 pairs (deviation form), held to the FP64 bars against the reference fixtures"""
    z = np.load(os.path.join(GOLDEN, f"ref_ns3d_{name}.npz"))
    s = _solver_df(hype, z)
    e_rhs = rel(s.RHSFunction(0.0, z["U"]), z["RHS"])
    assert abs(s.ctx.dt - float(z["dt"])) <= 1e-13 * float(z["dt"])
    s = _solver_df(hype, z)
    s.set_state(z["U"])
    s.step(3)
    e3 = rel(s.get_state(), z["U3"])
    print(f"ns3d df64 {name}: RHS {e_rhs:.2e}, 3 steps {e3:.2e}")
    assert e_rhs <= TOL_STEP and e3 <= TOL_STEP
    assert abs(s.t - float(z["t3"])) <= 1e-13 * float(z["t3"])


def test_ns3d_df64_taylor_green_matches_ke_csv(hype, oracle):
    """the reference's ke.csv rows 0-20 with the double-float form, as the FP64 form matches them"""
    ke = np.loadtxt(os.path.join(GOLDEN, "ns3d_tgv_ke.csv"), delimiter=",")
    n = 32
    h = 2.0 * np.pi / n
    cfg = oracle.euler_cfg(n, h, cfl=0.6, origin=(-np.pi,) * 3, recon=1, mu=0.01)
    ctx = hype.AppCtx(N_x=n, N_y=n, N_z=n, h=h, x_min=-np.pi, y_min=-np.pi, z_min=-np.pi, CFL=0.6,
                      recon=L.RECON_LINEAR4, mu=0.01, prandtl=1.0, cv=2.5, precision=L.PREC_DF64)
    s = hype.EulerSolver(ctx)
    s.set_state(oracle.tgv_ic(cfg))
    for r in range(0, 21):
        if r:
            s.step(10)
            assert abs(s.t - ke[r, 0]) <= 1e-8 * ke[r, 0]
        k, d = s.monitor()
        assert abs(k - ke[r, 1]) <= 1e-8 * ke[r, 1], (r, k, ke[r, 1])
        assert abs(d - ke[r, 2]) <= 1e-8 * ke[r, 2], (r, d, ke[r, 2])
