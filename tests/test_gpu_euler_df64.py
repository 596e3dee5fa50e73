"""The double-float reconstruction form of the 3D Euler RHS (HYPE_PREC_DF64: CWENO4 / R4 in
pairs of FP32 numbers on deviations from a per-variable reference, state, fluxes and stage
accumulation in FP64) held to the FP64 path's bars: relative L-inf max|gpu - ref| / max|ref|
<= 1e-12 after one step and <= 1e-10 after a run, against the reference's outputs and the
CPU checker, including the small-amplitude pulse of the 256^3 workload."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-12
TOL_RUN = 1e-10


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _solver(hype, n, bc=(0,) * 6, **kw):
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    kw.setdefault("precision", hype._lib.PREC_DF64)
    ctx = hype.AppCtx(N_x=nx, N_y=ny, N_z=nz, h=1.0 / nx, CFL=kw.pop("cfl", 0.4), boundaries=bc, **kw)
    return hype.EulerSolver(ctx)


NAMES = ["periodic", "walls", "mixed", "periodic_hllc", "walls_hllc", "periodic_rothllc"]


@pytest.mark.parametrize("name", NAMES)
def test_df64_rhs_and_steps_vs_reference(hype, name):
    z = np.load(os.path.join(GOLDEN, f"ref_euler_{name}.npz"))
    flux = int(z["flux"]) if "flux" in z else 0
    mk = lambda: _solver(hype, int(z["n"]), tuple(int(b) for b in z["bc"]), cfl=float(z["cfl"]), flux=flux)
    s = mk()
    e_rhs = rel(s.RHSFunction(0.0, z["U"]), z["RHS"])
    assert abs(s.ctx.dt - float(z["dt"])) <= 1e-14 * float(z["dt"])
    s = mk()
    s.set_state(z["U"])
    s.step(3)
    e3 = rel(s.get_state(), z["U3"])
    print(f"df64 {name}: RHS {e_rhs:.2e}, 3 steps {e3:.2e}")
    assert e_rhs <= TOL_STEP and e3 <= TOL_STEP
    assert abs(s.t - float(z["t3"])) <= 1e-13 * float(z["t3"])


def test_df64_small_amplitude_pulse_matches_oracle(hype, oracle):
    """the 256^3 workload's initial data (dp = 1e-3 on a uniform background) at 32^3: the
    RHS is small against the state, the case a shorter significand would fail first"""
    from acoustic_petsc_gb300 import workloads

    n = 32
    U0 = workloads.euler_pulse(n, amp=1e-3, sigma=0.1)
    cfg = oracle.euler_cfg(n, 1.0 / n, cfl=0.4)
    Ro, smax, rc, _ = oracle.euler_rhs(cfg, U0)
    assert rc == 0
    errs = {}
    for prec in (hype._lib.PREC_FP64, hype._lib.PREC_DF64):
        s = _solver(hype, n, precision=prec)
        errs[prec] = rel(s.RHSFunction(0.0, U0), Ro)
    Uo, t, dt, rc = oracle.euler_run(cfg, U0, 1)
    s = _solver(hype, n)
    s.set_state(U0)
    s.step(1)
    e1 = rel(s.get_state(), Uo)
    inc = rel(s.get_state() - U0, Uo - U0)
    print(f"small pulse 32^3: RHS error fp64 {errs[0]:.2e}, df64 {errs[2]:.2e}; one step {e1:.2e}, increment {inc:.2e}")
    # the RHS is ~1e-3 of the fluxes it is the difference of, so even the FP64 form's RHS
    # differs from the oracle's by a few 1e-12 of its size here; the double-float RHS stays
    # within twice that, and the state after a step within the 1e-12 bar
    assert errs[hype._lib.PREC_DF64] <= max(2.0 * errs[hype._lib.PREC_FP64], TOL_STEP)
    assert e1 <= TOL_STEP and inc <= 1e-9


def test_df64_run_vs_oracle(hype, oracle):
    from acoustic_petsc_gb300 import workloads

    n = 16
    U0 = workloads.euler_pulse(n, amp=0.2, sigma=0.1)
    s = _solver(hype, n)
    s.set_state(U0)
    s.step(20)
    Uo, t, dt, rc = oracle.euler_run(oracle.euler_cfg(n, 1.0 / n, cfl=0.4), U0, 20)
    assert rc == 0
    assert rel(s.get_state(), Uo) <= TOL_RUN
    assert abs(s.t - t) <= 1e-12 * t


@pytest.mark.parametrize("shape,bc", [((13, 7, 9), (1, 1, 2, 2, 1, 2)), ((10, 12, 11), (0, 0, 1, 1, 2, 2))])
def test_df64_odd_shapes_and_boundaries(hype, oracle, shape, bc):
    nx, ny, nz = shape
    rng = np.random.default_rng(nx * 100 + ny)
    U = np.zeros((nz, ny, nx, 5))
    U[..., 0] = 1.0 + 0.1 * rng.random((nz, ny, nx))
    U[..., 1:4] = 0.1 * rng.standard_normal((nz, ny, nx, 3))
    U[..., 4] = (1 / 1.4 + 0.1 * rng.random((nz, ny, nx))) / 0.4 + 0.5 * (U[..., 1:4] ** 2).sum(-1) / U[..., 0]
    s = _solver(hype, shape, bc)
    cfg = oracle.euler_cfg(shape, 1.0 / nx, cfl=0.4, bc=bc)
    Ro, smax, rc, _ = oracle.euler_rhs(cfg, U)
    assert rc == 0
    assert rel(s.RHSFunction(0.0, U), Ro) <= TOL_STEP
    s.set_state(U)
    s.step(2)
    Uo, t, dt, rc = oracle.euler_run(cfg, U, 2)
    assert rel(s.get_state(), Uo) <= TOL_STEP


def test_df64_linear_reconstruction(hype, oracle):
    from acoustic_petsc_gb300 import workloads

    n = 12
    U0 = workloads.euler_pulse(n, amp=0.1, sigma=0.1)
    s = _solver(hype, n, recon=hype._lib.RECON_LINEAR4)
    Ro, smax, rc, _ = oracle.euler_rhs(oracle.euler_cfg(n, 1.0 / n, cfl=0.4, recon=1), U0)
    assert rc == 0
    assert rel(s.RHSFunction(0.0, U0), Ro) <= TOL_STEP


def test_df64_blast_positivity_fallback_vs_oracle(hype, oracle):
    from acoustic_petsc_gb300 import workloads

    n = 20
    U0 = workloads.euler_blast(n)
    s = _solver(hype, n, positivity=1)
    s.set_state(U0)
    s.step(6)
    cfg = oracle.euler_cfg(n, 1.0 / n, cfl=0.4, positivity=1)
    Uo, t, dt, rc = oracle.euler_run(cfg, U0, 6)
    assert rc == 0
    assert rel(s.get_state(), Uo) <= TOL_RUN


def test_df64_rejects_what_it_does_not_cover(hype):
    from acoustic_petsc_gb300 import _lib as L

    with pytest.raises(Exception):
        _solver(hype, 8, recon=L.RECON_WENO3)
    with pytest.raises(Exception):  # viscous: Rusanov only
        _solver(hype, 8, mu=0.01, prandtl=0.71, cv=1.0, flux=L.FLUX_HLLC)
    s = _solver(hype, 8)
    with pytest.raises(Exception):
        s.set_recon(L.RECON_WENO3)


def _gated(hype, n, prob, positivity=0, seed=3):
    from acoustic_petsc_gb300 import indicator, workloads

    s = _solver(hype, n, recon=hype._lib.RECON_LEARNED, positivity=positivity)
    s.set_mlp(indicator.init_params(seed), prob)
    s.set_state(workloads.euler_blast(n, p_ratio=3.0, rho_ratio=2.0))
    return s


@pytest.mark.parametrize("prob,recon", [(1e-30, 0), (1.0 - 1e-7, 1)])
def test_df64_indicator_gate_limits(hype, prob, recon):
    """the indicator-gated double-float reconstruction: a gate that flags every cell is the
    double-float CWENO4, one that flags none its R4 limit, bit for bit"""
    from acoustic_petsc_gb300 import workloads

    n = 16
    g = _gated(hype, n, prob)
    g.step(3)
    p = _solver(hype, n, recon=recon, positivity=0)
    p.set_state(workloads.euler_blast(n, p_ratio=3.0, rho_ratio=2.0))
    p.step(3)
    assert np.array_equal(g.get_state(), p.get_state())
    flagged, _ = g.indicator_stats()
    assert (flagged > 0) == (recon == 0)


def test_df64_indicator_gate_matches_fp64_gate(hype, oracle):
    """the same network gating the FP64 and the double-float reconstructions on a blast: the
    networks see the FP64 form's stencils rounded to FP32 and the double-float form's deviations,
    so a cell whose logit sits within rounding of the threshold may go the other way; the
    flagged counts agree within 1 %, and the states to the FP64 bar unless a cell flipped"""
    from acoustic_petsc_gb300 import indicator, workloads

    n = 16
    params = indicator.init_params(5)
    # a threshold that flags about a fifth of the cells of this state
    probe = _solver(hype, n, precision=hype._lib.PREC_FP64)
    probe.set_state(workloads.euler_blast(n, p_ratio=3.0, rho_ratio=2.0))
    X, _ = indicator.sample(probe)
    thr = float(np.quantile(indicator.score(X, params), 0.8))
    prob = 1.0 / (1.0 + np.exp(-thr))
    states, flags = [], []
    for prec in (hype._lib.PREC_FP64, hype._lib.PREC_DF64):
        s = _solver(hype, n, precision=prec, recon=hype._lib.RECON_LEARNED, positivity=1)
        s.set_mlp(params, prob)
        s.set_state(workloads.euler_blast(n, p_ratio=3.0, rho_ratio=2.0))
        s.step(3)
        states.append(s.get_state())
        flags.append(s.indicator_stats())
    assert flags[0][0] > 0 and abs(flags[0][0] - flags[1][0]) <= 0.01 * flags[0][0]
    err = rel(states[1], states[0])
    print(f"gate fp64 vs df64: flagged {flags[0][0]} / {flags[1][0]}, state difference {err:.2e}")
    # a flipped cell next to the blast takes R4 in one run and CWENO4 in the other (1.6e-6 seen)
    assert err <= (1e-12 if flags[0] == flags[1] else 1e-4)


@pytest.mark.parametrize("shape,bc", [((3, 5, 4), (0, 0, 1, 1, 2, 2)), ((4, 3, 3), (1, 2, 0, 0, 0, 0))])
def test_smallest_grids_both_forms(hype, oracle, shape, bc):
    """the smallest grids the library takes (3 cells on an axis: the periodic ghost fill wraps
    more than once, reflective and transmissive ghosts reach past the opposite wall's mirror)
    in the FP64 and the double-float forms against the CPU checker"""
    nx, ny, nz = shape
    rng = np.random.default_rng(7 + nx)
    U = np.zeros((nz, ny, nx, 5))
    U[..., 0] = 1.0 + 0.1 * rng.random((nz, ny, nx))
    U[..., 1:4] = 0.1 * rng.standard_normal((nz, ny, nx, 3))
    U[..., 4] = (1 / 1.4 + 0.1 * rng.random((nz, ny, nx))) / 0.4 + 0.5 * (U[..., 1:4] ** 2).sum(-1) / U[..., 0]
    cfg = oracle.euler_cfg(shape, 1.0 / nx, cfl=0.4, bc=bc)
    Ro, smax, rc, _ = oracle.euler_rhs(cfg, U)
    assert rc == 0
    Uo, t, dt, rc = oracle.euler_run(cfg, U, 2)
    for prec in (hype._lib.PREC_FP64, hype._lib.PREC_DF64):
        s = _solver(hype, shape, bc, precision=prec)
        assert rel(s.RHSFunction(0.0, U), Ro) <= TOL_STEP
        s.set_state(U)
        s.step(2)
        assert rel(s.get_state(), Uo) <= TOL_STEP
