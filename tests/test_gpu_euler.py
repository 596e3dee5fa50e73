"""3D Euler CWENO4 + Rusanov on the GPU against the reference's outputs and the
CPU checker.  Tolerance (the bar of the FP64 path): relative L-inf
max|gpu - ref| / max|ref| <= 1e-12 after one step, <= 1e-10 after a run."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-12
TOL_RUN = 1e-10


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def solver(hype, n, bc=(0,) * 6, **kw):
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    ctx = hype.AppCtx(N_x=nx, N_y=ny, N_z=nz, h=1.0 / nx, CFL=kw.pop("cfl", 0.4), boundaries=bc, **kw)
    return hype.EulerSolver(ctx)


# walls_rothllc is checked separately below: the reference's rotated HLLC is discontinuous at reflective walls
NAMES = ["periodic", "walls", "mixed", "periodic_hllc", "walls_hllc", "periodic_rothllc", "periodic_weno3", "walls_weno3",
         "mixed_weno3"]


def _golden_solver(hype, z):
    n = int(z["n"])
    flux = int(z["flux"]) if "flux" in z else 0
    recon = int(z["recon"]) if "recon" in z else 0
    dt_mode = int(z["dt_mode"]) if "dt_mode" in z else 0
    return solver(hype, n, tuple(int(b) for b in z["bc"]), cfl=float(z["cfl"]), flux=flux, recon=recon,
                  dt_mode=dt_mode)


@pytest.mark.parametrize("name", NAMES)
def test_rhs_vs_reference(hype, name):
    z = np.load(os.path.join(GOLDEN, f"ref_euler_{name}.npz"))
    s = _golden_solver(hype, z)
    R = s.RHSFunction(0.0, z["U"])
    assert rel(R, z["RHS"]) <= TOL_STEP
    assert abs(s.ctx.dt - float(z["dt"])) <= 1e-14 * float(z["dt"])


@pytest.mark.parametrize("name", NAMES)
def test_three_steps_vs_reference(hype, name):
    z = np.load(os.path.join(GOLDEN, f"ref_euler_{name}.npz"))
    s = _golden_solver(hype, z)
    s.set_state(z["U"])
    s.step(1)
    s.step(2)
    assert rel(s.get_state(), z["U3"]) <= TOL_STEP
    assert abs(s.t - float(z["t3"])) <= 1e-13 * float(z["t3"])
    assert abs(s.next_dt - float(z["dt3"])) <= 1e-13 * float(z["dt3"])


def _pulse(n, amp=0.05):
    from acoustic_petsc_gb300 import workloads

    return workloads.euler_pulse(n, amp=amp, sigma=0.1)


def test_one_step_vs_oracle_pulse(hype, oracle):
    n = 24
    U0 = _pulse(n)
    s = solver(hype, n)
    s.set_state(U0)
    s.step(1)
    Uo, t, dt, rc = oracle.euler_run(oracle.euler_cfg(n, 1.0 / n, cfl=0.4), U0, 1)
    assert rc == 0
    assert rel(s.get_state(), Uo) <= TOL_STEP
    # the increment itself, not only the state, must agree
    assert rel(s.get_state() - U0, Uo - U0) <= 1e-9


def test_run_vs_oracle(hype, oracle):
    n = 16
    U0 = _pulse(n, amp=0.2)
    s = solver(hype, n)
    s.set_state(U0)
    for _ in range(4):
        s.step(5)
    Uo, t, dt, rc = oracle.euler_run(oracle.euler_cfg(n, 1.0 / n, cfl=0.4), U0, 20)
    assert rc == 0
    assert rel(s.get_state(), Uo) <= TOL_RUN
    assert abs(s.t - t) <= 1e-12 * t


@pytest.mark.parametrize("shape,bc", [((13, 7, 9), (1, 1, 2, 2, 1, 2)), ((33, 5, 6), (2, 2, 0, 0, 1, 1)),
                                      ((10, 12, 11), (0, 0, 1, 1, 2, 2))])
def test_odd_shapes_and_boundaries(hype, oracle, shape, bc):
    nx, ny, nz = shape
    rng = np.random.default_rng(nx * 100 + ny)
    U = np.zeros((nz, ny, nx, 5))
    U[..., 0] = 1.0 + 0.1 * rng.random((nz, ny, nx))
    U[..., 1:4] = 0.1 * rng.standard_normal((nz, ny, nx, 3))
    U[..., 4] = (1 / 1.4 + 0.1 * rng.random((nz, ny, nx))) / 0.4 + 0.5 * (U[..., 1:4] ** 2).sum(-1) / U[..., 0]
    ctx = hype.AppCtx(N_x=nx, N_y=ny, N_z=nz, h=1.0 / nx, CFL=0.4, boundaries=bc)
    s = hype.EulerSolver(ctx)
    cfg = oracle.euler_cfg((nx, ny, nz), 1.0 / nx, cfl=0.4, bc=bc)
    R = s.RHSFunction(0.0, U)
    Ro, smax, rc, _ = oracle.euler_rhs(cfg, U)
    assert rc == 0
    assert rel(R, Ro) <= TOL_STEP
    s.set_state(U)
    s.step(2)
    Uo, t, dt, rc = oracle.euler_run(cfg, U, 2)
    assert rel(s.get_state(), Uo) <= TOL_STEP


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_dt_semantics(hype, oracle, mode):
    n = 12
    U0 = _pulse(n, amp=0.3)
    ctx = hype.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, dt_mode=mode)
    s = hype.EulerSolver(ctx)
    s.set_state(U0)
    s.step(6, dt=0.003 if mode == 2 else 0.0)
    Uo, t, dt, rc = oracle.euler_run(oracle.euler_cfg(n, 1.0 / n, cfl=0.4), U0, 6, dt_mode=mode, dt=0.003)
    assert rel(s.get_state(), Uo) <= TOL_STEP * 10
    assert abs(s.t - t) <= 1e-13 * t and abs(s.next_dt - dt) <= 1e-13 * dt


def test_weno3_run_vs_oracle(hype, oracle):
    """the WENO3 program (3d/weno3/Euler: fixed dt from the first RHS) over 20 steps, walls and periodic"""
    n = 14
    U0 = _pulse(n, amp=0.2)
    for bc in ((0,) * 6, (1, 1, 2, 2, 1, 2)):
        s = solver(hype, n, bc, recon=hype._lib.RECON_WENO3, dt_mode=hype._lib.DT_FROZEN)
        s.set_state(U0)
        s.step(20)
        cfg = oracle.euler_cfg(n, 1.0 / n, cfl=0.4, bc=bc, recon=3)
        U, t, dt, rc = oracle.euler_run(cfg, U0, 20, dt_mode=1)
        assert rc == 0
        assert rel(s.get_state(), U) <= TOL_RUN
        assert abs(s.t - t) <= 1e-12 * t


def test_weno3_fp32_error_is_bounded(hype, oracle):
    n = 16
    U0 = _pulse(n, amp=0.2)
    s = solver(hype, n, recon=hype._lib.RECON_WENO3, precision=hype._lib.PREC_FP32)
    s.set_state(U0)
    s.step(5)
    U, t, dt, rc = oracle.euler_run(oracle.euler_cfg(n, 1.0 / n, cfl=0.4, recon=3), U0, 5)
    assert rel(s.get_state(), U) <= 1e-5


def test_linear_reconstruction(hype, oracle):
    n = 12
    U0 = _pulse(n, amp=0.3)
    ctx = hype.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, recon=hype._lib.RECON_LINEAR4)
    s = hype.EulerSolver(ctx)
    R = s.RHSFunction(0.0, U0)
    Ro, _, rc, _ = oracle.euler_rhs(oracle.euler_cfg(n, 1.0 / n, cfl=0.4, recon=1), U0)
    assert rel(R, Ro) <= TOL_STEP


def test_device_rhs_equals_host_rhs(hype):
    import ctypes as C

    n = 10
    U0 = _pulse(n)
    s = solver(hype, n)
    R_host = s.RHSFunction(0.0, U0)
    s.set_state(U0)
    L = hype.lib()
    import torch

    out = torch.empty(5 * n**3, dtype=torch.float64, device="cuda")
    dt = C.c_double()
    rc = L.hype_euler_rhs_device(s._h, 0.0, C.c_void_p(s.device_state_ptr()), C.c_void_p(out.data_ptr()), C.byref(dt))
    assert rc == 0
    R_dev = out.cpu().numpy().reshape(5, n, n, n).transpose(1, 2, 3, 0)
    assert np.array_equal(R_dev, R_host)


def test_fp32_recon_flux_error_is_bounded(hype, oracle):
    """FP32 reconstruction/flux with FP64 state: error against the FP64 oracle is
    stated, not claimed at parity (acoustic pulse amplitude 1e-3 as in the 256^3 workload)."""
    n = 24
    U0 = _pulse(n, amp=1e-3)
    ctx = hype.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, precision=hype._lib.PREC_FP32)
    s = hype.EulerSolver(ctx)
    s.set_state(U0)
    s.step(5)
    Uo, t, dt, rc = oracle.euler_run(oracle.euler_cfg(n, 1.0 / n, cfl=0.4), U0, 5)
    e_state = rel(s.get_state(), Uo)
    e_pert = float(np.abs(s.get_state()[..., 0] - Uo[..., 0]).max() / np.abs(Uo[..., 0] - 1.0).max())
    print(f"FP32 recon/flux: state rel err {e_state:.2e}, density-perturbation rel err {e_pert:.2e}")
    assert e_state <= 1e-6


def test_inadmissible_state_returns_error(hype):
    n = 8
    U0 = _pulse(n)
    U0[3, 4, 5, 0] = -0.5
    s = solver(hype, n)
    with pytest.raises(hype.HypeError) as ei:
        s.RHSFunction(0.0, U0)
    assert ei.value.code == hype._lib.HYPE_ERR_STATE
    # the context stays usable
    R = s.RHSFunction(0.0, _pulse(n))
    assert np.isfinite(R).all()


@pytest.mark.parametrize("flux", [1, 2])
def test_hllc_family_run_vs_oracle(hype, oracle, flux):
    n = 14
    U0 = _pulse(n, amp=0.3)
    rng = np.random.default_rng(5)
    U0[..., 1:4] += 0.05 * rng.standard_normal(U0[..., 1:4].shape)
    U0[..., 4] += 0.5 * (U0[..., 1:4] ** 2).sum(-1) / U0[..., 0]
    bc = (1, 1, 2, 2, 0, 0)
    ctx = hype.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, boundaries=bc, flux=flux)
    s = hype.EulerSolver(ctx)
    s.set_state(U0)
    s.step(8)
    Uo, t, dt, rc = oracle.euler_run(oracle.euler_cfg(n, 1.0 / n, cfl=0.4, bc=bc, flux=flux), U0, 8)
    assert rc == 0
    assert rel(s.get_state(), Uo) <= TOL_RUN
    assert abs(s.t - t) <= 1e-12 * t


def test_rothllc_at_reflective_walls(hype):
    """The reference's rotated HLLC picks the tangent frame of its inner HLLC by the
    sign of |t_y + t_z| - |t_y - t_z| of the velocity-jump direction, and its inner
    HLLC uses an uncorrected t2z (3d/weno4/Navier-Stokes-3D/pde.c:238, non-orthogonal
    frame).  At a reflective wall the jump is along the wall normal up to rounding
    noise, so the frame - and the flux, at O(1) - follows that noise.  Everywhere
    else the GPU matches the reference to the FP64 tolerance; the mismatch is
    confined to the cells next to the reflective walls."""
    z = np.load(os.path.join(GOLDEN, "ref_euler_walls_rothllc.npz"))
    s = _golden_solver(hype, z)
    R = s.RHSFunction(0.0, z["U"])
    bc = [int(b) for b in z["bc"]]
    n = int(z["n"])
    wall = np.zeros((n, n, n), dtype=bool)  # [k][j][i]
    if bc[0] == 1:
        wall[:, :, 0] = True
    if bc[1] == 1:
        wall[:, :, -1] = True
    if bc[2] == 1:
        wall[:, 0, :] = True
    if bc[3] == 1:
        wall[:, -1, :] = True
    if bc[4] == 1:
        wall[0, :, :] = True
    if bc[5] == 1:
        wall[-1, :, :] = True
    interior = ~wall
    err = np.abs(R - z["RHS"]).max(axis=-1)
    scale = np.abs(z["RHS"]).max()
    assert err[interior].max() <= TOL_STEP * scale


def test_blast_positivity_fallback_vs_oracle(hype, oracle):
    """Pressure-ratio-10 blast: the CWENO4 traces break positivity next to the shock;
    with the first-order fallback the run proceeds and matches the CPU checker."""
    from acoustic_petsc_gb300 import workloads

    n = 20
    U0 = workloads.euler_blast(n)
    ctx = hype.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, positivity=1)
    s = hype.EulerSolver(ctx)
    s.set_state(U0)
    s.step(6)
    flagged, fallbacks = s.indicator_stats()
    cfg = oracle.euler_cfg(n, 1.0 / n, cfl=0.4, positivity=1)
    oracle.lib().orc_positivity_fallbacks(1)
    Uo, t, dt, rc = oracle.euler_run(cfg, U0, 6)
    assert rc == 0
    assert rel(s.get_state(), Uo) <= TOL_RUN
    print(f"blast {n}^3: {fallbacks} GPU cell-stage fallbacks, oracle {oracle.lib().orc_positivity_fallbacks(1)}")


def test_restart_file_resumes_bit_for_bit(hype, tmp_path):
    """write the resident state as restart1.bin (PETSc binary Vec), load it into a fresh
    context, and the two runs continue identically; the VTK snapshot holds the same state"""
    n = 12
    a = solver(hype, n, (1, 1, 2, 2, 0, 0))
    a.set_state(_pulse(n, amp=0.2))
    a.step(3)
    a.write_restart(tmp_path / "restart1.bin")
    raw = np.frombuffer((tmp_path / "restart1.bin").read_bytes()[8:], dtype=">f8").astype(np.float64)
    assert np.array_equal(raw.reshape(a.shape), a.get_state())
    assert (tmp_path / "restart1.bin.info").read_text().strip() == "-vecload_block_size 5"
    b = solver(hype, n, (1, 1, 2, 2, 0, 0))
    b.read_restart(tmp_path / "restart1.bin")
    b.t, b.next_dt = a.t, a.next_dt
    a.step(4)
    b.step(4)
    assert np.array_equal(a.get_state(), b.get_state())
    a.write_vtk(tmp_path / "sol.vtk")
    lines = (tmp_path / "sol.vtk").read_text().splitlines()
    assert lines[4] == f"DIMENSIONS {n} {n} {n}" and lines[8] == "SCALARS density double 1"
    rho = np.array([float(t) for t in lines[10:10 + n**3]])
    assert np.array_equal(rho, a.get_state()[..., 0].ravel())


@pytest.mark.parametrize("precision,flux", [(0, 0), (2, 0), (0, 1)])
def test_graph_replayed_steps_equal_launched_steps(hype, precision, flux):
    """Steps after the first of a call replay a captured CUDA graph; with per-kernel profiling
    on they are launched one by one.  Same kernels, same arguments: bit-identical states, times
    and next dt, and the replayed kernels are counted as launches."""
    from acoustic_petsc_gb300 import _lib as L

    n = 20
    U0 = _pulse(n, amp=0.2)
    out = []
    for prof in (0, 1):
        s = solver(hype, n, precision=precision, flux=flux)
        s.set_state(U0)
        L.lib().hype_euler_profile(s._h, prof)
        l0 = L.launches()
        s.step(7)
        out.append((s.get_state(), s.t, s.next_dt, L.launches() - l0))
        s.step(3)  # a second call reuses the captured graph
        out.append((s.get_state(), s.t, s.next_dt, None))
        s.close()
    (Ug, tg, dg, lg), (Ug2, tg2, dg2, _), (Ue, te, de, le), (Ue2, te2, de2, _) = out
    assert np.array_equal(Ug, Ue) and tg == te and dg == de
    assert np.array_equal(Ug2, Ue2) and tg2 == te2 and dg2 == de2
    assert lg == le > 0
