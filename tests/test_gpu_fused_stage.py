"""The fused FP32 stage kernel (reconstruction, face traces in shared memory, Rusanov solves,
divergence and the SSP combination in one pass per RK stage) against the unfused kernels
(reconstruction into a face-trace buffer, three face-flux kernels, update).  Both use the same
device arithmetic with explicit roundings, so the results are required to be bit-identical:
RHS, states after steps, time, next dt, the positivity-fallback count and the first
inadmissible cell.  Grids cover partial tiles (the fused tile is 30 x 10 cells), the
smallest grids, every boundary kind, the three reconstructions and the three dt modes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _state(shape, seed, amp=0.1):
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    U = np.zeros((nz, ny, nx, 5))
    U[..., 0] = 1.0 + amp * rng.random((nz, ny, nx))
    U[..., 1:4] = amp * rng.standard_normal((nz, ny, nx, 3))
    U[..., 4] = (1 / 1.4 + amp * rng.random((nz, ny, nx))) / 0.4 + 0.5 * (U[..., 1:4] ** 2).sum(-1) / U[..., 0]
    return U


def _pair(hype, shape, **kw):
    nx, ny, nz = shape
    out = []
    for mode in (hype._lib.STAGE_AUTO, hype._lib.STAGE_UNFUSED):
        ctx = hype.AppCtx(N_x=nx, N_y=ny, N_z=nz, h=1.0 / nx, CFL=0.4, precision=hype._lib.PREC_FP32, **kw)
        s = hype.EulerSolver(ctx)
        s.set_stage_kernel(mode)
        out.append(s)
    return out


CASES = [((13, 7, 9), (1, 1, 2, 2, 1, 2), 0), ((33, 5, 6), (2, 2, 0, 0, 1, 1), 0), ((3, 3, 3), (0,) * 6, 0),
         ((61, 21, 17), (0, 0, 1, 1, 2, 2), 0), ((31, 11, 40), (1, 1, 1, 1, 0, 0), 1), ((30, 10, 8), (0,) * 6, 3),
         ((47, 33, 12), (2,) * 6, 3), ((64, 48, 40), (0,) * 6, 1)]


@pytest.mark.parametrize("shape,bc,recon", CASES)
def test_fused_equals_unfused_rhs_and_steps(hype, shape, bc, recon):
    a, b = _pair(hype, shape, boundaries=bc, recon=recon)
    U = _state(shape, sum(shape) + recon)
    Ra, Rb = a.RHSFunction(0.0, U), b.RHSFunction(0.0, U)
    assert np.array_equal(Ra, Rb)
    assert a.ctx.dt == b.ctx.dt
    for s in (a, b):
        s.set_state(U)
        s.step(1)
        s.step(5)
    assert np.array_equal(a.get_state(), b.get_state())
    assert a.t == b.t and a.next_dt == b.next_dt


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_fused_dt_modes(hype, mode):
    """the first stage whose dt comes from its own RHS (RHS, dt, then the combination) and the
    frozen / fixed dt modes"""
    from acoustic_petsc_gb300 import workloads

    n = 20
    U = workloads.euler_pulse(n, amp=0.3, sigma=0.1)
    a, b = _pair(hype, (n, n, n), dt_mode=mode)
    for s in (a, b):
        s.set_state(U)
        s.step(7, dt=0.003 if mode == 2 else 0.0)
    assert np.array_equal(a.get_state(), b.get_state())
    assert a.t == b.t and a.next_dt == b.next_dt


def test_fused_positivity_fallback(hype):
    """the pressure-ratio-10 blast with the first-order fallback: same states, same count"""
    from acoustic_petsc_gb300 import workloads

    n = 36
    U = workloads.euler_blast(n)
    a, b = _pair(hype, (n, n, n), positivity=1)
    counts = []
    for s in (a, b):
        s.set_state(U)
        s.indicator_stats(reset=True)
        s.step(12)
        counts.append(s.indicator_stats()[1])
    assert np.array_equal(a.get_state(), b.get_state())
    assert counts[0] == counts[1]
    print(f"blast {n}^3 FP32, 12 steps: {counts[0]} positivity fallbacks in both forms")


def test_fused_reports_the_same_first_bad_cell(hype):
    """an inadmissible state: both forms return HYPE_ERR_STATE with the same first bad cell"""
    import ctypes as C

    L = hype._lib
    n = 14
    U = _state((n, n, n), 3)
    U[6, 4, 9, 0] = -0.5
    U[9, 2, 3, 0] = -0.25
    bad = []
    for s in _pair(hype, (n, n, n)):
        with pytest.raises(hype.HypeError) as ei:
            s.RHSFunction(0.0, U)
        assert ei.value.code == L.HYPE_ERR_STATE
        s.set_state(U)
        status = L.Status()
        t, dt = C.c_double(0.0), C.c_double(0.0)
        rc = L.lib().hype_euler_step(s._h, 1, C.byref(t), C.byref(dt), C.byref(status))
        assert rc == L.HYPE_ERR_STATE
        bad.append(status.bad_cell)
    assert bad[0] == bad[1] >= 0


def test_fused_256_three_steps(hype):
    """the 256^3 pulse workload in the FP32 form: three steps of both stage forms"""
    from acoustic_petsc_gb300 import workloads

    n = 256
    U = workloads.euler_pulse(n)
    res = []
    for mode in (0, 1):
        ctx = hype.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, precision=hype._lib.PREC_FP32)
        s = hype.EulerSolver(ctx)
        s.set_stage_kernel(mode)
        s.set_state(U)
        s.step(3)
        res.append((s.get_state(), s.t, s.next_dt))
        s.close()
    assert np.array_equal(res[0][0], res[1][0])
    assert res[0][1] == res[1][1] and res[0][2] == res[1][2]


def test_fused_learned_gate_equals_unfused(hype):
    """the indicator gate folded into the fused stage (scoring on the tensor cores, R4 or CWENO4
    per cell, CWENO4 redo on an R4 positivity break, first order after that) against the
    unfused k_recon_learned path: bit-identical states and the same flagged / fallback counts"""
    from test_gpu_indicator import _train_on_blast

    from acoustic_petsc_gb300 import workloads

    p, _, _, _ = _train_on_blast(hype)
    n = 40
    U = workloads.euler_blast(n)
    a, b = _pair(hype, (n, n, n), recon=hype._lib.RECON_LEARNED, positivity=1)
    stats = []
    for s in (a, b):
        s.set_mlp(p, 0.2)
        s.set_state(U)
        s.indicator_stats(reset=True)
        s.step(1)
        s.step(9)
        stats.append(s.indicator_stats())
    assert np.array_equal(a.get_state(), b.get_state())
    assert a.t == b.t and a.next_dt == b.next_dt
    assert stats[0] == stats[1]
    assert stats[0][0] > 0
    print(f"learned blast {n}^3 FP32, 10 steps: flagged {stats[0][0]}, fallbacks {stats[0][1]} in both forms")
