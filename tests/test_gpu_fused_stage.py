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
    """the indicator gate of the fused stage (a scoring pass on the tensor cores writing one flag
    per cell, then R4 or CWENO4 per cell in the fused kernel, CWENO4 redo on an R4 positivity
    break, first order after that) against the unfused k_recon_learned path: bit-identical states
    and the same flagged / fallback counts"""
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


@pytest.fixture(scope="module")
def blast_net(hype):
    from test_gpu_indicator import _train_on_blast

    p, _, _, _ = _train_on_blast(hype)
    return p


def _widen(f):
    """the 3 x 3 x 3 maximum of a flag array (x fastest, zero outside it)"""
    pad = np.pad(f, 1)
    out = np.zeros_like(f)
    nz, ny, nx = f.shape
    for dk in range(3):
        for dj in range(3):
            for di in range(3):
                out |= pad[dk:dk + nz, dj:dj + ny, di:di + nx]
    return out


def test_gate_per_step_widens_the_first_stage_flags(hype, blast_net):
    """gate scored once per step: after a step, the widened flags are the 3x3x3 maximum of the
    network's flags, the network's flags equal the per-stage gate's on the same input (an
    RHS-only call scores its input in both modes), and the flagged count is the widened owned
    cells once in each of the step's four stages"""
    from acoustic_petsc_gb300 import workloads

    n = 40
    U = workloads.euler_blast(n)
    per_stage, per_step = (hype.EulerSolver(hype.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, positivity=1,
                                                        precision=hype._lib.PREC_FP32,
                                                        recon=hype._lib.RECON_LEARNED)) for _ in range(2))
    for s in (per_stage, per_step):
        s.set_mlp(blast_net, 0.2)
    per_step.set_gate_per_step(True)
    per_step.set_state(U)
    per_step.indicator_stats(reset=True)
    per_step.step(1)
    flagged, _ = per_step.indicator_stats()
    raw, wide = per_step.gate_flags(False), per_step.gate_flags(True)
    assert raw.any()
    assert np.array_equal(wide, _widen(raw))
    assert flagged == 4 * int(wide[1:-1, 1:-1, 1:-1].sum())
    per_step.RHSFunction(0.0, U)
    per_stage.RHSFunction(0.0, U)
    assert np.array_equal(per_step.gate_flags(False), per_stage.gate_flags(False))
    print(f"blast {n}^3: {int(raw[1:-1, 1:-1, 1:-1].sum())} cells flagged, {int(wide[1:-1, 1:-1, 1:-1].sum())} "
          "after widening")
    per_stage.close()
    per_step.close()


@pytest.mark.parametrize("bias", [1000.0, -1000.0], ids=["all", "none"])
def test_gate_per_step_limits(hype, blast_net, bias):
    """a network that flags every cell makes the per-step gated stage plain CWENO4 bit for bit; one
    that flags none makes it the per-stage gate's R4 with the CWENO4 redo, bit for bit"""
    from acoustic_petsc_gb300 import workloads

    n = 24
    U = workloads.euler_blast(n)
    p = np.array(blast_net, dtype=np.float32)
    p[-1] = bias
    out = []
    for recon, per_step in ((hype._lib.RECON_LEARNED, True),
                            (hype._lib.RECON_CWENO4 if bias > 0 else hype._lib.RECON_LEARNED, False)):
        s = hype.EulerSolver(hype.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, positivity=1,
                                         precision=hype._lib.PREC_FP32, recon=recon))
        if recon == hype._lib.RECON_LEARNED:
            s.set_mlp(p, 0.2)
            s.set_gate_per_step(per_step)
        s.set_state(U)
        s.indicator_stats(reset=True)
        s.step(1)
        s.step(4)
        out.append((s.get_state(), s.t, s.indicator_stats()))
        s.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][1] == out[1][1]
    assert out[0][2][0] == (5 * 4 * n**3 if bias > 0 else 0)


def test_gate_per_step_accuracy(hype, blast_net):
    """the per-step gate keeps the learned form's distance from plain CWENO4: blast 48^3, 20 steps,
    relative L1 of the density against the plain FP32 form no larger than the per-stage gate's
    (within 50 %) and below 1e-3"""
    from acoustic_petsc_gb300 import workloads

    n = 48
    U = workloads.euler_blast(n)
    rho = {}
    for name, recon, per_step in (("plain", hype._lib.RECON_CWENO4, False), ("stage", hype._lib.RECON_LEARNED, False),
                                  ("step", hype._lib.RECON_LEARNED, True)):
        s = hype.EulerSolver(hype.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, positivity=1,
                                         precision=hype._lib.PREC_FP32, recon=recon, dt_mode=hype._lib.DT_FIXED))
        if recon == hype._lib.RECON_LEARNED:
            s.set_mlp(blast_net, 0.2)
            s.set_gate_per_step(per_step)
        s.set_state(U)
        s.step(20, dt=0.25 / n)
        rho[name] = s.get_state()[..., 0]
        s.close()
    d_stage = float(np.abs(rho["stage"] - rho["plain"]).sum() / np.abs(rho["plain"]).sum())
    d_step = float(np.abs(rho["step"] - rho["plain"]).sum() / np.abs(rho["plain"]).sum())
    print(f"blast {n}^3, 20 steps: L1(rho) from plain CWENO4: per-stage gate {d_stage:.3e}, per-step gate {d_step:.3e}")
    assert d_step <= 1.5 * d_stage + 1e-7
    assert d_step < 1e-3
