"""2D multiphase RHS on the GPU: the diffuse-interface model against the
reference's own outputs (2d/weno4/bubble), the Kapila five-equation model and
the 1024^2-workload initial condition against the CPU checker."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("name", ["smooth", "sharp"])
def test_bubble_vs_reference(hype, name):
    z = np.load(os.path.join(GOLDEN, f"ref_bubble_{name}.npz"))
    L = hype._lib
    m = hype.Multiphase2D(int(z["nx"]), int(z["ny"]), float(z["h"]), float(z["xmin"]), float(z["ymin"]),
                          CFL=float(z["cfl"]), boundaries=tuple(int(b) for b in z["bc"]), model=L.MP_DI4,
                          eos=(4.4, 6000.0, 1.4, 0.0), stepper=L.STEP_SSPRK104)
    R = m.RHSFunction(0.0, z["U"])
    assert rel(R, z["RHS"]) <= 1e-12
    assert abs(m.dt - float(z["dt"])) <= 1e-13 * float(z["dt"])
    m.set_state(z["U"])
    m.step(int(z["steps"]))
    assert rel(m.get_state(), z["U3"]) <= 1e-12
    assert abs(m.t - float(z["t3"])) <= 1e-12 * float(z["t3"])
    if name == "sharp":
        assert m.fallback_cells > 0


def _kapila(hype, oracle, n, model, precision=0):
    from acoustic_petsc_gb300 import workloads as W

    U, h = W.kapila_bubble(n, model=model)
    L = hype._lib
    m = hype.Multiphase2D(n, n, h, CFL=0.4, boundaries=(2, 2, 2, 2), model=model, eos=W.KAPILA_EOS,
                          stepper=L.STEP_SSPRK43, precision=precision)
    cfg = oracle.mp2d_cfg(n, n, h, 0.0, 0.0, cfl=0.4, bc=(2, 2, 2, 2), model=model, eos=W.KAPILA_EOS)
    return m, cfg, U


@pytest.mark.parametrize("model", [0, 1])
def test_kapila_workload_rhs_and_steps_vs_oracle(hype, oracle, model):
    m, cfg, U = _kapila(hype, oracle, 96, model)
    R = m.RHSFunction(0.0, U)
    Ro, smax, rc, fb = oracle.mp2d_rhs(cfg, U)
    assert rc == 0
    assert rel(R, Ro) <= 1e-12
    m.set_state(U)
    m.step(12)
    Uo, t, dt, rc = oracle.mp2d_run(cfg, U, 12, stepper=0)
    assert rc == 0
    assert rel(m.get_state(), Uo) <= 1e-10
    assert abs(m.t - t) <= 1e-12 * t


@pytest.mark.parametrize("model", [0, 1], ids=["diffuse_interface", "kapila"])
def test_kapila_fp32_recon_flux_error_stated(hype, oracle, model):
    """the FP32 recon/flux form (FP32 primitives, mixture, fluxes; FP64 pressure, volume-fraction term
    and stage combination) against the FP64 checker after 12 steps, both 2D models"""
    m, cfg, U = _kapila(hype, oracle, 96, model, precision=1)
    m.set_state(U)
    m.step(12)
    Uo, t, dt, rc = oracle.mp2d_run(cfg, U, 12, stepper=0)
    assert rc == 0
    density = (lambda Q: Q[..., 0]) if model == 0 else (lambda Q: Q[..., 0] + Q[..., 1])
    rho, rho_o = density(m.get_state()), density(Uo)
    l1 = float(np.abs(rho - rho_o).mean() / np.abs(rho_o).mean())
    print(f"model {model} FP32 recon/flux: L1(rho) rel err {l1:.2e} after 12 steps, state rel {rel(m.get_state(), Uo):.2e}")
    assert l1 <= 1e-3
    assert np.isfinite(m.get_state()).all()


def _kapila_solver(hype, n, precision=0, recon=0):
    from acoustic_petsc_gb300 import workloads as W

    U, h = W.kapila_bubble(n, model=1)
    L = hype._lib
    m = hype.Multiphase2D(n, n, h, CFL=0.4, boundaries=(2, 2, 2, 2), model=L.MP_KAPILA5, eos=W.KAPILA_EOS,
                          stepper=L.STEP_SSPRK43, precision=precision, recon=recon)
    m.set_state(U)
    return m


def _kapila_training(hype, n=96, tau=1e-4):
    """labels: tau = 1e-4 of the variable's magnitude; in units of p + pi (pi = 6e8 Pa for
    water) the 1e8 Pa shock is weak and the nonlinear weights move traces by ~1e-3 at most"""
    from acoustic_petsc_gb300 import indicator

    m = _kapila_solver(hype, n)
    Xs, Ds = [], []
    for _ in range(6):
        m.step(15)
        X, D = indicator.sample(m)
        Xs.append(X)
        Ds.append(D)
    m.close()
    X, D = np.concatenate(Xs), np.concatenate(Ds)
    y = indicator.labels(D, tau)
    p, loss = indicator.train(X, y, epochs=20, batch=2048, lr=3e-3, seed=0)
    return p, X, y


def test_kapila_learned_indicator_trains_on_solver_labels(hype):
    """2D learned indicator (config 3): labels from the solver's own CWENO4 weights, training on the GPU"""
    from acoustic_petsc_gb300 import indicator

    p, X, y = _kapila_training(hype)
    assert 0.0 < y.mean() < 0.5
    recall, precision, flagged = indicator.recall_precision(indicator.score(X, p), y, 0.2)
    print(f"Kapila indicator: recall {recall:.3f} precision {precision:.3f} flagged {flagged:.3f} labels {y.mean():.3f}")
    assert recall >= 0.9 and flagged <= 0.6


def test_kapila_learned_gain_at_equal_error(hype):
    """FP32-flux forms on the 64^2 shock-bubble problem against a 128^2 FP64 run of the same
    problem (block averages of the mixture density): the learned form stays within 1.05x of
    plain CWENO4's L1 error while most cells take the R4 path."""
    L = hype._lib
    p, _, _ = _kapila_training(hype)
    n = 64
    ref = _kapila_solver(hype, 2 * n)
    plain = _kapila_solver(hype, n, precision=L.PREC_FP32)
    learned = _kapila_solver(hype, n, precision=L.PREC_FP32, recon=L.RECON_LEARNED)
    learned.set_mlp(p, 0.2)
    learned.indicator_stats(reset=True)
    T = 2.0e-4
    steps = {}
    for name, m in (("ref", ref), ("plain", plain), ("learned", learned)):
        steps[name] = 0
        while m.t < T:
            m.step(1)
            steps[name] += 1
    rho = lambda U: U[..., 0] + U[..., 1]  # noqa: E731
    r_ref = rho(ref.get_state()).reshape(n, 2, n, 2).mean(axis=(1, 3))
    e_plain = np.abs(rho(plain.get_state()) - r_ref).mean() / np.abs(r_ref).mean()
    e_learn = np.abs(rho(learned.get_state()) - r_ref).mean() / np.abs(r_ref).mean()
    frac = learned.indicator_stats() / (n * n * 4.0 * steps["learned"])
    print(f"Kapila L1(rho) vs 2x FP64: plain FP32 {e_plain:.3e} learned FP32 {e_learn:.3e}; flagged/cell-stage {frac:.3f}; "
          f"minmod fallbacks {learned.fallback_cells}")
    assert e_learn <= 1.05 * e_plain
    assert frac < 0.5


@pytest.fixture(scope="module")
def kapila_net(hype):
    p, _, _ = _kapila_training(hype)
    return p


def _widen2(f):
    pad = np.pad(f, 1)
    ny, nx = f.shape
    out = np.zeros_like(f)
    for dj in range(3):
        for di in range(3):
            out |= pad[dj:dj + ny, di:di + nx]
    return out


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_kapila_gate_per_step_flags(hype, kapila_net, precision):
    """gate scored once per step: the widened flags are the 3x3 maximum of the network's flags, the
    network's flags on an RHS-only call are the cells the per-stage gate flags on the same state
    (its counter), and a step counts the widened owned cells in each of its four stages"""
    L = hype._lib
    n = 64
    per_stage = _kapila_solver(hype, n, precision=precision, recon=L.RECON_LEARNED)
    per_step = _kapila_solver(hype, n, precision=precision, recon=L.RECON_LEARNED)
    for m in (per_stage, per_step):
        m.set_mlp(kapila_net, 0.2)
        m.step(20)  # the shock into the domain: some cells to flag
    per_step.set_gate_per_step(True)
    U = per_stage.get_state()
    per_step.set_state(U)
    per_step.indicator_stats(reset=True)
    per_step.step(1)
    flagged = per_step.indicator_stats(reset=True)
    raw, wide = per_step.gate_flags(False), per_step.gate_flags(True)
    assert raw.any()
    assert np.array_equal(wide, _widen2(raw))
    assert flagged == 4 * int(wide[1:-1, 1:-1].sum())
    per_step.set_state(U)
    per_step.RHSFunction(0.0, U)
    per_stage.indicator_stats(reset=True)
    per_stage.RHSFunction(0.0, U)
    assert int(per_step.gate_flags(False)[1:-1, 1:-1].sum()) == per_stage.indicator_stats(reset=True)
    print(f"Kapila {n}^2: {int(raw[1:-1, 1:-1].sum())} cells flagged, {int(wide[1:-1, 1:-1].sum())} after widening")
    per_stage.close()
    per_step.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("bias", [1000.0, -1000.0], ids=["all", "none"])
def test_kapila_gate_per_step_limits(hype, kapila_net, precision, bias):
    """a network that flags every cell makes the per-step gated form plain CWENO4 bit for bit; one
    that flags none makes it the per-stage gate's R4 with the CWENO4 redo, bit for bit"""
    L = hype._lib
    n = 48
    p = np.array(kapila_net, dtype=np.float32)
    p[-1] = bias
    out = []
    for recon, per_step in ((L.RECON_LEARNED, True), (L.RECON_CWENO4 if bias > 0 else L.RECON_LEARNED, False)):
        m = _kapila_solver(hype, n, precision=precision, recon=recon)
        if recon == L.RECON_LEARNED:
            m.set_mlp(p, 0.2)
            m.set_gate_per_step(per_step)
        m.step(6)
        out.append((m.get_state(), m.t))
        m.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][1] == out[1][1]


def test_kapila_gate_per_step_gain_at_equal_error(hype, kapila_net):
    """the per-step gate on the 64^2 shock-bubble problem against a 128^2 FP64 run: within 1.05x of
    plain FP32 CWENO4's L1 error, as the per-stage gate"""
    L = hype._lib
    n = 64
    ref = _kapila_solver(hype, 2 * n)
    plain = _kapila_solver(hype, n, precision=L.PREC_FP32)
    learned = _kapila_solver(hype, n, precision=L.PREC_FP32, recon=L.RECON_LEARNED)
    learned.set_mlp(kapila_net, 0.2)
    learned.set_gate_per_step(True)
    T = 2.0e-4
    for m in (ref, plain, learned):
        while m.t < T:
            m.step(1)
    rho = lambda U: U[..., 0] + U[..., 1]  # noqa: E731
    r_ref = rho(ref.get_state()).reshape(n, 2, n, 2).mean(axis=(1, 3))
    e_plain = np.abs(rho(plain.get_state()) - r_ref).mean() / np.abs(r_ref).mean()
    e_learn = np.abs(rho(learned.get_state()) - r_ref).mean() / np.abs(r_ref).mean()
    print(f"Kapila L1(rho) vs 2x FP64: plain FP32 {e_plain:.3e}, per-step gated FP32 {e_learn:.3e}")
    assert e_learn <= 1.05 * e_plain
    for m in (ref, plain, learned):
        m.close()


def test_multiphase_restart_round_trip(hype, tmp_path):
    L = hype._lib
    m = _kapila_solver(hype, 40)
    m.step(5)
    m.write_restart(tmp_path / "restart1.bin")
    assert (tmp_path / "restart1.bin.info").read_text().strip() == "-vecload_block_size 6"
    k = _kapila_solver(hype, 40)
    k.read_restart(tmp_path / "restart1.bin")
    assert np.array_equal(k.get_state(), m.get_state())
    m.write_vtk(tmp_path / "sol.vtk")
    assert (tmp_path / "sol.vtk").read_text().splitlines()[4] == "DIMENSIONS 40 40 1"
    assert L.MP_KAPILA5 == 1


def test_kapila_full_workload_vs_oracle(hype, oracle):
    """the Kapila workload at its full size (1024^2 cells, 1e8 Pa step driving the air bubble):
    RHS and two SSPRK(4,3) steps bit-identical to the multi-threaded checker (the FP64 form keeps
    the checker's operation order and is compiled without contractions)"""
    m, cfg, U = _kapila(hype, oracle, 1024, 1)
    R = m.RHSFunction(0.0, U)
    Ro, smax, rc, fb = oracle.mp2d_rhs(cfg, U)
    assert rc == 0
    e_rhs = rel(R, Ro)
    m.set_state(U)
    m.step(2)
    Uo, t, dt, rc = oracle.mp2d_run(cfg, U, 2, stepper=0)
    assert rc == 0
    e_run = rel(m.get_state(), Uo)
    print(f"Kapila 1024^2: RHS {e_rhs:.2e}, two steps {e_run:.2e}")
    assert np.array_equal(R, Ro) and np.array_equal(m.get_state(), Uo)
    assert m.t == t
