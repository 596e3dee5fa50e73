"""Each workload run to the length it is specified with, against the CPU checker.

The bars are the FP64 path's: relative L-inf max|gpu - ref| / max|ref| <= 1e-10 after the whole
run (<= 1e-12 after one step is covered by the shorter tests).  The reference's own time loop runs
its whole horizon through TSSolve (3d/weno3/Euler/hype.c:188-194: SSP RKS3 with 4 stages) and the
CTCS drivers' step loops (2d/ctcs/line_source/wave.c:98-111); these tests do the same on the GPU:

* 3D Euler CWENO4 + Rusanov + SSPRK(4,3), Gaussian pulse, CFL 0.4 with the monitor's dt: the
  200 steps of the workload at 64^3, in FP64 and in the double-float form; and 10 steps at the
  workload's own 256^3;
* the pressure-ratio-10 blast with the first-order positivity fallback: its 500 steps at 64^3,
  with the number of cell-stage fallbacks equal to the checker's;
* batched monopole CTCS (256 instances, sides log-uniform in 64..1024, seed 7): all 2000 steps,
  the four smallest, four median and two largest instances checked;
* the Kapila bubble at 1024^2: the 8 SSPRK(4,3) steps the benchmark runs (3 warm-up + 5 timed),
  bit-identical to the checker.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_RUN = 1e-10


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _euler(hype, n, **kw):
    ctx = hype.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, **kw)
    return hype.EulerSolver(ctx)


@pytest.fixture(scope="module")
def pulse64_oracle(oracle):
    from acoustic_petsc_gb300 import workloads

    n = 64
    U0 = workloads.euler_pulse(n)
    Uo, t, dt, rc = oracle.euler_run(oracle.euler_cfg(n, 1.0 / n, cfl=0.4), U0, 200)
    assert rc == 0
    return U0, Uo, t, dt


@pytest.mark.parametrize("precision", [0, 2], ids=["fp64", "df64"])
def test_pulse_200_steps_64(hype, pulse64_oracle, precision):
    U0, Uo, t, dt = pulse64_oracle
    s = _euler(hype, 64, precision=precision)
    s.set_state(U0)
    for _ in range(4):
        s.step(50)
    Ug = s.get_state()
    err = rel(Ug, Uo)
    inc = rel(Ug - U0, Uo - U0)
    print(f"pulse 64^3, 200 steps ({'FP64' if precision == 0 else 'double-float'}): state {err:.2e}, "
          f"increment {inc:.2e}, t {s.t:.6f}")
    assert err <= TOL_RUN
    assert inc <= 1e-7
    assert abs(s.t - t) <= 1e-12 * t
    assert abs(s.next_dt - dt) <= 1e-12 * dt
    s.close()


def test_pulse_ten_steps_256(hype, oracle):
    from acoustic_petsc_gb300 import workloads

    n = 256
    U0 = workloads.euler_pulse(n)
    s = _euler(hype, n)
    s.set_state(U0)
    s.step(10)
    Ug, tg = s.get_state(), s.t
    s.close()
    Uo, t, dt, rc = oracle.euler_run(oracle.euler_cfg(n, 1.0 / n, cfl=0.4), U0, 10)
    assert rc == 0
    err = rel(Ug, Uo)
    inc = rel(Ug - U0, Uo - U0)
    print(f"pulse 256^3, 10 steps: state {err:.2e}, increment {inc:.2e}")
    assert err <= TOL_RUN
    assert inc <= 1e-7
    assert abs(tg - t) <= 1e-12 * t


def test_blast_500_steps_64(hype, oracle):
    from acoustic_petsc_gb300 import workloads

    n = 64
    U0 = workloads.euler_blast(n)
    s = _euler(hype, n, positivity=1)
    s.set_state(U0)
    s.indicator_stats(reset=True)
    for _ in range(10):
        s.step(50)
    _, fb_gpu = s.indicator_stats()
    Ug, tg = s.get_state(), s.t
    s.close()
    cfg = oracle.euler_cfg(n, 1.0 / n, cfl=0.4, positivity=1)
    oracle.lib().orc_positivity_fallbacks(1)
    Uo, t, dt, rc = oracle.euler_run(cfg, U0, 500)
    fb_orc = oracle.lib().orc_positivity_fallbacks(1)
    assert rc == 0
    err = rel(Ug, Uo)
    print(f"blast 64^3, 500 steps: state {err:.2e}, t {tg:.5f}; fallbacks GPU {fb_gpu}, checker {fb_orc}")
    assert err <= TOL_RUN
    assert fb_gpu == fb_orc
    assert abs(tg - t) <= 1e-12 * t


def test_batch_2000_steps(hype, oracle):
    from acoustic_petsc_gb300 import workloads

    inst = workloads.monopole_batch(256, seed=7, nmin=64, nmax=1024)
    b = hype.BatchLeapfrog([hype.Monopole(**m) for m in inst])
    b.step(2000)
    order = sorted(range(len(inst)), key=lambda q: inst[q]["nx"] * inst[q]["ny"])
    mid = len(order) // 2
    pick = order[:4] + order[mid - 2:mid + 2] + order[-2:]
    worst = 0.0
    for q in pick:
        m = inst[q]
        a, p = b.get(q)
        cfg = oracle.MonoCfg()
        for f, _ in oracle.MonoCfg._fields_:
            if f != "it0":
                setattr(cfg, f, m[f])
        cfg.it0 = 0
        z = np.zeros((m["ny"], m["nx"]))
        ao, po = oracle.ctcs_monopole(cfg, z, z, 2000)
        e = max(rel(p, po), rel(a, ao))
        print(f"instance {q} ({m['nx']}x{m['ny']}): {e:.2e}")
        worst = max(worst, e)
    b.close()
    assert worst <= TOL_RUN


def test_kapila_1024_bench_horizon(hype, oracle):
    from acoustic_petsc_gb300 import workloads as W

    n = 1024
    U, h = W.kapila_bubble(n, model=1)
    L = hype._lib
    m = hype.Multiphase2D(n, n, h, CFL=0.4, boundaries=(2, 2, 2, 2), model=1, eos=W.KAPILA_EOS,
                          stepper=L.STEP_SSPRK43, precision=0)
    cfg = oracle.mp2d_cfg(n, n, h, 0.0, 0.0, cfl=0.4, bc=(2, 2, 2, 2), model=1, eos=W.KAPILA_EOS)
    m.set_state(U)
    m.step(3)
    m.step(5)
    Uo, t, dt, rc = oracle.mp2d_run(cfg, U, 8, stepper=0)
    assert rc == 0
    Ug = m.get_state()
    print(f"Kapila 1024^2, 8 steps: state {rel(Ug, Uo):.2e}")
    assert np.array_equal(Ug, Uo)
    assert m.t == t
    m.close()
