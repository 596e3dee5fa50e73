"""The 3D Euler CWENO4 + Rusanov + SSPRK(4,3) workload at its full size (256^3 cells on [0,1]^3,
periodic, Gaussian acoustic pulse dp = 1e-3 exp(-r^2/(2*0.04^2)), CFL 0.4) on the GPU: one step
against the CPU checker (relative L-inf <= 1e-12, its multi-threaded restatement of the
reference's RHSFunction), then size-independent properties over further steps: conservation
of mass, momentum and energy under periodic boundaries, and the pulse's symmetries (axis
permutations and reflections) kept to round-off."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 256


def _solver(hype, precision=0):
    ctx = hype.AppCtx(N_x=N, N_y=N, N_z=N, h=1.0 / N, CFL=0.4, precision=precision)
    return hype.EulerSolver(ctx)


@pytest.fixture(scope="module")
def pulse():
    from acoustic_petsc_gb300 import workloads

    return workloads.euler_pulse(N)


def test_one_step_vs_oracle_256(hype, oracle, pulse):
    s = _solver(hype)
    s.set_state(pulse)
    s.step(1)
    Ug = s.get_state()
    t_g = s.t
    s.close()
    Uo, t, dt, rc = oracle.euler_run(oracle.euler_cfg(N, 1.0 / N, cfl=0.4), pulse, 1)
    assert rc == 0
    err = float(np.abs(Ug - Uo).max() / np.abs(Uo).max())
    # the increment (dp ~ 1e-3 of the state) agrees as well
    inc = float(np.abs((Ug - pulse) - (Uo - pulse)).max() / np.abs(Uo - pulse).max())
    print(f"256^3 one step: state {err:.2e}, increment {inc:.2e}")
    assert err <= 1e-12
    assert inc <= 1e-9
    assert abs(t_g - t) <= 1e-14 * t


def _mirror(U, axis):
    """the state under the reflection x_axis -> 1 - x_axis (the normal momentum changes sign)"""
    V = np.flip(U, axis=2 - axis).copy()
    V[..., 1 + axis] = -V[..., 1 + axis]
    return V


def _swap_xy(U):
    V = np.swapaxes(U, 1, 2).copy()
    V[..., [1, 2]] = V[..., [2, 1]]
    return V


@pytest.mark.parametrize("precision", [0, 2])
def test_conservation_and_symmetry_256(hype, pulse, precision):
    s = _solver(hype, precision)
    s.set_state(pulse)
    s.step(6)
    U = s.get_state()
    s.close()
    dev = np.abs(U - pulse).max()
    assert 1e-6 < dev < 1e-2  # the pulse has moved, and stayed a small perturbation
    # conservation: periodic finite volumes change the totals only by round-off
    for c in (0, 4):
        tot0, tot = pulse[..., c].sum(dtype=np.float64), U[..., c].sum(dtype=np.float64)
        assert abs(tot - tot0) <= 1e-13 * abs(tot0), (c, tot, tot0)
    for c in (1, 2, 3):
        m = U[..., c]
        assert abs(m.sum()) <= 1e-10 * np.abs(m).sum(), c
    # symmetries of the centred pulse, relative to the perturbation
    bg = pulse[0, 0, 0]
    scale = np.abs(U - bg).max()
    for name, V in (("mirror x", _mirror(U, 0)), ("mirror y", _mirror(U, 1)), ("mirror z", _mirror(U, 2)),
                    ("swap x,y", _swap_xy(U))):
        sym = float(np.abs(V - U).max() / scale)
        assert sym <= 1e-9, (name, sym)
