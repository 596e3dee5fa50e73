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


def test_kapila_fp32_recon_flux_error_stated(hype, oracle):
    m, cfg, U = _kapila(hype, oracle, 96, 1, precision=1)
    m.set_state(U)
    m.step(12)
    Uo, t, dt, rc = oracle.mp2d_run(cfg, U, 12, stepper=0)
    rho = m.get_state()[..., 0] + m.get_state()[..., 1]
    rho_o = Uo[..., 0] + Uo[..., 1]
    l1 = float(np.abs(rho - rho_o).mean() / np.abs(rho_o).mean())
    print(f"Kapila FP32 recon/flux: L1(rho) rel err {l1:.2e} after 12 steps, state rel {rel(m.get_state(), Uo):.2e}")
    assert l1 <= 1e-3
