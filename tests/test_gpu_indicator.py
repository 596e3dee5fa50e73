"""Learned troubled-cell indicator (no counterpart in the reference: parity is
unpinned; it is checked by its gradients against a CPU FP64 restatement and by
the accuracy of the gated solver against full CWENO4)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rand(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(-0.8, 0.8, size=(n, 3, 25)).astype(np.float32)
    y = (rng.random(n) < 0.3).astype(np.float32)
    return X, y


def test_forward_matches_cpu_restatement(hype):
    from acoustic_petsc_gb300 import indicator
    from oracle import mlp_oracle

    X, _ = _rand(2000, 1)
    p = indicator.init_params(3)
    s_gpu = indicator.score(X, p)
    # tensor-core inference: BF16 inputs and first hidden layer, FP32 accumulation; the
    # FP32 sums can round a hidden value to the neighbouring BF16 number (2^-8 relative)
    s_cpu = mlp_oracle.logits(X, p, act_bf16=True).max(axis=1)
    err = np.abs(s_gpu - s_cpu)
    scale = max(1.0, np.abs(s_cpu).max())
    assert err.max() <= 2e-3 * scale
    assert np.median(err) <= 1e-5 * scale


def test_backward_matches_cpu_restatement(hype):
    """GPU backward kernel (FP32 accumulation, BF16 weights) vs FP64 gradient of the same network."""
    from acoustic_petsc_gb300 import indicator
    from oracle import mlp_oracle

    X, y = _rand(3000, 2)
    p = indicator.init_params(4)
    g_gpu, l_gpu = indicator.grad(X, y, p, pos_weight=2.5)
    l_cpu, g_cpu = mlp_oracle.loss_and_grad(X, y, p, pos_weight=2.5)
    assert abs(l_gpu - l_cpu) <= 1e-5 * abs(l_cpu)
    assert np.abs(g_gpu - g_cpu).max() <= 2e-4 * np.abs(g_cpu).max()


def _blast_solver(hype, n, precision=0, recon=0):
    from acoustic_petsc_gb300 import workloads

    U0 = workloads.euler_blast(n)
    ctx = hype.AppCtx(N_x=n, N_y=n, N_z=n, h=1.0 / n, CFL=0.4, precision=precision, recon=recon, positivity=1)
    s = hype.EulerSolver(ctx)
    s.set_state(U0)
    return s, U0


def _train_on_blast(hype, n=32, tau=0.01):
    from acoustic_petsc_gb300 import indicator

    s, _ = _blast_solver(hype, n)
    Xs, Ds = [], []
    for _ in range(4):
        s.step(3)
        X, D = indicator.sample(s)
        Xs.append(X)
        Ds.append(D)
    X, D = np.concatenate(Xs), np.concatenate(Ds)
    y = indicator.labels(D, tau)
    p, loss = indicator.train(X, y, epochs=12, batch=2048, lr=3e-3, seed=0)
    return p, X, y, loss


def test_training_learns_the_solver_labels(hype):
    from acoustic_petsc_gb300 import indicator

    p, X, y, loss = _train_on_blast(hype)
    assert 0.0 < y.mean() < 0.5
    recall, precision, flagged = indicator.recall_precision(indicator.score(X, p), y, 0.2)
    print(f"indicator: recall {recall:.3f} precision {precision:.3f} flagged {flagged:.3f} (labels {y.mean():.3f})")
    assert recall >= 0.9 and flagged <= 0.6


def test_learned_indicator_gain(hype):
    """Against the method without it: the gated solver sends most cells to the
    cheap R4 path, and its density stays within 1.05x of full CWENO4's distance
    from a finer-grid FP64 reference; the shadow step measures the deviation."""
    p, _, _, _ = _train_on_blast(hype)
    n = 32
    ref, _ = _blast_solver(hype, 2 * n)
    full, _ = _blast_solver(hype, n)
    learned, _ = _blast_solver(hype, n, recon=hype._lib.RECON_LEARNED)
    learned.set_mlp(p, 0.2)
    learned.indicator_stats(reset=True)
    T = 0.02
    nsteps = {}
    for name, s in (("ref", ref), ("full", full), ("learned", learned)):
        nsteps[name] = 0
        while s.t < T:
            s.step(1)
            nsteps[name] += 1
    rho_ref = ref.get_state()[..., 0].reshape(n, 2, n, 2, n, 2).mean(axis=(1, 3, 5))
    e_full = np.abs(full.get_state()[..., 0] - rho_ref).mean()
    e_learn = np.abs(learned.get_state()[..., 0] - rho_ref).mean()
    flagged, fallbacks = learned.indicator_stats()
    frac = flagged / (n**3 * 4.0 * nsteps["learned"])
    shadow = learned.shadow_step()
    print(f"L1 vs 2x reference: full {e_full:.3e} learned {e_learn:.3e}; flagged/cell-stage {frac:.3f} "
          f"positivity fallbacks {fallbacks}; shadow L1 {shadow:.2e}")
    assert e_learn <= 1.05 * e_full
    assert shadow < 1e-3
