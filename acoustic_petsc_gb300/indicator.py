"""Learned troubled-cell indicator (no counterpart in the reference).

A 25 -> 32 -> 32 -> 1 network (BF16 weights, FP32 accumulation) scores each
cell from the normalised 5-point stencils of its 5 conserved variables along x,
y and z (max of the three logits).  Labels come from the solver itself: a cell
is troubled when its CWENO4 nonlinear weights depart from the linear ones enough
to move one of its face traces by more than ``tau`` of the cell's magnitude
(``hype_euler_sample_features``).  Training, scoring and inference run in the library's own
CUDA kernels (``hype_mlp_*``, ``HYPE_RECON_LEARNED``).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import check

NIN, NH = 25, 32
NPARAM = NH * NIN + NH + NH * NH + NH + NH + 1


def _fp(a: np.ndarray):
    if a.dtype != np.float32 or not a.flags.c_contiguous:
        raise ValueError("float32 C-contiguous array required")
    return a.ctypes.data_as(L.F)


def init_params(seed: int = 0) -> np.ndarray:
    """He-initialised parameters, zero biases, output bias favouring 'smooth'."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, dtype=np.float32)
    o = 0
    p[o:o + NH * NIN] = rng.normal(0, np.sqrt(2.0 / NIN), NH * NIN)
    o += NH * NIN + NH
    p[o:o + NH * NH] = rng.normal(0, np.sqrt(2.0 / NH), NH * NH)
    o += NH * NH + NH
    p[o:o + NH] = rng.normal(0, np.sqrt(1.0 / NH), NH)
    p[-1] = -2.0
    return p


def sample(solver, stride: int = 1):
    """(X[n][3][25], D[n]) from the solver's resident state (3D Euler or 2D multiphase)."""
    if hasattr(solver, "sample_features"):
        return solver.sample_features(stride)
    n = (solver.ctx.N_x * solver.ctx.N_y * solver.ctx.N_z + stride - 1) // stride
    X = np.empty((n, 3, NIN), dtype=np.float32)
    D = np.empty(n, dtype=np.float32)
    ns = C.c_longlong()
    check(L.lib().hype_euler_sample_features(solver._h, stride, _fp(X), _fp(D), C.byref(ns)), "sample_features")
    return X, D


def score(X: np.ndarray, params: np.ndarray) -> np.ndarray:
    X = np.ascontiguousarray(X, dtype=np.float32)
    out = np.empty(X.shape[0], dtype=np.float32)
    check(L.lib().hype_mlp_score(_fp(X), X.shape[0], _fp(np.ascontiguousarray(params, np.float32)), _fp(out)), "mlp_score")
    return out


def grad(X: np.ndarray, y: np.ndarray, params: np.ndarray, pos_weight: float = 1.0):
    """(gradient of the summed loss, summed loss) computed by the GPU backward kernel"""
    X = np.ascontiguousarray(X, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    g = np.empty(NPARAM, dtype=np.float32)
    loss = C.c_double()
    check(L.lib().hype_mlp_grad(_fp(X), _fp(y), X.shape[0], _fp(np.ascontiguousarray(params, np.float32)),
                                float(pos_weight), _fp(g), C.byref(loss)), "mlp_grad")
    return g, loss.value


def train(X: np.ndarray, y: np.ndarray, params: np.ndarray | None = None, epochs: int = 6, batch: int = 4096,
          lr: float = 3e-3, pos_weight: float | None = None, seed: int = 0):
    """Adam training on the GPU; returns (params, mean loss of the last epoch)."""
    X = np.ascontiguousarray(X, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    p = init_params(seed) if params is None else np.array(params, dtype=np.float32, copy=True)
    if pos_weight is None:
        pos = float(y.mean())
        pos_weight = 1.0 if pos <= 0.0 or pos >= 1.0 else min(50.0, (1.0 - pos) / pos)
    loss = C.c_double()
    check(L.lib().hype_mlp_train(_fp(X), _fp(y), X.shape[0], _fp(p), epochs, batch, float(lr), float(pos_weight),
                                 int(seed) & 0xFFFFFFFF, C.byref(loss)), "mlp_train")
    return p, loss.value


def labels(D: np.ndarray, tau: float) -> np.ndarray:
    return (D > tau).astype(np.float32)


def recall_precision(score_logits: np.ndarray, y: np.ndarray, prob_threshold: float):
    thr = np.log(prob_threshold / (1.0 - prob_threshold))
    pred = score_logits > thr
    tp = float(np.sum(pred & (y > 0.5)))
    return tp / max(float(np.sum(y > 0.5)), 1.0), tp / max(float(np.sum(pred)), 1.0), float(pred.mean())
