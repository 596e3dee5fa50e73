"""The double-float primitives behind HYPE_PREC_DF64 (df64.cuh), elementwise on the GPU:
the split of an FP64 value into an FP32 pair (rounded bit pattern) and back, and the pair
arithmetic against FP64 at its stated accuracy (~2^-48 relative)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _probe(hype, x, y):
    from acoustic_petsc_gb300 import _lib as L

    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    out = np.empty((len(x), 7))
    L.check(L.probes().hype_df64_probe(x.ctypes.data_as(L.D), y.ctypes.data_as(L.D), len(x),
                                    out.ctypes.data_as(L.D)), "hype_df64_probe")
    return out


def test_split_and_arithmetic(hype):
    rng = np.random.default_rng(5)
    n = 200000
    mag = 10.0 ** rng.uniform(-30, 30, n)
    x = mag * rng.choice([-1.0, 1.0], n) * (1 + rng.random(n))
    y = 10.0 ** rng.uniform(-30, 30, n) * rng.choice([-1.0, 1.0], n) * (1 + rng.random(n))
    # near-cancelling pairs and exact values
    x[:1000] = 1.0 + rng.random(1000) * 1e-9
    y[:1000] = 1.0 + rng.random(1000) * 1e-9
    x[1000:1010] = [0.0, -0.0, 1.0, -2.5, 0.1, 3.0, 1e-20, -7.0, 2.0**-100, 2.0**100]
    o = _probe(hype, x, y)
    hi, lo, back = o[:, 0], o[:, 1], o[:, 2]
    # hi is x rounded to FP32 (ties away from zero on the bit pattern; numpy rounds ties to
    # even, which differs only on exact ties), lo the remainder rounded likewise
    assert np.mean(hi == x.astype(np.float32).astype(np.float64)) > 0.9999
    assert np.all(hi.astype(np.float32) == hi) and np.all(lo.astype(np.float32) == lo)
    assert np.all(np.abs(lo) <= np.abs(np.spacing(hi.astype(np.float32)).astype(np.float64)) / 2 * (1 + 1e-7))
    # hi + lo carries 48 bits of x, except that a remainder x - hi below the FP32 normal
    # range (possible for |x| < 2^-74) flushes to zero: absolute error < 2^-126
    assert np.all(np.abs(back - x) <= np.maximum(2.0**-48 * np.abs(x), 2.0**-126))
    assert back[1000] == 0.0 and back[1001] == 0.0
    xs, ys = back, _probe(hype, y, y)[:, 2]  # the values the pair arithmetic actually saw
    # full accuracy (~2^-46) where operands and results lie in [2^-70, 2^100] (every lo part
    # an FP32 normal number); smaller magnitudes lose a flushed lo part
    tol = 2.0**-45

    def inrange(v):
        return (np.abs(v) >= 2.0**-70) & (np.abs(v) <= 2.0**100)

    ops = inrange(xs) & inrange(ys)
    for col, ref, scale in ((3, xs + ys, np.abs(xs) + np.abs(ys)), (4, xs - ys, np.abs(xs) + np.abs(ys)),
                            (5, xs * ys, np.abs(xs * ys)), (6, xs / ys, np.abs(xs / ys))):
        ok = ops & inrange(ref)
        assert ok.sum() > n // 4
        err = np.abs(o[:, col] - ref)
        assert np.all(err[ok] <= tol * scale[ok]), (col, float(np.max(err[ok] / scale[ok])))
