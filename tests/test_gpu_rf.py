"""GPU: receiver functions (fdfk_rf_itdecon) against the oracle restatement of utils/makeRFitdecon.m.

Both sides compute in FP64; they differ only in the order of their sums, so the spike lags and the
iteration counts must agree exactly and the values to ~1e-9 of the largest."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import rf_oracle as RO  # noqa: E402

pytestmark = pytest.mark.gpu
RF_TOL = 1e-9


@pytest.fixture(scope="module")
def F():
    import fdfk2d_gb300 as F
    from fdfk2d_gb300 import build
    build.build()
    F.lib()
    return F


def _pulse(nt, dt, t0, f):
    t = np.arange(nt) * dt - t0
    a = (np.pi * f * t) ** 2
    return (1 - 2 * a) * np.exp(-a)


def _synthetic(rng, nt, dt, nspk):
    den = _pulse(nt, dt, rng.uniform(0.3, 0.5) * nt * dt, rng.uniform(0.8, 2.0))
    rf = np.zeros(nt)
    for _ in range(nspk):
        rf[rng.integers(0, nt // 4)] += rng.normal()
    num = np.convolve(den, rf)[:nt] + 0.01 * rng.normal(size=nt)
    return num.astype(np.float32), (den + 0.01 * rng.normal(size=nt)).astype(np.float32)


def _compare(F, num, den, dt, minlag, maxlag, tshift, f0, itmax, minderr):
    rf, rms, its = F.receiver_functions(num, den, dt, minlag, maxlag, tshift, f0, itmax, minderr)
    if num.ndim == 1:
        rf, rms, its = rf[:, None], [rms], np.array([its])
        num, den = num[:, None], den[:, None]
    for j in range(num.shape[1]):
        rref, mref, _ = RO.itdecon(num[:, j].astype(np.float64), den[:, j].astype(np.float64), dt, minlag, maxlag,
                                   tshift, f0, itmax, minderr)
        assert rf.shape[0] == rref.size
        assert its[j] == mref.size, (j, its[j], mref.size)
        scale = max(np.abs(rref).max(), 1e-300)
        assert np.abs(rf[:, j] - rref).max() <= RF_TOL * scale, j
        assert np.allclose(rms[j], mref, rtol=1e-8, atol=1e-14), j


@pytest.mark.parametrize("minlag,maxlag,tshift,f0,itmax", [(0.0, 10.0, 0.0, 2.5, 100),
                                                          (-5.0, 0.0, 0.0, 4.0, 60),
                                                          (-2.0, 8.0, 1.0, 2.5, 100),
                                                          (0.0, 6.0, -0.5, 8.0, 30),
                                                          (-40.0, 40.0, 0.0, 2.5, 50)])   # lags halved to fit
def test_synthetic_traces_match_oracle(F, minlag, maxlag, tshift, f0, itmax):
    rng = np.random.default_rng(17)
    nt, dt = 600, 0.05
    pairs = [_synthetic(rng, nt, dt, k) for k in (1, 3, 6)]
    num = np.stack([p[0] for p in pairs], axis=1)
    den = np.stack([p[1] for p in pairs], axis=1)
    _compare(F, num, den, dt, minlag, maxlag, tshift, f0, itmax, 1e-3)


def test_single_trace_and_length_query(F):
    rng = np.random.default_rng(3)
    num, den = _synthetic(rng, 400, 0.04, 4)
    _compare(F, num, den, 0.04, 0.0, 5.0, 0.0, 2.5, 100, 1e-3)


def test_solve_seismograms(F):
    """P receiver functions of a small hybrid solve's traces, as utils/plot_PRF.m forms them."""
    from test_gpu_batch import _session
    s = _session(F, "b", 500, 0.06e-3, True, 20.0)
    s.advance(501)
    sx, sz = s.seismograms()
    s.close()
    dt = 0.012
    cols = [0, sx.shape[1] // 2, sx.shape[1] - 1]
    _compare(F, np.asfortranarray(sx[:, cols]), np.asfortranarray(sz[:, cols]), dt, 0.0, 3.0, 0.0, 8.0, 100, 1e-3)
