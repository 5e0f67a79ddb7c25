"""CPU: the receiver-function oracle (oracle/rf_oracle.py, a restatement of utils/makeRFitdecon.m).

MATLAB is not available here, so the builtins it relies on are pinned to their documented outputs,
and the deconvolution to its known answers: a numerator equal to the denominator gives one spike
at lag 0 of unit area; a numerator delayed by k samples gives the spike at lag k.
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import rf_oracle as RO  # noqa: E402


def test_matlab_builtins():
    assert np.array_equal(RO.conv_same(np.array([1.0, 2, 3]), np.array([1.0, 1])), [3, 5, 3])
    assert np.array_equal(RO.conv_same(np.array([1.0, 2, 3]), np.array([1.0, 1, 1])), [3, 6, 5])
    assert np.array_equal(RO.xcorr(np.array([1.0, 2, 3]), np.array([1.0, 1, 1]), 2), [1, 3, 6, 5, 3])
    assert np.array_equal(RO.xcorr(np.array([1.0, 2]), np.array([1.0, 0]), 3), [0, 0, 0, 1, 2, 0, 0])
    assert [RO.mround(v) for v in (0.5, -0.5, 2.5, -2.5, 1.49)] == [1, -1, 3, -3, 1]


def _pulse(nt, dt, t0, f=1.5):
    t = np.arange(nt) * dt - t0
    a = (np.pi * f * t) ** 2
    return (1 - 2 * a) * np.exp(-a)


def test_identity_and_delay():
    nt, dt = 500, 0.05
    den = _pulse(nt, dt, 12.5)                   # inside the samples the lags leave to the denominator
    rf, rms, p0 = RO.itdecon(den, den, dt, -5.0, 10.0, 0.0, 2.5, 20, 1e-3)
    ml = max(100, 200)
    k = int(np.argmax(np.abs(p0)))
    assert k == ml                               # the spike at lag 0
    assert abs(p0[k] - 1.0) < 0.05               # of unit amplitude
    assert rms[-1] < 1e-3
    num = np.zeros(nt)
    num[40:] = den[:-40]                         # delayed by 40 samples = 2 s
    rf, rms, p0 = RO.itdecon(num, den, dt, -5.0, 10.0, 0.0, 2.5, 20, 1e-3)
    assert int(np.argmax(np.abs(p0))) == ml + 40
    assert rms[-1] < 1e-3


def test_lag_halving_and_windows():
    assert RO.plan(100, 0.1, -20.0, 20.0) == (50, 50)             # 200 + 200 lags > 100: halved twice
    assert RO.plan(100, 0.1, 0.0, 5.0) == (0, 50)
    ml = 50
    assert RO.output_window(ml, -50, 50, 101, 0.1, 0.0) == (0, 101)
    assert RO.output_window(ml, 0, 50, 101, 0.1, 0.0) == (50, 101)
    assert RO.output_window(ml, 0, 50, 101, 0.1, 1.0) == (40, 101)     # 1 s of lead time
    assert RO.output_window(ml, 0, 50, 101, 0.1, 9.0) == (0, 101)      # past the start: from the first sample
    assert RO.output_window(ml, 0, 50, 101, 0.1, -1.0) == (60, 101)    # negative shift: truncated
