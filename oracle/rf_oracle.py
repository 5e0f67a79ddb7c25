"""Oracle (test infrastructure only): CPU restatement in float64 of the iterative
time-domain receiver-function deconvolution of utils/makeRFitdecon.m (Ligorria and
Ammon 1999, time-domain variant of that file).  Only tests/ may import this module.

MATLAB semantics restated here (the reference runs under MATLAB, which this
project does not have: parity unpinned against MATLAB itself; the restatement
follows the documented meaning of each builtin):
  conv(a, b, 'same')      central part of the full convolution, length of a,
                          starting at full index floor(len(b)/2) (0-based);
  xcorr(x, y, L, 'none')  R(m) = sum_n x(n+m) y(n), m = -L..L (zero outside);
  normpdf(x, mu, s)       exp(-(x-mu)^2 / (2 s^2)) / (s sqrt(2 pi));
  round                   half away from zero;
  max(abs(v))             first index of the largest magnitude.
"""
from __future__ import annotations

import numpy as np


def mround(x: float) -> int:
    """MATLAB round: half away from zero."""
    return int(np.sign(x) * np.floor(abs(x) + 0.5))


def conv_same(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    full = np.convolve(a, b)
    s = len(b) // 2
    return full[s:s + len(a)]


def xcorr(x: np.ndarray, y: np.ndarray, maxlag: int) -> np.ndarray:
    """R(m) = sum_n x[n+m] y[n] for m = -maxlag..maxlag (x and y of one length N)."""
    n = len(x)
    full = np.correlate(x, y, "full")          # lags -(N-1) .. N-1
    out = np.zeros(2 * maxlag + 1)
    for i, m in enumerate(range(-maxlag, maxlag + 1)):
        if -(n - 1) <= m <= n - 1:
            out[i] = full[m + n - 1]
    return out


def normpdf(x, mu, sigma):
    return np.exp(-0.5 * ((x - mu) / sigma) ** 2) / (sigma * np.sqrt(2.0 * np.pi))


def plan(ntin: int, dt: float, minlag: float, maxlag: float):
    """Lag counts after the reference's halving rule (utils/makeRFitdecon.m:87-100)."""
    endnlag = max(mround(maxlag / dt), 0)
    begnlag = max(mround(-minlag / dt), 0)
    while begnlag + endnlag > ntin:
        if begnlag > 0:
            minlag = 0.5 * minlag
            begnlag = max(mround(-minlag / dt), 0)
        if endnlag > 0:
            maxlag = 0.5 * maxlag
            endnlag = max(mround(maxlag / dt), 0)
    return begnlag, endnlag


def gauss_filter(ntin: int, dt: float, f0: float) -> np.ndarray:
    """gaussT of utils/makeRFitdecon.m:117-118."""
    sigma = 1.0 / (np.sqrt(2.0) * f0)
    return dt * normpdf(dt * np.arange(ntin), dt * mround(0.5 * ntin - 0.5), sigma)


def output_window(maxlag_n: int, lag1: int, lag2: int, nrfp: int, dt: float, tshift: float):
    """0-based slice [i1, i2) of the final filtered spike train (utils/makeRFitdecon.m:203-223)."""
    idx1 = maxlag_n + lag1 + 1
    idx2 = maxlag_n + lag2 + 1
    shifti = mround(tshift / dt)
    if shifti == 0:
        return idx1 - 1, idx2
    if shifti > 0:
        idx1 -= shifti
        if idx1 <= 0:
            return 0, idx2          # the reference prepends zeros(1, 1 - shifti), which is empty here
        return idx1 - 1, idx2
    idx1 -= shifti
    idx2 = min(nrfp, idx2 - shifti)
    return idx1 - 1, idx2


def itdecon(uin, win, dt, minlag, maxlag, tshift, f0, itmax, minderr):
    """[RFI, RMS] of utils/makeRFitdecon.m for one trace (float64)."""
    uin = np.asarray(uin, np.float64)
    win = np.asarray(win, np.float64)
    ntin = len(uin)
    if ntin == 0:
        raise ValueError("Zero length numerator")
    if len(win) < ntin:
        raise ValueError("numerator and denominator dimensions dont match")
    win = win[:ntin]
    begnlag, endnlag = plan(ntin, dt, minlag, maxlag)
    W = np.zeros(ntin)
    W[begnlag:ntin - endnlag] = win[begnlag:ntin - endnlag]
    g = gauss_filter(ntin, dt, f0)
    U = conv_same(uin, g)
    W = conv_same(W, g)
    R = U.copy()
    invpowU = 1.0 / np.sum(U ** 2)
    invpowW = 1.0 / np.sum(conv_same(win, g) ** 2)
    lag1, lag2 = -begnlag, endnlag
    ml = max(begnlag, endnlag)
    P0 = np.zeros(2 * ml + 1)
    lags = np.arange(-ml, ml + 1)
    ok = np.nonzero((lags >= lag1) & (lags <= lag2))[0]
    rms = []
    it = 0
    sumsq_i = 1.0
    d_error = 100.0 * np.sum(U ** 2) + minderr
    while abs(d_error) > minderr and it < itmax:
        it += 1
        RW = xcorr(R, W, ml) * invpowW
        k = ok[int(np.argmax(np.abs(RW[ok])))]
        P0[k] += RW[k]
        RFP = conv_same(P0, g)
        UP = conv_same(win, RFP)
        R = U - UP
        sumsq = np.sum(R ** 2) * invpowU
        rms.append(sumsq)
        d_error = 100.0 * (sumsq_i - sumsq)
        sumsq_i = sumsq
    RFP = conv_same(P0, g)
    i1, i2 = output_window(ml, lag1, lag2, len(RFP), dt, tshift)
    return RFP[i1:i2], np.array(rms), P0
