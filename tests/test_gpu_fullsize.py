"""GPU: size-independent properties at the full config-2 size (4001 x 2001 cells at 100 m, 40-cell
absorbing layers, the dipping-Moho / basin / perturbed model, 401 surface receivers).

Receivers sit 20 cells above the bottom strips, where the upgoing plane wave enters in 400 steps.

* Linearity: the step is linear in the background, so doubling every background strip doubles
  every seismogram sample and field value, to rounding (not bit for bit: the plane wave's
  exponential tails reach the subnormal range, where rounding is absolute rather than relative, and
  the few-ulp differences spread through the field).
* Determinism: two runs give bit-identical traces (no order-dependent reductions, no races between
  the concurrent kernels of a step).
* The two kernel paths agree: with every cell on the tiled kernel (FDFK_TILED_ONLY=1) the traces
  match the fast-path run to rounding.
"""
import os

import numpy as np
import pytest

from fdfk2d_gb300 import workloads as WL

pytestmark = pytest.mark.gpu
NT = 400     # 2.4 s: the plane wave's pulse (peak at 1.5 s at the bottom strips) enters the grid


@pytest.fixture(scope="module")
def F():
    import fdfk2d_gb300 as F
    from fdfk2d_gb300 import build
    build.build()
    F.lib()
    return F


@pytest.fixture(scope="module")
def case():
    w = WL.config2(nt=NT)
    strips = WL.plane_wave_background(w, amp=1e-3)
    p = w["p"]
    w["rz"] = np.full_like(w["rz"], (p["nz"] - 21) * p["dz"])      # a row 20 cells above the bottom strips
    return w, strips


def _run(F, w, strips, scale=1.0, tiled_only=False):
    old = os.environ.get("FDFK_TILED_ONLY")
    os.environ["FDFK_TILED_ONLY"] = "1" if tiled_only else "0"
    try:
        with F.Session(w["p"], w["c"]) as s:
            s.upload_background({k: (v * np.float32(scale)).astype(np.float32, order="F") for k, v in strips.items()})
            s.set_receivers(w["rx"], w["rz"], w["x0"], w["z0"], 1, NT)
            s.advance(NT + 1)
            sx, sz = s.seismograms()
            snap_x, snap_z = s.snapshot()
    finally:
        if old is None:
            os.environ.pop("FDFK_TILED_ONLY", None)
        else:
            os.environ["FDFK_TILED_ONLY"] = old
    return sx, sz, snap_x, snap_z


def test_linear_and_deterministic(F, case):
    w, strips = case
    a = _run(F, w, strips)
    b = _run(F, w, strips)
    d = _run(F, w, strips, scale=2.0)
    assert np.abs(a[1]).max() > 0 and np.abs(a[3]).max() > 0          # the wave is inside the grid
    for x, y, z in zip(a, b, d):
        assert np.array_equal(x, y)                                  # deterministic
        dev = np.abs(z - 2.0 * x).max() / np.abs(2.0 * x).max()
        assert dev <= 1e-5, dev                                      # linear


def test_tiled_path_matches_fast_path(F, case):
    w, strips = case
    fast = _run(F, w, strips)
    tiled = _run(F, w, strips, tiled_only=True)
    for x, y in zip(fast, tiled):
        scale = np.abs(y).max()
        assert scale > 0
        assert np.abs(x - y).max() <= 1e-4 * scale
