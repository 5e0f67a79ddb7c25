"""GPU: the PML-on-top mode (is_PML_top: izt = 1 - npml, an absorbing layer of npml rows above row 1).

* The drop-in ``updatedispl_`` against the shipped library's step (fixtures step_top_*.npz made by
  tests/golden/make_golden.py): wavefield levels, memory variables and split fields.
* Whole time loops through the C ABI against the oracle's restatement of the mode
  (oracle/fdfk_oracle.c, item 5), receivers on the surface (whose 7 x 7 sampling reaches into
  the top layer) and below it.
* The fast path and the all-tiled path agree, every launch shape gives the same bits, and batched
  members (their top layers in one more launch after the step's interior) match their solves alone.
"""
import os

import numpy as np
import pytest

from conftest import STEP_CASES_TOP, load_npz, max_rel, rel_l2, step_inputs

pytestmark = pytest.mark.gpu

STEP_TOL = 2e-5      # one FP32 step against the shipped FP32 step
TRACE_TOL = 1e-4     # seismograms after hundreds of steps, relative L2 per component


@pytest.fixture(scope="module")
def F():
    import fdfk2d_gb300 as F
    from fdfk2d_gb300 import build
    build.build()
    F.lib()
    return F


def _top_case(seed, nx, nz, npml, norder, nt, dx=200.0, dz=200.0, dt=0.006):
    """Heterogeneous random material over rows 1-npml..nz+npml and a smooth seeded background."""
    rng = np.random.default_rng(seed)
    NZ, NX = nz + 2 * npml, nx + 2 * npml
    vp = 4000 + 3000 * rng.random((NZ, NX))
    vs = vp / (1.65 + 0.3 * rng.random((NZ, NX)))
    rho = 1740.0 * (vp / 1000.0) ** 0.25
    c = np.zeros((3, NZ, NX), np.float32, order="F")
    c[0], c[1], c[2] = rho, rho * (vp * vp - 2 * vs * vs), rho * vs * vs
    nbd = 2 * norder - 1
    import fdfk2d_gb300 as Fm
    t = np.arange(nt + 1) * dt
    strips = {}
    for k, s in Fm.strip_shapes(nx, nz, nbd, nt).items():
        ph = rng.random(s[:2])[..., None] * 0.3
        arg = (np.pi * 4.0 * (t[None, None, :] - 0.4 - ph)) ** 2
        strips[k] = np.asfortranarray(((1 - 2 * arg) * np.exp(-arg) * 1e-3).astype(np.float32))
    p = dict(norder=norder, nx=nx, nz=nz, npml=npml, nt=nt, dx=dx, dz=dz, dt=dt, is_PML_top=True,
             vpml=float(np.sqrt((c[1] + 2 * c[2]) / c[0]).max()), R0=1e-3, npower=2)
    rx = np.linspace(0.0, (nx - 1) * dx, 9).astype(np.float32)
    rz = np.concatenate([np.zeros(5), np.linspace(dz, (nz - 1) * dz * 0.6, 4)]).astype(np.float32)
    return p, c, strips, rx, rz


@pytest.mark.parametrize("name", STEP_CASES_TOP)
def test_dropin_step_matches_shipped(F, name):
    d = load_npz("step_" + name)
    p, strips, c, c0, c1, ux, uz, bp, bu = step_inputs(d)
    assert p["is_PML_top"] and p["izt"] == 1 - p["npml"]
    F.updatedispl(p, strips, c, c0, c1, ux, uz, bp, bu, int(d["it"]))
    assert max_rel(ux, d["out_ux"]) < STEP_TOL
    assert max_rel(uz, d["out_uz"]) < STEP_TOL
    for k, v in list(bp.items()) + list(bu.items()):
        if d["out_" + k].any():
            assert max_rel(v, d["out_" + k]) < STEP_TOL, k


@pytest.mark.parametrize("norder,npml,nstp", [(3, 10, 1), (2, 7, 2), (1, 3, 1), (4, 9, 1)])
def test_time_loop_matches_oracle(F, oracle_lib, norder, npml, nstp):
    nt = 180
    p, c, strips, rx, rz = _top_case(300 + norder, 70, 37, npml, norder, nt)
    nsis = nt // nstp
    gx, gz = F.simulate(p, c, strips, rx, rz, 0.0, 0.0, nstp, nsis)
    q = dict(p, izt=1 - npml, nbd=2 * norder - 1)
    ox, oz = oracle_lib.simulate(q, strips, c, rx, rz, 0.0, 0.0, nstp, nsis)
    assert np.abs(oz).max() > 0
    assert rel_l2(gx, ox) < TRACE_TOL
    assert rel_l2(gz, oz) < TRACE_TOL
    for r in range(len(rx)):
        assert rel_l2(gz[:, r], oz[:, r]) < TRACE_TOL


def _solve(F, p, c, strips, rx, rz, tune=None):
    with F.Session(p, c) as s:
        if tune is not None:
            s.set_tuning(*tune)
        s.upload_background(strips)
        s.set_receivers(rx, rz, 0.0, 0.0, 1, p["nt"])
        s.advance(p["nt"] + 1)
        return s.seismograms()


def test_fast_path_tiled_path_and_tunings_agree(F):
    p, c, strips, rx, rz = _top_case(41, 90, 60, 12, 3, 150)
    fast = _solve(F, p, c, strips, rx, rz)
    old = os.environ.get("FDFK_TILED_ONLY")
    os.environ["FDFK_TILED_ONLY"] = "1"
    try:
        tiled = _solve(F, p, c, strips, rx, rz)
    finally:
        if old is None:
            os.environ.pop("FDFK_TILED_ONLY", None)
        else:
            os.environ["FDFK_TILED_ONLY"] = old
    for a, b in zip(fast, tiled):
        assert np.abs(a).max() > 0
        assert rel_l2(a, b) < 1e-5
    for tune in ((16, 12), (96, 48), (24, 13)):
        other = _solve(F, p, c, strips, rx, rz, tune)
        assert np.array_equal(other[0], fast[0]) and np.array_equal(other[1], fast[1]), tune


def test_batch_with_top_sessions_matches_each_alone(F):
    """Members with the absorbing layer on top (and one with a free surface) in one batch, with
    graph replay: every member's seismograms are the bits it gets alone."""
    cases = [_top_case(61, 70, 37, 10, 3, 140), _top_case(62, 55, 30, 9, 3, 100)]
    free = _top_case(63, 60, 33, 8, 3, 120)
    p_free = dict(free[0], is_PML_top=False)
    c_free = np.asfortranarray(free[1][:, free[0]["npml"]:, :])
    cases.append((p_free, c_free, free[2], free[3], free[4]))
    ref = [_solve(F, *cs) for cs in cases]
    sessions = []
    for p, c, strips, rx, rz in cases:
        s = F.Session(p, c)
        s.upload_background(strips)
        s.set_receivers(rx, rz, 0.0, 0.0, 1, p["nt"])
        sessions.append(s)
    with F.Batch(3, graph_chunk=16) as b:
        for s in sessions:
            b.add(s)
        b.advance(141)
        assert b.live() == 0
        got = [s.seismograms() for s in sessions]
    for (gx, gz), (rx_, rz_) in zip(got, ref):
        assert np.abs(gz).max() > 0
        assert np.array_equal(gx, rx_) and np.array_equal(gz, rz_)
    for s in sessions:
        s.close()
