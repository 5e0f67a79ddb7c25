"""GPU parity: the sm_103a step and time loop against the reference's shipped libraries
(golden fixtures) and against the oracle, through the C ABI."""
import numpy as np
import pytest

from conftest import STEP_CASES, load_npz, max_rel, rel_l2, step_inputs

pytestmark = pytest.mark.gpu

# One FP32 GPU step vs one shipped step (float32 state): max |error| / max |value|.
STEP_TOL = 2e-5
# Seismograms after hundreds of steps: relative L2 per component, the bar of 1e-4.
TRACE_TOL = 1e-4


@pytest.fixture(scope="module")
def F():
    import fdfk2d_gb300 as F
    from fdfk2d_gb300 import build
    build.build()
    F.lib()
    return F


def _check_step(d, ux, uz, bp, bu, tol):
    assert max_rel(ux, d["out_ux"]) < tol
    assert max_rel(uz, d["out_uz"]) < tol
    for k, v in bp.items():
        if d["out_" + k].any():
            assert max_rel(v, d["out_" + k]) < tol, k
    for k, v in bu.items():
        if d["out_" + k].any():
            assert max_rel(v, d["out_" + k]) < tol, k


@pytest.mark.parametrize("name", STEP_CASES)
def test_dropin_updatedispl_matches_shipped(F, name):
    d = load_npz("step_" + name)
    p, strips, c, c0, c1, ux, uz, bp, bu = step_inputs(d)
    n0 = F.kernel_launches()
    F.updatedispl(p, strips, c, c0, c1, ux, uz, bp, bu, int(d["it"]))
    # the material conversion, then the step: tiled kernel, plus frame and fast path when they apply
    assert F.kernel_launches() - n0 in (2, 4)
    _check_step(d, ux, uz, bp, bu, STEP_TOL)


@pytest.mark.parametrize("name", STEP_CASES)
def test_session_step_matches_oracle(F, oracle_lib, name):
    d = load_npz("step_" + name)
    p, strips, c, c0, c1, ux, uz, bp, bu = step_inputs(d)
    ref = step_inputs(d)
    oracle_lib.updatedispl(*ref[:9], 0)
    with F.Session(p, c) as s:
        s.upload_background(strips)
        s.upload_state(ux, uz, bp, bu, 0)
        s.advance(1)
        s.download_state(ux, uz, bp, bu)
    assert max_rel(ux, ref[5]) < STEP_TOL
    assert max_rel(uz, ref[6]) < STEP_TOL
    for k in bu:
        if ref[8][k].any():
            assert max_rel(bu[k], ref[8][k]) < STEP_TOL, k


def test_time_loop_matches_shipped(F):
    d = load_npz("loop_layered")
    strips = {k: d[k] for k in F.STRIPS}
    sx, sz = F.simulate(d["p"], d["c"], strips, d["rx"], d["rz"], 0.0, 0.0, int(d["nstp"]), int(d["nsis"]))
    assert rel_l2(sx, d["seisx"]) < TRACE_TOL
    assert rel_l2(sz, d["seisz"]) < TRACE_TOL
    for r in range(sz.shape[1]):
        assert rel_l2(sz[:, r], d["seisz"][:, r]) < TRACE_TOL, r
        assert rel_l2(sx[:, r], d["seisx"][:, r]) < TRACE_TOL, r


def test_session_chunks_equal_one_shot(F):
    """Advancing in uneven chunks with background uploaded per chunk equals one call."""
    d = load_npz("loop_layered")
    p = d["p"]
    strips = {k: d[k] for k in F.STRIPS}
    ref = F.simulate(p, d["c"], strips, d["rx"], d["rz"], 0.0, 0.0, int(d["nstp"]), int(d["nsis"]))
    with F.Session(p, d["c"]) as s:
        s.set_receivers(d["rx"], d["rz"], 0.0, 0.0, int(d["nstp"]), int(d["nsis"]))
        t = 0
        for chunk in (1, 7, 50, 100, p["nt"] + 1):
            n = min(chunk, p["nt"] + 1 - t)
            if n <= 0:
                break
            s.upload_background(strips, t, n)
            s.advance(n)
            t += n
        s.synchronize()
        got = s.seismograms()
    np.testing.assert_array_equal(got[0], ref[0])
    np.testing.assert_array_equal(got[1], ref[1])


def _random_case(seed, nx, nz, npml, norder, nt, dx=200.0, dz=200.0, dt=0.006):
    rng = np.random.default_rng(seed)
    NZ, NX = nz + npml, nx + 2 * npml
    vp = 4000 + 3000 * rng.random((NZ, NX))
    vs = vp / (1.65 + 0.3 * rng.random((NZ, NX)))
    rho = 1740.0 * (vp / 1000.0) ** 0.25
    c = np.zeros((3, NZ, NX), np.float32, order="F")
    c[0], c[1], c[2] = rho, rho * (vp * vp - 2 * vs * vs), rho * vs * vs
    nbd = 2 * norder - 1
    import fdfk2d_gb300 as F
    t = np.arange(nt + 1) * dt
    strips = {}
    for k, s in F.strip_shapes(nx, nz, nbd, nt).items():
        # a smooth, seeded background: a Ricker pulse with random spatial phase per strip cell
        ph = rng.random(s[:2])[..., None] * 0.3
        arg = (np.pi * 4.0 * (t[None, None, :] - 0.4 - ph)) ** 2
        strips[k] = np.asfortranarray(((1 - 2 * arg) * np.exp(-arg) * 1e-3).astype(np.float32))
    p = dict(norder=norder, nx=nx, nz=nz, npml=npml, nt=nt, dx=dx, dz=dz, dt=dt,
             vpml=float(np.sqrt((c[1] + 2 * c[2]) / c[0]).max()), R0=1e-3, npower=2)
    rx = np.linspace(0.0, (nx - 1) * dx, 9).astype(np.float32)
    rz = np.linspace(0.0, (nz - 1) * dz * 0.6, 9).astype(np.float32)
    return p, c, strips, rx, rz


@pytest.mark.parametrize("norder,npml,nstp", [(3, 10, 1), (2, 6, 3), (4, 9, 2), (1, 3, 1), (8, 15, 4)])
def test_time_loop_matches_oracle(F, oracle_lib, norder, npml, nstp):
    nt = 180
    p, c, strips, rx, rz = _random_case(100 + norder, 70, 37, npml, norder, nt)
    nsis = nt // nstp
    gx, gz = F.simulate(p, c, strips, rx, rz, 0.0, 0.0, nstp, nsis)
    ox, oz = oracle_lib.simulate(dict(p, izt=1, nbd=2 * norder - 1), strips, c, rx, rz, 0.0, 0.0, nstp, nsis)
    assert rel_l2(gx, ox) < TRACE_TOL
    assert rel_l2(gz, oz) < TRACE_TOL


def test_errors_are_reported(F):
    p, c, strips, rx, rz = _random_case(1, 40, 20, 6, 3, 10)
    with F.Session(p, c) as s:
        with pytest.raises(F.FDFKError) as e:
            s.advance(1)
        assert e.value.code == -5
        s.upload_background(strips)
        with pytest.raises(F.FDFKError):
            s.set_receivers([1e9], [0.0], 0.0, 0.0, 1, 10)
        with pytest.raises(F.FDFKError):
            s.advance(p["nt"] + 2)
        s.advance(p["nt"] + 1)
        assert s.step_index == p["nt"] + 1


def _random_state(seed, p):
    rng = np.random.default_rng(seed)
    import fdfk2d_gb300 as F
    NZ, NX = p["nz"] + p["npml"], p["nx"] + 2 * p["npml"]
    ux = np.asfortranarray(rng.standard_normal((2, NZ, NX)).astype(np.float32))
    uz = np.asfortranarray(rng.standard_normal((2, NZ, NX)).astype(np.float32))
    ps = F.pml_shapes(p["nx"], p["nz"], p["npml"])
    bp = {k: np.asfortranarray((1e3 * rng.standard_normal(ps[k])).astype(np.float32)) for k in F.BP}
    bu = {k: np.asfortranarray(rng.standard_normal(ps[k]).astype(np.float32)) for k in F.BU}
    strips = {k: np.asfortranarray(rng.standard_normal(s).astype(np.float32))
              for k, s in F.strip_shapes(p["nx"], p["nz"], 2 * p["norder"] - 1, p["nt"]).items()}
    return ux, uz, bp, bu, strips


def _gpu_step(F, p, c, state, tiled_only, seg=0):
    import os
    ux, uz, bp, bu, strips = [x.copy() if isinstance(x, np.ndarray) else {k: v.copy(order="F") for k, v in x.items()}
                              for x in state]
    ux = np.asfortranarray(ux); uz = np.asfortranarray(uz)
    old = os.environ.get("FDFK_TILED_ONLY")
    os.environ["FDFK_TILED_ONLY"] = "1" if tiled_only else "0"
    try:
        with F.Session(p, c) as s:
            if seg:
                s.set_tuning(seg, 0)
            s.upload_background(strips)
            s.upload_state(ux, uz, bp, bu, 0)
            s.advance(1)
            s.download_state(ux, uz, bp, bu)
    finally:
        if old is None:
            os.environ.pop("FDFK_TILED_ONLY", None)
        else:
            os.environ["FDFK_TILED_ONLY"] = old
    return ux, uz


@pytest.mark.parametrize("norder", [1, 2, 3, 4])
def test_interior_fast_path_matches_tiled_path_and_oracle(F, oracle_lib, norder):
    """The marching interior kernel and the tiled kernel give the same step (random state, strips
    and heterogeneous material, a grid large enough for several bands and segments)."""
    npml = 2 * norder + 3
    p, c, _, _, _ = _random_case(7 + norder, 150, 141, npml, norder, 0)
    state = _random_state(70 + norder, p)
    mx, mz = _gpu_step(F, p, c, state, tiled_only=False)
    tx, tz = _gpu_step(F, p, c, state, tiled_only=True)
    assert max_rel(mx, tx) < STEP_TOL
    assert max_rel(mz, tz) < STEP_TOL
    ux, uz, bp, bu, strips = state
    ox, oz = ux.copy(order="F"), uz.copy(order="F")
    oracle_lib.updatedispl(dict(p, izt=1, nbd=2 * norder - 1), strips, c, oracle_lib.fd_coef0(norder),
                           oracle_lib.fd_coef1(norder), ox, oz, {k: v.copy(order="F") for k, v in bp.items()},
                           {k: v.copy(order="F") for k, v in bu.items()}, 0)
    assert max_rel(mx, ox) < STEP_TOL
    assert max_rel(mz, oz) < STEP_TOL


def test_tuning_changes_no_result(F):
    """Every launch shape gives the same bits (the autotuner may pick any of them)."""
    d = load_npz("loop_layered")
    p = dict(d["p"])
    strips = {k: d[k] for k in F.STRIPS}
    seg, run, ms = F.autotune(p, d["c"], steps=5)
    assert seg >= 16 and 12 <= run <= 48 and ms > 0
    out = []
    for tune in ((0, 0), (16, 12), (96, 48), (seg, run)):
        with F.Session(p, d["c"]) as s:
            s.set_tuning(*tune)
            s.upload_background(strips)
            s.set_receivers(d["rx"], d["rz"], 0.0, 0.0, int(d["nstp"]), int(d["nsis"]))
            s.advance(p["nt"] + 1)
            out.append(s.seismograms())
    for sx, sz in out[1:]:
        assert np.array_equal(sx, out[0][0]) and np.array_equal(sz, out[0][1])


def test_tuning_rejects_tiles_beyond_shared_memory(F):
    """At the highest order, 64-cell runs across a 40-cell layer need more shared memory than a
    block has: set_tuning refuses them (and keeps the current shapes), and the autotuner skips
    such candidates."""
    from test_gpu_batch import _layered
    nx, nz, npml, h = 40, 30, 40, 250.0
    c, fk, vmax = _layered(nx, nz, npml, h, 3000.0)
    p = dict(norder=8, nx=nx, nz=nz, npml=npml, nbd=15, nt=10, dx=h, dz=h, dt=0.004, vpml=vmax, npower=2, R0=1e-3)
    with F.Session(p, c) as s:
        before = s.tuning()
        with pytest.raises(F.FDFKError):
            s.set_tuning(0, 64)
        assert s.tuning() == before
        s.set_tuning(0, 16)
    seg, run, ms = F.autotune(p, c, steps=2)
    assert 12 <= run <= 48 and ms > 0


@pytest.mark.parametrize("nx,nz,npml,seg", [(10, 8, 5, 0),      # two fast-path rows, one short segment
                                            (97, 53, 5, 16),    # one partial band, ragged last segment, minimum layer
                                            (131, 59, 9, 24),   # a second band holding one row
                                            (64, 121, 7, 64)])  # segment length equal to nx
def test_ragged_shapes_fast_path_matches_tiled_path_and_oracle(F, oracle_lib, nx, nz, npml, seg):
    """Order 6 on grids whose rows and columns do not divide into the fast path's bands and
    segments, including the thinnest absorbing layer (material columns left of the grid)."""
    norder = 3
    p, c, _, _, _ = _random_case(nx + nz, nx, nz, npml, norder, 0)
    state = _random_state(nx * nz, p)
    mx, mz = _gpu_step(F, p, c, state, tiled_only=False, seg=seg)
    tx, tz = _gpu_step(F, p, c, state, tiled_only=True)
    assert max_rel(mx, tx) < STEP_TOL
    assert max_rel(mz, tz) < STEP_TOL
    ux, uz, bp, bu, strips = state
    ox, oz = ux.copy(order="F"), uz.copy(order="F")
    oracle_lib.updatedispl(dict(p, izt=1, nbd=2 * norder - 1), strips, c, oracle_lib.fd_coef0(norder),
                           oracle_lib.fd_coef1(norder), ox, oz, {k: v.copy(order="F") for k, v in bp.items()},
                           {k: v.copy(order="F") for k, v in bu.items()}, 0)
    assert max_rel(mx, ox) < STEP_TOL
    assert max_rel(mz, oz) < STEP_TOL
