"""GPU: batches of solves (different events, grid sizes and lengths) give each member exactly the
seismograms it gets alone, through the C ABI; graph replay and membership changes included."""
import numpy as np
import pytest

from conftest import load_npz

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F():
    import fdfk2d_gb300 as F
    from fdfk2d_gb300 import build
    build.build()
    F.lib()
    return F


def _layered(nx, nz, npml, h, moho):
    from fdfk2d_gb300 import workloads as W
    NZ, NX = nz + npml, nx + 2 * npml
    z = (np.arange(NZ) * h)[:, None] * np.ones((1, NX))
    vp = np.where(z < moho, 6300.0, 8100.0)
    vs = np.where(z < moho, 3600.0, 4500.0)
    fk = np.asfortranarray(np.array([[0.0, moho], [6300.0, 8100.0], [3600.0, 4500.0],
                                     list(W.gardner([6300.0, 8100.0]))], np.float32))
    return W.pack_c(vp, vs), fk, float(vp.max())


GRIDS = {
    "a": dict(norder=3, nx=40, nz=24, npml=8, nbd=5, dx=250.0, dz=250.0, dt=0.015, moho=3000.0),
    "b": dict(norder=3, nx=70, nz=33, npml=10, nbd=5, dx=200.0, dz=200.0, dt=0.012, moho=2400.0),
    "c": dict(norder=3, nx=24, nz=40, npml=6, nbd=5, dx=250.0, dz=250.0, dt=0.015, moho=5000.0),
}


def _session(F, grid, nt, rayp, p_wave, baz_deg, f0=2.0):
    g = GRIDS[grid]
    c, fk, vmax = _layered(g["nx"], g["nz"], g["npml"], g["dx"], g["moho"])
    p = dict(norder=g["norder"], nx=g["nx"], nz=g["nz"], npml=g["npml"], nbd=g["nbd"], nt=nt, dx=g["dx"],
             dz=g["dz"], dt=g["dt"], vpml=vmax, npower=2, R0=1e-3)
    fp = dict(nx=g["nx"], nz=g["nz"], npml=g["npml"], izt=1, nbd=g["nbd"], nt=nt, src_type=p_wave, x0=0.0, z0=0.0,
              dx=g["dx"], dz=g["dz"], dt=g["dt"], ds=1e-3, f0=f0, rayp=rayp)
    bazs = np.full(g["nx"] + 2 * g["npml"], np.deg2rad(baz_deg))
    s = F.Session(p, c)
    s.fk_background(fp, bazs, fk, fk)
    rx = np.arange(0.0, (g["nx"] - 1) * g["dx"] + 1, 3 * g["dx"], dtype=np.float32)
    s.set_receivers(rx, np.zeros_like(rx), 0.0, 0.0, 1, nt)
    return s


EVENTS = [("a", 240, 0.06e-3, True, 0.0), ("a", 240, 0.04e-3, True, 25.0), ("a", 240, 0.08e-3, True, 160.0),
          ("a", 240, 0.10e-3, False, 10.0), ("a", 240, 0.11e-3, False, 200.0), ("a", 240, 0.12e-3, False, 330.0)]


def _alone(F, spec):
    s = _session(F, *spec)
    s.advance(spec[1] + 1)
    out = s.seismograms()
    s.close()
    return out


@pytest.mark.parametrize("chunk", (32, 0))
def test_batch_of_events_matches_each_event_alone(F, chunk):
    ref = [_alone(F, e) for e in EVENTS]
    sessions = [_session(F, *e) for e in EVENTS]
    with F.Batch(3, graph_chunk=chunk) as b:
        for s in sessions:
            b.add(s)
        b.advance(241)
        assert b.live() == 0
        got = [s.seismograms() for s in sessions]
    for (gx, gz), (rx_, rz_) in zip(got, ref):
        assert np.abs(gz).max() > 0
        assert np.array_equal(gx, rx_) and np.array_equal(gz, rz_)
    for s in sessions:
        s.close()


def test_batch_of_uneven_solves_matches_alone(F):
    specs = [("a", 240, 0.06e-3, True, 0.0), ("b", 300, 0.07e-3, True, 15.0), ("c", 130, 0.11e-3, False, 180.0),
             ("b", 75, 0.05e-3, True, 350.0)]
    ref = [_alone(F, e) for e in specs]
    sessions = [_session(F, *e) for e in specs]
    n0 = F.kernel_launches()
    with F.Batch(3, graph_chunk=7) as b:
        for s in sessions:
            b.add(s)
        b.advance(150)
        b.advance(151)            # the longest member has 301 steps; the others stop at their own nt
        assert b.live() == 0
        # four launches per batch step (bump, tiled kernel, frame, fast path), whatever the number of members
        assert F.kernel_launches() - n0 == 4 * 301
        got = [s.seismograms() for s in sessions]
    for (gx, gz), (rx_, rz_) in zip(got, ref):
        assert np.array_equal(gx, rx_) and np.array_equal(gz, rz_)
    for s in sessions:
        s.close()


def test_member_leaves_midway_and_finishes_alone(F):
    specs = [("a", 240, 0.06e-3, True, 0.0), ("b", 200, 0.07e-3, True, 15.0), ("a", 240, 0.11e-3, False, 40.0)]
    ref = [_alone(F, e) for e in specs]
    sessions = [_session(F, *e) for e in specs]
    with F.Batch(3, graph_chunk=16) as b:
        for s in sessions:
            b.add(s)
        b.advance(100)
        b.remove(sessions[1])
        assert sessions[1].step_index == 100
        sessions[1].advance(101)          # finishes alone
        late = _session(F, "c", 120, 0.05e-3, True, 90.0)
        b.add(late)                        # joins while the others are half-way
        b.advance(141)
        got = [s.seismograms() for s in sessions]
        late_got = late.seismograms()
    for (gx, gz), (rx_, rz_) in zip(got, ref):
        assert np.array_equal(gx, rx_) and np.array_equal(gz, rz_)
    lx, lz = _alone(F, ("c", 120, 0.05e-3, True, 90.0))
    assert np.array_equal(late_got[0], lx) and np.array_equal(late_got[1], lz)
    for s in sessions + [late]:
        s.close()


def test_batch_refuses_member_calls(F):
    s = _session(F, "a", 40, 0.06e-3, True, 0.0)
    b = F.Batch(3)
    b.add(s)
    with pytest.raises(F.FDFKError) as e:
        s.advance(1)
    assert e.value.code == -5
    with pytest.raises(F.FDFKError) as e:
        b.add(s)
    assert e.value.code == -5
    b2 = F.Batch(2)
    t = _session(F, "a", 40, 0.06e-3, True, 0.0)
    with pytest.raises(F.FDFKError) as e:
        b2.add(t)
    assert e.value.code == -1
    b.close()
    s.advance(41)                          # an ordinary session again
    b2.close()
    s.close()
    t.close()


def test_batch_matches_shipped_loop(F):
    """The golden time loop (shipped step and FK) run as one member of a batch of two."""
    d = load_npz("loop_layered")
    p = dict(d["p"])
    strips = {k: d[k] for k in F.STRIPS}
    with F.Session(p, d["c"]) as s1, F.Session(p, d["c"]) as s2:
        for s in (s1, s2):
            s.upload_background(strips)
            s.set_receivers(d["rx"], d["rz"], 0.0, 0.0, int(d["nstp"]), int(d["nsis"]))
        with F.Batch(3) as b:
            b.add(s1)
            b.add(s2)
            b.advance(p["nt"] + 1)
            sx, sz = s1.seismograms()
            tx, tz = s2.seismograms()
    err = np.linalg.norm(sz - d["seisz"]) / np.linalg.norm(d["seisz"])
    assert err < 1e-4
    assert np.array_equal(sx, tx) and np.array_equal(sz, tz)


@pytest.mark.parametrize("seg,run", [(24, 16), (0, 13), (64, 0)])
def test_batch_tuning_changes_no_result(F, seg, run):
    """The batch's own launch shapes (segment columns, absorbing-layer tile length) give every
    member the bits it gets alone."""
    ref = [_alone(F, e) for e in EVENTS[:3]]
    sessions = [_session(F, *e) for e in EVENTS[:3]]
    with F.Batch(3, graph_chunk=16) as b:
        b.set_tuning(seg, run)
        for s in sessions:
            b.add(s)
        b.advance(120)
        b.set_tuning(0, 0)                 # back to the defaults half-way
        b.advance(121)
        got = [s.seismograms() for s in sessions]
    for (gx, gz), (rx_, rz_) in zip(got, ref):
        assert np.array_equal(gx, rx_) and np.array_equal(gz, rz_)
    with pytest.raises(F.FDFKError):
        b2 = F.Batch(3)
        try:
            b2.set_tuning(4, 0)
        finally:
            b2.close()
    for s in sessions:
        s.close()
