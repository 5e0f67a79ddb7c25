"""GPU: sessions bound to their own CUDA streams give the seismograms of sessions on the default
stream, bit for bit, including when the stream is bound right after creation (the state cleared
at creation is still queued on the default stream then) and when many sessions are created and
started while other sessions' FK backgrounds run (session setup waits for none of them)."""
import numpy as np
import pytest

from test_gpu_batch import GRIDS, _layered

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F():
    import fdfk2d_gb300 as F
    from fdfk2d_gb300 import build
    build.build()
    F.lib()
    return F


def _inputs(grid, nt, rayp, p_wave, baz_deg):
    g = GRIDS[grid]
    c, fk, vmax = _layered(g["nx"], g["nz"], g["npml"], g["dx"], g["moho"])
    p = dict(norder=g["norder"], nx=g["nx"], nz=g["nz"], npml=g["npml"], nbd=g["nbd"], nt=nt, dx=g["dx"],
             dz=g["dz"], dt=g["dt"], vpml=vmax, npower=2, R0=1e-3)
    fp = dict(nx=g["nx"], nz=g["nz"], npml=g["npml"], izt=1, nbd=g["nbd"], nt=nt, src_type=p_wave, x0=0.0, z0=0.0,
              dx=g["dx"], dz=g["dz"], dt=g["dt"], ds=1e-3, f0=2.0, rayp=rayp)
    bazs = np.full(g["nx"] + 2 * g["npml"], np.deg2rad(baz_deg))
    rx = np.arange(0.0, (g["nx"] - 1) * g["dx"] + 1, 3 * g["dx"], dtype=np.float32)
    return p, c, fp, bazs, fk, rx


EVENTS = [("b", 300, 0.06e-3, True, 0.0), ("b", 300, 0.11e-3, False, 120.0), ("a", 260, 0.05e-3, True, 300.0)]


def _start(F, ev, stream=None):
    p, c, fp, bazs, fk, rx = _inputs(*ev)
    s = F.Session(p, c, stream=stream)
    s.fk_background(fp, bazs, fk, fk)
    s.set_receivers(rx, np.zeros_like(rx), 0.0, 0.0, 1, p["nt"])
    s.advance(p["nt"] + 1)
    return s


def test_own_streams_match_default_stream(F):
    import torch
    ref = []
    for ev in EVENTS:
        s = _start(F, ev)
        ref.append(s.seismograms())
        s.close()
    streams = [torch.cuda.Stream() for _ in EVENTS]
    sessions = [_start(F, ev, st.cuda_stream) for ev, st in zip(EVENTS, streams)]   # all in flight at once
    for s, (rx_, rz_) in zip(sessions, ref):
        sx, sz = s.seismograms()
        assert np.array_equal(sx, rx_) and np.array_equal(sz, rz_)
        s.close()


def test_sessions_started_while_others_run(F):
    ref = []
    for ev in EVENTS:
        s = _start(F, ev)
        ref.append(s.seismograms())
        s.close()
    sessions = [_start(F, ev) for ev in EVENTS * 3]       # enqueued back to back, no waits in between
    for k, s in enumerate(sessions):
        sx, sz = s.seismograms()
        assert np.array_equal(sx, ref[k % len(EVENTS)][0]) and np.array_equal(sz, ref[k % len(EVENTS)][1])
        s.close()
