"""GPU: every receiver trace of the FP32 GPU solver (FK background on the GPU, single solves and
batch members) within 1e-4 relative L2 of the FP64 oracle (the restatement in double precision,
with the FK background restated in FP64)."""
import numpy as np
import pytest

from conftest import load_npz
from test_gpu_batch import GRIDS, _layered

import fk_oracle

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-4


@pytest.fixture(scope="module")
def F():
    import fdfk2d_gb300 as F
    from fdfk2d_gb300 import build
    build.build()
    F.lib()
    return F


def _per_trace(got, ref):
    g, r = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    return max(np.linalg.norm(g[:, i] - r[:, i]) / max(np.linalg.norm(r[:, i]), 1e-30) for i in range(r.shape[1]))


def _fp64(oracle_lib, p, c, fp, bazs, fl, fr, rx, rz, nstp, nsis):
    q = dict(p, izt=1)
    strips = fk_oracle.background(fp, bazs, fl, fr, x0=fp.get("x0", 0.0), z0=fp.get("z0", 0.0), dtype=np.float64)
    return oracle_lib.simulate64(q, strips, c, rx, rz, 0.0, 0.0, nstp, nsis)


def test_golden_loop_traces_vs_fp64(F, oracle_lib):
    d = load_npz("loop_layered")
    p = dict(d["p"])
    fp = dict(p, izt=1)
    with F.Session(p, d["c"]) as s:
        s.fk_background(fp, d["bazs"], d["fk_left"], d["fk_right"])
        s.set_receivers(d["rx"], d["rz"], 0.0, 0.0, int(d["nstp"]), int(d["nsis"]))
        s.advance(p["nt"] + 1)
        gx, gz = s.seismograms()
    ox, oz = _fp64(oracle_lib, p, d["c"], fp, d["bazs"], d["fk_left"], d["fk_right"], d["rx"], d["rz"],
                   int(d["nstp"]), int(d["nsis"]))
    assert _per_trace(gx, ox) < TRACE_TOL and _per_trace(gz, oz) < TRACE_TOL


EVENTS = [("a", 240, 0.05e-3, True, 15.0), ("b", 200, 0.11e-3, False, 200.0), ("c", 150, 0.08e-3, True, 330.0)]


def test_batch_member_traces_vs_fp64(F, oracle_lib):
    sessions, refs = [], []
    for grid, nt, rayp, p_wave, baz in EVENTS:
        g = GRIDS[grid]
        c, fk, vmax = _layered(g["nx"], g["nz"], g["npml"], g["dx"], g["moho"])
        p = dict(norder=3, nx=g["nx"], nz=g["nz"], npml=g["npml"], nbd=5, nt=nt, dx=g["dx"], dz=g["dz"], dt=g["dt"],
                 vpml=vmax, npower=2, R0=1e-3)
        fp = dict(nx=g["nx"], nz=g["nz"], npml=g["npml"], izt=1, nbd=5, nt=nt, src_type=p_wave, x0=0.0, z0=0.0,
                  dx=g["dx"], dz=g["dz"], dt=g["dt"], ds=1e-3, f0=2.0, rayp=rayp)
        bazs = np.full(g["nx"] + 2 * g["npml"], np.deg2rad(baz))
        rx = np.arange(0.0, (g["nx"] - 1) * g["dx"] + 1, 3 * g["dx"], dtype=np.float32)
        rz = np.zeros_like(rx)
        s = F.Session(p, c)
        s.fk_background(fp, bazs, fk, fk)
        s.set_receivers(rx, rz, 0.0, 0.0, 1, nt)
        sessions.append(s)
        refs.append(_fp64(oracle_lib, p, c, fp, bazs, fk, fk, rx, rz, 1, nt))
    with F.Batch(3) as b:
        for s in sessions:
            b.add(s)
        b.advance(max(e[1] for e in EVENTS) + 1)
        got = [s.seismograms() for s in sessions]
    for (gx, gz), (ox, oz) in zip(got, refs):
        assert np.abs(oz).max() > 0
        assert _per_trace(gx, ox) < TRACE_TOL and _per_trace(gz, oz) < TRACE_TOL
    for s in sessions:
        s.close()
