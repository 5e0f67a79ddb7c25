"""GPU: the serving loop (continuous batching under a device-memory budget).  Requests that
arrive while others run are admitted into the running batch, and every result is identical to
the same solve run alone."""
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


def _request(grid, nt, rayp, p_wave, baz_deg, f0=2.0):
    g = GRIDS[grid]
    c, fk, vmax = _layered(g["nx"], g["nz"], g["npml"], g["dx"], g["moho"])
    p = dict(norder=g["norder"], nx=g["nx"], nz=g["nz"], npml=g["npml"], nbd=g["nbd"], nt=nt, dx=g["dx"],
             dz=g["dz"], dt=g["dt"], vpml=vmax, npower=2, R0=1e-3)
    fp = dict(nx=g["nx"], nz=g["nz"], npml=g["npml"], izt=1, nbd=g["nbd"], nt=nt, src_type=p_wave, x0=0.0, z0=0.0,
              dx=g["dx"], dz=g["dz"], dt=g["dt"], ds=1e-3, f0=f0, rayp=rayp)
    bazs = np.full(g["nx"] + 2 * g["npml"], np.deg2rad(baz_deg))
    rx = np.arange(0.0, (g["nx"] - 1) * g["dx"] + 1, 3 * g["dx"], dtype=np.float32)
    return dict(p=p, c=c, fk=fp, bazs=bazs, fk_left=fk, fk_right=fk, rx=rx, rz=np.zeros_like(rx))


def _alone(F, r):
    with F.Session(r["p"], r["c"]) as s:
        s.fk_background(r["fk"], r["bazs"], r["fk_left"], r["fk_right"])
        s.set_receivers(r["rx"], r["rz"], 0.0, 0.0, 1, r["p"]["nt"])
        s.advance(r["p"]["nt"] + 1)
        return s.seismograms()


SPECS = [("a", 240, 0.06e-3, True, 0.0), ("b", 200, 0.07e-3, True, 20.0), ("c", 150, 0.11e-3, False, 190.0),
         ("a", 90, 0.05e-3, True, 300.0), ("b", 260, 0.10e-3, False, 45.0), ("c", 60, 0.08e-3, True, 120.0)]


def test_requests_arriving_mid_run_match_alone(F):
    reqs = [_request(*s) for s in SPECS]
    ref = [_alone(F, r) for r in reqs]
    with F.Server(3, budget_bytes=8 << 30, chunk=16) as srv:
        ids = [srv.submit(**reqs[0]), srv.submit(**reqs[1])]
        for _ in range(4):
            srv.pump()
        ids += [srv.submit(**r) for r in reqs[2:4]]     # arrive while the first two are running
        srv.pump()
        st = srv.stats()
        assert st["running"] + st["completed"] == 4 and st["queued"] == 0
        for _ in range(3):
            srv.pump()
        ids += [srv.submit(**r) for r in reqs[4:]]
        while srv.pump() > 0:
            pass
        assert srv.stats()["completed"] == len(SPECS)
        for rid, (rx_, rz_) in zip(ids, ref):
            state, t_sub, t_adm, t_done = srv.request(rid)
            assert state == F.api.REQ_DONE and t_sub <= t_adm <= t_done
            gx, gz = srv.result(rid)
            assert np.array_equal(gx, rx_) and np.array_equal(gz, rz_)


def test_budget_bounds_admission(F):
    reqs = [_request(*s) for s in SPECS[:4]]
    ref = [_alone(F, r) for r in reqs]
    need = max(F.session_device_bytes(r["p"], r["rx"].size, r["p"]["nt"]) for r in reqs)
    budget = int(2.5 * need)
    with F.Server(3, budget_bytes=budget, chunk=32) as srv:
        ids = [srv.submit(**r) for r in reqs]
        peak, waited = 0, False
        while True:
            left = srv.pump()
            st = srv.stats()
            assert st["bytes_in_use"] <= budget          # never more resident than the budget
            peak = max(peak, st["running"])
            waited |= st["queued"] > 0 and st["running"] > 0
            if left == 0:
                break
        assert 1 <= peak < len(reqs) and waited         # some requests waited for memory to free up
        for rid, (rx_, rz_) in zip(ids, ref):
            gx, gz = srv.result(rid)
            assert np.array_equal(gx, rx_) and np.array_equal(gz, rz_)


def test_request_larger_than_budget_is_refused(F):
    r = _request(*SPECS[0])
    with F.Server(3, budget_bytes=1 << 20) as srv:
        with pytest.raises(F.FDFKError) as e:
            srv.submit(**r)
        assert e.value.code == -1


def test_served_config3_traces_vs_fp64_oracle(F, oracle_lib):
    """A stream of config-3 requests (events on the 801 x 401 two-layer model, 4001 steps, P and S
    incidence, back-azimuths 0-360, 0.5-1 Hz) served with staggered arrivals; 8 requests chosen by a
    seeded draw are checked trace by trace against the FP64 GPU oracle fed the FP64 FK restatement:
    relative L2 of every trace at most 1e-4."""
    import fk_oracle
    from fdfk2d_gb300 import workloads as WL
    w = WL.config1()
    p = w["p"]
    events = WL.config3_events(24, seed=23)
    pick = sorted(np.random.default_rng(5).choice(len(events), 8, replace=False).tolist())
    ids = []
    with F.Server(3, budget_bytes=40 << 30, chunk=64) as srv:
        for i, ev in enumerate(events):
            fp, bazs, fl, fr = WL.event_inputs(w, ev)
            ids.append(srv.submit(p, w["c"], fp, bazs, fl, fr, w["rx"], w["rz"], w["x0"], w["z0"], 1, p["nt"]))
            if i % 3 == 2:                                  # later requests arrive while earlier ones run
                srv.pump()
        while srv.pump() > 0:
            pass
        got = {i: tuple(np.array(a) for a in srv.result(ids[i])) for i in pick}
    worst = 0.0
    for i in pick:
        fp, bazs, fl, fr = WL.event_inputs(w, events[i])
        strips = fk_oracle.background_device(fp, bazs, fl, fr, x0=w["x0"], z0=w["z0"])
        ox, oz = oracle_lib.simulate64_gpu(dict(p, izt=1), strips, w["c"], w["rx"], w["rz"], w["x0"], w["z0"], 1,
                                           p["nt"])
        del strips
        for g, o in zip(got[i], (ox, oz)):
            e = np.linalg.norm(g.astype(np.float64) - o, axis=0) / np.linalg.norm(o, axis=0)
            worst = max(worst, float(e.max()))
    print(f"\nserved config-3 requests {pick}: worst per-trace relative L2 vs FP64 oracle {worst:.3e}")
    assert worst <= 1e-4
