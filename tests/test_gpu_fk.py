"""GPU parity of the FK background (FP64 on the GPU, float32 strips) against the reference's
shipped comput_background_wavefield_ (golden fixtures) and the oracle restatement, through the C ABI."""
import os

import numpy as np
import pytest

from conftest import load_npz, max_rel, rel_l2

import fk_oracle as FO

pytestmark = pytest.mark.gpu

# FP64 spectra and transforms rounded to float32: max |error| / max |strip|.
FK_TOL = 1e-6
# Seismograms of the time loop driven by the GPU background: relative L2 per component.
TRACE_TOL = 1e-4


@pytest.fixture(scope="module")
def F():
    import fdfk2d_gb300 as F
    from fdfk2d_gb300 import build
    build.build()
    F.lib()
    return F


def _cmp(a, b, tol=FK_TOL):
    for k in FO.STRIPS:
        assert a[k].shape == b[k].shape, k
        assert max_rel(a[k], b[k]) < tol, (k, max_rel(a[k], b[k]))


@pytest.mark.parametrize("name", ("fk_p_ramp", "fk_s_left", "loop_layered"))
def test_fk_matches_shipped(F, name):
    d = load_npz(name)
    p = dict(d["p"])
    n0 = F.kernel_launches()
    got = F.fk_background(p, d["bazs"], d["fk_left"], d["fk_right"])
    assert F.kernel_launches() - n0 >= 7
    _cmp(got, {k: d[k] for k in FO.STRIPS})


def test_fk_dropin_entry_point_equals_c_api(F):
    d = load_npz("fk_s_left")
    p = dict(d["p"])
    a = F.fk_background(p, d["bazs"], d["fk_left"], d["fk_right"])
    b = {k: np.zeros_like(a[k], order="F") for k in FO.STRIPS}
    F.comput_background_wavefield(p, d["bazs"], d["fk_left"], d["fk_right"], b)
    for k in FO.STRIPS:
        assert np.array_equal(a[k], b[k]), k


def _random_models(rng):
    def model(nl):
        tops = np.concatenate([[0.0], np.sort(rng.uniform(300.0, 4000.0, nl - 1))])
        vp = np.sort(rng.uniform(4500.0, 8200.0, nl))
        vs = vp / rng.uniform(1.65, 1.85, nl)
        rho = 1740.0 * (vp / 1000.0) ** 0.25
        return np.asfortranarray(np.stack([tops, vp, vs, rho]).astype(np.float32))
    return model(int(rng.integers(1, 6))), model(int(rng.integers(1, 6)))


@pytest.mark.parametrize("seed,batch", ((1, None), (2, "7"), (3, "64")))
def test_fk_matches_oracle_random(F, seed, batch, monkeypatch):
    rng = np.random.default_rng(seed)
    nbd = int(rng.integers(1, 6))
    nx, nz = int(rng.integers(nbd + 2, 30)), int(rng.integers(nbd + 2, 20))
    npml = nbd + int(rng.integers(0, 4))
    p = dict(nx=nx, nz=nz, npml=npml, izt=1, nbd=nbd, nt=int(rng.integers(60, 300)), src_type=bool(seed % 2),
             x0=float(rng.uniform(-2000, 2000)), z0=0.0, dx=float(rng.choice([100.0, 200.0, 250.0])),
             dz=float(rng.choice([100.0, 150.0, 250.0])), dt=float(rng.uniform(0.005, 0.015)), ds=1e-3,
             f0=float(np.float32(rng.uniform(0.8, 2.5))), rayp=float(rng.uniform(0.04e-3, 0.08e-3)))
    ml, mr = _random_models(rng)
    c0 = rng.uniform(-30, 30) + (0 if seed != 3 else 180)
    bazs = np.deg2rad(c0 + rng.uniform(-5, 5, nx + 2 * npml))
    if batch:
        monkeypatch.setenv("FDFK_FK_BATCH", batch)
    got = F.fk_background(p, bazs, ml, mr)
    ref = FO.background(p, bazs, ml, mr, x0=p["x0"], z0=p["z0"])
    _cmp(got, ref)


def test_fk_linear_in_source_scale(F):
    """Size-independent property at a larger size (several FFT batches): strips scale with ds."""
    p = dict(nx=600, nz=300, npml=10, izt=1, nbd=5, nt=2500, src_type=True, x0=0.0, z0=0.0, dx=100.0, dz=100.0,
             dt=0.006, ds=1e-3, f0=1.0, rayp=0.07e-3)
    ml = np.asfortranarray(np.array([[0, 33e3], [6300, 8100], [3600, 4500], [2750, 3300]], np.float32))
    mr = np.asfortranarray(np.array([[0, 50e3], [6300, 8100], [3600, 4500], [2750, 3300]], np.float32))
    bazs = np.deg2rad(np.linspace(-10, 10, 620))
    a = F.fk_background(p, bazs, ml, mr)
    b = F.fk_background(dict(p, ds=4e-3), bazs, ml, mr)
    for k in FO.STRIPS:
        assert np.isfinite(a[k]).all(), k
        assert max_rel(b[k], 4.0 * a[k]) < 1e-6, k


def test_time_loop_with_gpu_background_matches_shipped(F):
    """FK background computed on the GPU into the session, then the time loop: the shipped run's traces."""
    d = load_npz("loop_layered")
    p = dict(d["p"])
    with F.Session(p, d["c"]) as s:
        s.fk_background(p, d["bazs"], d["fk_left"], d["fk_right"])
        s.set_receivers(d["rx"], d["rz"], 0.0, 0.0, int(d["nstp"]), int(d["nsis"]))
        s.advance(p["nt"] + 1)
        sx, sz = s.seismograms()
    assert rel_l2(sx, d["seisx"]) < TRACE_TOL
    assert rel_l2(sz, d["seisz"]) < TRACE_TOL
