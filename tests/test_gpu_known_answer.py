"""GPU: the hybrid method's known answer at the config-1 size (801 x 401 cells at 250 m, two flat
layers, 20-cell absorbing layers).

On a laterally homogeneous model identical to the FK models nothing scatters, so the field of the
regular domain is the FK background itself.  At vertical incidence that background is the same in
every column: every surface receiver must record the FK surface response, which the background
strips hold in their first row, sample for sample.  This exercises the injection on both strip
sides, the interior fast path, the tiled kernel (free-surface rows, absorbing layers) and receiver
sampling together.  What remains is discretisation error: the leapfrog step's phase lead (second
order in dt: at the config-1 step the arrivals lead by about half a sample), the spatial dispersion
of the 6th-order stencils (S waves at 5-7 cells per wavelength over 100 km) and, with layers, the
flat interface's position on the grid.  Dividing dt by three must cut the P misfit of a half-space
more than fourfold.
"""
import numpy as np
import pytest

from fdfk2d_gb300 import workloads as WL

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F():
    import fdfk2d_gb300 as F
    from fdfk2d_gb300 import build
    build.build()
    F.lib()
    return F


def _misfits(F, p_wave, dt, half_space=False, duration=30.0):
    nt = int(round(duration / dt))
    w = WL.config1(nt=nt)
    p = dict(w["p"], dt=dt)
    fp, bazs, fl, fr = WL.event_inputs(w, dict(p_wave=p_wave, rayp=1e-9, baz=0.0, f0=1.0))
    fp = dict(fp, dt=dt)
    if half_space:                             # the crust everywhere: no interface
        NZ, NX = p["nz"] + p["npml"], p["nx"] + 2 * p["npml"]
        w["c"] = WL.pack_c(np.full((NZ, NX), 6300.0), np.full((NZ, NX), 3600.0))
        fl = fr = np.array([[0.0], [6300.0], [3600.0], [WL.gardner(6300.0)]], np.float32)
        p["vpml"] = 6300.0
    strips = F.fk_background(fp, bazs, fl, fr)
    with F.Session(p, w["c"]) as s:
        s.upload_background(strips)
        s.set_receivers(w["rx"], w["rz"], w["x0"], w["z0"], 1, nt)
        s.advance(nt + 1)
        sx, sz = s.seismograms()
    comp = "uz" if p_wave else "ux"
    ref = strips[comp + "l_pml"][0, 0, :].astype(np.float64)        # row 1 of the left outer strip
    far = strips[comp + "r_pml"][0, -1, :].astype(np.float64)       # 200 km away
    assert np.linalg.norm(far - ref) <= 5e-3 * np.linalg.norm(ref)   # the same in every column
    main, other = (sz, sx) if p_wave else (sx, sz)
    out = []
    for j in range(5, main.shape[1] - 5, 5):                        # receivers away from the strips
        m = main[:, j].astype(np.float64)
        out.append(np.linalg.norm(m - ref) / np.linalg.norm(ref))
        assert np.abs(other[:, j]).max() <= 0.01 * np.abs(ref).max(), j   # the other component stays ~0
    return np.array(out)


@pytest.mark.parametrize("p_wave", [True, False])
def test_half_space_surface_equals_fk_response(F, p_wave):
    coarse = _misfits(F, p_wave, 0.015, half_space=True)     # the config-1 step
    fine = _misfits(F, p_wave, 0.005, half_space=True)
    print("known answer, half-space", "P" if p_wave else "S", coarse.max(), fine.max())
    assert coarse.max() < 0.15, coarse.max()
    if p_wave:
        assert fine.max() < 0.012, fine.max()
        assert fine.max() < coarse.max() / 4.0, (coarse.max(), fine.max())   # second-order time convergence
    else:
        assert fine.max() < 0.04, fine.max()        # spatial dispersion of S over the 100 km path


@pytest.mark.parametrize("p_wave", [True, False])
def test_flat_layers_surface_equals_fk_response(F, p_wave):
    coarse = _misfits(F, p_wave, 0.015)
    fine = _misfits(F, p_wave, 0.005)
    print("known answer, two layers", "P" if p_wave else "S", coarse.max(), fine.max())
    assert coarse.max() < 0.2, coarse.max()
    assert fine.max() < min(0.09, coarse.max()), (coarse.max(), fine.max())
