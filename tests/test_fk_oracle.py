"""CPU tests: the FK background restatement (oracle/fk_oracle.py) against strips made by the
reference's shipped comput_background_wavefield_ (lib_gnu/libFK3D.so), plus its formula parts."""
import numpy as np
import pytest

from conftest import load_npz, max_rel

import fk_oracle as FO

# Strips are float32; the restatement works in FP64 and differs from the shipped
# propagator/FFT arithmetic only by rounding.
FK_TOL = 5e-7


@pytest.mark.parametrize("name", ("fk_p_ramp", "fk_s_left"))
def test_fk_restatement_matches_shipped(name):
    d = load_npz(name)
    p = d["p"]
    mine = FO.background(p, d["bazs"], d["fk_left"], d["fk_right"], x0=p["x0"], z0=p["z0"])
    for k in FO.STRIPS:
        assert mine[k].shape == d[k].shape, k
        assert max_rel(mine[k], d[k]) < FK_TOL, k


def test_fk_restatement_matches_shipped_loop_background():
    # the background that drove the golden time loop (zero back-azimuth, same model both sides)
    d = load_npz("loop_layered")
    p = d["p"]
    mine = FO.background(p, d["bazs"], d["fk_left"], d["fk_right"])
    for k in FO.STRIPS:
        assert max_rel(mine[k], d[k]) < FK_TOL, k


def test_nfft_and_cutoff():
    assert FO.nfft(240) == 512
    assert FO.nfft(255) == 512
    assert FO.nfft(256) == 1024
    W, N, alpha = FO.source_spectrum(240, 0.015, 2.0, 1e-3)
    assert N == 512 and abs(alpha - 10.0 / 3.6) < 1e-15
    # Hermitian spectrum of a real source
    np.testing.assert_allclose(W[1:N // 2], np.conj(W[N - 1:N // 2:-1]), rtol=0, atol=1e-18)


def test_homogeneous_halfspace_free_surface_p():
    """A one-layer model at vertical P incidence: at the surface U_Z is twice the incident
    amplitude (free-surface doubling) and U_R vanishes."""
    m = np.array([[0.0], [6000.0], [3500.0], [2700.0]], np.float32)
    wc = np.array([1.0 - 0.1j, 5.0 - 0.1j])
    UR, UZ = FO.layered_response(m, 0.0, wc, [0.0], "P", z_ref=0.0)
    np.testing.assert_allclose(np.abs(UR), 0.0, atol=1e-12)
    np.testing.assert_allclose(np.abs(UZ[:, 0]), 2.0, rtol=1e-12)


def test_bottom_strip_model_switch():
    """Bottom strips take the model of the side the wave arrives from, except the nbd columns
    under the other side strip."""
    p = dict(nx=12, nz=8, npml=4, nbd=3, nt=60, dt=0.01, dx=250.0, dz=250.0, f0=2.0, ds=1e-3,
             rayp=6e-5, src_type=True)
    ml = np.array([[0.0], [6000.0], [3500.0], [2700.0]], np.float32)
    mr = np.array([[0.0], [5000.0], [2900.0], [2500.0]], np.float32)
    for baz, left_cols in ((0.0, 3 + 3), (np.pi, 3 + 12 - 3)):
        bazs = np.full(p["nx"] + 2 * p["npml"], baz)
        a = FO.background(p, bazs, ml, mr)["uzb_pml"]
        al = FO.background(p, bazs, ml, ml)["uzb_pml"]
        ar = FO.background(p, bazs, mr, mr)["uzb_pml"]
        for j in range(a.shape[1]):
            ref = al if j < left_cols else ar
            assert np.array_equal(a[:, j], ref[:, j]), (baz, j)


@pytest.mark.parametrize("name", ("fk_p_ramp", "fk_s_left"))
def test_batched_restatement_matches_per_column(name):
    """background_device (the batched form used for the full-size FP64 oracle, here on the CPU with
    small chunks) gives the per-column restatement's FP64 values to rounding."""
    d = load_npz(name)
    p = d["p"]
    a = FO.background(p, d["bazs"], d["fk_left"], d["fk_right"], x0=p["x0"], z0=p["z0"], dtype=np.float64)
    b = FO.background_device(p, d["bazs"], d["fk_left"], d["fk_right"], x0=p["x0"], z0=p["z0"], device="cpu",
                             chunk_bytes=1 << 16)
    for k in FO.STRIPS:
        got = b[k].numpy().transpose(2, 1, 0)
        assert got.shape == a[k].shape, k
        assert max_rel(got, a[k]) < 1e-12, k
