"""CPU tests of the input/output surface (src/Input.f90, src/FDFK2D.f90:537-561, the geodesy of
src/coord_transform.f90 and src/calc_backazimuth.f90, check_stability of src/Submain.f90)."""
import os

import numpy as np
import pytest

from io_folder import H, NPML, NX, NZ, write_folder


@pytest.fixture(scope="module")
def F():
    import fdfk2d_gb300 as F
    from fdfk2d_gb300 import build
    build.build()
    return F


def test_read_input_folder(F, tmp_path):
    write_folder(str(tmp_path))
    d = F.read_input(str(tmp_path), "inpar.dat", write_model_copies=True)
    assert (d["nx"], d["nz"], d["npml"], d["izt"], d["norder"]) == (NX, NZ, NPML, 1, 3)
    assert d["dt"] == 0.015 and d["tmax"] == np.float32(3.0) and d["tstp"] == np.float32(0.03)
    assert d["src_type"] == 1 and d["is_PML_top"] == 0 and d["outsnap"] == 0 and d["nstep"] == 50
    assert abs(d["rayp"] - 6.672 * 180.0 / (np.pi * 6371.0e3)) < 1e-18
    assert (d["lat_org"], d["lon_org"], d["az_org"], d["evla"], d["evlo"]) == (30.0, 100.0, 90.0, 0.0, 140.0)
    np.testing.assert_array_equal(d["rx"], np.float32([0.0, 1250.0, 4875.0, 7500.0, 9750.0]))
    fl = d["fk_left"]
    assert fl.shape == (4, 2)
    np.testing.assert_array_equal(fl[:, 1], np.float32([3000.0, 8100.0, 4500.0, (8100.0 + 980.0) / 2.76]))
    c = d["c"]
    assert c.shape == (3, NZ + NPML, NX + 2 * NPML)
    rho = np.float32((np.float32(6300.0) + np.float32(980.0)) / np.float32(2.76))
    assert c[0, 0, 0] == rho and c[2, 0, 0] == rho * np.float32(3600.0) * np.float32(3600.0)
    # the model without its absorbing frame, written next to the inputs
    heads, vp = F.read_su(str(tmp_path / "vp_without_pml.su"), NZ)
    assert vp.shape == (NZ, NX) and heads[0, 57] == NZ and heads[0, 58] == 1000 and vp[0, 0] == 6300.0


def test_norder_is_limited_by_the_pml(F, tmp_path):
    write_folder(str(tmp_path))
    txt = open(tmp_path / "FD_model.dat").read().replace("\n6\n", "\n16\n").replace(" 8 .false.", " 5 .false.")
    open(tmp_path / "FD_model.dat", "w").write(txt)
    assert F.read_input(str(tmp_path), "inpar.dat")["norder"] == 3     # int((npml + 1) / 2)


def test_input_errors(F, tmp_path):
    write_folder(str(tmp_path))
    open(tmp_path / "Receiver.dat", "w").write("# nrcv\n1\n# rx rz\n20000.0 0.0\n")
    with pytest.raises(F.FDFKError, match="outside the model"):
        F.read_input(str(tmp_path), "inpar.dat")
    write_folder(str(tmp_path))
    open(tmp_path / "FK_model_right.dat", "w").write("# n\n1\n# vp vs z\n7000.0 4000.0 0.0\n")
    with pytest.raises(F.FDFKError, match="half-space must be identical"):
        F.read_input(str(tmp_path), "inpar.dat")
    with pytest.raises(F.FDFKError, match="cannot open"):
        F.read_input(str(tmp_path / "missing"), "inpar.dat")


def test_su_round_trip(F, tmp_path):
    data = np.random.default_rng(1).standard_normal((17, 5)).astype(np.float32)
    F.write_su(str(tmp_path / "a.su"), data, 17, 15000)
    heads, back = F.read_su(str(tmp_path / "a.su"), 17)
    np.testing.assert_array_equal(back, data)
    assert heads.shape == (5, 120) and (heads[:, 57] == 17).all() and (heads[:, 58] == 15000).all()
    assert os.path.getsize(tmp_path / "a.su") == 5 * (240 + 17 * 4)


def test_backazimuth_directions(F):
    # profile through (lat 0, lon 0) along azimuth 0 (north): stations at x = 0
    b = np.rad2deg(F.backazimuths(0.0, 0.0, 0.0, 30.0, 0.0, [0.0]))[0]        # event to the north
    assert abs(b) < 1e-9 or abs(b - 360.0) < 1e-9
    assert abs(np.rad2deg(F.backazimuths(0.0, 0.0, 0.0, 0.0, 40.0, [0.0]))[0] - 90.0) < 1e-9      # east
    assert abs(np.rad2deg(F.backazimuths(0.0, 0.0, 0.0, -30.0, 0.0, [0.0]))[0] - 180.0) < 1e-9    # south
    # the profile azimuth is subtracted; moving along the profile changes the back-azimuth smoothly
    b2 = np.rad2deg(F.backazimuths(0.0, 0.0, 90.0, 0.0, 40.0, [0.0, 1e5, 2e5]))
    assert abs(b2[0]) < 1e-9 and np.all(np.abs(np.diff(b2)) < 1.0)


def test_stable_dt_matches_oracle(F, oracle_lib):
    from io_folder import write_folder as _w  # noqa: F401
    c = np.zeros((3, 10, 12), np.float32, order="F")
    c[0], c[1], c[2] = 2700.0, 2700.0 * (6000.0 ** 2 - 2 * 3500.0 ** 2), 2700.0 * 3500.0 ** 2
    dt = F.stable_dt(3, 8, 6, 2, 250.0, 250.0, c)
    ref = oracle_lib.dt_stable(8, 6, 2, 1, 3, 250.0, 250.0, c)
    assert abs(dt - ref) <= 1e-7 * ref
    # CFL of order 6 (src/Submain.f90:118-164): 0.5752 h / vpmax
    assert abs(dt * 6000.0 / 250.0 - 0.5752) < 1e-4
