"""CPU: the reference's own example input folders (examples/{test1..4,Altyn}/input, copied to
tests/golden/inputs) parsed by fdfk_input_read, checked against an independent reading of the same
files by the rules of src/Input.f90:75-186, 227-284 (FD order halved and capped by the absorbing
layer, grid sizes by NINT, ray parameter s/deg -> s/m, nlayer rows of each FK model with
rho = (vp + 980)/2.76, the first two values of each receiver record), and the profile geometry
(fdfk_backazimuths) against the geodesy restatement oracle/geodesy_oracle.py at every grid column
and receiver of each example, for every event the example lists."""
import os

import numpy as np
import pytest

from example_models import CASES, _numbers, make_case

import geodesy_oracle as GO

BAZ_TOL = 1e-12       # radians


@pytest.fixture(scope="module")
def F():
    import fdfk2d_gb300 as F
    from fdfk2d_gb300 import build
    build.build()
    return F


def _expected(folder):
    L = lambda name: open(os.path.join(folder, name)).read().splitlines()
    fd = L("FD_model.dat")
    order = int(_numbers(fd[1])[0])
    x0, xn, z0, zn, dx, dz, dt = _numbers(fd[3])[:7]
    t = fd[5].replace(",", " ").split()
    tmax, tstp, npml = float(t[0]), float(t[1]), int(t[2])
    lat, lon, az = _numbers(fd[7])[:3]
    norder = order // 2
    if 2 * norder > npml + 1:
        norder = (npml + 1) // 2
    src = L("Source.dat")
    f0, ds = _numbers(src[1].split()[0] + " " + src[1].split()[1])
    rayp_deg, evla, evlo = [float(v) for v in src[3].split()[:3]]
    events = []
    for line in src[3:]:
        tok = line.split("!")[0].split()
        if len(tok) >= 3:
            events.append((float(tok[1]), float(tok[2])))
    rc = L("Receiver.dat")
    nrcv = int(rc[1].split()[0])
    rcv = np.array([_numbers(rc[3 + i])[:2] for i in range(nrcv)], np.float32)
    fk = {}
    for side in ("left", "right"):
        lines = L(f"FK_model_{side}.dat")
        n = int(_numbers(lines[1])[0])
        rows = np.array([_numbers(lines[3 + i])[:3] for i in range(n)], np.float32)
        fk[side] = rows
    return dict(norder=norder, nx=int(round((xn - x0) / dx)) + 1, nz=int(round((zn - z0) / dz)) + 1, npml=npml,
                dx=dx, dz=dz, dt=dt, tmax=tmax, tstp=tstp, x0=x0, z0=z0, lat=lat, lon=lon, az=az, f0=f0, ds=ds,
                rayp=rayp_deg * 180.0 / (np.pi * 6371.0e3), evla=evla, evlo=evlo, events=events, rcv=rcv, fk=fk)


@pytest.mark.parametrize("case", CASES)
def test_example_folder_is_parsed_as_the_reference_reads_it(F, case, tmp_path):
    folder = make_case(case, str(tmp_path / case))
    e = _expected(folder)
    d = F.read_input(folder, "inpar.dat")
    assert (d["nx"], d["nz"], d["npml"], d["izt"], d["norder"]) == (e["nx"], e["nz"], e["npml"], 1, e["norder"])
    assert d["is_PML_top"] == 0
    assert d["dt"] == e["dt"] and d["tmax"] == np.float32(e["tmax"]) and d["tstp"] == np.float32(e["tstp"])
    assert d["dx"] == np.float32(e["dx"]) and d["dz"] == np.float32(e["dz"])
    assert (d["lat_org"], d["lon_org"], d["az_org"]) == (e["lat"], e["lon"], e["az"])
    assert (d["evla"], d["evlo"]) == (e["evla"], e["evlo"])
    assert abs(d["rayp"] - e["rayp"]) <= 1e-15 * e["rayp"]
    assert d["f0"] == np.float32(e["f0"]) and d["ds"] == np.float32(e["ds"])
    assert d["nrcv"] == len(e["rcv"])
    np.testing.assert_array_equal(d["rx"], e["rcv"][:, 0])
    np.testing.assert_array_equal(d["rz"], e["rcv"][:, 1])
    for side in ("left", "right"):
        rows = e["fk"][side]
        got = d["fk_" + side]
        assert got.shape == (4, len(rows)), side
        np.testing.assert_array_equal(got[0], rows[:, 2])
        np.testing.assert_array_equal(got[1], rows[:, 0])
        np.testing.assert_array_equal(got[2], rows[:, 1])
        np.testing.assert_allclose(got[3], (rows[:, 0] + np.float32(980.0)) / np.float32(2.76), rtol=1e-7)
    c = d["c"]
    assert c.shape == (3, e["nz"] + e["npml"], e["nx"] + 2 * e["npml"])
    assert (c[0] > 0).all() and (c[2] > 0).all()


def test_test1_order_16_becomes_norder_8(F, tmp_path):
    d = F.read_input(make_case("test1", str(tmp_path / "t1")), "inpar.dat")
    assert d["norder"] == 8


@pytest.mark.parametrize("case", CASES)
def test_profile_backazimuths_match_geodesy_restatement(F, case, tmp_path):
    folder = make_case(case, str(tmp_path / case))
    e = _expected(folder)
    npml, nx = e["npml"], e["nx"]
    coordx = np.float32(e["x0"]) + (np.arange(1 - npml, nx + npml + 1) - 1).astype(np.float32) * np.float32(e["dx"])
    for evla, evlo in e["events"]:
        for xs in (coordx, e["rcv"][:, 0]):
            got = F.backazimuths(e["lat"], e["lon"], e["az"], evla, evlo, xs)
            ref = GO.profile_bazs(e["lat"], e["lon"], e["az"], evla, evlo, xs)
            assert np.abs(got - ref).max() <= BAZ_TOL, (evla, evlo)


def test_geodesy_restatement_known_directions():
    # on the equator, events due north / east / south of a station at the profile origin
    for (evla, evlo), want in (((30.0, 0.0), 0.0), ((0.0, 40.0), 90.0), ((-30.0, 0.0), 180.0)):
        b = np.rad2deg(GO.backazimuth_grids(0.0, 0.0, 0.0, evla, evlo, [0.0]))[0]
        assert abs(b - want) < 1e-9
    R, Ri = GO.rotation_matrices(40.372214, 88.173868, 134.1466634471141)
    # the forward matrix is a rotation (orthonormal rows)
    np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-15)
