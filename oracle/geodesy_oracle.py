"""ORACLE (test infrastructure only): NumPy restatement of the profile geometry of FDFK2D.

The host program computes one back-azimuth per grid column (src/FDFK2D.f90:380-387) and per
receiver (src/FDFK2D.f90:537-539) with `compute_backazimuth_grids`:

* :func:`rotation_matrices` - src/define_rotation_matrix.f90:1-89 (the closed-form matrices at the
  end of the routine, both of them, entry for entry; the inverse matrix's (2,1) entry uses
  sin(lat) cos(lon) as the reference writes it);
* :func:`geogr2cart` / :func:`cart2geogr` - src/calc_backazimuth.f90:211-270 (spherical Earth of
  radius 6371 km, the radius a single-precision constant; near-zero angles snapped to 0);
* :func:`backaz` - src/calc_backazimuth.f90:72-207 (Bullen's flattened-sphere formulas with
  flattening 1/298.257, the quadrant-safe atan2 form, 360 -> 0);
* :func:`backazimuth_grids` - src/coord_transform.f90:1-61: each profile coordinate (float, along
  the local X axis) mapped through the inverse rotation into the Earth-centred frame around the
  profile origin, back to latitude/longitude, then the back-azimuth of the event there, in
  radians;  :func:`profile_bazs` subtracts the profile azimuth as src/FDFK2D.f90:387 and :539 do.

Everything is FP64 (the reference's real(8)), element by element with NumPy's libm-equivalent
functions.  Only tests use this module.
"""
from __future__ import annotations

import numpy as np

PI = 4.0 * np.arctan(1.0)
DEG2RAD = PI / 180.0
RAD2DEG = 180.0 / PI
EARTH_R = float(np.float32(6371.0e3))          # `real, parameter` in the reference
FLATTENING = 1.0 / 298.257
SNAP = float(np.float32(1.0e-9))               # the single-precision literal 1.e-9 of cart2geogr


def rotation_matrices(lat_org, lon_org, az_org):
    """(rotate_matrix, inv_rotate_matrix), 3 x 3 each, of the profile frame (X along az_org)."""
    az, lat, lon = az_org * DEG2RAD, lat_org * DEG2RAD, lon_org * DEG2RAD
    st, ct = np.sin(lat), np.cos(lat)
    sp, cp = np.sin(lon), np.cos(lon)
    sa, ca = np.sin(az), np.cos(az)
    f1, f2 = st * cp, st * sp
    R = np.array([[-sa * sp + ca * f1, sa * cp + ca * f2, -ca * ct],
                  [-ca * sp - sa * f1, ca * cp - sa * f2, sa * ct],
                  [ct * cp, ct * sp, st]])
    Ri = np.array([[-sa * sp + ca * f1, -ca * sp - sa * f2, -ct * cp],
                   [sa * cp + ca * f1, ca * cp - sa * f2, ct * cp],
                   [-ca * ct, sa * cp, st]])
    return R, Ri


def geogr2cart(lat, lon):
    colat = (90.0 - lat) * DEG2RAD
    lo = lon * DEG2RAD
    return (EARTH_R * np.sin(colat) * np.cos(lo), EARTH_R * np.sin(colat) * np.sin(lo), EARTH_R * np.cos(colat))


def cart2geogr(x, y, z):
    r = np.hypot(x, y)
    if r < 1.0e-6:
        return (90.0 if z > 0.0 else -90.0), 0.0
    lat = np.arctan2(z, r) * RAD2DEG
    lon = np.arctan2(y, x) * RAD2DEG
    if abs(lat) < SNAP:
        lat = 0.0
    if abs(lon) < SNAP:
        lon = 0.0
    return lat, lon


def backaz(evla, evlo, stla, stlo):
    """Back-azimuth (degrees) at station (stla, stlo) of the event (evla, evlo)."""
    coeff = (1.0 - FLATTENING) * (1.0 - FLATTENING)
    scola = 0.5 * PI - np.arctan(coeff * np.tan(stla * DEG2RAD))
    ecola = 0.5 * PI - np.arctan(coeff * np.tan(evla * DEG2RAD))
    slon, elon = stlo * DEG2RAD, evlo * DEG2RAD
    c = np.cos(scola)
    d, e = np.sin(slon), -np.cos(slon)
    g, h, k = -c * e, c * d, -np.sin(scola)
    aa = np.sin(ecola) * np.cos(elon)
    bb = np.sin(ecola) * np.sin(elon)
    cc = np.cos(ecola)
    rhs1 = (aa - d) ** 2 + (bb - e) ** 2 + cc * cc - 2.0
    rhs2 = (aa - g) ** 2 + (bb - h) ** 2 + (cc - k) ** 2 - 2.0
    dbaz = np.arctan2(rhs1, rhs2)
    if dbaz < 0.0:
        dbaz += 2.0 * PI
    baz = dbaz * RAD2DEG
    if abs(baz - 360.0) < 1.0e-5:
        baz = 0.0
    return baz


def backazimuth_grids(lat_org, lon_org, az_org, evla, evlo, coordx):
    """compute_backazimuth_grids: back-azimuths (radians) at the profile coordinates coordx (float)."""
    _, Ri = rotation_matrices(lat_org, lon_org, az_org)
    xo, yo, zo = geogr2cart(lat_org, lon_org)
    out = np.empty(len(coordx), np.float64)
    for i, X in enumerate(np.asarray(coordx, np.float32)):
        v = Ri @ np.array([float(X), 0.0, 0.0])
        stla, stlo = cart2geogr(v[0] + xo, v[1] + yo, v[2] + zo)
        out[i] = backaz(evla, evlo, stla, stlo) * DEG2RAD
    return out


def profile_bazs(lat_org, lon_org, az_org, evla, evlo, coordx):
    """Back-azimuths relative to the profile (bazs - az_org, radians), as the host passes them on."""
    return backazimuth_grids(lat_org, lon_org, az_org, evla, evlo, coordx) - az_org * DEG2RAD
