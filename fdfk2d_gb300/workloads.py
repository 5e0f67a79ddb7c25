"""Seeded synthetic workloads in the reference's input conventions (SI units).

* :func:`config1` - 200 km x 100 km at 250 m (801 x 401), two layers
  (crust 0-35 km Vp 6.3 / Vs 3.6 km/s over mantle Vp 8.1 / Vs 4.5 km/s),
  20-cell PML, free surface, dt = 0.015 s, nt = 4000, 101 surface receivers
  every 2 km, P incidence at 0.06 s/km, 1 Hz Ricker.
* :func:`config2` - 400 km x 200 km at 100 m (4001 x 2001), 40-cell PML,
  Moho dipping linearly 35 -> 55 km across the profile, a 60 km wide, 3 km
  deep sediment basin (Vp 3.0 / Vs 1.5 km/s), a 3 % (std) Gaussian-smoothed
  Vp/Vs perturbation with 5 km correlation length (seeded), dt = 0.006 s,
  nt = 12000, 401 surface receivers, P incidence at 0.07 s/km.

Density follows Gardner's rule rho = 1.74 Vp^0.25 g/cc with Vp in km/s
(stored in kg/m^3).  FD order 6 (norder = 3) for both.

:func:`plane_wave_background` fills the twelve background strips with an
analytic P plane wave (Ricker wavelet) in the half-space below the model: a
seeded stand-in for the FK background with the same shapes and value range,
used where only the cost of the time loop matters.  :func:`fk_inputs` gives the
arguments of the FK background (the 1-D models on either side) for the GPU
FK path.
"""
from __future__ import annotations

import math

import numpy as np

from .api import STRIPS, strip_shapes


def gardner(vp):
    return 1740.0 * (np.asarray(vp, np.float64) / 1000.0) ** 0.25


def pack_c(vp, vs):
    """c(1:3, NZ, NX) = rho, lambda, mu (src/Input.f90:364-378 with Gardner density)."""
    rho = gardner(vp)
    c = np.empty((3,) + vp.shape, np.float32, order="F")
    c[0] = rho
    c[1] = rho * (vp * vp - 2.0 * vs * vs)
    c[2] = rho * vs * vs
    return c


def _smooth_noise(rng, NZ, NX, h, corr, std):
    """Gaussian-smoothed white noise with correlation length `corr` (m), formed on a coarse grid."""
    step = max(1, int(round(corr / h / 5)))
    nzc, nxc = NZ // step + 3, NX // step + 3
    w = rng.standard_normal((nzc, nxc))
    sig = corr / (h * step)
    r = int(math.ceil(3 * sig))
    k = np.exp(-0.5 * (np.arange(-r, r + 1) / sig) ** 2)
    k /= k.sum()
    w = np.apply_along_axis(lambda v: np.convolve(v, k, mode="same"), 0, w)
    w = np.apply_along_axis(lambda v: np.convolve(v, k, mode="same"), 1, w)
    w = (w - w.mean()) / w.std() * std
    zi = np.arange(NZ) / step
    xi = np.arange(NX) / step
    z0 = np.floor(zi).astype(int)
    x0 = np.floor(xi).astype(int)
    fz = (zi - z0)[:, None]
    fx = (xi - x0)[None, :]
    a = w[z0][:, x0]
    b = w[z0 + 1][:, x0]
    c = w[z0][:, x0 + 1]
    d = w[z0 + 1][:, x0 + 1]
    return (a * (1 - fz) * (1 - fx) + b * fz * (1 - fx) + c * (1 - fz) * fx + d * fz * fx)


def _base(name, nx, nz, npml, h, dt, nt, nrcv, rayp_s_per_km, f0):
    p = dict(norder=3, nx=nx, nz=nz, npml=npml, nt=nt, dx=h, dz=h, dt=dt, npower=2, R0=1e-3,
             is_PML_top=False, nbd=5)
    rx = np.linspace(0.0, (nx - 1) * h, nrcv).astype(np.float32)
    rz = np.zeros(nrcv, np.float32)
    return dict(name=name, p=p, rx=rx, rz=rz, x0=0.0, z0=0.0, nstp=1, nsis=nt,
                rayp=rayp_s_per_km * 1e-3, f0=f0)


def config1(nt=4000):
    w = _base("config1: 200x100 km, 801x401 @ 250 m, 2 layers, P 0.06 s/km, nt=4000", 801, 401, 20, 250.0, 0.015,
              nt, 101, 0.06, 1.0)
    p = w["p"]
    NZ, NX = p["nz"] + p["npml"], p["nx"] + 2 * p["npml"]
    z = (np.arange(NZ) * p["dz"])[:, None] * np.ones((1, NX))
    vp = np.where(z < 35e3, 6300.0, 8100.0)
    vs = np.where(z < 35e3, 3600.0, 4500.0)
    w["c"] = pack_c(vp, vs)
    w["vp_half"] = 8100.0
    p["vpml"] = float(vp.max())
    return w


def config2(nt=12000, seed=2024):
    w = _base("config2: 400x200 km, 4001x2001 @ 100 m, dipping Moho + basin + 3% perturbation, P 0.07 s/km, "
              "nt=12000", 4001, 2001, 40, 100.0, 0.006, nt, 401, 0.07, 1.0)
    p = w["p"]
    rng = np.random.default_rng(seed)
    NZ, NX = p["nz"] + p["npml"], p["nx"] + 2 * p["npml"]
    h = p["dx"]
    x = ((np.arange(NX) - p["npml"]) * h)[None, :]
    z = (np.arange(NZ) * h)[:, None]
    L = (p["nx"] - 1) * h
    moho = 35e3 + 20e3 * np.clip(x / L, 0.0, 1.0)
    mantle = z >= moho
    vp = np.where(mantle, 8100.0, 6300.0)
    vs = np.where(mantle, 4500.0, 3600.0)
    basin = (np.abs(x - 0.3 * L) <= 30e3) & (z < 3e3)
    vp = np.where(basin, 3000.0, vp)
    vs = np.where(basin, 1500.0, vs)
    pert = _smooth_noise(rng, NZ, NX, h, 5e3, 0.03)
    vp = vp * (1.0 + pert)
    vs = vs * (1.0 + pert)
    w["c"] = pack_c(vp, vs)
    w["vp_half"] = 8100.0
    w["fk_moho"] = (33e3, 50e3)
    p["vpml"] = float(vp.max())
    return w


def strip_coords(p, name):
    """Fortran (iz, ix) of every element of a background strip (src/FDFK2D.f90:328-355)."""
    nx, nz, nbd = p["nx"], p["nz"], p["nbd"]
    side, kind = name[2], name[4:]
    if kind == "reg":
        if side == "l":
            iz, ix = np.arange(1, nz - nbd + 1), np.arange(1, nbd + 1)
        elif side == "r":
            iz, ix = np.arange(1, nz - nbd + 1), np.arange(nx - nbd + 1, nx + 1)
        else:
            iz, ix = np.arange(nz - nbd + 1, nz + 1), np.arange(1, nx + 1)
    else:
        if side == "l":
            iz, ix = np.arange(1, nz + 1), np.arange(1 - nbd, 1)
        elif side == "r":
            iz, ix = np.arange(1, nz + 1), np.arange(nx + 1, nx + nbd + 1)
        else:
            iz, ix = np.arange(nz + 1, nz + nbd + 1), np.arange(1 - nbd, nx + nbd + 1)
    return iz, ix


def plane_wave_background(w, t0_index=0, count=None, out=None, amp=1e-3):
    """Analytic upgoing P plane wave on the strips for time indices [t0_index, t0_index + count).

    Returns dict name -> float32 Fortran array (n1, n2, count) (or fills `out`, arrays of the same
    shape, e.g. views of pinned buffers).  u = amp * ricker(t - tau) * (sin th, -cos th),
    tau = t_s + p x - eta z, eta = sqrt(1/vp^2 - p^2).
    """
    p = w["p"]
    if count is None:
        count = p["nt"] + 1 - t0_index
    vp = w["vp_half"]
    ray = w["rayp"]
    eta = math.sqrt(max(1.0 / vp ** 2 - ray ** 2, 0.0))
    sin_t, cos_t = ray * vp, eta * vp
    f0 = w["f0"]
    zmax = (p["nz"] + p["npml"]) * p["dz"]
    ts = 1.5 / f0 + eta * zmax
    t = (np.arange(t0_index, t0_index + count) * p["dt"]).astype(np.float64)
    res = {} if out is None else out
    for name in STRIPS:
        iz, ix = strip_coords(p, name)
        x = w["x0"] + (ix - 1) * p["dx"]
        z = w["z0"] + (iz - 1) * p["dz"]
        tau = ts + ray * x[None, :] - eta * z[:, None]
        arg = (np.pi * f0 * (t[None, None, :] - tau[:, :, None])) ** 2
        val = amp * (1.0 - 2.0 * arg) * np.exp(-arg)
        comp = sin_t if name[1] == "x" else -cos_t
        v = (val * comp).astype(np.float32)
        if out is None:
            res[name] = np.asfortranarray(v)
        else:
            res[name][...] = v
    return res


def _fk_model(moho_m):
    """Two-layer FK model (4, 2): z_top, vp, vs, rho (crust over mantle)."""
    vp = np.array([6300.0, 8100.0])
    return np.asfortranarray(np.stack([[0.0, moho_m], vp, [3600.0, 4500.0], gardner(vp)]).astype(np.float32))


def fk_inputs(w, ds=1e-3):
    """Arguments of comput_background_wavefield for a workload: (params, bazs, fk_left, fk_right).

    config 1: the same crust (0-35 km) over mantle on both sides; config 2: crust 33 km thick on
    the left, 50 km on the right.  The profile lies along the back-azimuth (bazs = 0).
    """
    p = w["p"]
    fp = dict(nx=p["nx"], nz=p["nz"], npml=p["npml"], izt=1, nbd=p["nbd"], nt=p["nt"], src_type=True,
              x0=w["x0"], z0=w["z0"], dx=p["dx"], dz=p["dz"], dt=p["dt"], ds=ds, f0=w["f0"], rayp=w["rayp"])
    left, right = w.get("fk_moho", (35e3, 35e3))
    bazs = np.zeros(p["nx"] + 2 * p["npml"])
    return fp, bazs, _fk_model(left), _fk_model(right)


def config3_events(n=64, seed=7):
    """Plane-wave events of the batched workload (config 3, on the config-1 model): half P with
    ray parameters uniform in 0.04-0.08 s/km, half S in 0.10-0.12 s/km, back-azimuths uniform in
    0-360 degrees (taken along the profile), Ricker centre frequencies uniform in 0.5-1 Hz."""
    rng = np.random.default_rng(seed)
    ev = []
    for i in range(n):
        p_wave = i < n // 2
        lo, hi = (0.04, 0.08) if p_wave else (0.10, 0.12)
        ev.append(dict(p_wave=p_wave, rayp=float(rng.uniform(lo, hi)) * 1e-3, baz=float(rng.uniform(0.0, 360.0)),
                       f0=float(np.float32(rng.uniform(0.5, 1.0)))))
    return ev


def event_inputs(w, ev, ds=1e-3):
    """FK arguments (params, bazs, fk_left, fk_right) of one event on workload w."""
    fp, bazs, fl, fr = fk_inputs(w, ds=ds)
    fp = dict(fp, src_type=ev["p_wave"], rayp=ev["rayp"], f0=ev["f0"])
    bazs = np.full_like(bazs, np.deg2rad(ev["baz"]))
    return fp, bazs, fl, fr


def check_shapes(w, strips):
    p = w["p"]
    shp = strip_shapes(p["nx"], p["nz"], p["nbd"], p["nt"])
    for k in STRIPS:
        assert strips[k].shape[:2] == shp[k][:2], k


def config4_solves(n=96, seed=4):
    """The uneven batch (config 4): n solves with grid sizes nx log-uniform in 500-6000 and nz
    log-uniform in 250-2500, dx = dz uniform in 100-500 m, simulated length uniform in 20-120 s with
    dt from the CFL limit of FD order 6 (0.9 of it) and nt = length / dt; a random two- to four-layer
    crust/mantle model (crustal interfaces over a Moho at 30-55 km) with a 0-5 % Gaussian-smoothed
    Vp/Vs perturbation (5 km correlation); P (0.04-0.08 s/km) or S (0.10-0.12 s/km) incidence, back-
    azimuth uniform in 0-360 degrees, Ricker 0.5-1 Hz; 20-cell PML; receivers every 2 km at the
    surface.  Each entry: a workload dict as config1/config2 make, plus its event and FK models."""
    rng = np.random.default_rng(seed)
    cfl6 = 0.5752                         # sqrt(2 / ((cx + cz) (sum |c2| + sum c2))) of order 6
    out = []
    for i in range(n):
        nx = int(round(math.exp(rng.uniform(math.log(500), math.log(6000)))))
        nz = int(round(math.exp(rng.uniform(math.log(250), math.log(2500)))))
        h = float(np.float32(rng.uniform(100.0, 500.0)))
        length = float(rng.uniform(20.0, 120.0))
        nlayer = int(rng.integers(2, 5))
        moho = float(rng.uniform(30e3, 55e3))
        tops = [0.0] + sorted(float(t) for t in rng.uniform(2e3, moho - 2e3, nlayer - 2)) + [moho]
        vps = list(np.linspace(5600.0, 6800.0, nlayer - 1) + rng.uniform(-200.0, 200.0, nlayer - 1)) + [8100.0]
        vss = [v / 1.75 for v in vps[:-1]] + [4500.0]
        pert_std = float(rng.uniform(0.0, 0.05))
        npml = 20
        NZ, NX = nz + npml, nx + 2 * npml
        z = (np.arange(NZ) * h)[:, None]
        vp = np.zeros((NZ, 1))
        vs = np.zeros((NZ, 1))
        for t, a, b in zip(tops, vps, vss):
            vp = np.where(z >= t, a, vp)
            vs = np.where(z >= t, b, vs)
        vp = vp * np.ones((1, NX))
        vs = vs * np.ones((1, NX))
        if pert_std > 0.0:
            pert = _smooth_noise(rng, NZ, NX, h, 5e3, pert_std)
            vp = vp * (1.0 + pert)
            vs = vs * (1.0 + pert)
        vmax = float(vp.max())
        dt = float(0.9 * cfl6 * h / vmax)
        nt = int(math.ceil(length / dt))
        p_wave = bool(rng.random() < 0.5)
        lo, hi = (0.04, 0.08) if p_wave else (0.10, 0.12)
        ev = dict(p_wave=p_wave, rayp=float(rng.uniform(lo, hi)) * 1e-3, baz=float(rng.uniform(0.0, 360.0)),
                  f0=float(np.float32(rng.uniform(0.5, 1.0))))
        nrcv = max(2, int((nx - 1) * h // 2000.0) + 1)
        w = _base(f"config4 solve {i}: {nx}x{nz} @ {h:.0f} m, {nlayer} layers, {length:.0f} s", nx, nz, npml, h, dt,
                  nt, nrcv, ev["rayp"] * 1e3, ev["f0"])
        w["c"] = pack_c(vp, vs)
        w["p"]["vpml"] = vmax
        fkm = np.asfortranarray(np.stack([np.asarray(tops), np.asarray(vps), np.asarray(vss),
                                          gardner(np.asarray(vps))]).astype(np.float32))
        w["event"] = ev
        w["fk_model"] = fkm
        out.append(w)
    return out


def config4_inputs(w, ds=1e-3):
    """FK arguments (params, bazs, fk_left, fk_right) of a config-4 solve (same 1-D model both sides)."""
    p, ev = w["p"], w["event"]
    fp = dict(nx=p["nx"], nz=p["nz"], npml=p["npml"], izt=1, nbd=p["nbd"], nt=p["nt"], src_type=ev["p_wave"],
              x0=w["x0"], z0=w["z0"], dx=p["dx"], dz=p["dz"], dt=p["dt"], ds=ds, f0=ev["f0"], rayp=ev["rayp"])
    bazs = np.full(p["nx"] + 2 * p["npml"], np.deg2rad(ev["baz"]))
    return fp, bazs, w["fk_model"], w["fk_model"]
