"""Generate the golden fixtures in tests/golden/ from the reference's own shipped libraries.

Runs only where the reference tree is present and the x86-64 harness is built
(``make -C oracle ref``); the GPU machine never runs this.  Usage (from the repo root):

    LD_LIBRARY_PATH=oracle/_ref/rt python tests/golden/make_golden.py

Fixtures:

* ``step_<name>.npz`` - one call of the shipped ``updatedispl_`` on seeded
  random state (wavefield, PML split fields, memory variables, background
  strips) and heterogeneous material: inputs and outputs (``step_top_*``: the
  PML-on-top mode, izt = 1 - npml).
* ``loop_layered.npz`` - the time loop of src/FDFK2D.f90:465-532 driven by the
  shipped ``updatedispl_`` and ``loadseis`` restated from src/Submain.f90:33-116,
  with background strips from the shipped ``comput_background_wavefield_``
  (two-layer model, P incidence): FK inputs, strips, seismograms, final state.
* ``fk_<name>.npz`` - one call of the shipped ``comput_background_wavefield_``
  with different left and right layered models and back-azimuths that vary
  along the profile: its inputs and the 12 background strips.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import refharness as R  # noqa: E402


def _coefs(norder):
    h = R.load()[0]
    c0 = np.zeros((norder, norder), np.float64, order="F")
    c1 = np.zeros((norder, norder), np.float64, order="F")
    h.fdfk_op_fd_coef0(C.c_int(norder), c0.ctypes.data_as(C.c_void_p))
    h.fdfk_op_fd_coef1(C.c_int(norder), c1.ctypes.data_as(C.c_void_p))
    return c0, c1


def material(rng, NZ, NX, hetero=True):
    vp = 4000 + 4000 * rng.random((NZ, NX)) if hetero else np.full((NZ, NX), 6000.0)
    vs = vp / (1.6 + 0.6 * rng.random((NZ, NX))) if hetero else vp / 1.73
    rho = 1740.0 * (vp / 1000.0) ** 0.25
    c = np.zeros((3, NZ, NX), np.float32, order="F")
    c[0] = rho
    c[1] = rho * (vp * vp - 2 * vs * vs)
    c[2] = rho * vs * vs
    return c


def step_case(name, seed, nx, nz, npml, norder, dx=200.0, dz=200.0, dt=0.01, top=False):
    """top: the PML-on-top mode (is_PML_top, izt = 1 - npml: npml more rows above row 1)."""
    rng = np.random.default_rng(seed)
    nbd = 2 * norder - 1
    izt = 1 - npml if top else 1
    NZ, NX = nz + npml - izt + 1, nx + 2 * npml
    nt = 0
    p = dict(norder=norder, nx=nx, nz=nz, npml=npml, izt=izt, is_PML_top=top, npower=2, nbd=nbd, nt=nt,
             dx=dx, dz=dz, dt=dt, R0=1e-3)
    c = material(rng, NZ, NX)
    p["vpml"] = float(np.sqrt((c[1] + 2 * c[2]) / c[0]).max())
    strips = {k: np.asfortranarray(rng.standard_normal(s).astype(np.float32))
              for k, s in R.strip_shapes(nx, nz, nbd, nt).items()}
    ux = np.asfortranarray(rng.standard_normal((2, NZ, NX)).astype(np.float32))
    uz = np.asfortranarray(rng.standard_normal((2, NZ, NX)).astype(np.float32))
    ps = R.pml_shapes(nx, nz, npml)
    bp = {k: np.asfortranarray((1e3 * rng.standard_normal(ps[k])).astype(np.float32)) for k in R.BP}
    bu = {k: np.asfortranarray(rng.standard_normal(ps[k]).astype(np.float32)) for k in R.BU}
    c0, c1 = _coefs(norder)
    out = {"params": np.array([repr(p)]), "c": c, "coef0": c0, "coef1": c1, "it": np.array(0)}
    out.update({"in_" + k: v.copy(order="F") for k, v in strips.items()})
    out.update({"in_ux": ux.copy(order="F"), "in_uz": uz.copy(order="F")})
    out.update({"in_" + k: v.copy(order="F") for k, v in bp.items()})
    out.update({"in_" + k: v.copy(order="F") for k, v in bu.items()})
    R.updatedispl(p, strips, c, c0, c1, ux, uz, bp, bu, it=0)
    out.update({"out_ux": ux, "out_uz": uz})
    out.update({"out_" + k: v for k, v in bp.items()})
    out.update({"out_" + k: v for k, v in bu.items()})
    np.savez_compressed(os.path.join(HERE, f"step_{name}.npz"), **out)
    print("wrote", name)


def layered_model(NZ, NX, dz, moho, vp=(6300.0, 8100.0), vs=(3600.0, 4500.0)):
    zz = (np.arange(1, NZ + 1) - 1) * dz
    VP = np.where(zz < moho, vp[0], vp[1])[:, None] * np.ones((1, NX))
    VS = np.where(zz < moho, vs[0], vs[1])[:, None] * np.ones((1, NX))
    RHO = 1740.0 * (VP / 1000.0) ** 0.25
    c = np.zeros((3, NZ, NX), np.float32, order="F")
    c[0] = RHO
    c[1] = RHO * (VP ** 2 - 2 * VS ** 2)
    c[2] = RHO * VS ** 2
    fk = np.zeros((4, 2), np.float32, order="F")
    fk[0] = [0.0, moho]
    fk[1] = vp
    fk[2] = vs
    fk[3] = 1740.0 * (np.asarray(vp) / 1000.0) ** 0.25
    return c, fk


def loop_case():
    nx, nz, npml, norder = 40, 24, 8, 3
    nbd = 2 * norder - 1
    dx = dz = 250.0
    dt = 0.015
    nt = 240
    NZ, NX = nz + npml, nx + 2 * npml
    c, fk = layered_model(NZ, NX, dz, moho=3000.0)
    p = dict(norder=norder, nx=nx, nz=nz, npml=npml, izt=1, is_PML_top=False, npower=2, nbd=nbd, nt=nt,
             dx=dx, dz=dz, dt=dt, R0=1e-3, x0=0.0, z0=0.0, src_type=True, ds=1e-3, f0=2.0, rayp=0.06e-3)
    p["vpml"] = float(np.sqrt((c[1] + 2 * c[2]) / c[0]).max())
    strips = {k: np.zeros(s, np.float32, order="F") for k, s in R.strip_shapes(nx, nz, nbd, nt).items()}
    bazs = np.zeros(NX, np.float64)
    R.comput_background_wavefield(p, bazs, fk, fk.copy(order="F"), strips)
    rx = np.arange(0.0, (nx - 1) * dx + 1, 2 * dx, dtype=np.float32)
    rz = np.zeros_like(rx)
    rx = np.append(rx, np.float32(4875.0))
    rz = np.append(rz, np.float32(1130.0))    # one buried receiver off the grid nodes
    nstp = 2
    nsis = nt // nstp
    c0, c1 = _coefs(norder)
    ux = np.zeros((2, NZ, NX), np.float32, order="F")
    uz = np.zeros_like(ux, order="F")
    ps = R.pml_shapes(nx, nz, npml)
    bp = {k: np.zeros(ps[k], np.float32, order="F") for k in R.BP}
    bu = {k: np.zeros(ps[k], np.float32, order="F") for k in R.BU}
    h = R.load()[0]
    sx = np.zeros((nsis + 1, len(rx)), np.float32, order="F")
    sz = np.zeros_like(sx, order="F")
    isis = istp = 0
    for it in range(nt + 1):
        if isis == it and istp <= nsis:
            for r in range(len(rx)):
                a, b = C.c_float(), C.c_float()
                h.fdfk_op_loadseis(C.c_int(nx), C.c_int(nz), C.c_int(npml), C.c_int(1), C.c_float(0.0), C.c_float(0.0),
                                   C.c_float(dx), C.c_float(dz), C.c_float(rx[r]), C.c_float(rz[r]),
                                   ux.ctypes.data_as(C.c_void_p), uz.ctypes.data_as(C.c_void_p), C.byref(a), C.byref(b))
                sx[istp, r] = a.value
                sz[istp, r] = b.value
            istp += 1
            isis += nstp
        R.updatedispl(p, strips, c, c0, c1, ux, uz, bp, bu, it=it)
    out = {"params": np.array([repr(p)]), "c": c, "fk_left": fk, "fk_right": fk.copy(order="F"), "bazs": bazs,
           "rx": rx, "rz": rz, "nstp": np.array(nstp), "nsis": np.array(nsis), "seisx": sx, "seisz": sz,
           "out_ux": ux, "out_uz": uz}
    out.update({k: v for k, v in strips.items()})
    np.savez_compressed(os.path.join(HERE, "loop_layered.npz"), **out)
    print("wrote loop_layered", "max|uz| %.3e" % np.abs(sz).max())


FK_LEFT = np.array([[0.0, 2000.0], [6300.0, 8100.0], [3600.0, 4500.0], [2750.0, 3300.0]], np.float32)
FK_RIGHT = np.array([[0.0, 900.0, 2600.0], [5500.0, 6300.0, 8100.0], [3200.0, 3600.0, 4500.0],
                     [2600.0, 2750.0, 3300.0]], np.float32)


def fk_case(name, src_type, rayp, baz_deg, f0, nt, dt, x0, z0, nx=16, nz=12, npml=6, nbd=3, dx=250.0, dz=200.0):
    p = dict(nx=nx, nz=nz, npml=npml, izt=1, nbd=nbd, nt=nt, src_type=src_type, x0=x0, z0=z0, dx=dx, dz=dz,
             dt=dt, ds=1e-3, f0=f0, rayp=rayp)
    bazs = np.deg2rad(np.linspace(baz_deg[0], baz_deg[1], nx + 2 * npml))
    fl = np.asfortranarray(FK_LEFT)
    fr = np.asfortranarray(FK_RIGHT)
    strips = {k: np.zeros(s, np.float32, order="F") for k, s in R.strip_shapes(nx, nz, nbd, nt).items()}
    R.comput_background_wavefield(p, bazs, fl, fr, strips)
    out = {"params": np.array([repr(p)]), "fk_left": fl, "fk_right": fr, "bazs": bazs}
    out.update(strips)
    np.savez_compressed(os.path.join(HERE, f"fk_{name}.npz"), **out)
    print("wrote fk", name, "max %.3e" % max(np.abs(v).max() for v in strips.values()))


if __name__ == "__main__":
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    step_case("n3", 11, nx=30, nz=18, npml=12, norder=3)
    step_case("n1", 12, nx=24, nz=12, npml=4, norder=1)
    step_case("n8", 13, nx=40, nz=30, npml=16, norder=8)
    step_case("n3_minpml_aniso", 14, nx=20, nz=14, npml=5, norder=3, dx=250.0, dz=125.0)
    step_case("n2_odd", 15, nx=17, nz=11, npml=7, norder=2, dx=150.0, dz=175.0, dt=0.008)
    # PML on top
    step_case("top_n2", 16, nx=20, nz=14, npml=6, norder=2, top=True)
    step_case("top_n3", 17, nx=26, nz=18, npml=8, norder=3, dx=250.0, dz=200.0, top=True)
    step_case("top_n1", 18, nx=15, nz=9, npml=3, norder=1, dx=180.0, dz=220.0, dt=0.008, top=True)
    loop_case()
    # P from the right (cos of the mean back-azimuth > 0), grid offset
    fk_case("p_ramp", True, 0.07e-3, (-25.0, 20.0), 2.0, 120, 0.01, x0=-1500.0, z0=0.0)
    # S from the left (cos < 0), low corner frequency, buried grid top
    fk_case("s_left", False, 0.11e-3, (160.0, 200.0), 1.2, 110, 0.012, x0=500.0, z0=300.0)
