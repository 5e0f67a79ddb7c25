"""ORACLE (test infrastructure only): the reference's shipped libraries as a black box.

Loads FDFK2D's closed gfortran builds ``lib_gnu/libHybrid.so``, ``libPML.so``
and ``libFK3D.so`` together with ``oracle/_ref/libfdfk_refharness.so`` (which
provides the FD operators, an FFTW3 legacy-interface shim and LAPACK
zgetrf/zgetrs) and calls the two entry points the reference host calls:

* ``updatedispl_``  (68 arguments, src/FDFK2D.f90:516-522)
* ``comput_background_wavefield_`` (32 arguments, src/FDFK2D.f90:432-434)

Only usable on x86-64 with the reference tree present and the harness built
(``make -C oracle ref``).  The dynamic loader must find ``libgfortran.so.5``:
callers run inside :func:`env` (``LD_LIBRARY_PATH`` is read at process start,
so tests spawn a child process with it).

All arrays are numpy arrays in Fortran order with the reference's shapes
(``FDFK2D.f90:253-355``): e.g. ``ux`` has shape ``(2, nz+npml-izt+1, nx+2*npml)``.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
RT = os.path.join(REF, "rt")
LIBDIR = os.path.join(REF, "lib_gnu")
HARNESS = os.path.join(REF, "libfdfk_refharness.so")


def available() -> bool:
    return (platform.machine() in ("x86_64", "AMD64") and os.path.exists(HARNESS)
            and os.path.exists(os.path.join(LIBDIR, "libHybrid.so")))


def env() -> dict:
    e = dict(os.environ)
    e["LD_LIBRARY_PATH"] = RT + os.pathsep + e.get("LD_LIBRARY_PATH", "")
    return e


def run_child(args, **kw):
    """Run ``python args...`` with the loader path needed by the shipped libraries."""
    return subprocess.run([sys.executable] + list(args), env=env(), **kw)


_libs = None


def load():
    global _libs
    if _libs is not None:
        return _libs
    if not available():
        raise RuntimeError("reference harness unavailable (x86-64 + make -C oracle ref needed)")
    mode = C.RTLD_GLOBAL | os.RTLD_LAZY
    C.CDLL("libgomp.so.1", mode)
    C.CDLL(os.path.join(RT, "libgfortran.so.5"), mode)
    h = C.CDLL(HARNESS, mode)
    pml = C.CDLL(os.path.join(LIBDIR, "libPML.so"), mode)
    hyb = C.CDLL(os.path.join(LIBDIR, "libHybrid.so"), mode)
    fk = C.CDLL(os.path.join(LIBDIR, "libFK3D.so"), mode)
    _libs = (h, pml, hyb, fk)
    return _libs


def _i(v):
    return C.byref(C.c_int(int(v)))


def _f(v):
    return C.byref(C.c_float(float(v)))


def _d(v):
    return C.byref(C.c_double(float(v)))


def _l(v):
    return C.byref(C.c_int(1 if v else 0))


def _p(a: np.ndarray, dtype=np.float32):
    assert a.dtype == dtype and a.flags.f_contiguous, (a.dtype, a.flags)
    return a.ctypes.data_as(C.c_void_p)


STRIPS = ("uxl_reg", "uzl_reg", "uxr_reg", "uzr_reg", "uxb_reg", "uzb_reg",
          "uxl_pml", "uzl_pml", "uxr_pml", "uzr_pml", "uxb_pml", "uzb_pml")
BP = ("bpxlx", "bpzlx", "bpxrx", "bpzrx", "bpxtx", "bpxtz", "bpztx", "bpztz",
      "bpxbx", "bpxbz", "bpzbx", "bpzbz")
BU = tuple(f"bu{c}{k}{s}" for s in "lrbt" for c in "xz" for k in "123")


def strip_shapes(nx, nz, nbd, nt):
    """Background-strip shapes, src/FDFK2D.f90:328-355 (last axis = time 0..nt)."""
    T = nt + 1
    return {
        "uxl_reg": (nz - nbd, nbd, T), "uzl_reg": (nz - nbd, nbd, T),
        "uxr_reg": (nz - nbd, nbd, T), "uzr_reg": (nz - nbd, nbd, T),
        "uxb_reg": (nbd, nx, T), "uzb_reg": (nbd, nx, T),
        "uxl_pml": (nz, nbd, T), "uzl_pml": (nz, nbd, T),
        "uxr_pml": (nz, nbd, T), "uzr_pml": (nz, nbd, T),
        "uxb_pml": (nbd, nx + 2 * nbd, T), "uzb_pml": (nbd, nx + 2 * nbd, T),
    }


def pml_shapes(nx, nz, npml):
    """PML auxiliary-array shapes, src/FDFK2D.f90:260-306."""
    X = nx + 2 * npml
    s = {
        "bpxlx": (nz, npml), "bpzlx": (nz, npml), "bpxrx": (nz, npml), "bpzrx": (nz, npml),
    }
    for k in ("bpxtx", "bpxtz", "bpztx", "bpztz", "bpxbx", "bpxbz", "bpzbx", "bpzbz"):
        s[k] = (npml, X)
    for name in BU:
        side = name[-1]
        s[name] = (2, nz, npml) if side in "lr" else (2, npml, X)
    return s


def updatedispl(p: dict, strips: dict, c: np.ndarray, coef0, coef1, ux, uz, bp: dict, bu: dict, it: int):
    """One call of the shipped ``updatedispl_`` (src/FDFK2D.f90:516-522); mutates arrays in place."""
    _, _, hyb, _ = load()
    args = [_i(p["norder"]), _i(p["nx"]), _i(p["nz"]), _i(p["npml"]), _i(p["izt"]), _l(p["is_PML_top"]),
            _i(p["npower"]), _i(p["nbd"]), _i(it), _i(p["nt"]), _f(p["dx"]), _f(p["dz"]), _d(p["dt"]),
            _f(p["vpml"]), _d(p["R0"])]
    args += [_p(strips[k]) for k in STRIPS]
    args += [_p(c), _p(coef0, np.float64), _p(coef1, np.float64), _p(ux), _p(uz)]
    args += [_p(bp[k]) for k in BP]
    args += [_p(bu[k]) for k in BU]
    assert len(args) == 68
    hyb.updatedispl_(*args)


def comput_background_wavefield(p: dict, bazs: np.ndarray, fk_left: np.ndarray, fk_right: np.ndarray,
                                strips: dict):
    """One call of the shipped ``comput_background_wavefield_`` (src/FDFK2D.f90:432-434)."""
    _, _, _, fk = load()
    args = [_i(p["nx"]), _i(p["nz"]), _i(p["npml"]), _i(p["izt"]), _i(p["nbd"]), _i(p["nt"]),
            _i(fk_left.shape[1]), _i(fk_right.shape[1]), _l(p["src_type"]),
            _f(p["x0"]), _f(p["z0"]), _f(p["dx"]), _f(p["dz"]), _d(p["dt"]), _f(p["ds"]), _f(p["f0"]),
            _d(p["rayp"]), _p(bazs, np.float64), _p(fk_left), _p(fk_right)]
    args += [_p(strips[k]) for k in STRIPS]
    assert len(args) == 32
    fk.comput_background_wavefield_(*args)


class Trace(C.Structure):
    _fields_ = [("name", C.c_char * 16), ("norder", C.c_int), ("nx", C.c_int), ("nz", C.c_int),
                ("npml", C.c_int), ("izt", C.c_int), ("mat", C.c_void_p), ("u", C.c_void_p),
                ("out", C.c_void_p), ("dump_off", C.c_long)]


def trace_enable(on: bool, cap_floats: int = 0):
    h = load()[0]
    h.fdfk_ref_trace_enable(C.c_int(1 if on else 0), C.c_long(cap_floats))


def trace_records(ncell: int):
    """Return [(name, mat, u, out)] copies recorded by the operator hooks."""
    h = load()[0]
    h.fdfk_ref_trace_get.restype = C.POINTER(Trace)
    h.fdfk_ref_trace_dump.restype = C.POINTER(C.c_float)
    n = h.fdfk_ref_trace_count()
    dump = h.fdfk_ref_trace_dump()
    out = []
    for i in range(n):
        r = h.fdfk_ref_trace_get(i).contents
        if r.dump_off >= 0:
            base = r.dump_off
            arr = np.ctypeslib.as_array(dump, shape=(base + 3 * ncell,))[base:base + 3 * ncell].copy()
            out.append((r.name.decode(), arr[:ncell], arr[ncell:2 * ncell], arr[2 * ncell:], r.mat, r.u, r.out))
        else:
            out.append((r.name.decode(), None, None, None, r.mat, r.u, r.out))
    h.fdfk_ref_trace_diff1_calls.restype = C.c_long
    h.fdfk_ref_trace_diffx1_calls.restype = C.c_long
    return out, h.fdfk_ref_trace_diff1_calls(), h.fdfk_ref_trace_diffx1_calls()
