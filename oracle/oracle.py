"""ORACLE (test infrastructure only): Python bindings of the C restatement.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
use this module.  It loads ``oracle/_build/libfdfk_oracle.so`` (built by
``make -C oracle``) and exposes:

* :func:`updatedispl` - one restated time step, same arrays as the reference
  call (src/FDFK2D.f90:516-522);
* :func:`simulate` - the restated time loop with receiver sampling
  (src/FDFK2D.f90:465-532);
* :func:`simulate64` - the same time loop with every field in FP64
  (``oracle/_build/libfdfk_oracle64.so``): the FP64 oracle the FP32 traces are
  stated against;
* :func:`simulate64_gpu` - the same FP64 time loop on the GPU
  (``oracle/_build/libfdfk_oracle_gpu.so``), for the full-size workloads;
* :func:`fd_coef0` / :func:`fd_coef1` / :func:`fd_coef2` (src/Submain.f90:1111-1245).

Array conventions match ``oracle/refharness.py``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libfdfk_oracle.so")
LIB64 = os.path.join(HERE, "_build", "libfdfk_oracle64.so")

STRIPS = ("uxl_reg", "uzl_reg", "uxr_reg", "uzr_reg", "uxb_reg", "uzb_reg",
          "uxl_pml", "uzl_pml", "uxr_pml", "uzr_pml", "uxb_pml", "uzb_pml")
BP = ("bpxlx", "bpzlx", "bpxrx", "bpzrx", "bpxtx", "bpxtz", "bpztx", "bpztz",
      "bpxbx", "bpxbz", "bpzbx", "bpzbz")
BU = tuple(f"bu{c}{k}{s}" for s in "lrbt" for c in "xz" for k in "123")


class Params(C.Structure):
    _fields_ = [("norder", C.c_int), ("nx", C.c_int), ("nz", C.c_int), ("npml", C.c_int), ("izt", C.c_int),
                ("npower", C.c_int), ("nbd", C.c_int), ("nt", C.c_int), ("dx", C.c_float), ("dz", C.c_float),
                ("dt", C.c_double), ("vpml", C.c_float), ("R0", C.c_double)]


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = C.CDLL(LIB)
        _lib.fdfk_oracle_updatedispl.restype = C.c_int
        _lib.fdfk_oracle_simulate.restype = C.c_int
    return _lib


class Params64(C.Structure):
    _fields_ = [("norder", C.c_int), ("nx", C.c_int), ("nz", C.c_int), ("npml", C.c_int), ("izt", C.c_int),
                ("npower", C.c_int), ("nbd", C.c_int), ("nt", C.c_int), ("dx", C.c_double), ("dz", C.c_double),
                ("dt", C.c_double), ("vpml", C.c_double), ("R0", C.c_double)]


_lib64 = None


def lib64():
    global _lib64
    if _lib64 is None:
        if not os.path.exists(LIB64):
            build()
        _lib64 = C.CDLL(LIB64)
        _lib64.fdfk_oracle_simulate.restype = C.c_int
    return _lib64


def simulate64(p, strips, c, rx, rz, x0, z0, nstp, nsis, steps_limit=-1):
    """The restated time loop in FP64 (inputs widened); returns float64 (seisx, seisz), (nsis+1, nrcv)."""
    L = lib64()
    nrcv = len(rx)
    d = lambda a: np.asfortranarray(a, np.float64)
    seisx = np.zeros((nsis + 1, nrcv), np.float64, order="F")
    seisz = np.zeros((nsis + 1, nrcv), np.float64, order="F")
    st = {k: d(strips[k]) for k in STRIPS}
    sp = (C.c_void_p * 12)(*[st[k].ctypes.data_as(C.c_void_p) for k in STRIPS])
    cd = d(c)
    rxa = np.asarray(rx, np.float64)
    rza = np.asarray(rz, np.float64)
    prm = Params64(int(p["norder"]), int(p["nx"]), int(p["nz"]), int(p["npml"]), int(p["izt"]),
                   int(p.get("npower", 2)), int(p["nbd"]), int(p["nt"]), float(p["dx"]), float(p["dz"]),
                   float(p["dt"]), float(p["vpml"]), float(p.get("R0", 1e-3)))
    rc = L.fdfk_oracle_simulate(C.byref(prm), sp, cd.ctypes.data_as(C.c_void_p), C.c_int(nrcv),
                                rxa.ctypes.data_as(C.c_void_p), rza.ctypes.data_as(C.c_void_p), C.c_double(x0),
                                C.c_double(z0), C.c_int(nstp), C.c_int(nsis), seisx.ctypes.data_as(C.c_void_p),
                                seisz.ctypes.data_as(C.c_void_p), C.c_int(steps_limit))
    if rc != 0:
        raise RuntimeError(f"FP64 oracle simulate failed: {rc}")
    return seisx, seisz


def params(p: dict) -> Params:
    return Params(int(p["norder"]), int(p["nx"]), int(p["nz"]), int(p["npml"]), int(p["izt"]),
                  int(p.get("npower", 2)), int(p["nbd"]), int(p["nt"]), float(p["dx"]), float(p["dz"]),
                  float(p["dt"]), float(p["vpml"]), float(p.get("R0", 1e-3)))


def _ptr(a, dtype=np.float32):
    assert a.dtype == dtype and a.flags.f_contiguous
    return a.ctypes.data_as(C.c_void_p)


def _coef(fn, norder):
    out = np.zeros((norder, norder), np.float64, order="F")
    getattr(lib(), fn)(C.c_int(norder), _ptr(out, np.float64))
    return out


def fd_coef0(norder):
    return _coef("fdfk_op_fd_coef0", norder)


def fd_coef1(norder):
    return _coef("fdfk_op_fd_coef1", norder)


def fd_coef2(norder):
    return _coef("fdfk_op_fd_coef2", norder)


def dt_stable(nx, nz, npml, izt, norder, dx, dz, c):
    """check_stability's stable dt (src/Submain.f90:118-164), restated."""
    L = lib()
    L.fdfk_op_dt_stable.restype = C.c_float
    coef2 = fd_coef2(norder)
    return float(L.fdfk_op_dt_stable(C.c_int(nx), C.c_int(nz), C.c_int(npml), C.c_int(izt), C.c_int(norder),
                                     C.c_float(dx), C.c_float(dz), _ptr(coef2, np.float64),
                                     _ptr(np.asfortranarray(c, np.float32))))


def updatedispl(p, strips, c, coef0, coef1, ux, uz, bp, bu, it):
    L = lib()
    sp = (C.c_void_p * 12)(*[_ptr(strips[k]) for k in STRIPS])
    bpp = (C.c_void_p * 12)(*[_ptr(bp[k]) for k in BP])
    bup = (C.c_void_p * 24)(*[_ptr(bu[k]) for k in BU])
    prm = params(p)
    rc = L.fdfk_oracle_updatedispl(C.byref(prm), C.c_int(it), sp, _ptr(c), _ptr(coef0, np.float64),
                                   _ptr(coef1, np.float64), _ptr(ux), _ptr(uz), bpp, bup)
    if rc != 0:
        raise RuntimeError(f"oracle updatedispl failed: {rc}")


def simulate(p, strips, c, rx, rz, x0, z0, nstp, nsis, steps_limit=-1):
    """Restated time loop; returns (seisx, seisz) of shape (nsis+1, nrcv), Fortran order."""
    L = lib()
    nrcv = len(rx)
    seisx = np.zeros((nsis + 1, nrcv), np.float32, order="F")
    seisz = np.zeros((nsis + 1, nrcv), np.float32, order="F")
    sp = (C.c_void_p * 12)(*[_ptr(strips[k]) for k in STRIPS])
    rxa = np.asarray(rx, np.float32)
    rza = np.asarray(rz, np.float32)
    prm = params(p)
    rc = L.fdfk_oracle_simulate(C.byref(prm), sp, _ptr(c), C.c_int(nrcv), rxa.ctypes.data_as(C.c_void_p),
                                rza.ctypes.data_as(C.c_void_p), C.c_float(x0), C.c_float(z0), C.c_int(nstp),
                                C.c_int(nsis), _ptr(seisx), _ptr(seisz), C.c_int(steps_limit))
    if rc != 0:
        raise RuntimeError(f"oracle simulate failed: {rc}")
    return seisx, seisz


LIBGPU = os.path.join(HERE, "_build", "libfdfk_oracle_gpu.so")


class ParamsGpu(C.Structure):
    _fields_ = [("norder", C.c_int), ("nx", C.c_int), ("nz", C.c_int), ("npml", C.c_int), ("izt", C.c_int),
                ("npower", C.c_int), ("nbd", C.c_int), ("nt", C.c_int), ("dx", C.c_double), ("dz", C.c_double),
                ("dt", C.c_double), ("vpml", C.c_double), ("R0", C.c_double)]


_libgpu = None


def libgpu():
    """oracle/_build/libfdfk_oracle_gpu.so: the FP64 GPU oracle (oracle/fdfk_oracle_gpu.cu)."""
    global _libgpu
    if _libgpu is None:
        if not os.path.exists(LIBGPU):
            build()
        _libgpu = C.CDLL(LIBGPU)
        _libgpu.fdfk_oracle_gpu_simulate.restype = C.c_int
    return _libgpu


def strips_to_device(strips, device="cuda"):
    """Twelve background strips as float64 tensors on the GPU in the reference's memory layout.

    A strip of Fortran shape (n1, n2, nt+1) becomes a C-contiguous tensor of shape (nt+1, n2, n1),
    the same bytes.  Tensors already on the device pass through (they must have that form)."""
    import torch
    out = {}
    for k in STRIPS:
        a = strips[k]
        if isinstance(a, torch.Tensor):
            t = a.to(device=device, dtype=torch.float64)
        else:
            t = torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.float64).transpose(2, 1, 0))).to(device)
        out[k] = t.contiguous()
    return out


def simulate64_gpu(p, strips, c, rx, rz, x0, z0, nstp, nsis, steps_limit=-1, fields=False):
    """The restated time loop in FP64 on the GPU (oracle/fdfk_oracle_gpu.cu).

    strips: numpy arrays in the reference layout, or float64 CUDA tensors of shape (nt+1, n2, n1)
    (see :func:`strips_to_device`).  Returns float64 (seisx, seisz) of shape (nsis+1, nrcv), and
    with fields=True also level 1 of ux, uz after the last step, shape (nz+npml, nx+2npml)."""
    import torch
    L = libgpu()
    dev = strips_to_device(strips)
    sp = (C.c_void_p * 12)(*[C.c_void_p(dev[k].data_ptr()) for k in STRIPS])
    nrcv = len(rx)
    seisx = np.zeros((nsis + 1, nrcv), np.float64, order="F")
    seisz = np.zeros((nsis + 1, nrcv), np.float64, order="F")
    cf = np.asfortranarray(c, np.float32)
    rxa = np.ascontiguousarray(rx, np.float64)
    rza = np.ascontiguousarray(rz, np.float64)
    NZ, NX = int(p["nz"]) + int(p["npml"]), int(p["nx"]) + 2 * int(p["npml"])
    ux = np.zeros((NZ, NX), np.float64, order="F") if fields else None
    uz = np.zeros((NZ, NX), np.float64, order="F") if fields else None
    prm = ParamsGpu(int(p["norder"]), int(p["nx"]), int(p["nz"]), int(p["npml"]), int(p.get("izt", 1)),
                    int(p.get("npower", 2)), int(p["nbd"]), int(p["nt"]), float(p["dx"]), float(p["dz"]),
                    float(p["dt"]), float(p["vpml"]), float(p.get("R0", 1e-3)))
    torch.cuda.synchronize()
    rc = L.fdfk_oracle_gpu_simulate(C.byref(prm), sp, cf.ctypes.data_as(C.c_void_p), C.c_int(nrcv),
                                    rxa.ctypes.data_as(C.c_void_p), rza.ctypes.data_as(C.c_void_p), C.c_double(x0),
                                    C.c_double(z0), C.c_int(nstp), C.c_int(nsis), seisx.ctypes.data_as(C.c_void_p),
                                    seisz.ctypes.data_as(C.c_void_p), C.c_int(steps_limit),
                                    ux.ctypes.data_as(C.c_void_p) if fields else None,
                                    uz.ctypes.data_as(C.c_void_p) if fields else None)
    if rc != 0:
        raise RuntimeError(f"FP64 GPU oracle simulate failed: {rc}")
    return (seisx, seisz, ux, uz) if fields else (seisx, seisz)
