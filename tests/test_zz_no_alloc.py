"""GPU: the allocation-free single-step entry point fdfk_step_noalloc, called through the C ABI,
against the existing drop-in updatedispl_ on two calls in a row, and its first call against one
step of the reference's shipped libraries.

The entry point serves callers that cannot allocate device memory themselves: a host program that
owns a fixed device budget, or code that runs where cudaMalloc is not allowed.  It carves every
buffer from one static device array, so these tests also check that a call leaves the device's
free memory unchanged.  This file is collected last, so a run that stops at the first failure has
already run every other test; it passes alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_npz, max_rel, step_inputs

pytestmark = pytest.mark.gpu

# Both are the FP32 GPU step; the drop-in may route the deep interior through the
# marching kernel, which sums in another order: max |difference| / max |value|.
TOL = 2e-6


@pytest.fixture(scope="module")
def F():
    import fdfk2d_gb300 as F
    from fdfk2d_gb300 import build
    build.build()
    L = F.lib()
    vp = C.POINTER(C.c_void_p)
    L.fdfk_step_noalloc.restype = C.c_int
    L.fdfk_step_noalloc.argtypes = [C.POINTER(F.Params), C.c_int, vp, C.c_void_p, C.c_void_p, C.c_void_p, vp, vp,
                                    C.c_void_p]
    L.fdfk_step_noalloc_capacity.restype = C.c_longlong
    L.fdfk_step_noalloc_need.restype = C.c_longlong
    L.fdfk_step_noalloc_need.argtypes = [C.POINTER(F.Params)]
    return F


def _noalloc(F, p, it, strips, c, ux, uz, bp, bu):
    prm = F.Params.from_dict(p)
    sp = (C.c_void_p * 12)(*[strips[k].ctypes.data for k in F.STRIPS])
    bpp = (C.c_void_p * 12)(*[bp[k].ctypes.data if k in bp else None for k in F.BP])
    bup = (C.c_void_p * 24)(*[bu[k].ctypes.data if k in bu else None for k in F.BU])
    return F.lib().fdfk_step_noalloc(C.byref(prm), it, sp, c.ctypes.data, ux.ctypes.data, uz.ctypes.data, bpp, bup,
                                     None)


# One FP32 GPU step vs one step of the reference's shipped library (the fixture's out_* arrays).
SHIPPED_TOL = 2e-5


def _compare(ux, uz, bp, bu, rux, ruz, rbp, rbu, tol):
    assert max_rel(ux, rux) < tol
    assert max_rel(uz, ruz) < tol
    for k in bp:
        if rbp[k].any():
            assert max_rel(bp[k], rbp[k]) < tol, k
    for k in bu:
        if rbu[k].any():
            assert max_rel(bu[k], rbu[k]) < tol, k


@pytest.mark.parametrize("name", ("n3", "n1", "n2_odd", "n8", "n3_minpml_aniso"))
def test_noalloc_step_matches_dropin_on_two_calls(F, name):
    d = load_npz("step_" + name)
    p, strips, c, c0, c1, ux, uz, bp, bu = step_inputs(d)
    ref = step_inputs(d)
    it = int(d["it"])
    for call in range(2):
        F.updatedispl(*ref[:9], it)
        assert _noalloc(F, p, it, strips, c, ux, uz, bp, bu) == 0, F.lib().fdfk_last_error()
        if call == 0:
            # the first call is one step of the shipped libHybrid/libPML from the same state
            shipped_bp = {k: d["out_" + k] for k in bp}
            shipped_bu = {k: d["out_" + k] for k in bu}
            _compare(ux, uz, bp, bu, d["out_ux"], d["out_uz"], shipped_bp, shipped_bu, SHIPPED_TOL)
        _compare(ux, uz, bp, bu, ref[5], ref[6], ref[7], ref[8], TOL)


def test_noalloc_step_allocates_nothing(F):
    import torch
    d = load_npz("step_n3")
    p, strips, c, c0, c1, ux, uz, bp, bu = step_inputs(d)
    assert _noalloc(F, p, 0, strips, c, ux, uz, bp, bu) == 0      # first call: scratch address set up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert _noalloc(F, p, 0, strips, c, ux, uz, bp, bu) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_oversize_geometry(F):
    L = F.lib()
    big = dict(norder=3, nx=4001, nz=2001, npml=40, nt=0, dx=100.0, dz=100.0, dt=0.006, vpml=8000.0)
    need = L.fdfk_step_noalloc_need(C.byref(F.Params.from_dict(big)))
    assert need > L.fdfk_step_noalloc_capacity() == (1 << 24)
    dummy = np.zeros(4, np.float32)
    strips = {k: dummy for k in F.STRIPS}
    bp = {k: dummy for k in F.BP}
    bu = {k: dummy for k in F.BU}
    rc = _noalloc(F, big, 0, strips, dummy, dummy, dummy, bp, bu)
    assert rc == -1
    assert b"scratch" in L.fdfk_last_error()
