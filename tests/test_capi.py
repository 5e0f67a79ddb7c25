"""CPU tests of the C-ABI library: it builds for sm_103a, loads without a GPU, exports every
symbol include/fdfk_gb300.h declares, and rejects bad arguments before touching the device."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "fdfk_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^[A-Za-z_][\w\s\*]*?\b(\w+)\s*\(", text, flags=re.M)) - {"defined"})


@pytest.fixture(scope="module")
def built():
    from fdfk2d_gb300 import build
    return build.build()


def test_header_declares_the_entry_points():
    names = declared_functions()
    for must in ("fdfk_session_create", "fdfk_session_advance", "fdfk_simulate", "updatedispl_"):
        assert must in names


def test_library_exports_every_declared_symbol(built):
    out = subprocess.run(["nm", "-D", "--defined-only", built], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_library_loads_and_validates_without_gpu(built):
    import fdfk2d_gb300 as F
    L = F.lib()
    assert L.fdfk_version() >= 100
    base = dict(norder=3, nx=40, nz=24, npml=8, nt=10, dx=250.0, dz=250.0, dt=0.015, vpml=8000.0)
    c = np.ones((3, 32, 56), np.float32, order="F")
    bad = [dict(norder=0), dict(norder=9), dict(npml=4), dict(nbd=4), dict(nz=5), dict(dx=0.0), dict(R0=2.0),
           dict(nt=-1), dict(nx=6)]
    for change in bad:
        p = dict(base, **change)
        with pytest.raises(F.FDFKError) as e:
            F.Session(p, c)
        assert e.value.code == -1, change
    # the absorbing layer on top is validated the same way (npml rows more above row 1)
    for change in (dict(npml=4), dict(nz=5)):
        with pytest.raises(F.FDFKError) as e:
            F.Session(dict(base, is_PML_top=True, **change), np.ones((3, 40, 56), np.float32, order="F"))
        assert e.value.code == -1, change


def test_shapes_match_reference_allocations():
    import fdfk2d_gb300 as F
    s = F.strip_shapes(40, 24, 5, 10)
    assert s["uxl_reg"] == (19, 5, 11) and s["uxb_pml"] == (5, 50, 11)
    ps = F.pml_shapes(40, 24, 8)
    assert ps["bux1l"] == (2, 24, 8) and ps["bpxbx"] == (8, 56)
    assert len(F.BU) == 24 and F.BU[0] == "bux1l" and F.BU[12] == "bux1b" and F.BU[18] == "bux1t"


def test_fk_entry_points_validate_without_gpu(built):
    import fdfk2d_gb300 as F
    p = dict(nx=16, nz=12, npml=6, nbd=3, nt=50, dt=0.01, dx=250.0, dz=250.0, ds=1e-3, f0=2.0, rayp=6e-5)
    m = np.array([[0.0], [6000.0], [3500.0], [2700.0]], np.float32)
    baz = np.zeros(16 + 12)
    # the grid's top row is 1 (free surface) or 1 - npml (absorbing layer on top)
    for izt in (2, -6):
        with pytest.raises(F.FDFKError) as e:
            F.fk_background(dict(p, izt=izt), baz, m, m)
        assert e.value.code == -1, izt
    for change in (dict(nbd=7), dict(nz=3), dict(nt=0), dict(dt=0.0), dict(nx=0)):
        with pytest.raises((F.FDFKError, ValueError)) as e:
            F.fk_background(dict(p, **change), np.zeros(int(dict(p, **change)["nx"]) + 12), m, m)
        if isinstance(e.value, F.FDFKError):
            assert e.value.code == -1, change
    with pytest.raises(ValueError):
        F.fk_background(p, np.zeros(5), m, m)
    with pytest.raises(ValueError):
        F.fk_background(p, baz, m[:3], m)


def test_noalloc_source_names_no_allocating_call():
    """The allocation-free step's source file, and the bodies of the helpers it launches through,
    name no device allocation or release and no library call that allocates."""
    import re
    csrc = os.path.join(ROOT, "fdfk2d_gb300", "csrc")
    forbidden = re.compile(r"\b(cudaMalloc\w*|cudaFree\w*|cuMemAlloc\w*|cuMemFree\w*|cufft\w*|cublas\w*|"
                           r"cudaMemPool\w*|cudaHostAlloc|cudaHostRegister|malloc|calloc|realloc|new\b)")
    src = open(os.path.join(csrc, "fdfk_noalloc.cu")).read()
    code = re.sub(r"//[^\n]*|/\*.*?\*/", "", src, flags=re.S)
    assert not forbidden.findall(code), forbidden.findall(code)

    def body(fname, sig):
        text = re.sub(r"//[^\n]*|/\*.*?\*/", "", open(os.path.join(csrc, fname)).read(), flags=re.S)
        i = text.index(sig)
        j = text.index("{", i)
        depth = 0
        for k in range(j, len(text)):
            depth += {"{": 1, "}": -1}.get(text[k], 0)
            if depth == 0:
                return text[j:k + 1]
        raise AssertionError(sig)

    for fname, sig in (("fdfk_sweep.cu", "cudaError_t launch_step(const StepArgs& a, cudaStream_t s)"),
                       ("fdfk_sweep.cu", "cudaError_t set_coefficients(const float* stag, const float* coll)"),
                       ("fdfk_capi.cu", "cudaError_t ensure_coefficients()"),
                       ("fdfk_capi.cu", "int fdfk_step_noalloc(")):
        b = body(fname, sig)
        assert not forbidden.findall(b), (sig, forbidden.findall(b))
