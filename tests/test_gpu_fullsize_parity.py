"""GPU: every receiver trace of the FP32 solver against the FP64 oracle at the full workload sizes.

* The FP64 GPU oracle (oracle/fdfk_oracle_gpu.cu: the C restatement of the time step and loop,
  src/FDFK2D.f90:465-532, in double precision on the GPU) is first pinned against the FP64 CPU
  restatement (oracle/_build/libfdfk_oracle64.so) on small heterogeneous cases of every stencil
  order, on the 4001 x 2001 grid for a few steps, and on the whole 4001-step 801 x 401 workload.
* Then the FP32 solver (FK background computed on the GPU, FP32 strips, product kernels through
  the C ABI) runs each workload's whole record and every trace is compared with the FP64 oracle
  fed the FP64 FK restatement (oracle/fk_oracle.py) on the same inputs:
  - 801 x 401 cells at 250 m, 20-cell absorbing layers, two layers, P at 0.06 s/km, 4001 steps,
    101 surface receivers: against the CPU and the GPU FP64 oracles;
  - 4001 x 2001 cells at 100 m, 40-cell layers, dipping Moho, basin and 3 % smoothed perturbation,
    left and right FK models differing, P at 0.07 s/km, 12001 steps, 401 surface receivers:
    against the GPU FP64 oracle.
  The bar: relative L2 error of every trace (each receiver, each component) at most 1e-4.
"""
import numpy as np
import pytest

from conftest import load_npz
from fdfk2d_gb300 import workloads as WL

import fk_oracle

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-4          # FP32 solver vs FP64 oracle, relative L2 per trace
PIN_TOL = 1e-9            # FP64 GPU oracle vs FP64 CPU oracle, relative L2 per trace


@pytest.fixture(scope="module")
def F():
    import fdfk2d_gb300 as F
    from fdfk2d_gb300 import build
    build.build()
    F.lib()
    return F


def _trace_errors(got, ref):
    g, r = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    den = np.maximum(np.linalg.norm(r, axis=0), 1e-300)
    return np.linalg.norm(g - r, axis=0) / den


def _summary(label, ex, ez):
    e = np.concatenate([ex, ez])
    worst = int(np.argmax(e))
    comp = "x" if worst < len(ex) else "z"
    print(f"\n{label}: per-trace relative L2 max {e.max():.3e} median {np.median(e):.3e} "
          f"(x max {ex.max():.3e}, z max {ez.max():.3e}); worst receiver {worst % len(ex)} ({comp})")
    return e.max()


def _host_strips(dev):
    return {k: np.asfortranarray(v.cpu().numpy().transpose(2, 1, 0)) for k, v in dev.items()}


def _fp32_solve(F, w, fp, bazs, fl, fr):
    p = w["p"]
    with F.Session(p, w["c"]) as s:
        s.fk_background(fp, bazs, fl, fr)
        s.set_receivers(w["rx"], w["rz"], w["x0"], w["z0"], w["nstp"], w["nsis"])
        s.advance(p["nt"] + 1)
        return s.seismograms()


def _oracle_params(w):
    return dict(w["p"], izt=1)


# --------------------------------------------------------------------------- pinning the GPU oracle
def test_gpu_oracle_matches_cpu_oracle_golden_loop(oracle_lib):
    d = load_npz("loop_layered")
    p = dict(d["p"], izt=1)
    strips = fk_oracle.background(p, d["bazs"], d["fk_left"], d["fk_right"], dtype=np.float64)
    a = oracle_lib.simulate64(p, strips, d["c"], d["rx"], d["rz"], 0.0, 0.0, int(d["nstp"]), int(d["nsis"]))
    b = oracle_lib.simulate64_gpu(p, strips, d["c"], d["rx"], d["rz"], 0.0, 0.0, int(d["nstp"]), int(d["nsis"]))
    assert np.abs(a[1]).max() > 0
    for x, y in zip(a, b):
        assert _trace_errors(y, x).max() < PIN_TOL


@pytest.mark.parametrize("norder,npml,nstp", [(1, 3, 1), (2, 6, 3), (3, 10, 1), (4, 9, 2), (8, 15, 4)])
def test_gpu_oracle_matches_cpu_oracle_every_order(oracle_lib, norder, npml, nstp):
    from test_gpu_parity import _random_case
    nt = 180
    p, c, strips, rx, rz = _random_case(100 + norder, 70, 37, npml, norder, nt)
    p = dict(p, izt=1, nbd=2 * norder - 1)
    nsis = nt // nstp
    a = oracle_lib.simulate64(p, strips, c, rx, rz, 0.0, 0.0, nstp, nsis)
    b = oracle_lib.simulate64_gpu(p, strips, c, rx, rz, 0.0, 0.0, nstp, nsis)
    for x, y in zip(a, b):
        assert np.abs(x).max() > 0
        assert _trace_errors(y, x).max() < PIN_TOL


def test_gpu_oracle_matches_cpu_oracle_full_grid(oracle_lib):
    """The 4001 x 2001 grid for 40 steps, a plane-wave pulse already at the bottom strips, receivers
    8 cells above them (every cell of the grid is stepped; the CPU restatement takes about a minute)."""
    nt = 40
    w = WL.config2(nt=nt)
    p = _oracle_params(w)
    strips = WL.plane_wave_background(w, t0_index=220, count=nt + 1, amp=1e-3)
    rx = w["rx"][::20]
    rz = np.full_like(rx, (p["nz"] - 9) * p["dz"])
    a = oracle_lib.simulate64(p, strips, w["c"], rx, rz, 0.0, 0.0, 1, nt)
    b = oracle_lib.simulate64_gpu(p, strips, w["c"], rx, rz, 0.0, 0.0, 1, nt)
    for x, y in zip(a, b):
        assert np.abs(x).max() > 0
        assert _trace_errors(y, x).max() < PIN_TOL


# --------------------------------------------------------------------------- the FP32 solver at full size
def test_config1_every_trace_vs_fp64(F, oracle_lib):
    """801 x 401 cells, 4001 steps, 101 surface receivers: FP32 solver vs FP64 oracles (CPU and GPU)."""
    w = WL.config1()
    fp, bazs, fl, fr = WL.fk_inputs(w)
    gx, gz = _fp32_solve(F, w, fp, bazs, fl, fr)
    dev = fk_oracle.background_device(fp, bazs, fl, fr, x0=w["x0"], z0=w["z0"])
    p = _oracle_params(w)
    ox, oz = oracle_lib.simulate64_gpu(p, dev, w["c"], w["rx"], w["rz"], w["x0"], w["z0"], w["nstp"], w["nsis"])
    cx, cz = oracle_lib.simulate64(p, _host_strips(dev), w["c"], w["rx"], w["rz"], w["x0"], w["z0"], w["nstp"],
                                   w["nsis"])
    del dev
    assert _trace_errors(ox, cx).max() < PIN_TOL and _trace_errors(oz, cz).max() < PIN_TOL
    assert np.abs(gz).max() > 0 and np.abs(gx).max() > 0
    worst_cpu = _summary("config 1 (801x401, 4001 steps) FP32 vs FP64 CPU oracle",
                         _trace_errors(gx, cx), _trace_errors(gz, cz))
    worst_gpu = _summary("config 1 (801x401, 4001 steps) FP32 vs FP64 GPU oracle",
                         _trace_errors(gx, ox), _trace_errors(gz, oz))
    assert worst_cpu <= TRACE_TOL and worst_gpu <= TRACE_TOL


def test_config2_every_trace_vs_fp64(F, oracle_lib):
    """4001 x 2001 cells, 12001 steps, 401 surface receivers: FP32 solver vs the FP64 GPU oracle."""
    import torch
    w = WL.config2()
    fp, bazs, fl, fr = WL.fk_inputs(w)
    gx, gz = _fp32_solve(F, w, fp, bazs, fl, fr)
    dev = fk_oracle.background_device(fp, bazs, fl, fr, x0=w["x0"], z0=w["z0"])
    ox, oz = oracle_lib.simulate64_gpu(_oracle_params(w), dev, w["c"], w["rx"], w["rz"], w["x0"], w["z0"],
                                       w["nstp"], w["nsis"])
    del dev
    torch.cuda.empty_cache()
    assert np.abs(gz).max() > 0 and np.abs(gx).max() > 0
    worst = _summary("config 2 (4001x2001, 12001 steps) FP32 vs FP64 GPU oracle",
                     _trace_errors(gx, ox), _trace_errors(gz, oz))
    assert worst <= TRACE_TOL
