"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import ast
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

STEP_CASES = ("n3", "n1", "n8", "n3_minpml_aniso", "n2_odd")
# the PML-on-top mode (is_PML_top, izt = 1 - npml)
STEP_CASES_TOP = ("top_n1", "top_n2", "top_n3")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    import oracle
    return oracle


def load_npz(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: (np.asfortranarray(z[k]) if z[k].ndim > 1 else z[k]) for k in z.files}
    d["p"] = ast.literal_eval(str(z["params"][0]))
    return d


def step_inputs(d):
    """(p, strips, c, coef0, coef1, ux, uz, bp, bu) fresh copies of a step fixture's inputs."""
    from fdfk2d_gb300.api import BP, BU, STRIPS
    cp = lambda a: np.array(a, dtype=a.dtype, order="F", copy=True)
    strips = {k: cp(d["in_" + k]) for k in STRIPS}
    bp = {k: cp(d["in_" + k]) for k in BP}
    bu = {k: cp(d["in_" + k]) for k in BU}
    return (dict(d["p"]), strips, cp(d["c"]), cp(d["coef0"]), cp(d["coef1"]), cp(d["in_ux"]), cp(d["in_uz"]), bp, bu)


def max_rel(a, ref):
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.abs(a - ref).max() / max(np.abs(ref).max(), 1e-30))


def rel_l2(a, ref):
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.linalg.norm(a - ref) / max(np.linalg.norm(ref), 1e-300))


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
