"""CPU: the FP64 oracle (the restatement with every field in double) against the FP32 restatement
of the reference's arithmetic: the reference's own FP32 traces lie within the 1e-4 relative L2 bar
of FP64, which is the bar the GPU traces are held to (tests/test_gpu_fp64.py)."""
import numpy as np

from conftest import load_npz, rel_l2

import fk_oracle


def test_fp32_restatement_within_bar_of_fp64(oracle_lib):
    d = load_npz("loop_layered")
    p = dict(d["p"])
    strips32 = {k: d[k] for k in oracle_lib.STRIPS}
    sx, sz = oracle_lib.simulate(p, strips32, d["c"], d["rx"], d["rz"], 0.0, 0.0, int(d["nstp"]), int(d["nsis"]))
    strips64 = fk_oracle.background(p, d["bazs"], d["fk_left"], d["fk_right"], dtype=np.float64)
    dx, dz = oracle_lib.simulate64(p, strips64, d["c"], d["rx"], d["rz"], 0.0, 0.0, int(d["nstp"]), int(d["nsis"]))
    assert np.abs(dz).max() > 0
    ex, ez = rel_l2(sx, dx), rel_l2(sz, dz)
    assert ex < 1e-4 and ez < 1e-4
    assert ex > 0 and ez > 0          # the two precisions do differ
