"""Post-processing phase on the GPU (fvm_post_*, fvm_calc_vor) against the CPU
restatement run in the same order: CALC_VOR, the per-step POST_NU_CD_CL.PLT
records (lift extrema, Strouhal number, averages, rms) and the time-averaged
fields of POST_PROCESS."""
import numpy as np
import pytest

from fvm_gb300 import capi
from tests.helpers import make_case, make_gpu, make_oracle, rel_l2

pytestmark = pytest.mark.gpu

POST_KEYS = ("time", "nu", "cd", "cl", "cl_amp", "cpb", "st", "rms_cd", "rms_cl", "st_last", "cl_amp_last")


def test_calc_vor_of_solid_rotation():
    case = make_case(32, 16, skew=0.2)
    ctx = make_gpu(case)
    X, Y = ctx.get("X"), ctx.get("Y")
    ctx.set("U", -0.7 * Y)
    ctx.set("V", 0.7 * X)
    w = ctx.calc_vor()
    g = case["g"]
    assert np.allclose(w[1:g.nj, 1:g.ni], 1.4, rtol=1e-12, atol=1e-12)
    assert np.array_equal(w[0, :], w[g.nj - 1, :]) and np.array_equal(w[g.nj, :], w[1, :])


def test_post_processing_matches_the_restatement():
    # a rotating cylinder: the lift has extrema inside the window
    case = make_case(32, 16, re=100.0, dt=0.005, vel_rot=0.3, resimax=1e-12, nswpp=200000)
    o = make_oracle(case)
    ctx = make_gpu(case)
    o.step(5)
    ctx.step(5)
    o.post_begin()
    ctx.post_begin()
    extrema = 0
    for s in range(10):
        o.step(1)
        ctx.step(1)
        a, b = ctx.post_get(), o.post_record()
        assert a["niter"] == b["niter"] == s + 1
        for k in POST_KEYS:
            assert a[k] == pytest.approx(b[k], rel=1e-8, abs=1e-10), (s, k)
        extrema = extrema + (a["st_last"] > 0)
    assert extrema > 0
    fa, fields_a = ctx.post_final()
    fb, fields_b = o.post_final()
    for k in POST_KEYS:
        assert fa[k] == pytest.approx(fb[k], rel=1e-8, abs=1e-10), k
    for nm in ("U", "V", "P", "T", "VOR"):
        assert rel_l2(fields_a[nm], fields_b[nm]) <= 1e-9, nm
    # the sums are readable by name and the state is not overwritten
    assert np.allclose(ctx.get("U_TA") / 10.0, fields_a["U"], rtol=0, atol=0)
    assert rel_l2(ctx.get("U"), o.array("U")) <= 1e-9


def test_adjoint_recomputation_is_not_averaged():
    case = make_case(32, 16, re=100.0, dt=0.005, vel_rot=0.2, resimax=1e-12, nswpp=200000)
    ctx = make_gpu(case, capi.FP64)
    ctx.step(3)
    ctx.post_begin()
    ctx.set_controls(0.2, np.zeros(case["g"].nj - 1))
    ctx.adjoint_drag_grad(4, 2)
    assert ctx.post_get()["niter"] == 4
    ctx.step(1)
    assert ctx.post_get()["niter"] == 5
