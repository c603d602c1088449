"""GPU parity: the CUDA library (through the C-ABI) against the CPU restatement
in GPU order, on identical host inputs.  The FP64 path evaluates the Poisson
residual every second sweep (its two pressure buffers alternate), so the
restatement is run with the same interval.

Tolerances (FP64): geometry and explicit stencils agree to rounding (rel-L2
<= 1e-13); line solves differ only by the parallel elimination order (<= 1e-12);
full steps with the Poisson residual converged to 1e-12 agree to <= 1e-9
relative L2 (the acceptance bar for the FP64 path).
"""
import numpy as np
import pytest

import oracle
from fvm_gb300 import capi
from tests.helpers import copy_oracle_state_to_gpu, make_case, make_gpu, make_oracle, rel_l2

pytestmark = pytest.mark.gpu

GEOM = ["X", "Y", "DJAC", "XIX", "XIY", "ETX", "ETY", "Q11", "Q12", "Q22", "DE", "DW", "DN", "DS", "THETA"]


def interior(a, g):
    return a[1:g.nj, 1:g.ni]


@pytest.mark.parametrize("skew", [0.0, 0.4])
def test_geometry_matches(skew):
    case = make_case(32, 24, skew=skew)
    o, ctx = make_oracle(case), make_gpu(case)
    g = case["g"]
    for nm in GEOM:
        a, b = ctx.get(nm), o.array(nm)
        if nm in ("DE", "DW", "DN", "DS"):
            a, b = interior(a, g), interior(b, g)
        if nm == "Q12" and skew == 0.0:
            assert np.abs(a - b).max() <= 1e-12 * np.abs(ctx.get("Q11")).max(), nm
            continue
        assert rel_l2(a, b) <= 1e-13, nm
    area = ctx.get("AREA")[1:g.nj, 1]
    assert rel_l2(area, o.array("AREA")[1:g.nj, 1]) <= 1e-15


def test_init_state_matches():
    case = make_case(32, 24, vel_rot=0.3)
    o, ctx = make_oracle(case), make_gpu(case)
    for nm in ("U", "V", "P", "T", "U_N", "V_N", "T_N"):
        np.testing.assert_allclose(ctx.get(nm), o.array(nm), rtol=0, atol=1e-15, err_msg=nm)


def _check(ctx, o, names, g, tol, region="full"):
    for nm in names:
        a, b = ctx.get(nm), o.array(nm)
        if region == "interior":
            a, b = interior(a, g), interior(b, g)
        err = rel_l2(a, b)
        assert err <= tol, f"{nm}: rel-L2 {err:.3e} > {tol:.1e}"


@pytest.mark.parametrize("skew", [0.0, 0.4])
def test_substeps_match(skew):
    """Each reference call point, started from the same developed state."""
    case = make_case(32, 24, skew=skew, resimax=1e-12, vel_rot=0.2)
    g = case["g"]
    o = make_oracle(case)
    o.step(3)
    ctx = make_gpu(case)
    copy_oracle_state_to_gpu(o, ctx)

    o.call("begin_step"); ctx.begin_step()
    _check(ctx, o, ["U_N", "V_N", "T_N"], g, 0.0)
    o.call("contra_vel"); ctx.contra_vel()
    _check(ctx, o, ["UE", "UW", "VN", "VS"], g, 1e-14, "interior")
    o.call("explicit")
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_T):
        ctx.nl(f)
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_T):
        ctx.dif(f)
    ctx.p_source()
    _check(ctx, o, ["NLX", "NLY", "ADV", "NLX_NM1", "DIFX", "DIFY", "DIFT", "S_U", "S_V"], g, 1e-13, "interior")
    o.call("iter_u"); ctx.iter_u()
    _check(ctx, o, ["U"], g, 1e-12, "interior")
    o.call("iter_v"); ctx.iter_v()
    _check(ctx, o, ["V"], g, 1e-12, "interior")
    o.call("remove_grad"); ctx.remove_grad()
    _check(ctx, o, ["U", "V"], g, 1e-12)
    sweeps_o = o.call("iter_p")
    resid, sweeps, rc = ctx.iter_p()
    assert rc == capi.FVM_OK
    assert abs(sweeps - sweeps_o) <= 1, (sweeps, sweeps_o)
    assert resid <= 1e-12
    _check(ctx, o, ["P"], g, 1e-10)
    o.call("correct"); ctx.correct()
    _check(ctx, o, ["U", "V"], g, 1e-11)
    _check(ctx, o, ["S_U", "S_V"], g, 1e-10, "interior")
    o.call("iter_t"); ctx.iter_t()
    _check(ctx, o, ["T"], g, 1e-12)
    o.call("calccoef")
    co = o.coeffs()
    cg = ctx.calccoef()
    for k in ("cd", "cl", "cd_p", "cd_v", "cl_p", "cl_v", "nu", "cpb", "cfl"):
        assert abs(cg[k] - co[k]) <= 1e-9 * max(1.0, abs(co[k])), (k, cg[k], co[k])


@pytest.mark.parametrize("skew,thermal", [(0.0, True), (0.3, False)])
def test_full_steps_match(skew, thermal):
    """FP64 GPU path vs the restatement over 12 complete steps, Poisson at 1e-12."""
    case = make_case(32, 24, skew=skew, resimax=1e-12, thermal=thermal)
    g = case["g"]
    o, ctx = make_oracle(case), make_gpu(case)
    for s in range(12):
        o.step(1)
        cg = ctx.step(1)
        co = o.coeffs()
        assert abs(cg["sweeps"] - co["sweeps"]) <= 2
        assert abs(cg["cd"] - co["cd"]) <= 1e-8 * abs(co["cd"])
    names = ["U", "V", "P"] + (["T"] if thermal else [])
    for nm in names:
        err = rel_l2(ctx.get(nm), o.array(nm), (g.ni, g.nj))
        assert err <= 1e-9, f"{nm}: {err:.3e}"


def test_fused_step_equals_call_sequence():
    case = make_case(32, 24, skew=0.2, resimax=1e-12)
    a, b = make_gpu(case), make_gpu(case)
    a.step(2)
    b.step(1)
    b.begin_step(); b.contra_vel()
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_T):
        b.nl(f)
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_T):
        b.dif(f)
    b.p_source(); b.iter_u(); b.iter_v(); b.remove_grad(); b.iter_p(); b.correct(); b.iter_t()
    for nm in ("U", "V", "P", "T"):
        assert rel_l2(a.get(nm), b.get(nm)) <= 1e-12, nm


def test_sweep_cap_reports_noconv():
    case = make_case(32, 24, resimax=1e-15, nswpp=6)
    ctx = make_gpu(case)
    ctx.begin_step(); ctx.contra_vel()
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_T):
        ctx.nl(f)
        ctx.dif(f)
    ctx.p_source(); ctx.iter_u(); ctx.iter_v(); ctx.remove_grad()
    resid, sweeps, rc = ctx.iter_p()
    assert rc == capi.FVM_ERR_NOCONV and sweeps == 6 and resid > 1e-15
    c = ctx.step(1)
    assert c["sweeps"] == 6


def test_call_order_errors():
    case = make_case(16, 12)
    g = case["g"]
    p = capi.default_params(ni=g.ni, nj=g.nj)
    ctx = capi.Context(p)
    with pytest.raises(capi.FvmError) as e:
        ctx.step(1)
    assert e.value.code == capi.FVM_ERR_ARG
    with pytest.raises(capi.FvmError):
        ctx.get("NOPE")
    bad = g.xg.copy()
    bad[:, :] = 0.0   # degenerate grid: zero Jacobian everywhere
    with pytest.raises(capi.FvmError) as e:
        ctx.set_grid(bad, bad)
    assert e.value.code == capi.FVM_ERR_ARG


@pytest.mark.parametrize("skew", [0.0, 0.3])
def test_mixed_matches_fp64_and_oracle(skew):
    """FP32 sweeps inside FP64 refinement: same fields as the FP64 path and as the
    restatement once both converge the Poisson residual to 1e-12."""
    case = make_case(32, 24, skew=skew, resimax=1e-12)
    g = case["g"]
    o = make_oracle(case)
    a = make_gpu(case)
    b = make_gpu(case, precision=capi.MIXED, refine_sweeps=4, adi_refine=2)
    for s in range(6):
        o.step(1)
        ca = a.step(1)
        cb = b.step(1)
        assert cb["resid"] <= 1e-12
        assert abs(cb["cd"] - ca["cd"]) <= 1e-7 * abs(ca["cd"])
        assert cb["sweeps"] % 4 == 0
    for nm in ("U", "V", "P", "T"):
        assert rel_l2(b.get(nm), a.get(nm), (g.ni, g.nj)) <= 1e-8, nm
        assert rel_l2(b.get(nm), o.array(nm), (g.ni, g.nj)) <= 1e-8, nm


def test_mixed_predictor_single_pass_is_fp32_accurate():
    """One defect-correction pass leaves an FP32-sized error, two passes reach FP64."""
    case = make_case(32, 24, skew=0.2, resimax=1e-12)
    g = case["g"]
    ref = make_gpu(case)
    one = make_gpu(case, precision=capi.MIXED, adi_refine=1)
    two = make_gpu(case, precision=capi.MIXED, adi_refine=2)
    ref.step(2)
    for ctx in (one, two):
        for nm in ("U", "V", "P", "T", "NLX", "NLY", "ADV", "U_N", "V_N", "T_N"):
            ctx.set(nm, ref.get(nm))
    for ctx in (ref, one, two):
        ctx.begin_step(); ctx.contra_vel()
        for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_T):
            ctx.nl(f)
            ctx.dif(f)
        ctx.p_source(); ctx.iter_u()
    e1 = rel_l2(one.get("U"), ref.get("U"), (g.ni, g.nj))
    e2 = rel_l2(two.get("U"), ref.get("U"), (g.ni, g.nj))
    assert e2 <= 1e-12 and e2 < e1 <= 1e-6


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED], ids=["fp64", "mixed"])
def test_device_poisson_loop_equals_host_loop(precision):
    """The graph while-node Poisson loop (poisson_host_loop = 0) runs the same kernels
    in the same order as the host replay: identical fields, coefficients and sweeps."""
    case = make_case(32, 24, re=200.0, dt=0.002, resimax=1e-10, nswpp=3000)
    out = []
    for host_loop in (1, 0):
        g = case["g"]
        p = capi.default_params(ni=g.ni, nj=g.nj, re=200.0, pr=0.71, dt=0.002, resimax=1e-10, nswpp=3000,
                                thermal=1, precision=precision, poisson_host_loop=host_loop)
        ctx = capi.Context(p)
        ctx.set_grid(g.xg, g.yg)
        ctx.init(case["du"], case["dv"])
        co = [ctx.step(1) for _ in range(3)]
        out.append(([(c["sweeps"], c["cd"]) for c in co], {nm: ctx.get(nm) for nm in ("U", "V", "P", "T")}))
        ctx.close()
    assert out[0][0] == out[1][0]
    for nm in ("U", "V", "P", "T"):
        assert np.array_equal(out[0][1][nm], out[1][1][nm]), nm
