"""Shared case builders for the tests: one O-grid case run by the CUDA library and
by the CPU restatement on identical host inputs."""
from __future__ import annotations

import numpy as np

import oracle
from fvm_gb300 import capi
from fvm_gb300.grid import o_grid, perturbation

STATE = ["U", "V", "P", "T", "NLX", "NLY", "ADV"]


def rel_l2(a, b, interior_of=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if interior_of is not None:
        ni, nj = interior_of
        a = a[1:nj, 1:ni]
        b = b[1:nj, 1:ni]
    den = np.linalg.norm(b)
    num = np.linalg.norm(a - b)
    return num / den if den > 0 else num


def make_case(n_theta=32, n_r=24, re=100.0, pr=0.71, dt=0.005, skew=0.0, amp=1e-3, seed=0,
              resimax=1e-12, nswpp=200000, thermal=True, vel_rot=0.0, dr1=0.005, r_out=50.0):
    g = o_grid(n_theta, n_r, dr1=dr1, r_out=r_out, skew=skew)
    du, dv = perturbation(g.ni, g.nj, amp, seed)
    return dict(g=g, du=du, dv=dv, re=re, pr=pr, dt=dt, resimax=resimax, nswpp=nswpp,
                thermal=thermal, vel_rot=vel_rot)


def make_oracle(case, order=oracle.GPU, res_every=2, variant="check"):
    g = case["g"]
    o = oracle.Oracle(g.ni, g.nj, re=case["re"], pr=case["pr"], dt=case["dt"], vel_rot=case["vel_rot"],
                      order=order, resimax=case["resimax"], nswpp=case["nswpp"],
                      thermal=case["thermal"], res_every=res_every, variant=variant)
    o.set_grid(g.xg, g.yg)
    o.init(case["du"], case["dv"])
    return o


def case_params(case, precision=capi.FP64, res_every=2, refine_sweeps=4, adi_refine=2, **extra):
    g = case["g"]
    return capi.default_params(ni=g.ni, nj=g.nj, re=case["re"], pr=case["pr"], dt=case["dt"],
                               vel_rot=case["vel_rot"], resimax=case["resimax"], nswpp=case["nswpp"],
                               thermal=int(case["thermal"]), precision=precision, res_every=res_every,
                               refine_sweeps=refine_sweeps, adi_refine=adi_refine, **extra)


def make_gpu(case, precision=capi.FP64, res_every=2, refine_sweeps=4, adi_refine=2, **extra):
    g = case["g"]
    p = case_params(case, precision, res_every, refine_sweeps, adi_refine, **extra)
    ctx = capi.Context(p)
    ctx.set_grid(g.xg, g.yg)
    ctx.init(case["du"], case["dv"])
    return ctx


def copy_oracle_state_to_gpu(o, ctx, names=("U", "V", "P", "T", "NLX", "NLY", "ADV", "U_N", "V_N", "T_N",
                                          "NLX_NM1", "NLY_NM1", "ADV_NM1")):
    for nm in names:
        ctx.set(nm, o.array(nm))
    ctx.set_time(o.time)
