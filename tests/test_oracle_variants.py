"""The build variants of the CPU restatement (oracle/Makefile).

"par" runs the GPU-order zebra line sweeps of one colour and the stencil loops on
all host threads; because every parallel loop writes each cell once from inputs it
does not modify and every reduction stays serial, its fields must equal the serial
checker's bit for bit.  bench.py relies on that when it uses "par" as the checker
at the benchmark grid.
"""
import numpy as np
import pytest

import oracle
from fvm_gb300.grid import o_grid, perturbation


@pytest.mark.parametrize("skew,thermal", [(0.0, True), (0.3, False)])
def test_parallel_checker_is_bit_identical(skew, thermal):
    g = o_grid(64, 48, skew=skew)
    du, dv = perturbation(g.ni, g.nj, 1e-3, 3)
    out = {}
    for var in ("check", "par"):
        o = oracle.Oracle(g.ni, g.nj, re=150.0, pr=0.71, dt=0.004, order=oracle.GPU, resimax=1e-9, nswpp=64,
                          thermal=thermal, res_every=4, vel_rot=0.1, variant=var)
        o.set_grid(g.xg, g.yg)
        o.init(du, dv)
        o.step(3)
        out[var] = ({nm: o.array(nm).copy() for nm in ("U", "V", "P", "T", "NLX", "NLY")}, o.coeffs())
    for nm, a in out["check"][0].items():
        assert np.array_equal(a, out["par"][0][nm]), nm
    for k in ("cd", "cl", "nu", "resid", "sweeps"):
        assert out["check"][1][k] == out["par"][1][k], k


def test_timing_copy_tracks_the_checker():
    """The FMA-contracted timing copy runs the same algorithm: same sweep counts and
    fields equal to rounding."""
    g = o_grid(32, 24)
    du, dv = perturbation(g.ni, g.nj, 1e-3, 0)
    res = []
    for var in ("check", "fast"):
        o = oracle.Oracle(g.ni, g.nj, re=100.0, dt=0.005, order=oracle.FAITHFUL, resimax=1e-8, nswpp=500,
                          variant=var)
        o.set_grid(g.xg, g.yg)
        o.init(du, dv)
        o.step(2)
        res.append((o.array("U").copy(), o.coeffs()["sweeps"]))
    assert abs(res[0][1] - res[1][1]) <= 2
    assert np.linalg.norm(res[0][0] - res[1][0]) <= 1e-9 * np.linalg.norm(res[0][0])
