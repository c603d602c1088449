"""Every line tile the kernels are instantiated for, against the CPU restatement in
GPU order, through the C-ABI.

A line of n unknowns is solved by a group of NW warps with M elements per thread
(32*NW*M >= n); the per-thread chunk recurrences, the warp scan and the fold across
the group's warps differ per (NW, M), so each instantiation is its own code path.
Each case forces one tile on both line families of the 2-D step (radial lines: the
Poisson sweep and the first predictor factor; circumferential lines: the cyclic
second factor) on a grid whose lines need that tile, with the last chunk partly
filled, and runs three steps with the Poisson iteration capped at 16 sweeps (the
same capped iterate in both codes: the parity of the kernels the benchmark times,
at sizes the restatement finishes in seconds).

FP64 runs on a skewed grid (non-zero cross terms) and must agree to 1e-9 relative
L2, the acceptance bar of the FP64 path.  The mixed path runs on the orthogonal
grid, where its refinement and the FP64 iteration produce the same iterate up to
the FP32 rounding of the corrections: P within 2e-6 (built from zero in the first
step, so it carries that rounding relative to itself) and U, V, T within 1e-7.  A
wrong scan, fold or chunk index gives errors of order one.
"""
import numpy as np
import pytest

import oracle
from fvm_gb300 import capi, capi3d
from fvm_gb300.grid import o_grid_3d, perturbation_3d
from tests.helpers import make_case, make_gpu, make_oracle, rel_l2

pytestmark = pytest.mark.gpu

TILES_2D = [(1, 1), (1, 2), (1, 3), (1, 4), (1, 6), (1, 8), (1, 12), (2, 1), (2, 2), (2, 3), (2, 4), (2, 6),
            (2, 8), (4, 1), (4, 2), (4, 3), (4, 4)]
CAP = 16


def _grid_for(nw, m):
    """Circumferential and radial cell counts whose lines need tile (nw, m), both
    short of the tile's capacity so that the last chunk is partly filled.  The
    circumferential count is a multiple of 4: with 2 (mod 4) cells one wall face is
    vertical and the reference's wall-friction formula divides by its zero slope
    difference (calccoef.f90, LA = (YB-YA)/(XB-XA)), giving a NaN drag in both codes."""
    cap = 32 * nw * m
    return cap - 4, cap - 3


def _run_2d(tile, precision, skew):
    nw, m = tile
    n_theta, n_r = _grid_for(nw, m)
    case = make_case(n_theta, n_r, re=200.0, dt=0.002, skew=skew, resimax=1e-14, nswpp=CAP, vel_rot=0.1)
    o = make_oracle(case, res_every=2, variant="par")
    ctx = make_gpu(case, precision=precision, res_every=2, refine_sweeps=4, adi_refine=2,
                   tile_r_warps=nw, tile_r_m=m, tile_t_warps=nw, tile_t_m=m)
    rec = []
    for _ in range(3):
        o.step(1)
        rec.append((ctx.step(1), o.coeffs()))
    return case["g"], o, ctx, rec


@pytest.mark.parametrize("tile", TILES_2D, ids=[f"nw{a}m{b}" for a, b in TILES_2D])
def test_fp64_tile_matches_the_restatement(tile):
    g, o, ctx, rec = _run_2d(tile, capi.FP64, skew=0.2)
    for cg, co in rec:
        assert cg["sweeps"] == co["sweeps"] == CAP
        assert abs(cg["cd"] - co["cd"]) <= 1e-9 * abs(co["cd"])
    for nm in ("U", "V", "P", "T"):
        err = rel_l2(ctx.get(nm), o.array(nm), (g.ni, g.nj))
        assert err <= 1e-9, f"{nm}: {err:.3e}"
    ctx.close()


@pytest.mark.parametrize("tile", TILES_2D, ids=[f"nw{a}m{b}" for a, b in TILES_2D])
def test_mixed_tile_matches_the_restatement(tile):
    g, o, ctx, rec = _run_2d(tile, capi.MIXED, skew=0.0)
    for cg, co in rec:
        assert cg["sweeps"] == co["sweeps"] == CAP
        assert abs(cg["cd"] - co["cd"]) <= 1e-6 * abs(co["cd"])
    tol = {"U": 1e-7, "V": 1e-7, "P": 2e-6, "T": 1e-7}
    for nm, t in tol.items():
        err = rel_l2(ctx.get(nm), o.array(nm), (g.ni, g.nj))
        assert err <= t, f"{nm}: {err:.3e}"
    ctx.close()


# 3-D: I lines of 191 cells (the benchmark's 192-cell radial direction has 191
# unknowns), automatic one-warp tile with 6 elements per thread plus the other
# tiles that cover those lines; J (16) and K (8) lines take the one-warp tile.
TILES_3D = [(0, 0), (2, 3), (4, 2), (2, 4), (1, 8), (1, 12)]


def _run_3d(tile, precision, skew):
    nw, m = tile
    g = o_grid_3d(16, 191, 8, lz=np.pi, dr1=0.005, skew=skew)
    du, dv, dw = perturbation_3d(g.ni, g.nj, g.nk, 0.05, 5)
    kw = dict(re=3900.0, dt=0.002, resimax=1e-14, nswpp=CAP, use_les=True, les_zavg=False, thermal=True,
              res_every=2, ref_a=np.pi)
    o = oracle.Oracle3D(g.ni, g.nj, g.nk, order=oracle.O3_GPU, **kw)
    o.set_grid(g)
    o.init(du, dv, dw)
    p = capi3d.default_params(ni=g.ni, nj=g.nj, nk=g.nk, re=3900.0, dt=0.002, resimax=1e-14, nswpp=CAP,
                              use_les=1, les_zavg=0, thermal=1, res_every=2, ref_a=np.pi, precision=precision,
                              refine_sweeps=4, tile_i_warps=nw, tile_i_m=m)
    ctx = capi3d.Context3(p)
    ctx.set_grid(g)
    ctx.init(du, dv, dw)
    rec = []
    for _ in range(2):
        o.step(1)
        rec.append((ctx.step(1), o.coeffs()))
    return o, ctx, rec


@pytest.mark.parametrize("tile", TILES_3D, ids=["auto-nw1m6"] + [f"nw{a}m{b}" for a, b in TILES_3D[1:]])
def test_fp64_3d_i_tile_matches_the_restatement(tile):
    o, ctx, rec = _run_3d(tile, capi.FP64, skew=0.3)
    for cg, co in rec:
        assert cg["sweeps"] == co["sweeps"] == CAP
        assert cg["cd"] == pytest.approx(co["cd"], rel=1e-9)
    for nm in ("U", "V", "W", "P", "T"):
        err = rel_l2(ctx.get(nm), o.array(nm))
        assert err <= 1e-9, f"{nm}: {err:.3e}"
    ctx.close()


@pytest.mark.parametrize("tile", TILES_3D, ids=["auto-nw1m6"] + [f"nw{a}m{b}" for a, b in TILES_3D[1:]])
def test_mixed_3d_i_tile_matches_the_restatement(tile):
    o, ctx, rec = _run_3d(tile, capi.MIXED, skew=0.0)
    for cg, co in rec:
        assert cg["sweeps"] == co["sweeps"] == CAP
        assert cg["cd"] == pytest.approx(co["cd"], rel=1e-6)
    tol = {"U": 1e-7, "V": 1e-7, "W": 1e-7, "P": 2e-6, "T": 1e-7}
    for nm, t in tol.items():
        err = rel_l2(ctx.get(nm), o.array(nm))
        assert err <= t, f"{nm}: {err:.3e}"
    ctx.close()
