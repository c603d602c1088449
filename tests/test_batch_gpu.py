"""Batched ragged cases (fvm_batch_*) against the same cases run one by one through
single contexts with the same line tiles: the batched launches perform the same
arithmetic per case, so the results are identical bit for bit."""
import numpy as np
import pytest

from fvm_gb300 import capi
from tests.helpers import STATE, case_params, make_case, make_gpu

pytestmark = pytest.mark.gpu

# ragged grids (theta cells x radial cells), Reynolds numbers, skew and rotation
SPECS = [dict(n_theta=32, n_r=24, re=80.0, seed=1),
         dict(n_theta=48, n_r=16, re=150.0, seed=2, dt=0.004),
         dict(n_theta=64, n_r=40, re=120.0, seed=3, skew=0.3),
         dict(n_theta=40, n_r=20, re=200.0, seed=4, vel_rot=0.2, pr=1.0)]


def _cases(**kw):
    return [make_case(resimax=1e-10, nswpp=40000, **{**s, **kw}) for s in SPECS]


def _batch(cases, precision, **extra):
    b = capi.Batch([case_params(c, precision, **extra) for c in cases])
    for ctx, c in zip(b.cases, cases):
        ctx.set_grid(c["g"].xg, c["g"].yg)
        ctx.init(c["du"], c["dv"])
    return b


def _singles(cases, precision, tiles, **extra):
    t = dict(tile_r_warps=tiles[0], tile_r_m=tiles[1], tile_t_warps=tiles[2], tile_t_m=tiles[3])
    return [make_gpu(c, precision, **t, **extra) for c in cases]


def _compare(b, singles, recs, steps):
    for k, ctx in enumerate(singles):
        ref = [ctx.step(1) for _ in range(steps)]
        for s in range(steps):
            for key in ("time", "cd", "cl", "nu", "cfl", "cpb", "sweeps", "resid"):
                assert recs[s][k][key] == ref[s][key], (k, s, key)
        for nm in STATE:
            assert np.array_equal(b.cases[k].get(nm), ctx.get(nm)), (k, nm)


@pytest.mark.parametrize("precision", [capi.MIXED, capi.FP64], ids=["mixed", "fp64"])
def test_batch_matches_one_by_one(precision):
    cases = _cases()
    b = _batch(cases, precision)
    tiles = b.tiles()
    steps = 4
    recs = b.step(steps)
    assert len(recs) == steps and len(recs[0]) == len(cases)
    singles = _singles(cases, precision, tiles)
    _compare(b, singles, recs, steps)
    # every case converged on its own sweep count
    sw = [recs[-1][k]["sweeps"] for k in range(len(cases))]
    assert all(recs[-1][k]["resid"] <= 1e-10 for k in range(len(cases))), [r["resid"] for r in recs[-1]]
    assert len(set(sw)) > 1


def test_batch_continues_across_calls_and_history():
    cases = _cases()
    b = _batch(cases, capi.MIXED)
    r1 = b.step(2)
    r2 = b.step(3)
    singles = _singles(cases, capi.MIXED, b.tiles())
    _compare(b, singles, r1 + r2, 5)
    h = b.cases[1].history(3)
    assert [x["time"] for x in h] == [r2[s][1]["time"] for s in range(3)]


def test_autotune_keeps_state_and_matches_singles():
    cases = _cases()
    b = _batch(cases, capi.MIXED)
    u0 = [c.get("U") for c in b.cases]
    tiles, ms = b.autotune(sweeps=20)
    assert all(np.array_equal(c.get("U"), u) for c, u in zip(b.cases, u0))
    assert tiles == b.tiles() and ms[0] > 0 and ms[1] > 0
    nr = max(c["g"].ni - 1 for c in cases)
    nt = max(c["g"].nj - 1 for c in cases)
    assert 32 * tiles[0] * tiles[1] >= nr and 32 * tiles[2] * tiles[3] >= nt
    recs = b.step(3)
    _compare(b, _singles(cases, capi.MIXED, tiles), recs, 3)


def test_explicit_tiles_change_nothing_but_rounding():
    cases = _cases()
    b = _batch(cases, capi.MIXED)
    b.set_tiles((4, 1, 4, 1))
    recs = b.step(2)
    _compare(b, _singles(cases, capi.MIXED, (4, 1, 4, 1)), recs, 2)
    with pytest.raises(capi.FvmError):
        b.set_tiles((1, 1, 1, 1))          # 32 elements cannot cover the longest line
