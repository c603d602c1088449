"""Line-resident FP32 Poisson sweeps (poisson_resident) against the per-colour
launches they replace, through the C-ABI.

The resident kernel runs a whole refinement interval in one launch, each block
keeping its lines on chip and exchanging boundary lines with its neighbours, after
every sweep or (resident_depth 2) after every two sweeps with three more lines per
block solved redundantly; the arithmetic of every line is the per-colour kernel's,
so the fields must agree bit for bit after several steps, for every lines-per-block
choice, exchange depth, tile and Poisson loop form.  The bounded waits are checked
by a call whose exchange tags no block publishes: it must report FVM_ERR_TIMEOUT
and leave the context usable.
"""
import time

import numpy as np
import pytest

from fvm_gb300 import capi
from tests.helpers import make_case, make_gpu

pytestmark = pytest.mark.gpu

def resident_auto_tile(n_r):
    """The radial tile a MIXED context with resident sweeps picks when none is given:
    one warp up to 128 cells, else two-warp groups with the fewest elements per
    thread that cover the line."""
    if n_r <= 128:
        return (1, -(-n_r // 32))
    return (2, next(m for m in (1, 2, 3, 4, 6, 8) if 64 * m >= n_r))


CASES = [
    # n_theta, n_r, lines per block (1 = automatic), radial tile, sweeps per exchange
    (512, 384, 1, resident_auto_tile(384), 0),   # the benchmark grid, automatic choices
    (512, 384, 4, resident_auto_tile(384), 1),
    (512, 384, 4, (4, 3), 0),
    (128, 96, 2, resident_auto_tile(96), 0),     # the 128 x 96 grid
    (128, 96, 4, (0, 0), 1),
    (128, 96, 4, (0, 0), 2),
    (96, 300, 6, (2, 6), 0),      # two-warp groups of 6 elements per thread
    (64, 380, 2, (1, 12), 0),     # one-warp groups of 12
    (64, 380, 4, (1, 12), 2),
    (60, 120, 10, (1, 4), 0),
    (16, 40, 4, (2, 1), 2),       # four blocks of 4 lines around the ring
    (12, 40, 4, (1, 2), 2),       # three: the smallest ring of two-sweep windows
]


def _run(case, resident, tile, host_loop, steps=3, depth=0):
    ctx = make_gpu(case, precision=capi.MIXED, refine_sweeps=8, adi_refine=2, poisson_resident=resident,
                   poisson_host_loop=host_loop, tile_r_warps=tile[0], tile_r_m=tile[1], resident_depth=depth)
    rec = [ctx.step(1) for _ in range(steps)]
    out = {nm: ctx.get(nm) for nm in ("U", "V", "P", "T")}
    ctx.close()
    return rec, out


@pytest.mark.parametrize("n_theta,n_r,lines,tile,depth", CASES,
                         ids=[f"{a}x{b}-B{c}-t{d[0]}{d[1]}-x{e}" for a, b, c, d, e in CASES])
@pytest.mark.parametrize("host_loop", [1, 0], ids=["host-loop", "device-loop"])
def test_resident_sweeps_are_bit_identical(n_theta, n_r, lines, tile, depth, host_loop):
    case = make_case(n_theta, n_r, re=200.0, dt=0.002, skew=0.0, resimax=1e-14, nswpp=64)
    ra, fa = _run(case, lines, tile, host_loop, depth=depth)
    rb, fb = _run(case, 0, tile, host_loop)
    for a, b in zip(ra, rb):
        assert a["sweeps"] == b["sweeps"] == 64
        assert a["cd"] == b["cd"] and a["resid"] == b["resid"]
    for nm in ("U", "V", "P", "T"):
        assert np.array_equal(fa[nm], fb[nm]), nm


def test_automatic_tile_of_resident_contexts():
    """Left automatic, a resident MIXED context takes resident_auto_tile: its steps
    equal those of a context given that tile explicitly."""
    case = make_case(96, 300, re=200.0, dt=0.002, resimax=1e-14, nswpp=32)
    ra, fa = _run(case, 1, (0, 0), 1, steps=1)
    rb, fb = _run(case, 1, resident_auto_tile(300), 1, steps=1)
    for nm in ("U", "V", "P", "T"):
        assert np.array_equal(fa[nm], fb[nm]), nm


@pytest.mark.parametrize("depth", [1, 2])
def test_resident_sweeps_converge_like_the_per_colour_path(depth):
    """With the tolerance as the stopping rule: same sweep counts and fields."""
    case = make_case(64, 48, re=100.0, dt=0.005, skew=0.2, resimax=1e-11, nswpp=200000)
    ra, fa = _run(case, 4, resident_auto_tile(48), 1, steps=2, depth=depth)
    rb, fb = _run(case, 0, resident_auto_tile(48), 1, steps=2)
    assert [r["sweeps"] for r in ra] == [r["sweeps"] for r in rb]
    assert all(r["resid"] <= 1e-11 for r in ra)
    for nm in ("U", "V", "P", "T"):
        assert np.array_equal(fa[nm], fb[nm]), nm


@pytest.mark.parametrize("depth", [1, 2])
def test_resident_wait_runs_out_and_the_context_stays_usable(depth):
    case = make_case(128, 96, re=100.0, dt=0.005, resimax=1e-14, nswpp=64)
    a = make_gpu(case, precision=capi.MIXED, refine_sweeps=8, poisson_resident=4, resident_depth=depth)
    b = make_gpu(case, precision=capi.MIXED, refine_sweeps=8, poisson_resident=4, resident_depth=depth)
    a.step(1)
    b.step(1)
    t0 = time.perf_counter()
    rc = a.resident_wait_test(max_polls=2048)
    assert rc == capi.FVM_ERR_TIMEOUT, capi.STATUS_NAMES.get(rc, rc)
    assert time.perf_counter() - t0 < 10.0
    assert "bounded wait" in a.last_error()
    # the exchange state was cleared: the next steps equal those of a context that
    # never saw the failed wait
    ca, cb = a.step(2), b.step(2)
    assert ca["cd"] == cb["cd"] and ca["sweeps"] == cb["sweeps"]
    for nm in ("U", "V", "P", "T"):
        assert np.array_equal(a.get(nm), b.get(nm)), nm


def test_resident_path_needs_mixed_precision():
    case = make_case(64, 48)
    ctx = make_gpu(case, precision=capi.FP64)
    assert ctx.resident_wait_test(64) == capi.FVM_ERR_ARG
    with pytest.raises(capi.FvmError):
        make_gpu(case, precision=capi.MIXED, poisson_resident=3)      # odd lines per block
    with pytest.raises(capi.FvmError):
        make_gpu(case, precision=capi.MIXED, poisson_resident=22)     # does not divide 64 lines
    with pytest.raises(capi.FvmError):
        make_gpu(case, precision=capi.MIXED, poisson_resident=2, resident_depth=2)   # two-sweep windows need 4
    with pytest.raises(capi.FvmError):
        make_gpu(case, precision=capi.MIXED, resident_depth=3)
