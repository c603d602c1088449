"""The block schedules of the resident Poisson sweeps, modelled on the CPU.

Each radial line of the zebra line Gauss-Seidel is reduced to one unknown x_j with
the same dependency structure: a line solve replaces x_j by a function of rf_j and
its two neighbours x_{j-1}, x_{j+1} (periodic in j), odd lines first, then even
lines.  The model runs the global zebra sweeps and the schedules of the resident
kernels - one block of B lines per CTA, the window rows and half-sweeps the
kernels solve, the lines they take from other blocks and when - and requires the
same bits for every line after S sweeps.  This pins the schedule logic (window
extents, which rows a half-sweep may solve, which lines cross between blocks) that
the GPU tests exercise through the C-ABI.
"""
import numpy as np
import pytest


def _system(L, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.5, 1.0, L), rng.uniform(0.5, 1.0, L), rng.uniform(3.0, 4.0, L), rng.uniform(-1, 1, L)


def _solve(an, as_, dg, rf, j, xs, xn):
    return (rf[j] + an[j] * xn + as_[j] * xs) / dg[j]


def zebra(L, S, sysm):
    """Global zebra sweeps from zero: lines are 1-based, odd lines first."""
    an, as_, dg, rf = sysm
    x = np.zeros(L)
    for _ in range(S):
        for parity in (1, 0):
            for j in range(1, L + 1):
                if j % 2 == parity:
                    x[j - 1] = _solve(an, as_, dg, rf, j - 1, x[(j - 2) % L], x[j % L])
    return x


# the four half-sweeps of a pair: (first row, last row, odd rows)
PAIR_HALVES = ((1, 4 + 5, True), (2, 4 + 4, False), (3, 4 + 3, True), (4, 4 + 2, False))


def two_sweep_windows(L, S, sysm, B=4, halves=PAIR_HALVES):
    """k_pois32_resident2: window rows w = 0 .. B+6 hold lines j0-3+w; one exchange
    (the four outer even rows, from the neighbours' own even lines) per two sweeps;
    a pair solves the rows of `halves` in turn."""
    an, as_, dg, rf = sysm
    nb = L // B
    wrap = lambda j: (j - 1) % L + 1
    rows = [np.zeros(B + 7) for _ in range(nb)]
    published = None            # every block's own even lines after the last pair
    for sw in range(1, S + 1, 2):
        if sw > 1:
            for b in range(nb):
                j0 = b * B + 1
                for hrow in (0, 2, B + 4, B + 6):
                    rows[b][hrow] = published[wrap(j0 - 3 + hrow) - 1]
        for b in range(nb):
            j0 = b * B + 1
            r = rows[b]
            for lo, hi, odd in halves:
                new = r.copy()
                for w in range(lo, hi + 1):
                    if (w % 2 == 1) == odd:
                        new[w] = _solve(an, as_, dg, rf, wrap(j0 - 3 + w) - 1, r[w - 1], r[w + 1])
                r[:] = new
        published = np.zeros(L)
        for b in range(nb):
            j0 = b * B + 1
            for w in range(4, B + 3, 2):
                published[wrap(j0 - 3 + w) - 1] = rows[b][w]
    x = np.zeros(L)
    for b in range(nb):
        j0 = b * B + 1
        for w in range(3, B + 3):
            x[wrap(j0 - 3 + w) - 1] = rows[b][w]
    return x


def one_sweep_blocks(L, S, sysm, B):
    """k_pois32_resident: lines j0 .. j0+B-1 plus the next block's first line solved
    again; lines j0-1 and j0+B+1 from the neighbours once per sweep."""
    an, as_, dg, rf = sysm
    nb = L // B
    wrap = lambda j: (j - 1) % L + 1
    own = [np.zeros(B + 1) for _ in range(nb)]   # lines j0 .. j0+B
    halo = [[0.0, 0.0] for _ in range(nb)]
    for sw in range(1, S + 1):
        if sw > 1:
            glob = np.zeros(L)
            for b in range(nb):
                for g in range(B):
                    glob[b * B + g] = own[b][g]
            for b in range(nb):
                j0 = b * B + 1
                halo[b] = [glob[wrap(j0 - 1) - 1], glob[wrap(j0 + B + 1) - 1]]
        for b in range(nb):
            j0 = b * B + 1
            v = own[b]
            new = v.copy()
            for g in range(0, B + 1, 2):       # odd lines and the redundant one
                xs = halo[b][0] if g == 0 else v[g - 1]
                xn = halo[b][1] if g == B else v[g + 1]
                new[g] = _solve(an, as_, dg, rf, wrap(j0 + g) - 1, xs, xn)
            v[:] = new
            for g in range(1, B, 2):           # even lines, both neighbours on chip
                new[g] = _solve(an, as_, dg, rf, wrap(j0 + g) - 1, v[g - 1], v[g + 1])
            v[:] = new
    x = np.zeros(L)
    for b in range(nb):
        for g in range(B):
            x[b * B + g] = own[b][g]
    return x


@pytest.mark.parametrize("L", [12, 16, 64, 512])
@pytest.mark.parametrize("S", [2, 4, 8, 32])
def test_two_sweeps_per_exchange_equal_the_zebra_sweeps(L, S):
    sysm = _system(L, L + S)
    assert np.array_equal(two_sweep_windows(L, S, sysm), zebra(L, S, sysm))


@pytest.mark.parametrize("L,B", [(12, 2), (16, 4), (64, 4), (60, 10), (96, 6)])
@pytest.mark.parametrize("S", [1, 3, 8])
def test_one_sweep_per_exchange_equals_the_zebra_sweeps(L, B, S):
    sysm = _system(L, L * B + S)
    assert np.array_equal(one_sweep_blocks(L, S, sysm, B), zebra(L, S, sysm))


def test_a_narrower_window_would_differ():
    """The model is sharp: solving the first sweep's even rows only on 4 .. B+2 (the
    second sweep's extent) leaves rows the second sweep reads stale."""
    L, S = 16, 4
    sysm = _system(L, 1)
    ref = zebra(L, S, sysm)
    assert np.array_equal(two_sweep_windows(L, S, sysm), ref)
    narrowed = (PAIR_HALVES[0], (4, 4 + 2, False), PAIR_HALVES[2], PAIR_HALVES[3])
    assert not np.array_equal(two_sweep_windows(L, S, sysm, halves=narrowed), ref)
