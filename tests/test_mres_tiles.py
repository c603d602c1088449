"""Index arithmetic of the mixed residual kernel's tiles, checked on the CPU.

k_mres (fvm_gb300/csrc/fvm_mixed.cu) gives each 256-thread block a tile of
32 radial x 8 circumferential cells (block b: tile column b mod ceil((NI-1)/32),
tile row b div that), loads the pressure of rows j0-2 .. j0+8 and columns
i0-2 .. i0+32 into shared memory (zero outside 0..NI x 0..NJ) and evaluates the
residual of every interior cell of the tile from there.  This enumerates those
index maps for grids of several shapes: every interior cell is evaluated by
exactly one thread, and every shared-memory value a cell reads is a loaded
in-range pressure, never the zero fill, for both cross-term pairings.
"""
import itertools

import pytest

TI, TJ = 32, 8
W, H = TI + 3, TJ + 3


def reads(i, j, NI, NJ, dd_pos):
    """Offsets (a, b) of P(i+a, j+b) read from the tile by cell (i, j)."""
    out = [(1, 0), (-1, 0), (0, 0)]
    if j + 1 != NJ:
        out.append((0, 1))        # else row 1 through the periodic wrap, from global memory
    if j != 1:
        out.append((0, -1))       # else row NJ-1, from global memory
    if not dd_pos:
        out += [(1, 1), (1, -1), (-1, 1), (-1, -1)]
    elif i > 1 and j > 1:
        out += [(0, 0), (0, -2), (-2, 0), (-2, -2)]
    return out


@pytest.mark.parametrize("NI,NJ", [(33, 25), (97, 129), (384, 513), (40, 17), (65, 9), (1025, 1025)])
def test_tiles_cover_the_interior_once_and_read_loaded_values(NI, NJ):
    ti = (NI - 1 + TI - 1) // TI
    nblk = ti * ((NJ - 1 + TJ - 1) // TJ)
    seen = {}
    for b in range(nblk):
        i0, j0 = (b % ti) * TI + 1, (b // ti) * TJ + 1
        loaded = set()
        for r, q in itertools.product(range(H), range(W)):
            ih, jh = i0 - 2 + q, j0 - 2 + r
            if 0 <= ih <= NI and 0 <= jh <= NJ:
                loaded.add((q, r))
        for t in range(256):
            tx, ty = t & 31, t >> 5
            i, j = i0 + tx, j0 + ty
            if not (i <= NI - 1 and j <= NJ - 1):
                continue
            seen[(i, j)] = seen.get((i, j), 0) + 1
            for dd_pos in (0, 1):
                for a, bb in reads(i, j, NI, NJ, dd_pos):
                    q, r = tx + 2 + a, ty + 2 + bb
                    assert 0 <= q < W and 0 <= r < H
                    assert (q, r) in loaded, (i, j, a, bb)
    assert len(seen) == (NI - 1) * (NJ - 1)
    assert set(seen.values()) == {1}
