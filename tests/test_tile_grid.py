"""The tile grid a batch gets (host logic, no GPU): sfwi_debug_tile_grid runs
the engine's own planner.  Checked against a brute force written from the
definitions: the tiles of a shot cover its update region [NOP, n-NOP) in both
directions, the z start keeps TMA box columns 16-byte aligned for 16-bit
snapshots (NOP - 8k), a tile holds PML cells exactly when one of its updated
cells is damped (index < pml or > n-pml), and no other allowed start has
fewer tiles plus PML tiles."""
import ctypes as C

import numpy as np
import pytest

NOP = 4


def _plan(pml, nzpml, tx, tz, widths):
    from sfwi_gb300 import _lib
    lib = _lib.load()
    n = len(widths)
    w = (C.c_int * n)(*widths)
    zs = C.c_int()
    xs, tiles, frame = (C.c_int * n)(), (C.c_int * n)(), (C.c_int * n)()
    _lib.check(lib.sfwi_debug_tile_grid(pml, nzpml, tx, tz, w, n, C.byref(zs), xs, tiles, frame))
    return zs.value, list(xs), list(tiles), list(frame)


def _axis(n, pml, t, start):
    """(tiles, tiles holding a damped updated index) of one axis, cell by cell."""
    count = frame = 0
    t0 = start
    while t0 < n - NOP:
        cells = [i for i in range(t0, t0 + t) if NOP <= i < n - NOP]
        assert cells, (n, t, start, t0)
        count += 1
        frame += any(i < pml or i > n - pml for i in cells)
        t0 += t
    return count, frame


def _shot(nx, nz, pml, tx, tz, xs, zs):
    cx, fx = _axis(nx, pml, tx, xs)
    cz, fz = _axis(nz, pml, tz, zs)
    return cx * cz, cx * cz - (cx - fx) * (cz - fz)


def _best_cost(pml, nzpml, tx, tz, widths):
    best = None
    for zs in range(NOP, NOP - tz, -8):
        cost = 0
        for nx in widths:
            cost += min(sum(_shot(nx, nzpml, pml, tx, tz, xs, zs)) for xs in range(NOP, NOP - tx, -1))
        best = cost if best is None else min(best, cost)
    return best


CASES = [
    (20, 241, 16, 32, [416] * 3),                 # 38-shot 376x201 batch (three of its shots)
    (20, 241, 8, 32, [416]),                      # one shot on 8x32 tiles
    (20, 341, 16, 32, [190, 254, 300, 441, 377]),  # 401x301 salt batch, uneven apertures
    (20, 341, 16, 64, [190, 441]),
    (20, 841, 32, 32, [2041, 2041]),              # 2001x801
    (11, 105, 16, 32, [67, 44, 47]),              # the small grid of the shape-identity tests
    (8, 46, 16, 32, [40, 52, 60]),                # the golden-vector grids: every tile holds PML cells
]


@pytest.mark.parametrize("pml,nzpml,tx,tz,widths", CASES)
def test_tile_grid_covers_the_update_region_and_is_optimal(pml, nzpml, tx, tz, widths):
    zs, xs, tiles, frame = _plan(pml, nzpml, tx, tz, widths)
    assert (NOP - zs) % 8 == 0 and NOP - tz < zs <= NOP, zs
    total = 0
    for nx, x0, t, f in zip(widths, xs, tiles, frame):
        assert NOP - tx < x0 <= NOP, x0
        assert (t, f) == _shot(nx, nzpml, pml, tx, tz, x0, zs)
        total += t + f
    assert total == _best_cost(pml, nzpml, tx, tz, widths)


def test_fewer_pml_tiles_on_the_376x201_batch():
    zs, xs, tiles, frame = _plan(20, 241, 16, 32, [416])
    share = frame[0] / tiles[0]
    base_t, base_f = _shot(416, 241, 20, 16, 32, NOP, NOP)
    print("PML tiles %d of %d (%.0f %%), from %d of %d starting at NOP" % (frame[0], tiles[0], 100 * share, base_f,
                                                                         base_t))
    assert tiles[0] == base_t and frame[0] < base_f and share < 0.35


def test_bad_arguments_are_refused():
    from sfwi_gb300 import _lib
    with pytest.raises(_lib.SfwiError, match="tile-grid"):
        _plan(20, 241, 16, 30, [416])  # z tiles must be a multiple of 8 columns
    with pytest.raises(_lib.SfwiError, match="too small"):
        _plan(20, 241, 16, 32, [416, 30])
