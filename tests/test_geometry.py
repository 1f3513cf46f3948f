"""CPU: the strip geometry of the advance kernel (the engine's own host code,
through an internal export).  For every grid, blocking and CPML/NTFF layout:
each column is owned by exactly one item; no item owns more columns than its
layout allows; the column window of every item lies inside the zero padding
of the field rows; wide windows start on a multiple of COLS (the row copies
move COLS elements at once); and no wide window -- owned columns and halo --
touches a column that needs the general path (PEC boundary, CPML, vertical
NTFF faces)."""
from __future__ import annotations

import ctypes as C

import pytest

PAD_LEFT, PAD_RIGHT = 32, 160


def _items(lib, nx, nc, d, T, cols, ny=None, nseg=1):
    buf = (C.c_int * 50000)()
    n = lib.tomo_internal_work_items(nx, nx if ny is None else ny, nc, d, T, cols, nseg, buf, 10000)
    assert n > 0, lib.tomo_last_error()
    return [tuple(buf[5 * i + j] for j in range(5)) for i in range(n)]


@pytest.mark.parametrize("T,cols", [(1, 1), (2, 1), (2, 2), (2, 4), (3, 1), (3, 2), (4, 1), (4, 2), (6, 1), (8, 1)])
def test_strip_geometry(tomo, T, cols):
    lib = tomo.library()
    grids = list(range(16, 140, 3)) + [200, 255, 256, 257, 400, 401, 512, 600, 601, 1024, 2048]
    wide_seen = 0
    for nx in grids:
        for nc in (0, 8, 10, 12, 16, 32):
            if 2 * nc + 4 > nx:
                continue
            for d in (-1, nc + 3):
                if d >= 0 and 2 * d + 4 > nx:
                    continue
                owned = [0] * (nx + 1)
                for x0, x1, narrow, y0, y1 in _items(lib, nx, nc, d, T, cols):
                    assert (y0, y1) == (0, nx + 1)
                    c = cols if (cols > 1 and not narrow) else 1
                    P = 32 * c
                    xs = x1 + T - P
                    assert 0 <= x0 < x1 <= nx + 1 and x1 - x0 <= P - 2 * T
                    assert xs <= x0 - T and xs >= -PAD_LEFT and xs + P <= nx + 1 + PAD_RIGHT
                    assert xs % c == 0, (nx, nc, d, x0, x1)
                    for x in range(x0, x1):
                        owned[x] += 1
                    if c > 1:
                        wide_seen += 1
                        for x in range(xs, xs + P):
                            special = x <= nc or x >= nx - nc or (d >= 0 and x in (d, nx - d - 1))
                            assert not special, (nx, nc, d, T, cols, x0, x1, x)
                assert owned == [1] * (nx + 1), (nx, nc, d)
    if cols > 1:
        assert wide_seen > 0


@pytest.mark.parametrize("nseg", [2, 3, 7])
def test_row_segments_cover_every_cell_once(tomo, nseg):
    lib = tomo.library()
    for nx, ny, nc, d in ((96, 96, 8, 11), (200, 150, 10, 13), (400, 400, 12, 15)):
        cover = [[0] * (ny + 1) for _ in range(nx + 1)]
        for x0, x1, _, y0, y1 in _items(lib, nx, nc, d, 2, 2, ny=ny, nseg=nseg):
            assert 0 <= y0 < y1 <= ny + 1
            for x in range(x0, x1):
                for y in range(y0, y1):
                    cover[x][y] += 1
        assert all(v == 1 for col in cover for v in col), (nx, ny, nseg)


def _blockings(lib, precision, mode):
    f = lib.tomo_internal_blockings
    f.restype, f.argtypes = C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int]
    buf = (C.c_int * 512)()
    n = f(precision, mode, buf, 512)
    assert n > 0, lib.tomo_last_error()
    return [tuple(buf[4 * i + j] for j in range(4)) for i in range(n)]


SMEM_PER_SM = 228 * 1024          # sm_100 family: 228 KB per SM, 1 KB of it reserved per resident block
SMEM_PER_BLOCK = 227 * 1024


def test_offered_blockings_are_launchable(tomo):
    """Every blocking the autotuner offers has a compiled kernel and a block
    small enough to launch; the FP32 variants' requested blocks per SM (the
    MINB their registers were capped for) also fit the SM's shared memory,
    so the cap buys the occupancy it was made for.  The bench's blockings
    (T 4 COLS 2 MINB 2, T 2 COLS 2 MINB 3) are offered in the breast mode, and
    the autotuner's first choice there is T 2 COLS 2 MINB 3."""
    lib = tomo.library()
    for prec in (tomo.FP32, tomo.FP64):
        for mode in (0, 1, 2):
            bs = _blockings(lib, prec, mode)
            for T, cols, minb, smem in bs:
                assert 0 < smem <= SMEM_PER_BLOCK, (prec, mode, T, cols, smem)
                if prec == tomo.FP32:
                    assert minb * (smem + 1024) <= SMEM_PER_SM, (mode, T, cols, minb, smem)
                else:
                    assert cols == 1
    breast = [b[:3] for b in _blockings(lib, tomo.FP32, 2)]
    assert breast[0] == (2, 2, 3) and (4, 2, 2) in breast and len(breast) == len(set(breast))
    # FP64, T 2, MINB 3: three blocks need 3 x 81.8 KB > 228 KB, so shared memory
    # holds it to two; the autotuner times it beside MINB 2 and keeps the faster
    f64 = {b[:3]: b[3] for b in _blockings(lib, tomo.FP64, 2)}
    assert 3 * (f64[(2, 1, 3)] + 1024) > SMEM_PER_SM
