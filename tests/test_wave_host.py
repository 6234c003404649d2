"""Host-side facts the persistent wavefront kernel (stag_wave_kernel, stages 4) rests on,
checked without a GPU:

* tile_row: the tile's row of tiles by a multiplier and shift instead of an integer
  division, tile_row(t) = (t * ceil(2^(32+l) / tiles_x)) >> (32 + l) with
  l = ceil(log2(tiles_x)), equals t // tiles_x for every tile index below 2^31;
* the dependency rule: a tile of row ty waits until rows ty - 1 .. ty + 1 finished the
  previous step. Every cell its staged region reads (rows y0 - 1 .. y0 + TY + 1,
  columns x0 - 4 .. x0 + TX + 3, the out-of-row columns taken from the neighbouring
  rows through the flat index) lies in those rows of tiles, for the tile shapes that
  have a wavefront kernel and for ragged grids; so does every tile that reads a cell
  this tile owns (the symmetric condition that orders overwrites after reads).
"""
import numpy as np
import pytest


def tile_divider(tiles_x):
    l = 0
    while (1 << l) < tiles_x:
        l += 1
    return ((1 << (32 + l)) + tiles_x - 1) // tiles_x, 32 + l


@pytest.mark.parametrize("tiles_x", list(range(1, 70)) + [127, 128, 129, 1000, 4095, 65537,
                                                           (1 << 20) + 7, (1 << 30) - 1])
def test_tile_row_divider_is_exact(tiles_x):
    mul, shift = tile_divider(tiles_x)
    assert mul < (1 << 33)
    rng = np.random.default_rng(tiles_x)
    t = np.concatenate([np.arange(0, 5000), rng.integers(0, 1 << 31, 20000),
                        np.array([(1 << 31) - 1, tiles_x * 37 - 1, tiles_x * 37])])
    t = t[t < (1 << 31)].astype(object)  # exact integers
    got = [(int(v) * mul) >> shift for v in t]
    assert got == [int(v) // tiles_x for v in t]


def _region_cells(x0, y0, tx, ty, nx, ny):
    """Flat indices of the staged region of a tile that exist in the field."""
    n = nx * ny
    ys = np.arange(y0 - 1, y0 + ty + 2)
    xs = np.arange(x0 - 4, x0 + tx + 4)
    f = (ys[:, None] * nx + xs[None, :]).reshape(-1)
    return f[(f >= 0) & (f < n)]


@pytest.mark.parametrize("tx,ty", [(64, 16), (64, 12)])
@pytest.mark.parametrize("nx,ny", [(2048, 2048), (256, 96), (204, 77), (200, 3), (64, 48),
                                   (130, 61), (64, 13)])
def test_wavefront_dependencies_cover_the_region(tx, ty, nx, ny):
    if nx * ny > 300000:
        nx, ny = 512, 200  # the same geometry at a size the test enumerates quickly
    tiles_x = (nx + tx - 1) // tx
    tiles_y = (ny + ty - 1) // ty
    readers = {}
    for tyi in range(tiles_y):
        for txi in range(tiles_x):
            cells = _region_cells(txi * tx, tyi * ty, tx, ty, nx, ny)
            rows_of_tiles = np.unique((cells // nx) // ty)
            # the cells this tile reads lie in tile rows tyi - 1 .. tyi + 1
            assert rows_of_tiles.min() >= tyi - 1 and rows_of_tiles.max() <= tyi + 1
            for r in rows_of_tiles:
                readers.setdefault(int(r), set()).add(tyi)
    # a tile's own cells are read only by tiles within one row of tiles of it, which
    # are exactly the rows whose completion it waits for before it overwrites them
    for r, rs in readers.items():
        assert max(rs) - r <= 1 and r - min(rs) <= 1
