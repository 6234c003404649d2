"""Host-side table compilation, checked through a NumPy model of the tile kernel
(tests/helpers.py:KernelModel) that reads the same tables: on small tiles (many
tiles, partial tiles, row-end wraps at tile seams) it must reproduce the oracle
bit for bit, for every field kind and boundary/output mode."""
import os

import numpy as np
import pytest

from oracle import fds_oracle as O
from oracle import scenarios as S
from helpers import KernelModel, build_field

CASES = []
for seed in range(30):
    kind = S.ALL_KINDS[seed % 6]
    if kind.endswith("1D"):
        CASES.append((seed, kind, [17, 9, 33, 5, 12][seed % 5], None, (4, 1)))
    else:
        CASES.append((seed, kind, [9, 7, 5, 11, 8][seed % 5], [7, 6, 9, 4, 5][(seed // 5) % 5],
                      [(4, 3), (3, 2), (2, 2), (8, 4), (1, 1)][seed % 5]))


@pytest.mark.parametrize("seed,kind,nx,ny,tile", CASES)
def test_kernel_model_matches_oracle(seed, kind, nx, ny, tile):
    spec = S.random_scenario(seed, kind, nx, ny, steps=6, mu=(seed % 3 != 0))
    st_o, sg_o = O.simulate(spec, spec["steps"])
    f = build_field(spec, exact=True)
    st_m, sg_m = KernelModel(f, tile=tile).run(spec["steps"])
    for c in st_o:
        assert np.array_equal(st_o[c], st_m[c]), c
        for a, b in zip(sg_o[c], sg_m[c]):
            assert np.array_equal(a, b), c


def test_kernel_model_segmented_start_step():
    spec = S.random_scenario(3, "Acoustic2D", 9, 6, steps=8)
    st_o, sg_o = O.simulate(spec, spec["steps"])
    f = build_field(spec, exact=True)
    m = KernelModel(f, tile=(4, 3))
    st1, sg1 = m.run(5, step0=0)
    for c, v in st1.items():
        getattr(f, c).values = v
    st2, sg2 = m.run(3, step0=5)
    for c in st_o:
        assert np.array_equal(st_o[c], st2[c])
        for a, b1, b2 in zip(sg_o[c], sg1[c], sg2[c]):
            assert np.array_equal(a, np.concatenate([b1, b2], axis=1))


def test_short_signal_raises_index_error_before_launch():
    import pyfds_gb300 as fds
    from pyfds_gb300 import _tables
    from pyfds_gb300.regions import Region
    geo = _tables.TileGeometry(6, 5, 4, 3, True)
    for value in (np.ones(10), np.ones((10, 2)), [np.ones(10), np.ones(10)]):
        b = fds.Boundary(Region([1, 2]), value=value, additive=True)
        _tables.compile_bounds([b], 30, _tables.SignalPool(), 10, geo, 0)
        with pytest.raises(IndexError):
            _tables.compile_bounds([b], 30, _tables.SignalPool(), 11, geo, 0)
    # ragged per-point signals: np.ndim raises ValueError, as in Boundary.apply
    b = fds.Boundary(Region([1, 2]), value=[np.ones(10), np.ones(12)], additive=True)
    with pytest.raises(ValueError):
        _tables.compile_bounds([b], 30, _tables.SignalPool(), 10, geo, 0)


def test_value_shape_errors():
    import pyfds_gb300 as fds
    from pyfds_gb300 import _tables
    from pyfds_gb300.regions import Region
    geo = _tables.TileGeometry(6, 5, 4, 3, True)
    b = fds.Boundary(Region([1, 2, 3]), value=[np.ones(5), np.ones(5)])
    with pytest.raises(ValueError):
        _tables.compile_bounds([b], 30, _tables.SignalPool(), 5, geo, 0)
    b = fds.Boundary(Region([1, 2]), value=[np.ones(5)] * 3)
    with pytest.raises(IndexError):
        _tables.compile_bounds([b], 30, _tables.SignalPool(), 5, geo, 0)
    b = fds.Boundary(Region([1, 2, 99]), value=1.0)
    with pytest.raises(IndexError):
        _tables.compile_bounds([b], 30, _tables.SignalPool(), 5, geo, 0)


def test_negative_indices_wrap_like_numpy():
    spec = S.random_scenario(2, "Acoustic1D", 12, None, steps=5, boundary_modes=["dirichlet"])
    spec["bounds"]["pressure"].append({"indices": [-1, -3], "value": 0.25, "additive": False})
    st_o, _ = O.simulate(spec, spec["steps"])
    f = build_field(spec, exact=True)
    st_m, _ = KernelModel(f, tile=(4, 1)).run(spec["steps"])
    assert np.array_equal(st_o["pressure"], st_m["pressure"])


def _decode(geo, tile, pos):
    """Flat cell of a tile slot (inverse of the slot numbering of each layout)."""
    tx, ty = tile % geo.tiles_x, tile // geo.tiles_x
    x0, y0 = tx * geo.tx, ty * geo.ty
    lx = pos % geo.rx - geo.ox
    ly = pos // geo.rx - geo.oy
    return (y0 + ly) * geo.nx + x0 + lx


@pytest.mark.parametrize("layout,tile", [(0, (64, 16)), (0, (4, 3)), (1, (62, 16)), (1, (30, 8)),
                                         (1, (6, 3))])
@pytest.mark.parametrize("nx,ny", [(200, 77), (62, 31), (7, 40), (130, 9)])
def test_table_slots_decode_to_their_cells(layout, tile, nx, ny):
    """Every boundary group and probe sits in slots that hold its own cell, and each
    flux cell is present in every tile that reads it (owner, right/bottom halo,
    row-end wrap)."""
    from pyfds_gb300 import _tables
    import pyfds_gb300 as fds
    from pyfds_gb300.regions import Region
    geo = _tables.TileGeometry(nx, ny, tile[0], tile[1], True, layout)
    n = nx * ny
    rng = np.random.default_rng(nx * 1000 + ny)
    cells = np.unique(np.concatenate([rng.integers(0, n, 300), np.arange(0, n, nx),
                                      np.arange(nx - 1, n, nx), np.arange(nx)]))
    for role in (0, 1, 2):
        b = fds.Boundary(Region(cells), value=1.0)
        bt = _tables.compile_bounds([b], n, _tables.SignalPool(), 1, geo, role)
        ts = bt["tile_start"]
        for t in range(geo.ntiles):
            grp = bt["groups"][ts[t]:ts[t + 1]]
            assert np.all(np.diff(grp["pos"]) >= 0)  # sorted by slot within a tile
            for g in grp:
                assert _decode(geo, t, g["pos"]) == g["cell"]
        # each flux cell appears in the tiles whose extended region reads it
        placed = {(int(t), int(g["cell"])) for t in range(geo.ntiles)
                  for g in bt["groups"][ts[t]:ts[t + 1]]}
        for t in range(geo.ntiles):
            x0, y0 = (t % geo.tiles_x) * geo.tx, (t // geo.tiles_x) * geo.ty
            x1, y1 = min(x0 + geo.tx, nx), min(y0 + geo.ty, ny)
            if role == 1:   # U-ext: [x0, x1] x [y0, y1)
                need = [(y * nx + x) for y in range(y0, y1) for x in range(x0, x1 + 1)]
            elif role == 2:  # V-ext: [x0, x1) x [y0, y1]
                need = [(y * nx + x) for y in range(y0, y1 + 1) for x in range(x0, x1)]
            else:
                need = [(y * nx + x) for y in range(y0, y1) for x in range(x0, x1)]
            for c in need:
                if c < n and c in set(cells.tolist()):
                    assert (t, c) in placed, (role, t, c)
    pt, ncols = _tables.compile_probes([fds.Output(Region(cells))], n, geo)
    ts = pt["tile_start"]
    for t in range(geo.ntiles):
        for q in pt["probes"][ts[t]:ts[t + 1]]:
            assert _decode(geo, t, q["pos"]) == q["cell"]


@pytest.mark.parametrize("nx,ny,tx,ty", [(37, 19, 8, 4), (5, 9, 8, 4), (1, 7, 8, 4), (64, 24, 16, 8),
                                         (3, 1, 8, 4), (17, 2, 4, 4), (9, 7, 1, 1), (7, 5, 2, 1),
                                         (6, 6, 3, 2)])
def test_two_step_ring_placements_match_brute_force(nx, ny, tx, ty):
    """Layout 2 (two steps per tile): a cell's bound group is placed at exactly the
    slots of each tile's first-step ring whose flat index is that cell, for every
    component's ring, including row-end wrap aliases and grids narrower than a tile."""
    from pyfds_gb300 import _tables as T
    geo = T.TileGeometry(nx, ny, tx, ty, True, layout=2)
    n = nx * ny
    cells = np.arange(n)
    for role, (ml, mr, ma, mb) in T.TileGeometry.RING.items():
        want = set()
        for t in range(geo.ntiles):
            x0 = (t % geo.tiles_x) * tx
            y0 = (t // geo.tiles_x) * ty
            for Y in range(y0 - ma, y0 + ty + mb):
                for X in range(x0 - ml, x0 + tx + mr):
                    f = Y * nx + X
                    if 0 <= f < n:
                        pos = (Y - y0 + geo.oy) * geo.rx + (X - x0) + geo.ox
                        want.add((t, pos, f))
        tiles, pos, src, primary = geo.placements(cells, role)
        got = set(zip(tiles.tolist(), pos.tolist(), cells[src].tolist()))
        assert got == want, (role, len(got), len(want))
        assert len(got) == tiles.size  # no duplicates
        # one primary placement per cell: its owner's slot
        assert np.array_equal(np.sort(src[primary == 1]), cells)
        own_t, own_p = geo.owner(cells[src[primary == 1]])
        assert np.array_equal(own_t, tiles[primary == 1])
        assert np.array_equal(own_p, pos[primary == 1])


TWO_STEP_CASES = []
for seed in range(40, 64):
    kind = ["Acoustic2D", "Thermal2D", "Acoustic3DAxi", "Thermal3DAxi"][seed % 4]
    TWO_STEP_CASES.append((seed, kind, [9, 7, 5, 11, 8, 3, 1][seed % 7],
                           [7, 6, 9, 4, 5, 2][(seed // 7) % 6],
                           [(4, 3), (3, 2), (2, 2), (8, 4), (1, 1), (4, 4)][seed % 6],
                           [6, 7, 1, 2][seed % 4]))


@pytest.mark.parametrize("seed,kind,nx,ny,tile,steps", TWO_STEP_CASES)
def test_two_step_kernel_model_matches_oracle(seed, kind, nx, ny, tile, steps):
    """Two steps per tile (layout-2 tables, the first step on a ring around the
    tile): bit for bit the oracle, for odd and even step counts, on tiny tiles and
    grids narrower than a tile, every boundary and output mode."""
    spec = S.random_scenario(seed, kind, nx, ny, steps=steps, mu=False)
    st_o, sg_o = O.simulate(spec, spec["steps"])
    f = build_field(spec, exact=True)
    st_m, sg_m = KernelModel(f, tile=tile, two_step=True).run(spec["steps"])
    for c in st_o:
        assert np.array_equal(st_o[c], st_m[c]), c
        for a, b in zip(sg_o[c], sg_m[c]):
            assert np.array_equal(a, b), c


def test_batched_launch_count():
    """Launches of a batched run (mirrors the loop of fds_stag_batch_run): with two
    steps per tile the count is even for every step count of two or more, so a
    captured graph ends with the ping-pong buffers where it started."""
    from pyfds_gb300.batch import launch_count
    assert [launch_count(n, 1) for n in range(6)] == [0, 1, 2, 3, 4, 5]
    assert [launch_count(n, 2) for n in range(1, 9)] == [1, 2, 2, 2, 4, 4, 4, 4]
    for n in range(2, 200):
        k = launch_count(n, 2)
        assert k % 2 == 0 and n / 2 <= k <= n / 2 + 2


FUZZ_CASES = int(os.environ.get("PYFDS_GB300_FUZZ_CASES", "1000"))


def test_kernel_model_fuzz():
    """Seeded random cases, one and two steps per tile: every field kind (two steps:
    the 2-D kinds), grids of 1 to 13 x 1 to 10 cells (1 to 39 in 1-D), tiles of 1 to 8
    x 1 to 5 cells, 1 to 7 steps, every boundary and output mode: the model on the
    compiled tables reproduces the oracle bit for bit. PYFDS_GB300_FUZZ_CASES sets
    the count (68 000 cases ran clean)."""
    rng = np.random.default_rng(12345)
    for _ in range(FUZZ_CASES):
        seed = int(rng.integers(1000, 10 ** 6))
        two = bool(rng.integers(0, 2))
        kinds = ["Acoustic2D", "Thermal2D", "Acoustic3DAxi", "Thermal3DAxi"]
        if not two:
            kinds += ["Acoustic1D", "Thermal1D"]
        kind = kinds[int(rng.integers(0, len(kinds)))]
        if kind.endswith("1D"):
            nx, ny, tile = int(rng.integers(1, 40)), None, (int(rng.integers(1, 9)), 1)
        else:
            nx, ny = int(rng.integers(1, 14)), int(rng.integers(1, 11))
            tile = (int(rng.integers(1, 9)), int(rng.integers(1, 6)))
        steps = int(rng.integers(1, 8))
        mu = False if two else bool(rng.integers(0, 2))
        case = (seed, kind, nx, ny, tile, steps, two, mu)
        spec = S.random_scenario(seed, kind, nx, ny, steps=steps, mu=mu)
        st_o, sg_o = O.simulate(spec, steps)
        f = build_field(spec, exact=True)
        st_m, sg_m = KernelModel(f, tile=tile, two_step=two).run(steps)
        for c in st_o:
            assert np.array_equal(st_o[c], st_m[c]), (case, c)
            for a, b in zip(sg_o[c], sg_m[c]):
                assert np.array_equal(a, b), (case, c)


def test_signal_steps_bounds_table_reuse():
    """Compiled tables serve every call that ends within the shortest signal of the
    boundaries (signal_steps); scalar values do not limit them."""
    from pyfds_gb300 import regions as R
    from pyfds_gb300._tables import signal_steps
    reg = R.Region([1, 2], "b")
    assert signal_steps([R.Boundary(reg, value=3.0)]) is None
    assert signal_steps([R.Boundary(reg, value=np.zeros(50)),
                         R.Boundary(reg, value=np.zeros((40, 2)))]) == 40
    assert signal_steps([R.Boundary(reg, value=[np.zeros(30), np.zeros(35)]),
                         R.Boundary(reg, value=1.0)]) == 30
