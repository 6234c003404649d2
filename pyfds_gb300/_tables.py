"""Compile a field's boundaries and outputs into the per-tile device tables.

Semantics reproduced (pyfds/fields.py:591-611, pyfds/regions.py:125-165):

- boundaries of one component apply in list order; one boundary assigns
  ``values[idx] = additive * values[idx] + value`` with numpy fancy indexing, so
  for a repeated index the LAST point of that boundary wins (and an additive
  boundary adds once);
- the value is a scalar, ``value[step]`` of an ndarray (1-D: broadcast; 2-D: one
  row of per-point values), or ``signal_k[step]`` of a list of per-point signals;
- outputs sample every index of their region, in order, once per step.

Each component's boundary cells become *groups*: one per distinct cell, holding
the chain of operations (one per boundary touching the cell, in list order). A
group is listed under every tile whose shared-memory region holds a copy of the
cell that the kernel updates: its owner tile and, for the x flux, the tile to its
left (which recomputes the column at its right edge) or, for column 0, the last
tile of the previous row (the row-end wrap); for the y flux, the tile above.
"""
import numpy as np

from . import _capi

ROLE_POTENTIAL, ROLE_UX, ROLE_VY = 0, 1, 2


class TileGeometry:
    """Tiling used by the kernel: ``tx`` x ``ty`` owned cells per tile, and how a
    tile numbers its slots (layout 0: the one-step tile kernel, layout 1: the
    register-marching kernel, layout 2: the two-step tile kernel; stag_kernel.cuh,
    march_kernel.cuh)."""

    # layout 2: margins (left, right, above, below) of the ring on which a tile
    # computes each component in its first step (the second step computes a subset)
    RING = {ROLE_POTENTIAL: (1, 1, 1, 1), ROLE_UX: (1, 2, 1, 1), ROLE_VY: (1, 1, 1, 2)}

    def __init__(self, nx, ny, tx, ty, has_v, layout=0):
        self.nx, self.ny, self.tx, self.ty = int(nx), int(ny), int(tx), int(ty)
        self.has_v = bool(has_v)
        self.layout = int(layout)
        self.tiles_x = (self.nx + self.tx - 1) // self.tx
        self.tiles_y = (self.ny + self.ty - 1) // self.ty
        self.ntiles = self.tiles_x * self.tiles_y
        if self.layout == 0:
            # shared-memory region: one halo row above, columns x0-4 .. x0+tx+3
            self.oy = 1 if has_v else 0
            self.ox = 4
            self.rx = self.tx + 8
        elif self.layout == 2:
            # two-step region: two halo rows above, columns x0-4 .. x0+tx+3
            self.oy = 2
            self.ox = 4
            self.rx = self.tx + 8
        else:
            # register-marching warp strip: cells x0-1 .. x0+tx per row, rows from y0
            self.oy = 0
            self.ox = 1
            self.rx = self.tx + 2

    def owner(self, cell):
        x = cell % self.nx
        y = cell // self.nx
        tx = x // self.tx
        ty = y // self.ty
        tile = ty * self.tiles_x + tx
        pos = (y - ty * self.ty + self.oy) * self.rx + (x - tx * self.tx) + self.ox
        return tile, pos

    def placements(self, cell, role):
        """(tile, pos, index into ``cell``, primary) of every tile slot a cell
        occupies; ``primary`` marks one placement per cell (the owning tile's slot)."""
        if self.layout == 2:
            return self._ring_placements(cell, role)
        tiles, poss = self.owner(cell)
        src = np.arange(cell.size)
        out_t, out_p, out_s = [tiles], [poss], [src]
        x = cell % self.nx
        y = cell // self.nx
        if role == ROLE_UX:
            # right-edge column of the left neighbour tile
            m = (x % self.tx == 0) & (x > 0)
            if m.any():
                tx = x[m] // self.tx - 1
                ty = y[m] // self.ty
                out_t.append(ty * self.tiles_x + tx)
                out_p.append((y[m] - ty * self.ty + self.oy) * self.rx + self.tx + self.ox)
                out_s.append(src[m])
            # column 0 of row y is column nx of row y-1 (flat-index wrap)
            m = (x == 0) & (y > 0)
            if m.any():
                yy = y[m] - 1
                tx = self.tiles_x - 1
                ty = yy // self.ty
                lx = self.nx - tx * self.tx
                out_t.append(ty * self.tiles_x + tx)
                out_p.append((yy - ty * self.ty + self.oy) * self.rx + lx + self.ox)
                out_s.append(src[m])
        elif role == ROLE_VY:
            m = (y % self.ty == 0) & (y > 0)
            if m.any():
                tx = x[m] // self.tx
                ty = y[m] // self.ty - 1
                out_t.append(ty * self.tiles_x + tx)
                out_p.append((self.ty + self.oy) * self.rx + (x[m] - tx * self.tx) + self.ox)
                out_s.append(src[m])
        primary = np.zeros(sum(t.size for t in out_t), np.int32)
        primary[:cell.size] = 1
        return np.concatenate(out_t), np.concatenate(out_p), np.concatenate(out_s), primary

    def _ring_placements(self, cell, role):
        """Layout 2: every slot of every tile's first-step ring where ``cell`` is
        computed. Slots are addressed by flat index, so a cell (x, y) also sits at
        (x + k*nx, y - k) wherever that column lies in a tile's ring (row-end wrap;
        several aliases per tile on grids narrower than the ring)."""
        ml, mr, ma, mb = self.RING[role]
        x0 = cell % self.nx
        y0 = cell // self.nx
        src0 = np.arange(cell.size)
        own_t0, own_p0 = self.owner(cell)
        # ring columns of all tiles: -ml .. W - 1 + mr; alias k exists for a cell when
        # x + k*nx falls there (k in {-1, 0, 1} unless the grid is narrower than that)
        W = self.tiles_x * self.tx
        kmin = -((ml + self.nx - 1) // self.nx)
        kmax = (W - 1 + mr) // self.nx
        out_t, out_p, out_s, out_q = [], [], [], []
        for k in range(kmin, kmax + 1):
            X = x0 + k * self.nx
            sel = np.nonzero((X >= -ml) & (X <= W - 1 + mr))[0]
            if sel.size == 0:
                continue
            X = X[sel]
            Y = y0[sel] - k
            src = src0[sel]
            own_t, own_p = own_t0[sel], own_p0[sel]
            # tiles whose ring [t*tx - ml, t*tx + tx - 1 + mr] contains X: at most
            # ceil((ml + mr) / tx) + 1 consecutive tile columns (two for the kernel's
            # tiles; more for tiles narrower than the margins)
            for dtx in range((ml + mr + self.tx - 1) // self.tx + 1):
                tx = (X + ml) // self.tx - dtx
                okx = (tx >= 0) & (tx < self.tiles_x) & (X >= tx * self.tx - ml) & \
                    (X <= tx * self.tx + self.tx - 1 + mr)
                for dty in range((ma + mb + self.ty - 1) // self.ty + 1):
                    ty = (Y + ma) // self.ty - dty
                    ok = okx & (ty >= 0) & (ty < self.tiles_y) & (Y >= ty * self.ty - ma) & \
                        (Y <= ty * self.ty + self.ty - 1 + mb)
                    if not ok.any():
                        continue
                    t = ty[ok] * self.tiles_x + tx[ok]
                    pos = (Y[ok] - ty[ok] * self.ty + self.oy) * self.rx + \
                        (X[ok] - tx[ok] * self.tx) + self.ox
                    out_t.append(t)
                    out_p.append(pos)
                    out_s.append(src[ok])
                    out_q.append(((t == own_t[ok]) & (pos == own_p[ok])).astype(np.int32))
        if not out_t:
            z = np.zeros(0, np.int64)
            return z, z, z, np.zeros(0, np.int32)
        return (np.concatenate(out_t), np.concatenate(out_p), np.concatenate(out_s),
                np.concatenate(out_q))


class SignalPool:
    """Float64 pool of boundary signal samples (one segment per distinct array)."""

    def __init__(self):
        self.parts = []
        self.size = 0
        self._seen = {}

    def add(self, arr, key=None):
        k = id(arr) if key is None else key
        if k in self._seen:
            return self._seen[k][0]
        a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64)).reshape(-1)
        off = self.size
        self.parts.append(a)
        self.size += a.size
        self._seen[k] = (off, arr)  # keep arr alive so its id stays unique
        return off

    def array(self):
        if not self.parts:
            return np.zeros(1)
        return np.concatenate(self.parts)


def _norm_indices(indices, n):
    idx = np.asarray(indices, dtype=np.int64).reshape(-1)
    if idx.size and (idx.min() < -n or idx.max() >= n):
        bad = idx[(idx < -n) | (idx >= n)][0]
        raise IndexError("index %d is out of bounds for axis 0 with size %d" % (bad, n))
    return np.where(idx < 0, idx + n, idx)


def _boundary_ops(b, n, pool, step_end):
    """Per-point operations of one boundary, after numpy's last-write-wins dedup.

    Returns (cells, ops) with ops a BOUND_OP_DTYPE array aligned with cells. Raises
    the exception the reference would raise when a signal is too short
    (IndexError) or the value does not fit the region (ValueError / IndexError /
    TypeError)."""
    idx = _norm_indices(b.region.indices, n)
    npts = idx.size
    value = b.value
    mul = float(b.additive)
    if np.ndim(value) == 0:  # (ragged per-point signals raise here, as in the reference)
        kind = "scalar"
    elif isinstance(value, np.ndarray):
        kind = "array%d" % value.ndim
    else:
        kind = "list"
    # keep the last occurrence of every repeated index (numpy fancy assignment)
    if npts:
        _, first_rev = np.unique(idx[::-1], return_index=True)
        keep = np.sort(npts - 1 - first_rev)
    else:
        keep = np.zeros(0, dtype=np.int64)
    cells = idx[keep]
    ops = np.zeros(keep.size, dtype=_capi.BOUND_OP_DTYPE)
    ops["mul"] = mul
    if kind == "scalar":
        ops["scalar"] = float(value)
        return cells, ops
    if kind == "array1":
        if value.shape[0] < step_end:
            raise IndexError("index %d is out of bounds for axis 0 with size %d"
                             % (step_end - 1, value.shape[0]))
        off = pool.add(value)
        ops["off"] = off
        ops["stride"] = 1
        ops["flags"] = _capi.BOP_SIGNAL
        return cells, ops
    if kind == "array2":
        rows, m = value.shape
        if rows < step_end:
            raise IndexError("index %d is out of bounds for axis 0 with size %d"
                             % (step_end - 1, rows))
        if m != npts and m != 1:
            raise ValueError("shape mismatch: value array of shape (%d,) could not be "
                             "broadcast to indexing result of shape (%d,)" % (m, npts))
        off = pool.add(value)
        ops["off"] = off + (keep if m > 1 else 0)
        ops["stride"] = m
        ops["flags"] = _capi.BOP_SIGNAL
        return cells, ops
    if kind.startswith("array"):
        raise ValueError("boundary value arrays must have 1 or 2 dimensions")
    # list of per-point signals
    sigs = list(value)
    m = len(sigs)
    if m > npts:
        raise IndexError("index %d is out of bounds for axis 0 with size %d" % (npts, npts))
    if m != npts and m != 1:
        raise ValueError("shape mismatch: value array of shape (%d,) could not be broadcast "
                         "to indexing result of shape (%d,)" % (m, npts))
    if m == 1 and npts > 1 and mul != 0.0:
        # the reference would add the FIRST point's old value to every point
        raise ValueError("one per-point signal for %d points is only supported with "
                         "additive=False" % npts)
    offs = np.zeros(m, dtype=np.int64)
    for k, sig in enumerate(sigs):
        if np.ndim(sig) != 1:
            raise TypeError("per-point boundary signals must be 1-D sequences")
        if len(sig) < step_end:
            raise IndexError("index %d is out of bounds for axis 0 with size %d"
                             % (step_end - 1, len(sig)))
        offs[k] = pool.add(sig)
    ops["off"] = offs[keep] if m > 1 else offs[0]
    ops["stride"] = 1
    ops["flags"] = _capi.BOP_SIGNAL
    return cells, ops


def signal_steps(boundaries):
    """Steps the signal values of a boundary list cover (the shortest signal's length;
    None without signals): tables compiled from them serve every step range ending
    there, the pool holding each signal whole."""
    best = None
    for b in boundaries:
        value = b.value
        if isinstance(value, (list, tuple)):
            lengths = [len(sig) for sig in value if np.ndim(sig) == 1]
            length = min(lengths) if lengths else None
        elif np.ndim(value) == 0:
            continue
        elif isinstance(value, np.ndarray):
            length = value.shape[0]
        else:
            lengths = [len(sig) for sig in value if np.ndim(sig) == 1]
            length = min(lengths) if lengths else None
        if length is not None:
            best = length if best is None else min(best, length)
    return best


def compile_bounds(boundaries, n, pool, step_end, geo, role, offset=0.0):
    """Group/op/tile tables of one component's boundary list (None if empty).

    ``offset``: the component is stored as value - offset on the device, so every
    operation new = mul*old + v becomes new' = mul*old' + v + (mul - 1)*offset (for
    signal operations the constant rides in the op's ``scalar`` field)."""
    cells_l, ops_l = [], []
    for b in boundaries:
        c, o = _boundary_ops(b, n, pool, step_end)
        if offset:
            o["scalar"] = o["scalar"] + (o["mul"] - 1.0) * offset
        cells_l.append(c)
        ops_l.append(o)
    if not cells_l or sum(c.size for c in cells_l) == 0:
        return None
    cells = np.concatenate(cells_l)
    ops = np.concatenate(ops_l)
    order = np.argsort(cells, kind="stable")  # chains keep boundary order
    cells = cells[order]
    ops = ops[order]
    ucells, start = np.unique(cells, return_index=True)
    end = np.append(start[1:], cells.size)
    tiles, pos, src, primary = geo.placements(ucells, role)
    o2 = np.lexsort((pos, tiles))  # by tile, then slot (row-major within the tile)
    tiles, pos, src, primary = tiles[o2], pos[o2], src[o2], primary[o2]
    groups = np.zeros(tiles.size, dtype=_capi.BOUND_GROUP_DTYPE)
    groups["cell"] = ucells[src]
    groups["pos"] = pos
    groups["primary"] = primary
    groups["op_begin"] = start[src]
    groups["op_end"] = end[src]
    tile_start = np.searchsorted(tiles, np.arange(geo.ntiles + 1)).astype(np.int32)
    return {"tile_start": tile_start, "groups": groups, "ops": ops}


def compile_probes(outputs, n, geo):
    """Probe table of one component's outputs (None if empty) and its column count."""
    cells_l = []
    for o in outputs:
        cells_l.append(_norm_indices(o.region.indices, n))
    if not cells_l:
        return None, 0
    cells = np.concatenate(cells_l) if cells_l else np.zeros(0, np.int64)
    ncols = int(cells.size)
    if ncols == 0:
        return None, 0
    cols = np.arange(ncols)
    tiles, pos = geo.owner(cells)
    o = np.lexsort((cols, pos, tiles))
    probes = np.zeros(ncols, dtype=_capi.PROBE_DTYPE)
    probes["cell"] = cells[o]
    probes["pos"] = pos[o]
    probes["col"] = cols[o]
    tile_start = np.searchsorted(tiles[o], np.arange(geo.ntiles + 1)).astype(np.int32)
    return {"tile_start": tile_start, "probes": probes}, ncols


def output_column_slices(outputs):
    """(output, first column, number of points) of every output, in order."""
    res = []
    c = 0
    for o in outputs:
        k = int(np.asarray(o.region.indices).reshape(-1).size)
        res.append((o, c, k))
        c += k
    return res
