"""Shared test helpers: build pyfds_gb300 fields from oracle scenario specs, compare
results, and a NumPy model of the tile kernel that runs on the compiled tables."""
import numpy as np

from pyfds_gb300 import _capi, _tables, workloads


def build_field(spec, **kwargs):
    """A pyfds_gb300 field equivalent to the scenario ``spec``."""
    return workloads.build_field(spec, **kwargs)


def field_results(f):
    """(state, signals) of a field in the oracle's format."""
    from oracle.fds_oracle import components_of
    kind = type(f).__name__
    state = {c: np.array(getattr(f, c).values, dtype=np.float64) for c in components_of(kind)}
    sig = {}
    for c in components_of(kind):
        comp = getattr(f, c)
        sig[c] = [np.array(o.signals, dtype=np.float64).reshape(
            len(np.asarray(o.region.indices).reshape(-1)), -1) for o in comp.outputs]
    return state, sig


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    if nb == 0:
        return 0.0 if np.linalg.norm(a) == 0 else np.inf
    return float(np.linalg.norm(a - b) / nb)


def max_rel_l2_signals(sig_a, sig_b):
    """Largest per-point relative L2 error over every recorded output signal."""
    worst = 0.0
    for c in sig_b:
        for A, B in zip(sig_a[c], sig_b[c]):
            assert A.shape == B.shape, (c, A.shape, B.shape)
            for k in range(B.shape[0]):
                worst = max(worst, rel_l2(A[k], B[k]))
    return worst


# --------------------------------------------------------------------------------------
# NumPy model of stag_step_kernel (exact arithmetic), driven by the compiled tables
# --------------------------------------------------------------------------------------

class KernelModel:
    """Runs a field through the same per-tile algorithm and tables as the CUDA kernel
    (pyfds_gb300/csrc/stag_kernel.cuh), with reference-order float64 arithmetic.

    A tile shape other than the kernel's may be given to exercise the bucketing
    of boundary and probe tables on small grids."""

    def __init__(self, field, tile=None, two_step=False):
        f = field
        if not f.matrices_assembled:
            f.assemble_matrices()
        self.f = f
        flags = f._stag_flags()
        self.has_v = bool(flags & _capi.FLAG_HAS_V)
        self.absorb = bool(flags & _capi.FLAG_ABSORB)
        self.axi = bool(flags & _capi.FLAG_AXI)
        self.memory = f._stag_family == _capi.FAMILY_ACOUSTIC
        # two steps per tile (layout 2): lossless 2-D only, as in the kernel
        self.two_step = bool(two_step)
        assert not self.two_step or (self.has_v and not self.absorb)
        tx, ty = tile if tile else (_capi.tile_shape(f._stag_family, 0, flags, f._nx, f._ny))
        self.geo = _tables.TileGeometry(f._nx, f._ny, tx, ty, self.has_v,
                                        layout=2 if self.two_step else 0)
        c = dict(f._stag_coefs)
        n = f.num_points
        z = np.zeros(n)
        self.c = {k: (c[k] if c.get(k) is not None else None) for k in c}
        if self.c.get("by") is None:
            self.c["by"] = self.c["bx"]
        if self.c.get("ky") is None:
            self.c["ky"] = self.c["kx"]
        for k in ("aym", "axm", "ad", "axp", "ayp", "ex"):
            if self.c.get(k) is None:
                self.c[k] = z

    def run(self, nsteps, step0=0):
        f, geo = self.f, self.geo
        n = f.num_points
        comps = f._stag_components
        st = [np.array(getattr(f, c).values, dtype=np.float64).copy() for c in comps]
        while len(st) < 3:
            st.append(np.zeros(n))
        pool = _tables.SignalPool()
        tabs = []
        for k, name in enumerate(comps):
            comp = getattr(f, name)
            bt = _tables.compile_bounds(comp.boundaries, n, pool, step0 + nsteps, geo, k)
            pt, ncols = _tables.compile_probes(comp.outputs, n, geo)
            tabs.append((bt, pt, ncols))
        while len(tabs) < 3:
            tabs.append((None, None, 0))
        poolv = pool.array()
        outs = [np.full((nsteps, max(t[2], 1)), np.nan) for t in tabs]

        def opval(op, step):
            return poolv[op["off"] + step * op["stride"]] if op["flags"] & _capi.BOP_SIGNAL \
                else op["scalar"]

        def apply_groups(bt, tile, s, step):
            if bt is None:
                return
            for g in bt["groups"][bt["tile_start"][tile]:bt["tile_start"][tile + 1]]:
                v = s[g["pos"]]
                for op in bt["ops"][g["op_begin"]:g["op_end"]]:
                    v = op["mul"] * v + opval(op, step)
                s[g["pos"]] = v

        def probes(pt, tile, s, out, row):
            if pt is None or row >= out.shape[0]:
                return
            for q in pt["probes"][pt["tile_start"][tile]:pt["tile_start"][tile + 1]]:
                out[row, q["col"]] = s[q["pos"]]

        # prologue
        bt0, pt0, _ = tabs[0]
        if bt0 is not None:
            for g in bt0["groups"]:
                if not g["primary"]:
                    continue
                v = st[0][g["cell"]]
                for op in bt0["ops"][g["op_begin"]:g["op_end"]]:
                    v = op["mul"] * v + opval(op, step0)
                st[0][g["cell"]] = v
        if pt0 is not None:
            for q in pt0["probes"]:
                outs[0][0, q["col"]] = st[0][q["cell"]]

        RX = geo.rx
        OY = geo.oy
        RY = geo.ty + OY + 2 if self.has_v else geo.ty
        nx = geo.nx
        c = self.c

        def g0(a, i):
            return a[i] if 0 <= i < n else 0.0

        def fluxnew(is_x, pos, i, x, sF, sP):
            back = 1 if is_x else RX
            ib = i - (1 if is_x else nx)
            bc = c["bx"] if is_x else c["by"]
            t = (-(g0(bc, ib) * sP[pos - back])) + bc[i] * sP[pos]
            if not self.memory:
                return -t
            u = sF[pos]
            r = t
            if self.absorb:
                acc = 0.0
                if self.has_v:
                    acc = acc + g0(c["aym"], i - nx) * sF[pos - RX]
                acc = acc + g0(c["axm"], i - 1) * sF[pos - 1]
                acc = acc + c["ad"][i] * sF[pos]
                acc = acc + g0(c["axp"], i + 1) * sF[pos + 1]
                if self.has_v:
                    acc = acc + g0(c["ayp"], i + nx) * sF[pos + RX]
                r = r - acc
            if self.axi and self.absorb and is_x:
                rad = c["rx"][x]
                r = r + (c["ex"][i] * u) / (rad * rad)
            return u - r

        def potnew(pos, i, x, sP, sU, sV):
            w, wn = sU[pos], sU[pos + 1]
            if self.axi and f.exact:
                xn = 0 if x + 1 == nx else x + 1
                w, wn = w * c["rx"][x], wn * c["rx"][xn]
            sx = (-(c["kx"][i] * w)) + g0(c["kx"], i + 1) * wn
            if self.has_v:
                sy = (-(c["ky"][i] * sV[pos])) + g0(c["ky"], i + nx) * sV[pos + RX]
                sx = sx + sy
            return sP[pos] - sx

        def ring_step(tile, x0, y0, sP, sU, sV, step, row):
            """Step `step` on the ring one cell around the tile (first of two)."""
            for ly in range(-1, geo.ty + 1):
                for lx in range(-1, geo.tx + 2):
                    i = (y0 + ly) * nx + x0 + lx
                    if 0 <= i < n:
                        pos = (ly + OY) * RX + lx + geo.ox
                        sU[pos] = fluxnew(True, pos, i, 0, sU, sP)
            for ly in range(-1, geo.ty + 2):
                for lx in range(-1, geo.tx + 1):
                    i = (y0 + ly) * nx + x0 + lx
                    if 0 <= i < n:
                        pos = (ly + OY) * RX + lx + geo.ox
                        sV[pos] = fluxnew(False, pos, i, 0, sV, sP)
            apply_groups(tabs[1][0], tile, sU, step)
            apply_groups(tabs[2][0], tile, sV, step)
            probes(tabs[1][1], tile, sU, outs[1], row)
            probes(tabs[2][1], tile, sV, outs[2], row)
            for ly in range(-1, geo.ty + 1):
                for lx in range(-1, geo.tx + 1):
                    i = (y0 + ly) * nx + x0 + lx
                    if 0 <= i < n:
                        pos = (ly + OY) * RX + lx + geo.ox
                        sP[pos] = potnew(pos, i, i % nx, sP, sU, sV)
            apply_groups(tabs[0][0], tile, sP, step + 1)
            probes(tabs[0][1], tile, sP, outs[0], row + 1)

        def tile_step(tile, x0, y0, x1, y1, sP, sU, sV, step, row, apply_next, new):
            """One step on the tile (the one-step kernel's compute_tile); stores."""
            uN = {}
            for ly in range(geo.ty):
                for lx in range(geo.tx + 1):
                    x, y = x0 + lx, y0 + ly
                    i = y * nx + x
                    pos = (ly + OY) * RX + lx + geo.ox
                    val = 0.0
                    if x <= x1 and y < y1 and i < n:
                        val = fluxnew(True, pos, i, 0 if x == nx else x, sU, sP)
                    uN[pos] = val
            vN = {}
            if self.has_v:
                for ly in range(geo.ty + 1):
                    for lx in range(geo.tx):
                        x, y = x0 + lx, y0 + ly
                        i = y * nx + x
                        pos = (ly + OY) * RX + lx + geo.ox
                        val = 0.0
                        if x < x1 and y <= y1 and i < n:
                            val = fluxnew(False, pos, i, x, sV, sP)
                        vN[pos] = val
            for pos, v in uN.items():
                sU[pos] = v
            for pos, v in vN.items():
                sV[pos] = v
            apply_groups(tabs[1][0], tile, sU, step)
            if self.has_v:
                apply_groups(tabs[2][0], tile, sV, step)
            probes(tabs[1][1], tile, sU, outs[1], row)
            if self.has_v:
                probes(tabs[2][1], tile, sV, outs[2], row)
            pN = {}
            for ly in range(geo.ty):
                for lx in range(geo.tx):
                    x, y = x0 + lx, y0 + ly
                    if x >= x1 or y >= y1:
                        continue
                    i = y * nx + x
                    pos = (ly + OY) * RX + lx + geo.ox
                    new[1][i] = sU[pos]
                    if self.has_v:
                        new[2][i] = sV[pos]
                    pN[pos] = potnew(pos, i, x, sP, sU, sV)
            for pos, v in pN.items():
                sP[pos] = v
            if apply_next:
                apply_groups(tabs[0][0], tile, sP, step + 1)
                probes(tabs[0][1], tile, sP, outs[0], row + 1)
            for ly in range(geo.ty):
                for lx in range(geo.tx):
                    x, y = x0 + lx, y0 + ly
                    if x < x1 and y < y1:
                        new[0][y * nx + x] = sP[(ly + OY) * RX + lx + geo.ox]

        s = 0
        while s < nsteps:
            take = 2 if (self.two_step and s + 1 < nsteps) else 1
            step = step0 + s
            new = [x.copy() for x in st]
            for tile in range(geo.ntiles):
                ttx, tty = tile % geo.tiles_x, tile // geo.tiles_x
                x0, y0 = ttx * geo.tx, tty * geo.ty
                x1, y1 = min(x0 + geo.tx, nx), min(y0 + geo.ty, geo.ny)
                flat = np.zeros(RX * RY, dtype=np.int64)
                for e in range(RX * RY):
                    flat[e] = (y0 + e // RX - OY) * nx + x0 + e % RX - geo.ox
                ok = (flat >= 0) & (flat < n)
                sP = np.where(ok, st[0][np.clip(flat, 0, n - 1)], 0.0)
                sU = np.where(ok, st[1][np.clip(flat, 0, n - 1)], 0.0) if self.memory \
                    else np.zeros(RX * RY)
                sV = np.where(ok, st[2][np.clip(flat, 0, n - 1)], 0.0) if self.memory \
                    else np.zeros(RX * RY)
                if take == 2:
                    ring_step(tile, x0, y0, sP, sU, sV, step, s)
                    tile_step(tile, x0, y0, x1, y1, sP, sU, sV, step + 1, s + 1,
                              s + 2 < nsteps, new)
                else:
                    tile_step(tile, x0, y0, x1, y1, sP, sU, sV, step, s, s + 1 < nsteps, new)
            st = new
            s += take
        state = {name: st[k] for k, name in enumerate(comps)}
        sig = {}
        for k, name in enumerate(comps):
            comp = getattr(f, name)
            sig[name] = []
            for o, c0, npts in _tables.output_column_slices(comp.outputs):
                sig[name].append(outs[k][:, c0:c0 + npts].T.copy())
        return state, sig
