"""Device side of a staggered field: PyTorch-owned buffers and the C-ABI call.

A field keeps its reference-style host API (``component.values`` as a float64
numpy array, boundary/output lists); the engine mirrors the state on the GPU,
uploads what the host changed, compiles the boundary/output tables, calls
``fds_stag_run`` and turns the device output buffer back into
``Output.signals`` samples. All device memory is allocated here as torch
tensors; libfdsgpu.so only borrows the pointers.
"""
import ctypes as C
import warnings
import zlib

import numpy as np

from . import _capi
from . import _tables

PRECISIONS = {"f64": _capi.PREC_F64, "f32": _capi.PREC_F32, "f32_t64": _capi.PREC_F32_T64,
              "dw": _capi.PREC_DW}

_ALIGN = 256

# What a diverged field (NaN or infinity in the potential after a call, reported by
# the kernels' status word) does: "raise" FieldDiverged (a FloatingPointError),
# "warn" (RuntimeWarning, as numpy does on invalid values) or "ignore".
NONFINITE_ACTIONS = ("raise", "warn", "ignore")
_nonfinite_action = "raise"


def set_nonfinite_action(action):
    """Choose what a diverged field does: "raise" (default), "warn" or "ignore"."""
    global _nonfinite_action
    if action not in NONFINITE_ACTIONS:
        raise ValueError("action must be one of %s" % (NONFINITE_ACTIONS,))
    _nonfinite_action = action


def split_dw(vals):
    """float64 values -> (n, 2) float32 double words: hi = fl32(x), lo = fl32(x - hi)
    (x - hi is exact in float64), so hi + lo holds 48 bits of x."""
    v = np.ascontiguousarray(vals, dtype=np.float64).reshape(-1)
    hi = v.astype(np.float32)
    lo = (v - hi.astype(np.float64)).astype(np.float32)
    return np.stack([hi, lo], axis=1)


def join_dw(pairs):
    """(n, 2) float32 double words -> float64 values hi + lo."""
    pairs = np.asarray(pairs, dtype=np.float32).reshape(-1, 2)
    return pairs[:, 0].astype(np.float64) + pairs[:, 1].astype(np.float64)


def upload_dw(torch, dev, vals, out=None):
    """Host float64 values -> device (n, 2) float32 double words: the float64 copy
    goes up (8 bytes per value, as the pairs would) and fds_dw_split splits it where
    it lands, with the roundings of split_dw."""
    v = torch.from_numpy(np.ascontiguousarray(vals, dtype=np.float64).reshape(-1)).to(dev)
    if out is None:
        out = torch.empty((v.numel(), 2), dtype=torch.float32, device=dev)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _capi.check(_capi.load().fds_dw_split(C.c_void_p(v.data_ptr()), C.c_void_p(out.data_ptr()),
                                          v.numel(), stream))
    return out


def device_join_dw(torch, pairs):
    """Device (n, 2) float32 double words -> device float64 values (fds_dw_join)."""
    out = torch.empty(pairs.shape[0], dtype=torch.float64, device=pairs.device)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _capi.check(_capi.load().fds_dw_join(C.c_void_p(pairs.data_ptr()), C.c_void_p(out.data_ptr()),
                                         pairs.shape[0], stream))
    return out


def _torch():
    import torch
    return torch


def require_cuda():
    """The time-stepping path runs on the GPU only: fail loudly without one."""
    torch = _torch()
    if not torch.cuda.is_available():
        raise RuntimeError("pyfds_gb300 time stepping needs a CUDA GPU (none is visible); "
                           "there is no CPU fallback")
    _capi.load()
    return torch


class _Blob:
    """Packs host arrays into one device byte buffer (one host-to-device copy)."""

    def __init__(self):
        self.parts = []
        self.size = 0

    def add(self, arr):
        if arr is None:
            return None
        b = np.ascontiguousarray(arr).view(np.uint8).reshape(-1)
        off = self.size
        self.parts.append((off, b))
        self.size = (off + b.size + _ALIGN - 1) // _ALIGN * _ALIGN
        return off

    def upload(self, torch, device):
        host = np.zeros(max(self.size, _ALIGN), dtype=np.uint8)
        for off, b in self.parts:
            host[off:off + b.size] = b
        dev = torch.from_numpy(host).to(device)
        return dev


_PINNED = {"buf": None, "event": None}


_HOST_ACCESS = {}


def _host_access():
    """Whether the current device reads pageable host memory (fds_host_access), per
    device."""
    import torch
    dev = torch.cuda.current_device()
    if dev not in _HOST_ACCESS:
        _HOST_ACCESS[dev] = bool(_capi.load().fds_host_access())
    return _HOST_ACCESS[dev]


class HostUpload:
    """Host arrays bound for many device tensors, sent in few copies.

    ``add`` records (host array, destination tensor); ``flush`` packs the small arrays
    into one pinned staging buffer (kept between calls, grown on demand), copies it to
    the device in one transfer and then fills every destination on the device: a copy
    with the dtype conversion the destination asks for, or for double words the split
    of float64 values into float32 pairs (fds_dw_split). A batch of fields thus pays
    one host-to-device transfer instead of a few per field. Arrays of ``DIRECT_BYTES``
    or more go straight from the caller's memory instead (on the GB300's Grace host a
    pageable copy runs at 125 GB/s, while packing into the staging buffer moves bytes
    at about 20 GB/s): where the device reads pageable host memory (fds_host_access)
    the float64 ones in one gather kernel that converts as it writes
    (fds_host_gather), else one copy each."""

    DIRECT_BYTES = 1 << 20

    def __init__(self, torch, device):
        self.torch, self.device = torch, device
        self.items = []
        self.size = 0

    def add(self, host, dst, dword=False):
        b = np.ascontiguousarray(host)
        off = self.size
        self.items.append((off, b, dst, dword))
        self.size = (off + b.nbytes + _ALIGN - 1) // _ALIGN * _ALIGN
        return dst

    def flush(self):
        torch = self.torch
        if not self.items:
            return
        lib = _capi.load()
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        dtypes = {np.dtype(np.float64): torch.float64, np.dtype(np.float32): torch.float32,
                  np.dtype(np.uint8): torch.uint8}
        small, direct, convert = [], [], []
        stage_bytes = 0
        for item in self.items:
            off, b, dst, dword = item
            if b.nbytes < self.DIRECT_BYTES or b.dtype not in dtypes or not b.flags.writeable:
                small.append(item)
            elif not dword and dst.dtype == dtypes[b.dtype]:
                direct.append((b, dst, dword, None))
            else:
                direct.append((b, dst, dword, stage_bytes))
                stage_bytes = (stage_bytes + b.nbytes + _ALIGN - 1) // _ALIGN * _ALIGN
        if direct and _host_access():
            # the device reads the float64 arrays where they are, in one kernel that
            # converts as it writes; the stream is synchronised before the arrays (and
            # the item table) may go
            kinds = {torch.float64: _capi.GATHER_F64, torch.float32: _capi.GATHER_F32}
            gather, rest, stage_bytes = [], [], 0
            for b, dst, dword, so in direct:
                kind = _capi.GATHER_DW if dword else kinds.get(dst.dtype)
                if b.dtype == np.float64 and kind is not None and dst.is_contiguous():
                    gather.append((b, dst, kind))
                else:
                    so = None if so is None else stage_bytes
                    if so is not None:
                        stage_bytes = (stage_bytes + b.nbytes + _ALIGN - 1) // _ALIGN * _ALIGN
                    rest.append((b, dst, dword, so))
            if gather:
                table = np.zeros(len(gather), dtype=_capi.GATHER_ITEM_DTYPE)
                for k, (b, dst, kind) in enumerate(gather):
                    table[k] = (b.ctypes.data, dst.data_ptr(), b.size, kind, 0)
                _capi.check(lib.fds_host_gather(C.c_void_p(table.ctypes.data), len(gather),
                                                stream))
                torch.cuda.current_stream().synchronize()
                del table, gather
            direct = rest
        # arrays that the device converts land in one staging buffer first; a copy from
        # pageable memory waits for the stream's earlier work, so all of them go before
        # any conversion is queued
        stage = torch.empty(stage_bytes, dtype=torch.uint8, device=self.device) if stage_bytes else None
        for b, dst, dword, so in direct:
            src = torch.from_numpy(b).view(-1)
            if so is None:
                dst.view(-1).copy_(src)
                continue
            staged = stage[so:so + b.nbytes].view(src.dtype)
            staged.copy_(src)
            convert.append((staged, dst, dword))
        for staged, dst, dword in convert:
            if dword:
                _capi.check(lib.fds_dw_split(C.c_void_p(staged.data_ptr()),
                                             C.c_void_p(dst.data_ptr()), staged.numel(), stream))
            else:
                dst.view(-1).copy_(staged)  # converts to dst's dtype
        size = 0
        packed = []
        for _, b, dst, dword in small:
            packed.append((size, b, dst, dword))
            size = (size + b.nbytes + _ALIGN - 1) // _ALIGN * _ALIGN
        self.items, self.size = packed, size
        if not packed:
            self.items = []
            self.size = 0
            return
        ev = _PINNED["event"]
        if ev is not None:
            ev.synchronize()  # the previous flush's copy has left the pinned buffer
        buf = _PINNED["buf"]
        if buf is None or buf.numel() < self.size:
            buf = torch.empty(max(self.size, 1 << 20), dtype=torch.uint8, pin_memory=True)
            _PINNED["buf"] = buf
        host = buf.numpy()
        for off, b, _, _ in self.items:
            host[off:off + b.nbytes] = b.view(np.uint8).reshape(-1)
        staged = torch.empty(self.size, dtype=torch.uint8, device=self.device)
        staged.copy_(buf[:self.size], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream())
        _PINNED["event"] = ev
        for off, b, dst, dword in self.items:
            src = staged[off:off + b.nbytes]
            if dword:
                _capi.check(lib.fds_dw_split(C.c_void_p(src.data_ptr()),
                                             C.c_void_p(dst.data_ptr()), b.size, stream))
            else:
                dst.view(-1).copy_(src.view(dtypes[b.dtype]))  # converts to dst's dtype
        self.items = []
        self.size = 0


class StagEngine:
    """GPU state, coefficients and tables of one staggered field."""

    def __init__(self, field):
        self.field = field
        self.coef_key = None
        self.coef_tensors = {}
        self.buffers = {}  # component name -> [cur, nxt] tensors
        self.table_cache = None
        self.launches = 0
        self.status = None  # device int32: FDS_STATUS_* bits reported by the kernels
        self.sync = None  # device int32 scratch of the wavefront run (stages 4)
        self.offset = None  # the potential is stored as value - offset (see potential_offset)

    # ------------------------------------------------------------------ dtypes
    def dtypes(self):
        torch = _torch()
        prec = self.field.precision
        if prec == "f64":
            return torch.float64, torch.float64, torch.float64
        if prec in ("f32", "dw"):  # dw: (n, 2) float32 pairs
            return torch.float32, torch.float32, torch.float32
        return torch.float64, torch.float32, torch.float32  # f32_t64: potential in float64

    # ------------------------------------------------------------ coefficients
    def _upload_coefs(self, torch, dev, up=None):
        key = self.field._coef_version
        if key == self.coef_key:
            return
        _, _, tc = self.dtypes()
        self.coef_tensors = {}
        for name, arr in self.field._stag_coefs.items():
            if arr is None:
                continue
            vals = np.ascontiguousarray(arr, dtype=np.float64).reshape(-1)
            if up is not None:
                dword = self.field.precision == "dw"
                dst = torch.empty((vals.size, 2) if dword else (vals.size,),
                                  dtype=torch.float32 if dword else tc, device=dev)
                self.coef_tensors[name] = up.add(vals, dst, dword)
                continue
            if self.field.precision == "dw":
                self.coef_tensors[name] = upload_dw(torch, dev, arr)
                continue
            self.coef_tensors[name] = torch.from_numpy(vals).to(dev).to(tc)
        self.coef_key = key

    def _flow_periods(self, torch, dev):
        """Device copy (int64) of a moving-medium field's per-row shift periods."""
        per = np.ascontiguousarray(self.field._flow_periods(), dtype=np.int64)
        cached = getattr(self, "_flow_cache", None)
        if cached is None or not np.array_equal(cached[0], per):
            self._flow_cache = (per.copy(), torch.from_numpy(per).to(dev))
        return self._flow_cache[1]

    def flow_shift(self, step):
        """The moving-medium shift of ``step`` on the device state (fds_stag_flow_shift)."""
        torch = require_cuda()
        plan = self.prepare(step, 0)
        state = _capi.FdsStagState()
        for k, name in enumerate(self.field._stag_components):
            cur, nxt = self.buffers[name]
            state.cur[k] = cur.data_ptr()
            state.nxt[k] = nxt.data_ptr()
        lib = _capi.load()
        _capi.check(lib.fds_stag_flow_shift(C.byref(plan["prob"]), C.byref(state), int(step),
                                            C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        for name in self.field._stag_components:
            getattr(self.field, name)._where = "device"

    # ------------------------------------------------------------------- state
    def _potential_offset(self):
        """Offset of the stored potential (0 unless below). Float32 thermal fields keep
        T - T_ref, with T_ref the field's ``potential_offset`` or the mean initial
        temperature (the float32 spacing near 0 K of deviation is fine, near 300 K it
        is 2^-15 K). Double-word thermal fields use ``potential_offset`` when it is
        set: it pays when every temperature stays close to it (the 48 bits then
        resolve the deviation), and costs accuracy on cells far from it, so there is
        no automatic choice. The other precisions store the temperature itself."""
        if self.offset is None:
            f = self.field
            off = 0.0
            if f._stag_family == _capi.FAMILY_THERMAL and f.precision in ("f32", "dw"):
                off = getattr(f, "potential_offset", None)
                if off is None:
                    off = 0.0
                    if f.precision == "f32":
                        vals = np.asarray(getattr(f, f._stag_components[0])._values,
                                          dtype=np.float64)
                        off = float(np.mean(vals)) if vals.size else 0.0
            self.offset = float(off)
        return self.offset

    def _sync_state_to_device(self, torch, dev, up=None):
        tp, tf, _ = self.dtypes()
        names = self.field._stag_components
        off = self._potential_offset()
        memory = self.field._stag_family == _capi.FAMILY_ACOUSTIC
        dword = self.field.precision == "dw"
        for k, name in enumerate(names):
            comp = getattr(self.field, name)
            dt = tp if k == 0 else tf
            bufs = self.buffers.get(name)
            n = self.field.num_points
            if bufs is None:
                shape = (n, 2) if dword else (n,)
                cur = torch.empty(shape, dtype=dt, device=dev)
                nxt = torch.empty(shape, dtype=dt, device=dev) if (k == 0 or memory) else cur
                bufs = self.buffers[name] = [cur, nxt]
                comp._attach(self, name)
                comp._where = "host"
            if comp._where == "host":
                vals = np.asarray(comp._values, dtype=np.float64).reshape(-1)
                if vals.size != n:
                    raise ValueError("component %s has %d values, field has %d points"
                                     % (name, vals.size, n))
                if k == 0 and off:
                    vals = vals - off
                if up is not None:
                    up.add(vals, bufs[0], dword)
                elif dword:
                    upload_dw(torch, dev, vals, out=bufs[0])
                else:
                    bufs[0].copy_(torch.from_numpy(np.ascontiguousarray(vals)).to(dev).to(dt))
                comp._where = "both"

    def device_values(self, name):
        """Current values of a component as a float64 device tensor (offset added)."""
        torch = _torch()
        b = self.buffers[name][0]
        if self.field.precision == "dw":
            v = device_join_dw(torch, b)
        else:
            v = b.to(dtype=torch.float64)
        if name == self.field._stag_components[0] and self.offset:
            v = v + self.offset
        return v

    def download(self, name):
        """The component's values as a new float64 host array: read from the device
        into pinned memory (torch's caching host allocator; the array keeps its block)."""
        torch = _torch()
        bufs = self.buffers[name]
        src = device_join_dw(torch, bufs[0]) if self.field.precision == "dw" else bufs[0]
        src = src.detach().reshape(-1).to(torch.float64)
        host = torch.empty(src.numel(), dtype=torch.float64, pin_memory=True)
        host.copy_(src)
        v = host.numpy()
        if name == self.field._stag_components[0] and self.offset:
            v += self.offset
        return v

    # ------------------------------------------------------------------ stages
    # precisions and families where two steps per tile are the faster default
    # (measured on the 2048^2 and axisymmetric steps: float32 +26 %, double words
    # +7 %; double-word thermal fields lose 10 % and keep one step)
    TWO_STEP_AUTO = {("f32", _capi.FAMILY_ACOUSTIC), ("f32", _capi.FAMILY_THERMAL),
                     ("dw", _capi.FAMILY_ACOUSTIC)}

    # precisions and families where every step of a call in one persistent launch
    # (stages 4, the wavefront kernel) is the faster default: float64 acoustic fields,
    # bound by the FP64 pipe, lose the wave tail and ramp of one launch per step
    # (2048^2: 59.7 -> 64.0 Gcell/s; axisymmetric 1024 x 4096: 60.9 -> 65.1); thermal
    # fields are faster with one launch per step (float64 68.6 vs 63.5, double words
    # 95.7 vs 53.1), float32 and double-word acoustic fields with two steps per tile
    WAVE_AUTO = {("f64", _capi.FAMILY_ACOUSTIC)}
    WAVE_TILES = ((64, 16), (64, 12))

    def stages(self, batched=False):
        """FdsStagProblem.stages of the next launch: the field's ``stages`` when set;
        for 0 (automatic) every step in one persistent launch (4) or two steps per
        tile (3) where that is the faster default and the variant has such a kernel
        (lossless 2-D, not exact, no moving medium, a tile with that kernel), else 0.
        Batched runs take the field's 1, 2 or 3 (the autotuner's choice; 4 counts as
        0); for 0 two steps per tile whenever the tile has a two-step kernel
        (measured faster for every precision in the batched kernel: float32 +22 %,
        double words +20 %, float64 +8 %)."""
        f = self.field
        st = int(getattr(f, "stages", 0) or 0)
        if batched and st == 4:
            st = 0
        if st:
            return st
        flags = f._stag_flags()
        lossless_2d = (flags & _capi.FLAG_HAS_V) and not (
            flags & (_capi.FLAG_ABSORB | _capi.FLAG_EXACT | _capi.FLAG_FLOW))
        if not lossless_2d:
            return 0
        tile = self._tile_shape()
        if batched:
            return 3 if f.precision != "f32_t64" and tile in _capi.TWO_STEP_TILES else 0
        if (f.precision, f._stag_family) in self.WAVE_AUTO and tile in self.WAVE_TILES:
            return 4
        if tile in _capi.TWO_STEP_TILES and (f.precision, f._stag_family) in self.TWO_STEP_AUTO:
            return 3
        return 0

    def _tile_shape(self):
        f = self.field
        prec = PRECISIONS[f.precision]
        flags = f._stag_flags()
        tx, ty = _capi.tile_shape(f._stag_family, prec, flags, f._nx, f._ny)
        tile = getattr(f, "tile", None)
        if tile is not None and (flags & _capi.FLAG_HAS_V):
            tx, ty = int(tile[0]), int(tile[1])
        return tx, ty

    # ------------------------------------------------------------------ tables
    def _geometry(self, batched=False):
        f = self.field
        flags = f._stag_flags()
        tx, ty = self._tile_shape()
        layout = _capi.tile_layout(tx, ty) if (flags & _capi.FLAG_HAS_V) else 0
        if self.stages(batched) == 3:
            layout = 2  # two steps per tile
        return _tables.TileGeometry(f._nx, f._ny, tx, ty, (flags & _capi.FLAG_HAS_V) != 0,
                                    layout)

    def _fingerprint(self):
        """What the tables are compiled from: the boundaries (objects, index lists and
        values, with checksums of their contents so that in-place edits count) and the
        outputs' index lists."""
        def crc(a):
            return zlib.crc32(np.ascontiguousarray(a).view(np.uint8).reshape(-1))

        parts = []
        for name in self.field._stag_components:
            comp = getattr(self.field, name)
            bp = []
            for b in comp.boundaries:
                v = b.value
                if np.ndim(v) == 0:
                    vk = float(v)
                elif isinstance(v, np.ndarray):
                    vk = (np.shape(v), str(v.dtype), crc(v))
                else:
                    vk = (len(v), tuple(crc(np.asarray(x, dtype=np.float64)) for x in v))
                idx = np.asarray(b.region.indices)
                bp.append((id(b), id(b.region), id(b.region.indices), crc(idx), id(v), vk,
                           b.additive))
            op = tuple((id(o), id(o.region), id(o.region.indices),
                        crc(np.asarray(o.region.indices))) for o in comp.outputs)
            parts.append((tuple(bp), op))
        return tuple(parts)

    def _compile_tables(self, torch, dev, step_end, geo, up=None):
        f = self.field
        n = f.num_points
        pool = _tables.SignalPool()
        comps = []
        for k, name in enumerate(f._stag_components):
            comp = getattr(f, name)
            bt = _tables.compile_bounds(comp.boundaries, n, pool, step_end, geo, k,
                                        offset=self._potential_offset() if k == 0 else 0.0)
            pt, ncols = _tables.compile_probes(comp.outputs, n, geo)
            comps.append((bt, pt, ncols))
        blob = _Blob()
        offs = []
        for bt, pt, ncols in comps:
            o = {}
            if bt is not None:
                o["bts"] = blob.add(bt["tile_start"])
                o["grp"] = blob.add(bt["groups"])
                o["ops"] = blob.add(bt["ops"])
            if pt is not None:
                o["pts"] = blob.add(pt["tile_start"])
                o["prb"] = blob.add(pt["probes"])
            offs.append(o)
        pool_arr = pool.array()
        pool_off = blob.add(pool_arr)
        if up is not None:
            host = np.zeros(max(blob.size, _ALIGN), dtype=np.uint8)
            for off, b in blob.parts:
                host[off:off + b.size] = b
            dev_blob = up.add(host, torch.empty(host.size, dtype=torch.uint8, device=dev))
        else:
            dev_blob = blob.upload(torch, dev)
        return {"blob": dev_blob, "offs": offs, "ncols": [c[2] for c in comps],
                "pool_off": pool_off, "pool_len": int(pool_arr.size)}

    def _tables_struct(self, tabs, outs, nsteps):
        base = tabs["blob"].data_ptr()
        st = _capi.FdsStagTables()
        for k in range(3):
            ct = st.comp[k]
            if k < len(tabs["offs"]):
                o = tabs["offs"][k]
                if "bts" in o:
                    ct.bound_tile_start = base + o["bts"]
                    ct.groups = base + o["grp"]
                    ct.ops = base + o["ops"]
                if "pts" in o:
                    ct.probe_tile_start = base + o["pts"]
                    ct.probes = base + o["prb"]
                    ct.out = outs[k].data_ptr()
                    ct.ncols = tabs["ncols"][k]
                    ct.out_rows = nsteps
        st.pool = base + tabs["pool_off"]
        st.pool_len = tabs["pool_len"]
        return st

    # --------------------------------------------------------------------- run
    def prepare(self, step0, nsteps, cache_tables=False, batched=False, up=None):
        """Upload what the host changed and compile the tables for steps
        ``step0 .. step0+nsteps-1``; returns a launch plan for ``launch``. With a
        HostUpload ``up`` the host arrays go to the device when the caller flushes
        it (before launching)."""
        torch = require_cuda()
        f = self.field
        dev = torch.device("cuda", torch.cuda.current_device())
        self._upload_coefs(torch, dev, up)
        self._sync_state_to_device(torch, dev, up)
        geo = self._geometry(batched)
        step_end = step0 + nsteps
        if cache_tables:
            # the tables depend on the tiling too (tile shape, slot layout); they serve
            # every call that ends within the signals (a call past them recompiles,
            # which raises the reference's error for a signal that is too short)
            fp = (self._fingerprint(), geo.tx, geo.ty, geo.layout)
            if self.table_cache is not None and self.table_cache[0] == fp and \
                    self.table_cache[2] >= step_end:
                tabs = self.table_cache[1]
            else:
                tabs = self._compile_tables(torch, dev, max(step_end, 1), geo, up)
                covered = [_tables.signal_steps(getattr(f, name).boundaries)
                           for name in f._stag_components]
                covered = [c for c in covered if c is not None]
                self.table_cache = (fp, tabs, max(step_end, min(covered)) if covered
                                    else float("inf"))
        else:
            tabs = self._compile_tables(torch, dev, step_end, geo, up)
        outs = [torch.empty((nsteps, max(nc, 1)), dtype=torch.float64, device=dev)
                if nc else None for nc in tabs["ncols"]]
        prob = _capi.FdsStagProblem()
        prob.family = f._stag_family
        prob.precision = PRECISIONS[f.precision]
        prob.flags = f._stag_flags()
        prob.nx = f._nx
        prob.ny = f._ny
        prob.tile_x = geo.tx
        prob.tile_y = geo.ty
        prob.stages = self.stages(batched)
        prob.offset = self._potential_offset()
        for name in ("bx", "by", "kx", "ky", "aym", "axm", "ad", "axp", "ayp", "ex", "rx"):
            t = self.coef_tensors.get(name)
            setattr(prob.coefs, name, t.data_ptr() if t is not None else None)
        if prob.flags & _capi.FLAG_FLOW:
            prob.flow_period = self._flow_periods(torch, dev).data_ptr()
            prob.flow_period_host = self._flow_cache[0].ctypes.data  # kept by the cache
        if self.status is None:
            self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        tstruct = self._tables_struct(tabs, outs, nsteps)
        tstruct.status = self.status.data_ptr()
        if prob.stages == 4:
            # scratch counters of the wavefront run (zeroed by the library per launch)
            words = int(_capi.load().fds_stag_sync_words(C.byref(prob)))
            if words < 0:
                _capi.check(words)
            if self.sync is None or self.sync.numel() < words:
                self.sync = torch.zeros(words, dtype=torch.int32, device=dev)
            tstruct.sync = self.sync.data_ptr()
            tstruct.sync_words = self.sync.numel()
        return {"prob": prob, "tabs": tabs, "outs": outs, "tstruct": tstruct,
                "step0": int(step0), "nsteps": int(nsteps), "geo": geo}

    def launch(self, plan):
        """Enqueue the steps of a plan on the current stream (no host sync)."""
        torch = _torch()
        lib = _capi.load()
        f = self.field
        names = f._stag_components
        state = _capi.FdsStagState()
        for k in range(3):
            if k < len(names):
                cur, nxt = self.buffers[names[k]]
                state.cur[k] = cur.data_ptr()
                state.nxt[k] = nxt.data_ptr()
        stream = torch.cuda.current_stream().cuda_stream
        store_flux = 1 if f._stag_family == _capi.FAMILY_ACOUSTIC else 0
        code = lib.fds_stag_run(C.byref(plan["prob"]), C.byref(state), C.byref(plan["tstruct"]),
                                plan["step0"], plan["nsteps"], store_flux, C.c_void_p(stream))
        _capi.check(code)
        self.launches += plan["nsteps"]
        # the call swapped cur/nxt as often as it stepped
        for k, name in enumerate(names):
            bufs = self.buffers[name]
            if state.cur[k] != bufs[0].data_ptr():
                bufs.reverse()
            getattr(f, name)._where = "device"
        self._last = plan  # keeps the tables and output buffers alive

    def finish(self, plan, status=None, host_outs=None):
        """Copy the output buffers to the host and append them to Output.signals;
        raise if a kernel reported a failed bounded wait. Returns True when the
        kernels reported a non-finite potential (see ``report_nonfinite``).
        ``status`` / ``host_outs``: the status word and the outputs (one host array
        per component, None where it has no outputs) when the caller already copied
        them to the host, as a batch does for all its fields at once."""
        f = self.field
        st = int(self.status.item()) if status is None else int(status)
        if st:
            self.status.zero_()
        if st & _capi.STATUS_TMA_TIMEOUT:
            raise _capi.FdsError(_capi.FDS_E_TIMEOUT,
                                 "a kernel reported status 0x%x (a bounded wait gave up: TMA "
                                 "copies that did not land, or tiles of the previous step that "
                                 "did not finish); the field state is not valid" % st)
        for k, name in enumerate(f._stag_components):
            out_t = plan["outs"][k]
            if out_t is None:
                continue
            host = out_t.to("cpu").numpy() if host_outs is None else host_outs[k]
            if k == 0 and self.offset:
                host = host + self.offset
            comp = getattr(f, name)
            for out, c0, npts in _tables.output_column_slices(comp.outputs):
                # one contiguous row per point; the reference's lists of float64
                # samples (Python floats: tolist is twice as fast as numpy scalars)
                # are built from it when Output.signals is read
                out._record(np.ascontiguousarray(host[:, c0:c0 + npts].T))
        return bool(st & _capi.STATUS_NONFINITE)

    def report_nonfinite(self, step):
        """Act on a diverged field as set_nonfinite_action chose (after the caller
        advanced the field's step to ``step``)."""
        msg = ("%s diverged: its %s holds NaN or infinity after step %d (the time step "
               "exceeds the explicit scheme's stability limit)"
               % (type(self.field).__name__, self.field._stag_components[0], step - 1))
        if _nonfinite_action == "raise":
            raise _capi.FieldDiverged(msg)
        if _nonfinite_action == "warn":
            warnings.warn(msg, RuntimeWarning, stacklevel=3)

    def run(self, step0, nsteps, cache_tables=False):
        """Advance the field by ``nsteps`` steps starting at global step ``step0``;
        True when the potential came out non-finite (the caller reports it with
        ``report_nonfinite`` once its step counter is advanced)."""
        if nsteps <= 0:
            return False
        plan = self.prepare(step0, nsteps, cache_tables)
        self.launch(plan)
        return self.finish(plan)
