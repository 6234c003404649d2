"""ctypes binding of libfdsgpu.so (declared in include/fds_capi.h).

The structures below mirror the C declarations field for field; numpy structured
dtypes mirror the table records so that host-built tables can be uploaded as raw
bytes. Loading fails loudly when the library has not been built: there is no
CPU fallback for the time-stepping path.
"""
import ctypes as C
import os

import numpy as np

from ._build import LIB_PATH

FDS_ABI_VERSION = 5

FDS_OK = 0
FDS_E_ARG = -1
FDS_E_LAUNCH = -2
FDS_E_NOKERNEL = -3
FDS_E_TIMEOUT = -4
FDS_E_SIZE = -5

FAMILY_ACOUSTIC = 0
FAMILY_THERMAL = 1

PREC_F64 = 0
PREC_F32 = 1
PREC_F32_T64 = 2
PREC_DW = 3

# tiles built for two steps per tile (FdsStagProblem.stages = 3; FDS_TB2_MENU in
# csrc/fds_internal.h)
TWO_STEP_TILES = ((64, 16), (64, 12), (64, 8), (32, 32))

FLAG_HAS_V = 1
FLAG_ABSORB = 2
FLAG_AXI = 4
FLAG_EXACT = 8
FLAG_FLOW = 16

NL1D_IDEAL_GAS = 0
NL1D_SECOND_ORDER = 1
NL1D_CONVECTIVE = 1
NL1D_NL_STATE = 2

BOP_SIGNAL = 2

# exported symbols, in header order
EXPORTED_SYMBOLS = ("fds_abi_version", "fds_last_error", "fds_stag_tile_shape",
                    "fds_stag_tile_menu", "fds_stag_run", "fds_stag_sync_words",
                    "fds_stag_batch_workspace_bytes",
                    "fds_stag_batch_run", "fds_selftest_bounded_wait", "fds_stag_batch_run_static",
                    "fds_stag_flow_shift",
                    "fds_nl1d_run", "fds_thermoacoustic_run", "fds_dw_split", "fds_dw_join",
                    "fds_host_access", "fds_host_gather",
                    # include/fds_surrogate.h
                    "fds_conv3x3", "fds_conv_packed_elems", "fds_conv_pack", "fds_conv3x3_wgrad",
                    "fds_conv_wgrad_max_grid", "fds_adamw", "fds_surr_pack", "fds_surr_loss",
                    "fds_surr_loss_parts", "fds_surr_unpack", "fds_surr_compare")

CONV_FWD_GELU = 0
CONV_FWD_LINEAR = 1
CONV_BWD_DATA = 2
SURR_STATUS_TIMEOUT = 1
SURR_STATUS_ALIGN = 2


class FdsCoefs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in
                ("bx", "by", "kx", "ky", "aym", "axm", "ad", "axp", "ayp", "ex", "rx")]


class FdsStagProblem(C.Structure):
    _fields_ = [("family", C.c_int32), ("precision", C.c_int32), ("flags", C.c_uint32),
                ("nx", C.c_int32), ("ny", C.c_int32), ("tile_x", C.c_int32),
                ("tile_y", C.c_int32), ("stages", C.c_int32), ("coefs", FdsCoefs),
                ("offset", C.c_double), ("flow_period", C.c_void_p),
                ("flow_period_host", C.c_void_p)]


class FdsStagState(C.Structure):
    _fields_ = [("cur", C.c_void_p * 3), ("nxt", C.c_void_p * 3)]


class FdsCompTables(C.Structure):
    _fields_ = [("bound_tile_start", C.c_void_p), ("groups", C.c_void_p), ("ops", C.c_void_p),
                ("probe_tile_start", C.c_void_p), ("probes", C.c_void_p), ("out", C.c_void_p),
                ("ncols", C.c_int32), ("out_rows", C.c_int32)]


class FdsStagTables(C.Structure):
    _fields_ = [("comp", FdsCompTables * 3), ("pool", C.c_void_p), ("pool_len", C.c_int64),
                ("status", C.c_void_p), ("sync", C.c_void_p), ("sync_words", C.c_int64)]


STATUS_TMA_TIMEOUT = 1
STATUS_NONFINITE = 2

BATCH_UPLOAD = 1
BATCH_LAUNCH = 2
BATCH_STATIC_MAX_BYTES = 8 << 20


# numpy mirrors of the table records (sizes asserted against the header's comments)
BOUND_OP_DTYPE = np.dtype([("scalar", "<f8"), ("mul", "<f8"), ("off", "<i8"),
                           ("stride", "<i4"), ("flags", "<i4")], align=True)
BOUND_GROUP_DTYPE = np.dtype([("cell", "<i8"), ("pos", "<i4"), ("op_begin", "<i4"),
                              ("op_end", "<i4"), ("primary", "<i4")], align=True)
PROBE_DTYPE = np.dtype([("cell", "<i8"), ("pos", "<i4"), ("col", "<i4")], align=True)
GATHER_ITEM_DTYPE = np.dtype([("src", "<u8"), ("dst", "<u8"), ("n", "<i8"), ("kind", "<i4"),
                              ("pad", "<i4")], align=True)
GATHER_F64, GATHER_F32, GATHER_DW = 0, 1, 2
assert GATHER_ITEM_DTYPE.itemsize == 32
assert BOUND_OP_DTYPE.itemsize == 32
assert BOUND_GROUP_DTYPE.itemsize == 24
assert PROBE_DTYPE.itemsize == 16


class FdsNl1dProblem(C.Structure):
    _fields_ = [("kind", C.c_int32), ("flags", C.c_uint32), ("n", C.c_int32),
                ("tile_x", C.c_int32), ("f1", C.c_double), ("fc", C.c_double),
                ("a", C.c_void_p), ("rho0", C.c_void_p), ("e1", C.c_void_p), ("e2", C.c_void_p),
                ("sync", C.c_void_p), ("status", C.c_void_p)]


class FdsConvArgs(C.Structure):
    _fields_ = [("batch", C.c_int32), ("height", C.c_int32), ("width", C.c_int32),
                ("cin", C.c_int32), ("cout", C.c_int32), ("dilation", C.c_int32),
                ("mode", C.c_int32), ("reserved", C.c_int32),
                ("x", C.c_void_p), ("weight", C.c_void_p), ("bias", C.c_void_p),
                ("resid", C.c_void_p), ("zin", C.c_void_p), ("out_z", C.c_void_p),
                ("out_h", C.c_void_p), ("out_f32", C.c_void_p), ("status", C.c_void_p)]


class FdsWgradArgs(C.Structure):
    _fields_ = [("batch", C.c_int32), ("height", C.c_int32), ("width", C.c_int32),
                ("cin", C.c_int32), ("cout", C.c_int32), ("dilation", C.c_int32),
                ("x", C.c_void_p), ("dz", C.c_void_p), ("partial", C.c_void_p),
                ("grid", C.c_int32), ("reserved", C.c_int32), ("status", C.c_void_p)]


class FdsAdamArgs(C.Structure):
    _fields_ = [("cin", C.c_int32), ("cout", C.c_int32), ("nparts", C.c_int32),
                ("step", C.c_int32), ("lr", C.c_float), ("beta1", C.c_float),
                ("beta2", C.c_float), ("eps", C.c_float), ("weight_decay", C.c_float),
                ("grad_scale", C.c_float), ("partial", C.c_void_p), ("weight", C.c_void_p),
                ("bias", C.c_void_p), ("m", C.c_void_p), ("v", C.c_void_p),
                ("wfwd", C.c_void_p), ("wbwd", C.c_void_p), ("grad_out", C.c_void_p)]


class FdsSurrData(C.Structure):
    _fields_ = [("count", C.c_int32), ("height", C.c_int32), ("width", C.c_int32),
                ("state_f64", C.c_int32), ("nsnap", C.c_int32), ("edge_zero_p", C.c_int32),
                ("inst", C.c_void_p), ("snap", C.c_void_p), ("state", C.c_void_p),
                ("media", C.c_void_p), ("freq", C.c_void_p), ("zref", C.c_void_p),
                ("scale", C.c_void_p), ("x", C.c_void_p), ("s", C.c_void_p), ("t", C.c_void_p)]


class FdsError(RuntimeError):
    """A libfdsgpu.so call failed; carries the library's status code."""

    def __init__(self, code, message):
        super().__init__("libfdsgpu error %d: %s" % (code, message))
        self.code = code


class FieldDiverged(FloatingPointError):
    """The potential after a ``simulate()`` call holds NaN or infinity: the time step
    exceeds the explicit scheme's stability limit (the reference's ``is_stable()``,
    pyfds/acoustics.py:54-63, would have said so). Raised after the call's outputs
    are recorded and the field's step advanced, so the state can be inspected."""


_lib = None


def library_path():
    return LIB_PATH


def load(path=None):
    """Load (once) and return the CDLL. Raises RuntimeError if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(
            "libfdsgpu.so is not built (%s); run `python -m pyfds_gb300._build`" % path)
    lib = C.CDLL(path)
    lib.fds_abi_version.restype = C.c_int32
    lib.fds_abi_version.argtypes = []
    lib.fds_last_error.restype = C.c_int32
    lib.fds_last_error.argtypes = [C.c_char_p, C.c_size_t]
    lib.fds_stag_tile_shape.restype = C.c_int32
    lib.fds_stag_tile_shape.argtypes = [C.c_int32, C.c_int32, C.c_uint32, C.c_int32, C.c_int32,
                                        C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    lib.fds_stag_tile_menu.restype = C.c_int32
    lib.fds_stag_tile_menu.argtypes = [C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                       C.POINTER(C.c_int32), C.c_int32]
    lib.fds_stag_run.restype = C.c_int32
    lib.fds_stag_run.argtypes = [C.POINTER(FdsStagProblem), C.POINTER(FdsStagState),
                                 C.POINTER(FdsStagTables), C.c_int64, C.c_int32, C.c_int32,
                                 C.c_void_p]
    lib.fds_stag_sync_words.restype = C.c_int64
    lib.fds_stag_sync_words.argtypes = [C.POINTER(FdsStagProblem)]
    lib.fds_stag_batch_workspace_bytes.restype = C.c_size_t
    lib.fds_stag_batch_workspace_bytes.argtypes = [C.c_int32, C.c_int64]
    lib.fds_stag_batch_run.restype = C.c_int32
    lib.fds_stag_batch_run.argtypes = [C.POINTER(FdsStagProblem), C.POINTER(FdsStagState),
                                       C.POINTER(FdsStagTables), C.c_int32, C.c_void_p,
                                       C.c_size_t, C.c_int64, C.c_int32, C.c_int32, C.c_uint32,
                                       C.c_void_p]
    lib.fds_selftest_bounded_wait.restype = C.c_int32
    lib.fds_selftest_bounded_wait.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_int64,
                                              C.c_void_p]
    lib.fds_stag_batch_run_static.restype = C.c_int32
    lib.fds_stag_batch_run_static.argtypes = [C.POINTER(FdsStagProblem), C.POINTER(FdsStagState),
                                              C.POINTER(FdsStagTables), C.c_int32, C.c_int64,
                                              C.c_int32, C.c_int32, C.c_void_p]
    lib.fds_thermoacoustic_run.restype = C.c_int32
    lib.fds_thermoacoustic_run.argtypes = [
        C.POINTER(FdsStagProblem), C.POINTER(FdsStagState), C.POINTER(FdsStagTables),
        C.POINTER(FdsStagProblem), C.POINTER(FdsStagState), C.POINTER(FdsStagTables),
        C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int32), C.c_double, C.c_int32,
        C.c_int32, C.c_int64, C.c_int32, C.c_void_p]
    lib.fds_nl1d_run.restype = C.c_int32
    lib.fds_nl1d_run.argtypes = [C.POINTER(FdsNl1dProblem), C.POINTER(FdsStagState),
                                 C.POINTER(FdsStagTables), C.c_int64, C.c_int32, C.c_void_p]
    lib.fds_stag_flow_shift.restype = C.c_int32
    lib.fds_stag_flow_shift.argtypes = [C.POINTER(FdsStagProblem), C.POINTER(FdsStagState),
                                        C.c_int64, C.c_void_p]
    lib.fds_host_access.restype = C.c_int32
    lib.fds_host_access.argtypes = []
    lib.fds_host_gather.restype = C.c_int32
    lib.fds_host_gather.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
    lib.fds_dw_split.restype = C.c_int32
    lib.fds_dw_split.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    lib.fds_dw_join.restype = C.c_int32
    lib.fds_dw_join.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    # include/fds_surrogate.h
    P = C.c_void_p
    lib.fds_conv3x3.restype = C.c_int32
    lib.fds_conv3x3.argtypes = [C.POINTER(FdsConvArgs), P]
    lib.fds_conv_packed_elems.restype = C.c_int64
    lib.fds_conv_packed_elems.argtypes = [C.c_int32, C.c_int32]
    lib.fds_conv_pack.restype = C.c_int32
    lib.fds_conv_pack.argtypes = [C.c_int32, C.c_int32, P, P, P, P]
    lib.fds_conv3x3_wgrad.restype = C.c_int32
    lib.fds_conv3x3_wgrad.argtypes = [C.POINTER(FdsWgradArgs), P]
    lib.fds_conv_wgrad_max_grid.restype = C.c_int32
    lib.fds_conv_wgrad_max_grid.argtypes = []
    lib.fds_adamw.restype = C.c_int32
    lib.fds_adamw.argtypes = [C.POINTER(FdsAdamArgs), P]
    lib.fds_surr_pack.restype = C.c_int32
    lib.fds_surr_pack.argtypes = [C.POINTER(FdsSurrData), P]
    lib.fds_surr_loss.restype = C.c_int32
    lib.fds_surr_loss.argtypes = [C.POINTER(FdsSurrData), P, P, P, P]
    lib.fds_surr_loss_parts.restype = C.c_int32
    lib.fds_surr_loss_parts.argtypes = [C.c_int32, C.c_int32, C.c_int32]
    lib.fds_surr_unpack.restype = C.c_int32
    lib.fds_surr_unpack.argtypes = [C.POINTER(FdsSurrData), P, P]
    lib.fds_surr_compare.restype = C.c_int32
    lib.fds_surr_compare.argtypes = [C.c_int32, C.c_int32, C.c_int32, P, P, P, P, P, P]
    v = lib.fds_abi_version()
    if v != FDS_ABI_VERSION:
        raise RuntimeError("libfdsgpu.so ABI version %d, expected %d (rebuild)" % (v, FDS_ABI_VERSION))
    _lib = lib
    return lib


def last_error():
    lib = load()
    buf = C.create_string_buffer(1024)
    lib.fds_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(code):
    if code != FDS_OK:
        raise FdsError(code, last_error())
    return code


def tile_menu(with_layout=False):
    """Tile shapes (x, y) built for the lossless 2-D variants; with ``with_layout``
    (x, y, layout): 0 = shared-memory tile, 1 = register-marching warp strip."""
    lib = load()
    n = lib.fds_stag_tile_menu(None, None, None, 0)
    xs = (C.c_int32 * n)()
    ys = (C.c_int32 * n)()
    ls = (C.c_int32 * n)()
    lib.fds_stag_tile_menu(xs, ys, ls, n)
    if with_layout:
        return [(xs[k], ys[k], ls[k]) for k in range(n)]
    return [(xs[k], ys[k]) for k in range(n)]


def tile_layout(tx, ty):
    """Slot layout of a tile shape (0 for every shape outside the menu)."""
    for x, y, lay in tile_menu(with_layout=True):
        if (x, y) == (tx, ty):
            return lay
    return 0


def tile_shape(family, precision, flags, nx, ny):
    lib = load()
    tx = C.c_int32()
    ty = C.c_int32()
    check(lib.fds_stag_tile_shape(family, precision, flags, nx, ny, C.byref(tx), C.byref(ty)))
    return tx.value, ty.value
