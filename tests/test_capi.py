"""The C-ABI library: loads without a GPU, exports every function include/*.h
declares, its structs match the header's layout, argument errors come back as
status codes with a message (no GPU work is issued by these calls)."""
import ctypes as C
import glob
import os
import re

import pytest

from pyfds_gb300 import _build, _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _capi.load()


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*[a-zA-Z_][\w\s\*]*?\b(fds_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert "fds_stag_run" in names and len(names) >= 4
    for n in names:
        assert hasattr(lib, n), n
    assert set(_capi.EXPORTED_SYMBOLS) <= set(names)


def test_abi_version(lib):
    assert lib.fds_abi_version() == _capi.FDS_ABI_VERSION


def test_struct_layouts_match_header():
    assert C.sizeof(_capi.FdsCoefs) == 11 * 8
    assert C.sizeof(_capi.FdsStagProblem) == 8 * 4 + 11 * 8 + 8 + 8 + 8
    assert C.sizeof(_capi.FdsStagState) == 6 * 8
    assert C.sizeof(_capi.FdsCompTables) == 6 * 8 + 8
    assert C.sizeof(_capi.FdsStagTables) == 3 * 56 + 40
    assert _capi.BOUND_OP_DTYPE.itemsize == 32
    assert _capi.BOUND_GROUP_DTYPE.itemsize == 24
    assert _capi.PROBE_DTYPE.itemsize == 16


def test_tile_shapes(lib):
    assert _capi.tile_shape(0, 0, _capi.FLAG_HAS_V, 100, 100) == (64, 16)
    assert _capi.tile_shape(0, 0, 0, 1000, 1) == (1024, 1)
    dw = _capi.PREC_DW
    assert _capi.tile_shape(0, dw, _capi.FLAG_HAS_V, 100, 100) == (64, 12)
    assert _capi.tile_shape(1, dw, _capi.FLAG_HAS_V | _capi.FLAG_AXI, 100, 100) == (64, 12)
    assert _capi.tile_shape(0, dw, _capi.FLAG_HAS_V | _capi.FLAG_ABSORB, 100, 100) == (64, 16)
    assert _capi.tile_shape(0, dw, 0, 1000, 1) == (1024, 1)


def test_argument_errors_are_reported(lib):
    st = _capi.FdsStagState()
    tb = _capi.FdsStagTables()
    pr = _capi.FdsStagProblem()
    assert lib.fds_stag_run(None, C.byref(st), C.byref(tb), 0, 1, 1, None) == _capi.FDS_E_ARG
    assert "null" in _capi.last_error()
    pr.nx, pr.ny = 0, 1
    assert lib.fds_stag_run(C.byref(pr), C.byref(st), C.byref(tb), 0, 1, 1, None) == _capi.FDS_E_ARG
    assert "bad grid" in _capi.last_error()
    pr.nx, pr.ny, pr.flags = 8, 4, 0
    pr.tile_x, pr.tile_y = 1024, 1
    assert lib.fds_stag_run(C.byref(pr), C.byref(st), C.byref(tb), 0, 1, 1, None) == _capi.FDS_E_ARG
    assert "1-D field" in _capi.last_error()
    pr.flags = _capi.FLAG_HAS_V
    pr.tile_x, pr.tile_y = 64, 16
    assert lib.fds_stag_run(C.byref(pr), C.byref(st), C.byref(tb), 0, 1, 1, None) == _capi.FDS_E_ARG
    assert "coefficient" in _capi.last_error()
    with pytest.raises(_capi.FdsError):
        _capi.check(_capi.FDS_E_ARG)


def test_wavefront_scratch_size_and_checks(lib):
    pr = _capi.FdsStagProblem()
    pr.nx, pr.ny, pr.tile_x, pr.tile_y = 2048, 2048, 64, 16
    assert lib.fds_stag_sync_words(C.byref(pr)) == 1 + 128
    pr.ny = 17
    assert lib.fds_stag_sync_words(C.byref(pr)) == 1 + 2
    pr.ny = 0
    assert lib.fds_stag_sync_words(C.byref(pr)) == _capi.FDS_E_ARG
    assert lib.fds_stag_sync_words(None) == _capi.FDS_E_ARG
    # stages beyond 4 are rejected before any GPU work
    st, tb = _capi.FdsStagState(), _capi.FdsStagTables()
    pr.ny, pr.stages = 16, 5
    assert lib.fds_stag_run(C.byref(pr), C.byref(st), C.byref(tb), 0, 1, 1, None) == _capi.FDS_E_ARG
    assert "stages" in _capi.last_error()


def test_selftest_argument_checks(lib):
    assert lib.fds_selftest_bounded_wait(2, None, None, 10, None) == _capi.FDS_E_ARG
    assert lib.fds_selftest_bounded_wait(0, None, None, 10, None) == _capi.FDS_E_ARG
    assert lib.fds_selftest_bounded_wait(0, C.c_void_p(256), None, 0, None) == _capi.FDS_E_ARG
    assert lib.fds_selftest_bounded_wait(1, C.c_void_p(256), None, 10, None) == _capi.FDS_E_ARG


def test_host_gather_argument_checks(lib):
    """fds_host_gather rejects a negative count or a null table before any GPU work,
    and an empty gather is a no-op."""
    assert lib.fds_host_gather(None, -1, None) == _capi.FDS_E_ARG
    assert lib.fds_host_gather(None, 1, None) == _capi.FDS_E_ARG
    assert lib.fds_host_gather(None, 0, None) == _capi.FDS_OK
    assert _capi.GATHER_ITEM_DTYPE.itemsize == 32
    # without a device the answer is 0 (and the gather is refused), never an error
    assert lib.fds_host_access() in (0, 1)
