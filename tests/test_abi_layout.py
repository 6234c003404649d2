"""The C ABI's records as a C compiler lays them out: every struct of include/*.h,
compiled with the host C compiler, has the size and field offsets of its ctypes or
numpy mirror in pyfds_gb300/_capi.py, and the headers compile as strict C99 and
C++11 (what a cgo, JNI or ctypes binding would include). No GPU is used."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from pyfds_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")

STRUCTS = [_capi.FdsCoefs, _capi.FdsStagProblem, _capi.FdsStagState, _capi.FdsCompTables,
           _capi.FdsStagTables, _capi.FdsNl1dProblem, _capi.FdsConvArgs, _capi.FdsWgradArgs,
           _capi.FdsAdamArgs, _capi.FdsSurrData]
RECORDS = {"FdsBoundOp": _capi.BOUND_OP_DTYPE, "FdsBoundGroup": _capi.BOUND_GROUP_DTYPE,
           "FdsProbe": _capi.PROBE_DTYPE, "FdsGatherItem": _capi.GATHER_ITEM_DTYPE}

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None, reason="needs a host C compiler")


def _expected():
    """(struct, field or '', size or offset) from the Python mirrors."""
    rows = []
    for s in STRUCTS:
        rows.append((s.__name__, "", C.sizeof(s)))
        for name, _ in s._fields_:
            rows.append((s.__name__, name, getattr(s, name).offset))
    for sname, dt in RECORDS.items():
        rows.append((sname, "", dt.itemsize))
        for name in dt.names:
            rows.append((sname, name, dt.fields[name][1]))
    return rows


def _probe_source(rows):
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "fds_capi.h"',
             '#include "fds_surrogate.h"', "int main(void) {"]
    for sname, field, _ in rows:
        expr = "offsetof(%s, %s)" % (sname, field) if field else "sizeof(%s)" % sname
        lines.append('  printf("%s %s %%zu\\n", (size_t)%s);' % (sname, field or "-", expr))
    lines += ["  return 0;", "}"]
    return "\n".join(lines) + "\n"


def test_struct_layouts_as_compiled(tmp_path):
    rows = _expected()
    src = tmp_path / "layout.c"
    exe = tmp_path / "layout"
    src.write_text(_probe_source(rows))
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I" + INCLUDE, str(src), "-o",
                    str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            sname, field, value = line.split()
            got[(sname, "" if field == "-" else field)] = int(value)
    bad = [(s, f, v, got.get((s, f))) for s, f, v in rows if got.get((s, f)) != v]
    assert not bad, bad


def test_every_header_struct_has_a_mirror():
    import re
    names = set()
    for h in ("fds_capi.h", "fds_surrogate.h"):
        names |= set(re.findall(r"typedef struct (Fds\w+) \{", open(os.path.join(INCLUDE, h)).read()))
    mirrored = {s.__name__ for s in STRUCTS} | set(RECORDS)
    assert names == mirrored, (names - mirrored, mirrored - names)


@pytest.mark.parametrize("compiler,std,ext", [("gcc", "c99", "c"), ("g++", "c++11", "cpp")])
def test_headers_compile_strictly(tmp_path, compiler, std, ext):
    if shutil.which(compiler) is None:
        pytest.skip("needs " + compiler)
    src = tmp_path / ("h." + ext)
    src.write_text('#include "fds_capi.h"\n#include "fds_surrogate.h"\nint main(void) { return 0; }\n')
    r = subprocess.run([compiler, "-std=" + std, "-Wall", "-Wextra", "-pedantic", "-Werror",
                        "-I" + INCLUDE, "-fsyntax-only", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
