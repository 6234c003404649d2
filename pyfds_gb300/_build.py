"""Build libfdsgpu.so (the CUDA engine) in-tree for sm_103a with nvcc.

Each ``csrc/*.cu`` translation unit is compiled in parallel and linked into
``pyfds_gb300/_lib/libfdsgpu.so``. A unit is recompiled only when it or a header
is newer than its object file. The CUDA runtime is linked statically, so the
library loads on machines without a GPU driver (the driver is only needed when
a kernel is launched).
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
SRC_DIR = os.path.join(PKG_DIR, "csrc")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
OBJ_DIR = os.path.join(PKG_DIR, "_lib", "obj")
INCLUDE_DIR = os.path.join(os.path.dirname(PKG_DIR), "include")
LIB_PATH = os.path.join(LIB_DIR, "libfdsgpu.so")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
            "-I" + INCLUDE_DIR, "-I" + SRC_DIR]


def _nvcc():
    exe = shutil.which("nvcc")
    if exe is None:
        cand = "/usr/local/cuda/bin/nvcc"
        if os.path.exists(cand):
            return cand
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfdsgpu.so")
    return exe


def _headers():
    return glob.glob(os.path.join(SRC_DIR, "*.cuh")) + glob.glob(os.path.join(SRC_DIR, "*.h")) + \
        glob.glob(os.path.join(INCLUDE_DIR, "*.h"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, jobs=None):
    """Compile and link libfdsgpu.so; returns its path."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = _nvcc()
    sources = sorted(glob.glob(os.path.join(SRC_DIR, "*.cu")))
    headers = _headers()
    objs = []
    todo = []
    for src in sources:
        obj = os.path.join(OBJ_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            todo.append((src, obj))

    def compile_one(item):
        src, obj = item
        cmd = [nvcc] + ARCH_FLAGS + CU_FLAGS + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return src

    if todo:
        n = jobs or min(len(todo), max(1, os.cpu_count() or 1))
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            for src in ex.map(compile_one, todo):
                if verbose:
                    print("compiled", os.path.basename(src))
    if todo or _stale(LIB_PATH, objs):
        cmd = [nvcc] + ARCH_FLAGS + ["-shared", "-o", LIB_PATH] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        if verbose:
            print("linked", LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    build(verbose=True)
