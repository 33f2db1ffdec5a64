"""In-tree build of libsep.so: the sep C API (C99 host layer) over the CUDA
kernels, for sm_103a only.

    python -m seplib_gb300.build          # or seplib_gb300.build.build()

Objects go to seplib_gb300/lib/obj, the library to seplib_gb300/lib/libsep.so.
Translation units compile in parallel; a unit is rebuilt when its source or
any header it may include is newer than its object.
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIB = os.path.join(LIBDIR, "libsep.so")
E2E = os.path.join(LIBDIR, "sep_e2e_loop")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
CC = os.environ.get("CC", "gcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
           "-I", INC, "-I", CSRC] + ARCH
CFLAGS = ["-std=c99", "-O2", "-fPIC", "-Wall", "-Wno-unused-function", "-D_GNU_SOURCE",
          "-I", INC, "-I", CSRC, "-I", "/usr/local/cuda/include"]


def _headers():
    return (glob.glob(os.path.join(INC, "*.h")) + glob.glob(os.path.join(CSRC, "*.h")) +
            glob.glob(os.path.join(CSRC, "*", "*.h")) + glob.glob(os.path.join(CSRC, "*", "*.cuh")))


def _stale(src, obj, newest_header):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or newest_header > t


def _compile(job):
    cmd, src = job
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (src, r.stdout, r.stderr))
    return src, r.stderr


def build(verbose=False, jobs=None):
    """Compile every translation unit that changed and link libsep.so."""
    os.makedirs(OBJDIR, exist_ok=True)
    hdr = max([os.path.getmtime(h) for h in _headers()] + [0])
    cu = sorted(glob.glob(os.path.join(CSRC, "cuda", "*.cu")))
    cs = sorted(glob.glob(os.path.join(CSRC, "host", "*.c")))
    objs, todo = [], []
    for src in cu:
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(src, obj, hdr):
            todo.append(([NVCC] + NVFLAGS + ["-c", src, "-o", obj], src))
    for src in cs:
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(src, obj, hdr):
            todo.append(([CC] + CFLAGS + ["-c", src, "-o", obj], src))
    if todo:
        with ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for src, log in ex.map(_compile, todo):
                if verbose and log.strip():
                    print(os.path.basename(src), log, file=sys.stderr)
    newest = max(os.path.getmtime(o) for o in objs)
    if todo or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [NVCC, "-shared", "-o", LIB] + objs + ARCH + ["-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed\n%s\n%s" % (r.stdout, r.stderr))
    # the prgs-style loop driver that times the C API end to end
    src = os.path.join(CSRC, "driver", "e2e_loop.c")
    if not os.path.exists(E2E) or os.path.getmtime(E2E) < max(os.path.getmtime(LIB), os.path.getmtime(src)):
        cmd = [CC, "-std=c99", "-O2", "-Wall", "-I", INC, src, "-o", E2E, "-L", LIBDIR,
               "-Wl,-rpath," + LIBDIR, "-lsep", "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("driver build failed\n%s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
