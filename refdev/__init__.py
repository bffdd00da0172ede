"""Device-to-device baseline: the reference's device GatherScatter algorithm
(libs/ogs/okl/ogsKernels.okl:32-81, row blocks of ogsOperator.cpp:447-512)
restated in CUDA (okl_equiv.cu), built for sm_103a into refdev/_build/.

Benchmark and test infrastructure only: the library never calls it.  It runs
on the T maps of a library handle, which equal the reference's maps.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "okl_equiv.cu")
LIB = os.path.join(HERE, "_build", "librefdev.so")

_lib = None


def _cmd():
    nvcc = os.environ.get("NVCC") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc")
                                      else shutil.which("nvcc"))
    return [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-lineinfo",
            "-Xcompiler", "-fPIC", "-shared", "-cudart", "static", "-o", LIB, SRC]


def start_build():
    """Start compiling librefdev.so (if stale); returns a Popen or None."""
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return None
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    return subprocess.Popen(_cmd(), stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)


def finish_build(p):
    if p is None:
        return LIB
    out, _ = p.communicate()
    if p.returncode != 0:
        raise RuntimeError(f"refdev build failed:\n{out}")
    return LIB


def build():
    return finish_build(start_build())


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError("refdev/_build/librefdev.so is missing: run refdev.build()")
        L = C.CDLL(LIB)
        L.refdev_create.argtypes = [C.c_void_p, C.c_int64, C.c_void_p]
        L.refdev_create.restype = C.c_void_p
        L.refdev_nblocks.argtypes = [C.c_void_p]
        L.refdev_nblocks.restype = C.c_int
        L.refdev_gather_scatter.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.refdev_gather_scatter.restype = C.c_int
        L.refdev_free.argtypes = [C.c_void_p]
        L.refdev_free.restype = None
        _lib = L
    return _lib


class RefDevOgs:
    """The reference-device-equivalent GatherScatter (Sym) over a library
    handle's T maps.  gather_scatter(ptr, k, type_code, op_code, stream)."""

    def __init__(self, g):
        import numpy as np
        rsT, ciT, _, _ = g.maps()
        self._rs = np.ascontiguousarray(rsT, dtype=np.int32)
        self._ci = np.ascontiguousarray(ciT, dtype=np.int32)
        self._h = lib().refdev_create(self._rs.ctypes.data, int(g.NlocalT), self._ci.ctypes.data)
        if not self._h:
            raise RuntimeError("refdev_create failed (a row above 512 members, or no device memory)")
        self.nblocks = lib().refdev_nblocks(self._h)

    def gather_scatter(self, ptr, k, type_code, op_code, stream=None):
        return lib().refdev_gather_scatter(self._h, ptr, int(k), int(type_code), int(op_code), stream)

    def free(self):
        if self._h:
            lib().refdev_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
