"""ctypes bindings for the CPU oracle.

TEST INFRASTRUCTURE ONLY.  ``OracleOgs`` wraps oracle/ogs_oracle.c, the C
restatement of libParanumal's host ogs (libs/ogs/ogsSetup.cpp,
libs/ogs/ogsOperator.cpp); ``GsRef`` wraps gslib built from the reference tree
(oracle/_ref/libgsref.so) and ``RefOperator`` the reference's own host
operator, libs/ogs/ogsOperator.cpp compiled unmodified against stand-ins for
OCCA and MPI (oracle/_ref/libogsref.so); both exist only where the reference
sources are.  Only
tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
module; the dawgs_gb300 package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libogs_oracle.so")
GSREF_SO = os.path.join(HERE, "_ref", "libgsref.so")
OGSREF_SO = os.path.join(HERE, "_ref", "libogsref.so")


def gslib_src() -> str | None:
    """The reference's vendored gslib sources: $GSLIB_SRC, else the default of
    the build recipe (oracle/Makefile); None when that directory is absent."""
    src = os.environ.get("GSLIB_SRC")
    if not src:
        try:
            src = subprocess.run(["make", "-s", "-C", HERE, "print-gslib-src"], check=True,
                                 capture_output=True, text=True).stdout.strip()
        except (OSError, subprocess.CalledProcessError):
            return None
    return src if src and os.path.isdir(src) else None


def ref_root() -> str | None:
    """The reference tree: $REF_ROOT, else the build recipe's default; None
    when its host operator source is absent."""
    root = os.environ.get("REF_ROOT")
    if not root:
        try:
            root = subprocess.run(["make", "-s", "-C", HERE, "print-ref-root"], check=True,
                                  capture_output=True, text=True).stdout.strip()
        except (OSError, subprocess.CalledProcessError):
            return None
    ok = root and os.path.isfile(os.path.join(root, "libs", "ogs", "ogsOperator.cpp"))
    return root if ok else None

TYPES = {"float32": 0, "float64": 1, "int32": 2, "int64": 3}
NP_OF = {0: np.float32, 1: np.float64, 2: np.int32, 3: np.int64}
OPS = {"add": 0, "mul": 1, "max": 2, "min": 3}
TRANS = {"sym": 0, "notrans": 1, "trans": 2}
KINDS = {"unsigned": 0, "signed": 1}


def build(ref: bool | None = None) -> None:
    """Compile the oracle (and gslib when the reference tree is present)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    src = gslib_src() if ref is not False else None
    if ref and src is None:
        raise FileNotFoundError("gslib sources not found: set GSLIB_SRC to the reference's 3rdParty/gslib/src")
    if src is not None:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"GSLIB_SRC={src}"], check=True)
    root = ref_root() if ref is not False else None
    if root is not None:
        subprocess.run(["make", "-s", "-C", HERE, "refop", f"REF_ROOT={root}"], check=True)


_lib = None
_gs = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        L = C.CDLL(ORACLE_SO)
        L.oracle_sizeof_handle.restype = C.c_int64
        L.oracle_setup.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int, C.c_int]
        L.oracle_setup.restype = C.c_int
        L.oracle_free.argtypes = [C.c_void_p]
        L.oracle_gather.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.oracle_scatter.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.oracle_gather_scatter.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.oracle_counts.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_maps.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        L.oracle_num_threads.restype = C.c_int
        L.oracle_set_num_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def gsref_available() -> bool:
    return os.path.exists(GSREF_SO)


def gslib():
    global _gs
    if _gs is None:
        L = C.CDLL(GSREF_SO)
        L.gsref_setup.argtypes = [C.c_void_p, C.c_int64, C.c_int]
        L.gsref_setup.restype = C.c_void_p
        L.gsref_gs.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.gsref_gs_vec.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.gsref_gs_many.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.gsref_unique.argtypes = [C.c_void_p, C.c_int64]
        L.gsref_free.argtypes = [C.c_void_p]
        _gs = L
    return _gs


def ogsref_available() -> bool:
    return os.path.exists(OGSREF_SO)


_ogsref = None


def ogsref():
    global _ogsref
    if _ogsref is None:
        L = C.CDLL(OGSREF_SO)
        L.ogsref_create.restype = C.c_void_p
        L.ogsref_create.argtypes = [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                    C.c_void_p]
        L.ogsref_free.argtypes = [C.c_void_p]
        L.ogsref_gather_scatter.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int,
                                            C.c_int]
        L.ogsref_time_gather_scatter.restype = C.c_double
        L.ogsref_time_gather_scatter.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int,
                                                 C.c_int, C.c_int, C.c_int]
        L.ogsref_gather.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int, C.c_int,
                                    C.c_int, C.c_int]
        L.ogsref_scatter.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int, C.c_int,
                                     C.c_int]
        _ogsref = L
    return _ogsref


class RefOperator:
    """The reference's own host ogs operator (ogsOperator_t, ogsOperator.cpp)
    over the maps of an ``OracleOgs`` handle: its GatherScatter, Gather and
    Scatter run the reference's code on those maps."""

    def __init__(self, o: "OracleOgs"):
        self._maps = o.maps()
        rsT, ciT, rsN, ciN = self._maps
        self.Ngather = o.Ngather
        self._h = ogsref().ogsref_create(o.N, o.NlocalT, _ptr(rsT), _ptr(ciT), o.NlocalP, _ptr(rsN), _ptr(ciN))

    def __del__(self):
        if _ogsref is not None and getattr(self, "_h", None):
            _ogsref.ogsref_free(self._h)
            self._h = None

    def gather_scatter(self, v: np.ndarray, k: int, op="add", trans="sym"):
        ogsref().ogsref_gather_scatter(self._h, _ptr(v), v.size, TYPES[v.dtype.name], k, _code(OPS, op),
                                       _code(TRANS, trans))
        return v

    def time_gather_scatter(self, v: np.ndarray, k: int, op="add", trans="sym", warm=2, reps=5) -> float:
        """Mean seconds per GatherScatter of the reference's code on one held field."""
        return ogsref().ogsref_time_gather_scatter(self._h, _ptr(v), v.size, TYPES[v.dtype.name], k,
                                                   _code(OPS, op), _code(TRANS, trans), warm, reps)

    def gather(self, gv: np.ndarray, v: np.ndarray, k: int, op="add", trans="trans"):
        ogsref().ogsref_gather(self._h, _ptr(gv), gv.size, _ptr(v), v.size, TYPES[v.dtype.name], k,
                               _code(OPS, op), _code(TRANS, trans))
        return gv

    def scatter(self, v: np.ndarray, gv: np.ndarray, k: int, trans="notrans"):
        ogsref().ogsref_scatter(self._h, _ptr(v), v.size, _ptr(gv), gv.size, TYPES[v.dtype.name], k,
                                _code(TRANS, trans))
        return v


def _code(table, x):
    return table[x] if isinstance(x, str) else int(x)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class OracleOgs:
    """Single-rank host ogs handle (the oracle).  ids is modified in place when unique."""

    def __init__(self, ids: np.ndarray, kind="unsigned", unique=False):
        assert ids.dtype == np.int64 and ids.flags.c_contiguous
        L = lib()
        self._buf = C.create_string_buffer(int(L.oracle_sizeof_handle()))
        rc = L.oracle_setup(self._buf, ids.size, _ptr(ids), _code(KINDS, kind), int(bool(unique)))
        if rc != 0:
            raise ValueError(f"oracle setup rejected the options (code {rc})")
        c = np.zeros(8, np.int64)
        L.oracle_counts(self._buf, _ptr(c))
        (self.N, self.NlocalP, self.NlocalT, self.Ngather, self.NgatherGlobal,
         self.nnzT, self.nnzN, gd) = (int(x) for x in c)
        self.gather_defined = bool(gd)

    def __del__(self):
        if _lib is not None and getattr(self, "_buf", None) is not None:
            _lib.oracle_free(self._buf)
            self._buf = None

    def maps(self):
        rsT = np.zeros(self.NlocalT + 1, np.int32)
        ciT = np.zeros(max(self.nnzT, 1), np.int32)
        rsN = np.zeros(self.NlocalT + 1, np.int32)
        ciN = np.zeros(max(self.nnzN, 1), np.int32)
        lib().oracle_maps(self._buf, _ptr(rsT), _ptr(ciT), _ptr(rsN), _ptr(ciN))
        return rsT, ciT[: self.nnzT], rsN, ciN[: self.nnzN]

    def gather_scatter(self, v: np.ndarray, k: int, op="add", trans="sym"):
        lib().oracle_gather_scatter(self._buf, _ptr(v), k, TYPES[v.dtype.name],
                                    _code(OPS, op), _code(TRANS, trans))
        return v

    def gather(self, gv: np.ndarray, v: np.ndarray, k: int, op="add", trans="trans"):
        lib().oracle_gather(self._buf, _ptr(gv), _ptr(v), k, TYPES[v.dtype.name],
                            _code(OPS, op), _code(TRANS, trans))
        return gv

    def scatter(self, v: np.ndarray, gv: np.ndarray, k: int, trans="notrans"):
        lib().oracle_scatter(self._buf, _ptr(v), _ptr(gv), k, TYPES[v.dtype.name],
                             _code(TRANS, trans))
        return v


def set_threads(n: int) -> None:
    lib().oracle_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().oracle_num_threads())


class GsRef:
    """gslib gs handle built from the reference tree (single rank, MPI off)."""

    def __init__(self, ids: np.ndarray, unique=False):
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        self._h = gslib().gsref_setup(_ptr(ids), ids.size, int(unique))

    def gs(self, v: np.ndarray, op="add", transpose=0):
        gslib().gsref_gs(_ptr(v), TYPES[v.dtype.name], _code(OPS, op), int(transpose), self._h)
        return v

    def gs_vec(self, v: np.ndarray, k: int, op="add", transpose=0):
        gslib().gsref_gs_vec(_ptr(v), k, TYPES[v.dtype.name], _code(OPS, op), int(transpose), self._h)
        return v

    def gs_many(self, vs, op="add", transpose=0):
        arr = (C.c_void_p * len(vs))(*[v.ctypes.data for v in vs])
        gslib().gsref_gs_many(arr, len(vs), TYPES[vs[0].dtype.name], _code(OPS, op), int(transpose), self._h)
        return vs

    def __del__(self):
        if _gs is not None and getattr(self, "_h", None):
            _gs.gsref_free(self._h)
            self._h = None
