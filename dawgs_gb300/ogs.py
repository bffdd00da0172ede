"""Python mirror of libParanumal's ``ogs::ogs_t`` (include/ogs.hpp:216-345 of
the reference) over the C ABI of libdawgs_ogs.so.

Names, argument order and meaning follow the reference::

    g = ogs_t()
    g.Setup(N, ids, comm, Unsigned, Auto, unique=False, verbose=False, platform=None)
    g.GatherScatter(o_v, k, Add, Sym)     # torch CUDA tensor: runs on its stream
    g.GatherScatter(v, k, Add, Sym)       # host buffer (numpy / CPU tensor): copied
                                          # through the GPU and back
    g.Gather(o_gv, o_v, k, Add, Trans)
    g.Scatter(o_v, o_gv, k, NoTrans)

Errors raise ``OgsError`` with the library's status and message, where the
reference raises ``libp::exception`` through LIBP_ABORT.  ``comm``, ``method``
and ``platform`` are accepted and ignored: the path runs at one rank.
"""
from __future__ import annotations

import ctypes as C
import enum

import numpy as np

from . import _lib
from ._lib import OgsCounts, OgsError, OgsLayoutStats, check, lib


class Type(enum.IntEnum):  # include/ogs.hpp:179
    Float = 0
    Double = 1
    Int32 = 2
    Int64 = 3


class Op(enum.IntEnum):  # include/ogs.hpp:186
    Add = 0
    Mul = 1
    Max = 2
    Min = 3


class Transpose(enum.IntEnum):  # include/ogs.hpp:189
    Sym = 0
    NoTrans = 1
    Trans = 2


class Method(enum.IntEnum):  # include/ogs.hpp:192
    Auto = 0
    Pairwise = 1
    CrystalRouter = 2
    AllToAll = 3


class Kind(enum.IntEnum):  # include/ogs.hpp:195
    Unsigned = 0
    Signed = 1
    Halo = 2


Float, Double, Int32, Int64 = Type
Add, Mul, Max, Min = Op
Sym, NoTrans, Trans = Transpose
Auto, Pairwise, CrystalRouter, AllToAll = Method
Unsigned, Signed, Halo = Kind

_NP_TYPES = {np.dtype(np.float32): Float, np.dtype(np.float64): Double,
             np.dtype(np.int32): Int32, np.dtype(np.int64): Int64}


def _type_of(buf) -> Type:
    if isinstance(buf, np.ndarray):
        t = _NP_TYPES.get(buf.dtype)
    else:
        import torch
        t = {torch.float32: Float, torch.float64: Double,
             torch.int32: Int32, torch.int64: Int64}.get(buf.dtype)
    if t is None:
        raise OgsError(_lib.OGS_EINVAL, f"unsupported field dtype {buf.dtype}")
    return t


def _is_device(buf) -> bool:
    return not isinstance(buf, np.ndarray) and getattr(buf, "is_cuda", False)


def _ptr(buf) -> int:
    if isinstance(buf, np.ndarray):
        if not buf.flags.c_contiguous:
            raise OgsError(_lib.OGS_EINVAL, "field buffers must be contiguous")
        return buf.ctypes.data
    if not buf.is_contiguous():
        raise OgsError(_lib.OGS_EINVAL, "field buffers must be contiguous")
    return buf.data_ptr()


def _stream_of(stream):
    if stream is not None:
        return getattr(stream, "cuda_stream", stream)
    import torch
    if torch.cuda.is_available():
        return torch.cuda.current_stream().cuda_stream
    return None


def extract(out, q, ids, k, stream=None):
    """out[n*k+c] = q[ids[n]*k+c]: the exchange's send-buffer packing
    (ogsKernels.okl:167-177).  Device tensors; ids int32."""
    t = _type_of(q)
    if _type_of(out) != t:
        raise OgsError(_lib.OGS_EINVAL, "out and q must have the same dtype")
    check(lib().ogs_extract(int(ids.numel()), int(k), int(t), _ptr(ids), _ptr(q), _ptr(out), _stream_of(stream)))
    return out


class ogs_t:
    """One single-rank gather-scatter handle (ogs::ogs_t)."""

    def __init__(self, platform=None):
        self._h = None
        self.N = self.Ngather = self.NgatherGlobal = self.NlocalT = self.NlocalP = 0
        self.NhaloT = self.NhaloP = 0
        self.nnzT = self.nnzN = 0
        self.gather_defined = False
        self.unique = False
        self.kind = Unsigned
        self.max_degree = 0

    # ogs_t::Setup, include/ogs.hpp:221-228 / libs/ogs/ogsSetup.cpp:44-53
    def Setup(self, N, ids, comm=None, kind=Unsigned, method=Auto, unique=False,
              verbose=False, platform=None, host_only=False, maps=None):
        """maps: None (GPU for N >= 65536 unless host_only), "device" or "host"
        -- where the N/T maps are built; the handle is the same either way."""
        self.Free()
        if not (isinstance(ids, np.ndarray) and ids.dtype == np.int64 and ids.flags.c_contiguous):
            raise OgsError(_lib.OGS_EINVAL, "ids must be a contiguous int64 numpy array")
        if len(ids) < N:
            raise OgsError(_lib.OGS_EINVAL, "ids is shorter than N")
        h = C.c_void_p()
        flags = (_lib.SETUP_VERBOSE if verbose else 0) | (_lib.SETUP_HOST_ONLY if host_only else 0)
        if maps not in (None, "device", "host"):
            raise OgsError(_lib.OGS_EINVAL, "maps must be None, 'device' or 'host'")
        flags |= {None: 0, "device": _lib.SETUP_DEVICE_MAPS, "host": _lib.SETUP_HOST_MAPS}[maps]
        check(lib().ogs_setup_ex(C.byref(h), int(N), ids.ctypes.data, int(kind), int(bool(unique)), flags))
        self._h = h
        return self._refresh()

    def SetupMaps(self, N, rowStartsT, colIdsT, rowStartsN=None, colIdsN=None, NrowsN=None, host_only=False):
        """An operator over caller-built CSR maps (ogsOperator_t: the
        reference's gatherLocal, gatherHalo and postmpi are such operators).
        Without N maps the N map is the T map."""
        self.Free()
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        rsT, ciT = i32(rowStartsT), i32(colIdsT)
        NrowsT = rsT.size - 1
        rsN = ciN = None
        if rowStartsN is not None:
            rsN, ciN = i32(rowStartsN), i32(colIdsN if colIdsN is not None else [])
            if NrowsN is None:
                NrowsN = NrowsT
        h = C.c_void_p()
        flags = _lib.SETUP_HOST_ONLY if host_only else 0
        check(lib().ogs_setup_maps(C.byref(h), int(N), int(NrowsN if NrowsN is not None else NrowsT), int(NrowsT),
                                   rsN.ctypes.data if rsN is not None else None,
                                   ciN.ctypes.data if ciN is not None and ciN.size else None,
                                   rsT.ctypes.data, ciT.ctypes.data if ciT.size else None, flags))
        self._h = h
        return self._refresh()

    def _refresh(self):
        c = OgsCounts()
        check(lib().ogs_get_counts(self._h, C.byref(c)))
        self.N, self.Ngather, self.NgatherGlobal = c.N, c.Ngather, c.NgatherGlobal
        self.NlocalP, self.NlocalT = c.NlocalP, c.NlocalT
        self.nnzT, self.nnzN = c.nnzT, c.nnzN
        self.gather_defined = bool(c.gather_defined)
        self.kind, self.unique, self.max_degree = Kind(c.kind), bool(c.unique), c.max_degree
        return self

    def Free(self):
        if self._h is not None and _lib._lib is not None:
            lib().ogs_free(self._h)
        self._h = None

    def __del__(self):
        try:
            self.Free()
        except Exception:
            pass

    @property
    def handle(self):
        if self._h is None:
            raise OgsError(_lib.OGS_EINVAL, "ogs handle is not set up")
        return self._h

    def ReserveHost(self, k, dtype=Double):
        """Reserve the staging of the host-buffer calls for fields of k
        components of dtype (a Type or numpy dtype): later host-buffer calls no
        larger allocate nothing (no reference counterpart; the reference
        allocates exchange buffers in every call, libs/ogs/ogs.cpp:53)."""
        t = dtype if isinstance(dtype, Type) else _NP_TYPES[np.dtype(dtype)]
        check(lib().ogs_reserve_host(self.handle, int(k), int(t)))
        return self

    # ---- GatherScatter (include/ogs.hpp:232-265) ----
    def GatherScatter(self, v, k, op=Add, trans=Sym, stream=None):
        t = _type_of(v)
        if _is_device(v):
            check(lib().ogs_gather_scatter(self.handle, _ptr(v), int(k), int(t), int(op), int(trans),
                                           _stream_of(stream)))
        else:
            check(lib().ogs_gather_scatter_host(self.handle, _ptr(v), int(k), int(t), int(op),
                                                int(trans), _stream_of(stream)))
        return v

    GatherScatterStart = GatherScatter

    def GatherScatterFinish(self, v, k, op=Add, trans=Sym, stream=None):
        return v

    def GatherScatterMany(self, vs, op=Add, trans=Sym, stream=None):
        """k separate device arrays (gslib's gs_many layout)."""
        t = _type_of(vs[0])
        arr = (C.c_void_p * len(vs))(*[_ptr(x) for x in vs])
        check(lib().ogs_gather_scatter_many(self.handle, arr, len(vs), int(t), int(op), int(trans),
                                            _stream_of(stream)))
        return vs

    # ---- Gather (include/ogs.hpp:268-306) ----
    def Gather(self, gv, v, k, op=Add, trans=Trans, stream=None):
        t = _type_of(v)
        if _type_of(gv) != t:
            raise OgsError(_lib.OGS_EINVAL, "gv and v must have the same dtype")
        if _is_device(v) != _is_device(gv):
            raise OgsError(_lib.OGS_EINVAL, "gv and v must both be device or both be host buffers")
        fn = lib().ogs_gather if _is_device(v) else lib().ogs_gather_host
        check(fn(self.handle, _ptr(gv), _ptr(v), int(k), int(t), int(op), int(trans), _stream_of(stream)))
        return gv

    GatherStart = Gather

    def GatherFinish(self, gv, v, k, op=Add, trans=Trans, stream=None):
        return gv

    # ---- Scatter (include/ogs.hpp:309-341) ----
    def Scatter(self, v, gv, k, trans=NoTrans, stream=None):
        t = _type_of(v)
        if _type_of(gv) != t:
            raise OgsError(_lib.OGS_EINVAL, "gv and v must have the same dtype")
        if _is_device(v) != _is_device(gv):
            raise OgsError(_lib.OGS_EINVAL, "gv and v must both be device or both be host buffers")
        fn = lib().ogs_scatter if _is_device(v) else lib().ogs_scatter_host
        check(fn(self.handle, _ptr(v), _ptr(gv), int(k), int(t), int(trans), _stream_of(stream)))
        return v

    ScatterStart = Scatter

    def ScatterFinish(self, v, gv, k, trans=NoTrans, stream=None):
        return v

    # ---- introspection ----
    def maps(self):
        """Host copies of (rowStartsT, colIdsT, rowStartsN, colIdsN)."""
        rsT = np.zeros(self.NlocalT + 1, np.int32)
        ciT = np.zeros(max(self.nnzT, 1), np.int32)
        rsN = np.zeros(self.NlocalT + 1, np.int32)
        ciN = np.zeros(max(self.nnzN, 1), np.int32)
        check(lib().ogs_get_maps(self.handle, rsT.ctypes.data, ciT.ctypes.data, rsN.ctypes.data,
                                 ciN.ctypes.data))
        return rsT, ciT[: self.nnzT], rsN, ciN[: self.nnzN]

    def checked_id_errors(self) -> int:
        """Ids out of range seen by a checked build's kernels (0 otherwise)."""
        n = C.c_uint64()
        check(lib().ogs_checked_id_errors(self.handle, C.byref(n)))
        return n.value

    def layout_stats(self) -> dict:
        s = OgsLayoutStats()
        check(lib().ogs_get_layout_stats(self.handle, C.byref(s)))
        return {"rows_by_degree": {d: int(s.rows_by_degree[d]) for d in range(1, 9) if s.rows_by_degree[d]},
                "rows_general": int(s.rows_by_degree[0]), "nnz_general": int(s.nnz_general),
                "ntiles": int(s.ntiles), "nwarp_tiles": int(s.nwarp_tiles),
                "ngeneral_tiles": int(s.ngeneral_tiles), "device_bytes": int(s.device_bytes),
                "phases": [tuple(int(x) for x in s.phases[p]) for p in range(int(s.nphases))],
                "phase_rows": [tuple(int(x) for x in s.phase_rows[p]) for p in range(int(s.nphases))]}


class halo_t:
    """libParanumal's halo_t (include/ogs.hpp:346-397; libs/ogs/ogsHalo.cpp):
    Exchange gives every copy of a halo row its owner's value, Combine gives
    the owner the sum of all copies.  The exchange between ranks (MPI in the
    reference) is the caller's: set_exchange(start, finish) with callables
    (d_buf, k, type, trans, stream) -> status, called around the library's
    device steps.  At one rank (Setup) the halo has no rows."""

    def __init__(self, platform=None):
        self._h = None
        self._x = None
        self._keep = None
        self.N = self.Nhalo = self.NlocalT = self.NhaloP = self.NhaloT = self.Nrecv = 0
        self.gathered_halo = False

    def _adopt(self, h):
        self.Free()
        self._h = h
        c = _lib.OgsHaloCounts()
        check(lib().ogs_halo_get_counts(h, C.byref(c)))
        self.N, self.NlocalT, self.NhaloP, self.NhaloT = int(c.N), int(c.NlocalT), int(c.NhaloP), int(c.NhaloT)
        self.Nhalo, self.Nrecv, self.gathered_halo = int(c.Nhalo), int(c.Nrecv), bool(c.gathered)
        return self

    # halo_t::Setup, ogsSetup.cpp:55-64 (one rank)
    def Setup(self, N, ids, comm=None, method=Auto, verbose=False, platform=None):
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        h = C.c_void_p()
        check(lib().ogs_halo_setup(C.byref(h), int(N), ids.ctypes.data, int(method), int(bool(verbose))))
        return self._adopt(h)

    def SetupMaps(self, N, NhaloP, rowStartsT, colIdsT, rowStartsN=None, colIdsN=None, Nrecv=0):
        """A halo over the gatherHalo maps of a multi-rank setup."""
        rsT = np.ascontiguousarray(rowStartsT, dtype=np.int32)
        ciT = np.ascontiguousarray(colIdsT, dtype=np.int32)
        rsN = None if rowStartsN is None else np.ascontiguousarray(rowStartsN, dtype=np.int32)
        ciN = None if colIdsN is None else np.ascontiguousarray(colIdsN, dtype=np.int32)
        h = C.c_void_p()
        check(lib().ogs_halo_setup_maps(C.byref(h), int(N), int(NhaloP), int(rsT.size - 1),
                                        None if rsN is None else rsN.ctypes.data,
                                        None if ciN is None or ciN.size == 0 else ciN.ctypes.data,
                                        rsT.ctypes.data, ciT.ctypes.data if ciT.size else None, int(Nrecv), 0))
        return self._adopt(h)

    # halo_t::SetupFromGather, ogsSetup.cpp:888-913
    def SetupFromGather(self, g=None, NlocalT=None, NhaloP=0, NhaloT=0, Nrecv=0):
        if g is not None:
            if not g.gather_defined:
                raise OgsError(_lib.OGS_EUNDEFINED, "Gather operation not well-defined.")
            NlocalT, NhaloP, NhaloT = g.NlocalT, g.NhaloP, g.NhaloT
        h = C.c_void_p()
        check(lib().ogs_halo_setup_from_gather(C.byref(h), int(NlocalT), int(NhaloP), int(NhaloT), int(Nrecv)))
        return self._adopt(h)

    def set_exchange(self, start=None, finish=None):
        def wrap(f):
            if f is None:
                return _lib.EXCHANGE_FN()
            return _lib.EXCHANGE_FN(lambda user, buf, k, t, tr, st: int(f(buf or 0, k, t, tr, st) or 0))
        fs = (wrap(start), wrap(finish))
        self._keep = fs
        self._x = _lib.OgsExchange(fs[0], fs[1], None)
        return self

    def reserve(self, k, dtype=Double) -> int:
        t = dtype if isinstance(dtype, Type) else _NP_TYPES[np.dtype(dtype)]
        p = C.c_void_p()
        check(lib().ogs_halo_reserve(self._h, int(k), int(t), C.byref(p)))
        return p.value or 0

    def _call(self, name, v, k, stream):
        x = C.byref(self._x) if self._x is not None else None
        host = not _is_device(v)
        fn = getattr(lib(), f"ogs_halo_{name}_host" if host else f"ogs_halo_{name}")
        check(fn(self._h, _ptr(v), int(k), int(_type_of(v)), x, _stream_of(stream)))
        return v

    def Exchange(self, v, k, stream=None):
        return self._call("exchange", v, k, stream)

    def ExchangeStart(self, v, k, stream=None):
        return self._call("exchange" if not _is_device(v) else "exchange_start", v, k, stream)

    def ExchangeFinish(self, v, k, stream=None):
        return v if not _is_device(v) else self._call("exchange_finish", v, k, stream)

    def Combine(self, v, k, stream=None):
        return self._call("combine", v, k, stream)

    def CombineStart(self, v, k, stream=None):
        return self._call("combine" if not _is_device(v) else "combine_start", v, k, stream)

    def CombineFinish(self, v, k, stream=None):
        return v if not _is_device(v) else self._call("combine_finish", v, k, stream)

    @property
    def handle(self):
        return self._h

    def Free(self):
        if getattr(self, "_h", None) is not None and _lib._lib is not None:
            lib().ogs_halo_free(self._h)
        self._h = None

    def __del__(self):
        try:
            self.Free()
        except Exception:
            pass


class ogs_batch_t:
    """Many meshes' GatherScatters in one persistent launch (no reference
    counterpart: dawgs calls ogs_t::GatherScatter once per mesh).

    entries: list of (ogs_t, device field tensor, k, op, trans); all fields
    share one dtype.  graph=True captures the launch in a CUDA graph on first
    use and replays it afterwards."""

    def __init__(self, entries, graph=False):
        self._b = None
        if not entries:
            raise OgsError(_lib.OGS_EINVAL, "a batch needs at least one entry")
        t = _type_of(entries[0][1])
        arr = (_lib.OgsBatchEntry * len(entries))()
        for i, (g, field, k, op, trans) in enumerate(entries):
            if _type_of(field) != t:
                raise OgsError(_lib.OGS_EINVAL, "all batch fields must share one dtype")
            arr[i] = _lib.OgsBatchEntry(g.handle, _ptr(field), int(k), int(op), int(trans), 0)
        b = C.c_void_p()
        check(lib().ogs_batch_create(C.byref(b), int(t), arr, len(entries),
                                     _lib.BATCH_GRAPH if graph else 0))
        self._b = b
        self.entries = entries

    def GatherScatter(self, stream=None):
        check(lib().ogs_batch_gather_scatter(self._b, _stream_of(stream)))

    def set_fields(self, fields, stream=None):
        arr = (C.c_void_p * len(fields))(*[_ptr(x) for x in fields])
        check(lib().ogs_batch_set_fields(self._b, arr, _stream_of(stream)))

    def tune(self, stream=None, use_cache=True) -> dict:
        """Run the tuner (times candidates on scratch copies of the fields,
        or takes a cached choice); returns the configuration chosen."""
        c = _lib.OgsBatchConfig()
        check(lib().ogs_batch_tune_ex(self._b, _stream_of(stream), 0 if use_cache else _lib.TUNE_NO_CACHE,
                                      C.byref(c)))
        return self._cfg_dict(c)

    @staticmethod
    def _cfg_dict(c):
        return {"pipeline": c.pipeline, "block": c.block, "occupancy": c.occupancy or 2, "ctas_per_sm": c.ctas_per_sm,
                "solo_items": c.solo_items, "solo_streams": c.solo_streams, "sms": c.sms,
                "from_cache": bool(c.from_cache), "ms": c.ms}

    @property
    def config(self) -> dict:
        c = _lib.OgsBatchConfig()
        check(lib().ogs_batch_get_config(self._b, C.byref(c)))
        return self._cfg_dict(c)

    def set_config(self, block=256, ctas_per_sm=0, solo_items=0, solo_streams=1, occupancy=2, pipeline=0,
                   stream=None):
        c = _lib.OgsBatchConfig(int(block), int(ctas_per_sm), int(solo_items), int(solo_streams), 0, 0,
                                int(occupancy), 0.0, int(pipeline), 0)
        check(lib().ogs_batch_set_config(self._b, C.byref(c), _stream_of(stream)))

    @property
    def items(self) -> int:
        n = C.c_int64()
        check(lib().ogs_batch_items(self._b, C.byref(n)))
        return n.value

    def Free(self):
        if self._b is not None and _lib._lib is not None:
            lib().ogs_batch_free(self._b)
        self._b = None

    def __del__(self):
        try:
            self.Free()
        except Exception:
            pass


class ogs_server_t:
    """Served gather-scatter (no reference counterpart): resident meshes,
    requests admitted against an HBM budget, continuous batching."""

    def __init__(self, field_budget_bytes=16 << 30, max_inflight=4096, max_batch=256):
        cfg = _lib.OgsServerConfig(int(field_budget_bytes), int(max_inflight), int(max_batch))
        s = C.c_void_p()
        check(lib().ogs_server_create(C.byref(s), C.byref(cfg)))
        self._s = s
        self.meshes = []

    def add_mesh(self, g: ogs_t) -> int:
        mid = C.c_int()
        check(lib().ogs_server_add_mesh(self._s, g.handle, C.byref(mid)))
        self.meshes.append(g)
        return mid.value

    def submit(self, mesh: int, host, k: int, op=Add, trans=Sym, arrival: float = 0.0) -> int:
        t = _type_of(host)
        r = _lib.OgsServerRequest(int(mesh), int(t), int(k), int(op), int(trans), 0, _ptr(host))
        rid = C.c_int64()
        check(lib().ogs_server_submit(self._s, C.byref(r), float(arrival), C.byref(rid)))
        return rid.value

    def submit_many(self, reqs, arrivals=None) -> int:
        """reqs: (mesh, host field, k, op, trans) tuples; arrivals: one
        ogs_server_clock time each (future times are scheduled), or None for
        now.  Returns the first id; the others follow in order."""
        n = len(reqs)
        arr = (_lib.OgsServerRequest * max(n, 1))()
        for i, (mesh, host, k, op, trans) in enumerate(reqs):
            arr[i] = _lib.OgsServerRequest(int(mesh), int(_type_of(host)), int(k), int(op), int(trans), 0,
                                           _ptr(host))
        a = None if arrivals is None else np.ascontiguousarray(arrivals, dtype=np.float64)
        first = C.c_int64()
        check(lib().ogs_server_submit_many(self._s, arr, None if a is None else a.ctypes.data, n,
                                           C.byref(first)))
        return first.value

    @staticmethod
    def clock() -> float:
        return float(lib().ogs_server_clock())

    def wait(self, rid: int, timeout: float | None = None):
        """Until the request is done or cancelled; with a timeout (seconds),
        OgsError(OGS_ETIMEOUT) when it runs out."""
        if timeout is None:
            check(lib().ogs_server_wait(self._s, int(rid)))
        else:
            check(lib().ogs_server_wait_for(self._s, int(rid), float(timeout)))

    def cancel(self, rid: int) -> bool:
        """Withdraw a request not admitted yet; False when it already runs or ran."""
        c = C.c_int()
        check(lib().ogs_server_cancel(self._s, int(rid), C.byref(c)))
        return bool(c.value)

    PENDING, ADMITTED, DONE, CANCELLED = range(4)

    def state(self, rid: int) -> int:
        st = C.c_int()
        check(lib().ogs_server_state(self._s, int(rid), C.byref(st)))
        return st.value

    def drain(self):
        check(lib().ogs_server_drain(self._s))

    def times(self, first: int, n: int, launched: bool = False):
        """(arrival, done) or, with launched=True, (arrival, launched, done)."""
        a = np.zeros(n)
        lt = np.zeros(n)
        d = np.zeros(n)
        check(lib().ogs_server_times(self._s, int(first), int(n), a.ctypes.data, lt.ctypes.data, d.ctypes.data))
        return (a, lt, d) if launched else (a, d)

    def stats(self) -> dict:
        """The worker thread's timing (passes, long gaps, long launches)."""
        st = _lib.OgsServerStats()
        check(lib().ogs_server_get_stats(self._s, C.byref(st)))
        return {f: getattr(st, f) for f, _ in st._fields_}

    def counters(self):
        l, b = C.c_int64(), C.c_int64()
        check(lib().ogs_server_counters(self._s, C.byref(l), C.byref(b)))
        return l.value, b.value

    def Free(self):
        if getattr(self, "_s", None) is not None and _lib._lib is not None:
            lib().ogs_server_free(self._s)
        self._s = None

    def __del__(self):
        try:
            self.Free()
        except Exception:
            pass


class gslib_t:
    """gslib-compatible gather-scatter on the GPU (gs_setup / gs / gs_vec /
    gs_many of the gslib that dawgs vendors, single rank, unique=0).  Negative
    ids are flagged; transpose 0 or 1 as in gslib."""

    def __init__(self, ids: np.ndarray, host_only=False):
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        h = C.c_void_p()
        check(lib().ogs_gslib_setup(C.byref(h), ids.ctypes.data, ids.size,
                                    _lib.SETUP_HOST_ONLY if host_only else 0))
        self._h = h
        self.n = ids.size

    def gs(self, u, op=Add, transpose=0, stream=None):
        check(lib().ogs_gslib_gs(self._h, _ptr(u), int(_type_of(u)), int(op), int(transpose), _stream_of(stream)))
        return u

    def gs_vec(self, u, vn, op=Add, transpose=0, stream=None):
        check(lib().ogs_gslib_gs_vec(self._h, _ptr(u), int(vn), int(_type_of(u)), int(op), int(transpose),
                                     _stream_of(stream)))
        return u

    def gs_many(self, us, op=Add, transpose=0, stream=None):
        arr = (C.c_void_p * len(us))(*[_ptr(x) for x in us])
        check(lib().ogs_gslib_gs_many(self._h, arr, len(us), int(_type_of(us[0])), int(op), int(transpose),
                                      _stream_of(stream)))
        return us

    def Free(self):
        if getattr(self, "_h", None) is not None and _lib._lib is not None:
            lib().ogs_free(self._h)
        self._h = None

    def __del__(self):
        try:
            self.Free()
        except Exception:
            pass
