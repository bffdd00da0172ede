"""ctypes binding of libdawgs_ogs.so, the C ABI declared in include/ogs_c.h.

The library must have been built (``python -m dawgs_gb300.build`` or
``__graft_entry__.build()``); there is no fallback implementation, so a missing
library is an ImportError-style failure at first use.  DAWGS_OGS_LIB names
another build of the same library (for instance one compiled with other
tile settings).
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB

OGS_OK, OGS_EINVAL, OGS_ENOMEM, OGS_EDEVICE, OGS_ETIMEOUT, OGS_ERANGE, OGS_EUNDEFINED = range(7)
STATUS_NAMES = {0: "OGS_OK", 1: "OGS_EINVAL", 2: "OGS_ENOMEM", 3: "OGS_EDEVICE",
                4: "OGS_ETIMEOUT", 5: "OGS_ERANGE", 6: "OGS_EUNDEFINED"}

SETUP_VERBOSE = 1
SETUP_HOST_ONLY = 2
SETUP_DEVICE_MAPS = 4
SETUP_HOST_MAPS = 8
DEVICE_MAPS_MIN_N = 65536

# every symbol include/ogs_c.h declares: (name, restype, argtypes)
_vp, _i, _i64, _u = C.c_void_p, C.c_int, C.c_int64, C.c_uint
SIGNATURES = {
    "ogs_setup": (_i, [C.POINTER(_vp), _i64, _vp, _i, _i, _i, _i]),
    "ogs_setup_ex": (_i, [C.POINTER(_vp), _i64, _vp, _i, _i, _u]),
    "ogs_free": (_i, [_vp]),
    "ogs_setup_maps": (_i, [C.POINTER(_vp), _i64, _i64, _i64, _vp, _vp, _vp, _vp, _u]),
    "ogs_extract": (_i, [_i64, _i, _i, _vp, _vp, _vp, _vp]),
    "ogs_gather_scatter": (_i, [_vp, _vp, _i, _i, _i, _i, _vp]),
    "ogs_gather_scatter_many": (_i, [_vp, _vp, _i, _i, _i, _i, _vp]),
    "ogs_gather": (_i, [_vp, _vp, _vp, _i, _i, _i, _i, _vp]),
    "ogs_scatter": (_i, [_vp, _vp, _vp, _i, _i, _i, _vp]),
    "ogs_gather_scatter_host": (_i, [_vp, _vp, _i, _i, _i, _i, _vp]),
    "ogs_reserve_host": (_i, [_vp, _i, _i]),
    "ogs_debug_fail_alloc": (_i, [_i64]),
    "ogs_debug_allocations": (_i, [_vp, _vp, _vp, _vp]),
    "ogs_gather_host": (_i, [_vp, _vp, _vp, _i, _i, _i, _i, _vp]),
    "ogs_scatter_host": (_i, [_vp, _vp, _vp, _i, _i, _i, _vp]),
    "ogs_gather_scatter_host_noalloc": (_i, [_vp, _vp, _i, _i, _i, _i, _vp]),
    "ogs_get_counts": (_i, [_vp, _vp]),
    "ogs_get_maps": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "ogs_get_layout_stats": (_i, [_vp, _vp]),
    "ogs_checked_id_errors": (_i, [_vp, _vp]),
    "ogs_gslib_setup": (_i, [C.POINTER(_vp), _vp, _i64, _u]),
    "ogs_gslib_gs": (_i, [_vp, _vp, _i, _i, _i, _vp]),
    "ogs_gslib_gs_vec": (_i, [_vp, _vp, _i, _i, _i, _i, _vp]),
    "ogs_gslib_gs_many": (_i, [_vp, _vp, _i, _i, _i, _i, _vp]),
    "ogs_batch_create": (_i, [C.POINTER(_vp), _i, _vp, _i, _u]),
    "ogs_batch_set_fields": (_i, [_vp, _vp, _vp]),
    "ogs_batch_gather_scatter": (_i, [_vp, _vp]),
    "ogs_batch_tune": (_i, [_vp, _vp, _vp]),
    "ogs_batch_tune_ex": (_i, [_vp, _vp, _u, _vp]),
    "ogs_batch_get_config": (_i, [_vp, _vp]),
    "ogs_batch_set_config": (_i, [_vp, _vp, _vp]),
    "ogs_batch_tune_key": (_i, [_i, _i, _i, _vp, _vp, _vp]),
    "ogs_batch_tune_cache_clear": (_i, []),
    "ogs_batch_items": (_i, [_vp, _vp]),
    "ogs_batch_free": (_i, [_vp]),
    "ogs_halo_setup": (_i, [C.POINTER(_vp), _i64, _vp, _i, _i]),
    "ogs_halo_setup_maps": (_i, [C.POINTER(_vp), _i64, _i64, _i64, _vp, _vp, _vp, _vp, _i64, _u]),
    "ogs_halo_setup_from_gather": (_i, [C.POINTER(_vp), _i64, _i64, _i64, _i64]),
    "ogs_halo_free": (_i, [_vp]),
    "ogs_halo_get_counts": (_i, [_vp, _vp]),
    "ogs_halo_reserve": (_i, [_vp, _i, _i, C.POINTER(_vp)]),
    "ogs_halo_exchange": (_i, [_vp, _vp, _i, _i, _vp, _vp]),
    "ogs_halo_exchange_start": (_i, [_vp, _vp, _i, _i, _vp, _vp]),
    "ogs_halo_exchange_finish": (_i, [_vp, _vp, _i, _i, _vp, _vp]),
    "ogs_halo_combine": (_i, [_vp, _vp, _i, _i, _vp, _vp]),
    "ogs_halo_combine_start": (_i, [_vp, _vp, _i, _i, _vp, _vp]),
    "ogs_halo_combine_finish": (_i, [_vp, _vp, _i, _i, _vp, _vp]),
    "ogs_halo_exchange_host": (_i, [_vp, _vp, _i, _i, _vp, _vp]),
    "ogs_halo_combine_host": (_i, [_vp, _vp, _i, _i, _vp, _vp]),
    "ogs_server_create": (_i, [C.POINTER(_vp), _vp]),
    "ogs_server_add_mesh": (_i, [_vp, _vp, _vp]),
    "ogs_server_submit": (_i, [_vp, _vp, C.c_double, _vp]),
    "ogs_server_submit_many": (_i, [_vp, _vp, _vp, _i64, _vp]),
    "ogs_server_clock": (C.c_double, []),
    "ogs_server_wait": (_i, [_vp, _i64]),
    "ogs_server_wait_for": (_i, [_vp, _i64, C.c_double]),
    "ogs_server_cancel": (_i, [_vp, _i64, _vp]),
    "ogs_server_state": (_i, [_vp, _i64, _vp]),
    "ogs_server_times": (_i, [_vp, _i64, _i64, _vp, _vp, _vp]),
    "ogs_server_drain": (_i, [_vp]),
    "ogs_server_latencies": (_i, [_vp, _i64, _i64, _vp, _vp]),
    "ogs_server_counters": (_i, [_vp, _vp, _vp]),
    "ogs_server_get_stats": (_i, [_vp, _vp]),
    "ogs_server_free": (_i, [_vp]),
    "ogs_last_error_string": (C.c_char_p, []),
    "ogs_version": (_i, []),
}


class OgsCounts(C.Structure):
    _fields_ = [("N", C.c_int64), ("Ngather", C.c_int64), ("NgatherGlobal", C.c_int64),
                ("NlocalP", C.c_int64), ("NlocalT", C.c_int64), ("nnzT", C.c_int64),
                ("nnzN", C.c_int64), ("gather_defined", C.c_int32), ("kind", C.c_int32),
                ("unique", C.c_int32), ("max_degree", C.c_int32)]


class OgsLayoutStats(C.Structure):
    _fields_ = [("rows_by_degree", C.c_int64 * 9), ("nnz_general", C.c_int64),
                ("ntiles", C.c_int64), ("device_bytes", C.c_int64), ("nphases", C.c_int64),
                ("phases", (C.c_int64 * 4) * 32), ("nwarp_tiles", C.c_int64), ("ngeneral_tiles", C.c_int64),
                ("phase_rows", (C.c_int64 * 2) * 32)]


class OgsBatchEntry(C.Structure):
    _fields_ = [("h", C.c_void_p), ("d_v", C.c_void_p), ("k", C.c_int32), ("op", C.c_int32),
                ("trans", C.c_int32), ("reserved", C.c_int32)]


BATCH_GRAPH = 1
TUNE_NO_CACHE = 1


class OgsBatchConfig(C.Structure):
    _fields_ = [("block", C.c_int32), ("ctas_per_sm", C.c_int32), ("solo_items", C.c_int64),
                ("solo_streams", C.c_int32), ("sms", C.c_int32), ("from_cache", C.c_int32),
                ("occupancy", C.c_int32), ("ms", C.c_double), ("pipeline", C.c_int32), ("reserved", C.c_int32)]


class OgsHaloCounts(C.Structure):
    _fields_ = [("N", C.c_int64), ("NlocalT", C.c_int64), ("NhaloP", C.c_int64), ("NhaloT", C.c_int64),
                ("Nhalo", C.c_int64), ("Nrecv", C.c_int64), ("gathered", C.c_int32), ("reserved", C.c_int32)]


# ogs_exchange_fn and ogs_exchange
EXCHANGE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p)


class OgsExchange(C.Structure):
    _fields_ = [("start", EXCHANGE_FN), ("finish", EXCHANGE_FN), ("user", C.c_void_p)]


class OgsServerConfig(C.Structure):
    _fields_ = [("field_budget_bytes", C.c_int64), ("max_inflight", C.c_int32), ("max_batch", C.c_int32)]


class OgsServerStats(C.Structure):
    _fields_ = [("passes", C.c_int64), ("gaps_over_1ms", C.c_int64), ("launches_over_1ms", C.c_int64),
                ("max_gap_ms", C.c_double), ("max_launch_ms", C.c_double), ("max_retire_ms", C.c_double)]


class OgsServerRequest(C.Structure):
    _fields_ = [("mesh", C.c_int32), ("type", C.c_int32), ("k", C.c_int32), ("op", C.c_int32),
                ("trans", C.c_int32), ("reserved", C.c_int32), ("host", C.c_void_p)]


class OgsError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_lib = None


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        path = os.environ.get("DAWGS_OGS_LIB") or LIB
        if not os.path.exists(path):
            raise ImportError(f"{path} is missing: build it with `python -m dawgs_gb300.build`; "
                              "the gather-scatter path has no CPU fallback")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != OGS_OK:
        raise OgsError(status, lib().ogs_last_error_string().decode())
