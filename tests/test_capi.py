"""The C ABI library loads without a GPU, exports every function that
include/ogs_c.h declares, and rejects bad arguments with the documented status
codes (the reference's LIBP_ABORT cases, ogsSetup.cpp:98-100, 861-864) before
touching a device."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from dawgs_gb300 import _lib, ogs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?!typedef\b)(?:const\s+)?[a-z_]+\s*\**\s*(ogs_[a-z_0-9]+)\s*\(", src, flags=re.M)
    return names


def test_library_exports_every_declared_symbol(built_lib):
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(built_lib, n), f"{n} is declared in include/ but not exported"
    assert set(names) == set(_lib.SIGNATURES), "ctypes binding and header disagree"


def test_version(built_lib):
    assert built_lib.ogs_version() >= 10000


def _setup(ids, kind=0, unique=0, flags=_lib.SETUP_HOST_ONLY):
    h = C.c_void_p()
    st = _lib.lib().ogs_setup_ex(C.byref(h), ids.size, ids.ctypes.data, kind, unique, flags)
    return st, h


def test_rejects_invalid_setups(built_lib):
    ids = np.arange(1, 11, dtype=np.int64)
    assert _setup(ids, kind=0, unique=1)[0] == _lib.OGS_EINVAL  # Unsigned + unique
    assert b"Invalid ogs setup" in built_lib.ogs_last_error_string()
    assert _setup(ids, kind=2)[0] == _lib.OGS_EINVAL  # Halo
    assert _setup(ids, kind=7)[0] == _lib.OGS_EINVAL
    bad = np.array([1, -(2 ** 63), 3], np.int64)
    assert _setup(bad)[0] == _lib.OGS_ERANGE
    # device indices are 32-bit (dlong = int, types.h:59-63): N is checked before ids are read
    h0 = C.c_void_p()
    assert built_lib.ogs_setup_ex(C.byref(h0), 2 ** 31, ids.ctypes.data, 0, 0, _lib.SETUP_HOST_ONLY) == \
        _lib.OGS_ERANGE
    h = C.c_void_p()
    assert built_lib.ogs_setup_ex(C.byref(h), -1, None, 0, 0, _lib.SETUP_HOST_ONLY) == _lib.OGS_EINVAL
    assert built_lib.ogs_setup_ex(C.byref(h), 5, None, 0, 0, _lib.SETUP_HOST_ONLY) == _lib.OGS_EINVAL
    assert built_lib.ogs_setup_ex(None, 5, ids.ctypes.data, 0, 0, _lib.SETUP_HOST_ONLY) == _lib.OGS_EINVAL
    assert built_lib.ogs_setup(C.byref(h), 10, ids.ctypes.data, 0, 9, 0, 0) == _lib.OGS_EINVAL  # method
    # maps on the GPU exclude a host-only handle and the host-maps flag
    for flags in (_lib.SETUP_DEVICE_MAPS | _lib.SETUP_HOST_ONLY, _lib.SETUP_DEVICE_MAPS | _lib.SETUP_HOST_MAPS):
        assert built_lib.ogs_setup_ex(C.byref(h), 10, ids.ctypes.data, 0, 0, flags) == _lib.OGS_EINVAL
    assert b"DEVICE_MAPS" in built_lib.ogs_last_error_string()


def test_host_only_handle_rejects_ops(built_lib):
    ids = np.array([1, 2, 1, 3], np.int64)
    st, h = _setup(ids)
    assert st == _lib.OGS_OK
    v = np.zeros(4)
    assert built_lib.ogs_gather_scatter(h, v.ctypes.data, 1, 1, 0, 0, None) == _lib.OGS_EINVAL
    assert b"host-only" in built_lib.ogs_last_error_string()
    assert built_lib.ogs_free(h) == _lib.OGS_OK
    assert built_lib.ogs_free(None) == _lib.OGS_OK
    assert built_lib.ogs_gather_scatter(None, v.ctypes.data, 1, 1, 0, 0, None) == _lib.OGS_EINVAL


def test_noalloc_size_check_cannot_wrap(built_lib):
    """The fixed staging array's size check is done by division: k near
    INT_MAX with 8-byte values (a product past 2^64 for large N) is refused
    with OGS_ERANGE before anything is copied, whatever the handle."""
    ids = np.arange(1, 1001, dtype=np.int64)
    st, h = _setup(ids)
    assert st == _lib.OGS_OK
    v = np.zeros(8)
    try:
        for k in (2 ** 31 - 1, 2 ** 30, 4195):  # 1000 nodes x 8 B x 4195 > 32 MiB
            assert built_lib.ogs_gather_scatter_host_noalloc(h, v.ctypes.data, k, 1, 0, 0, None) == _lib.OGS_ERANGE
            assert b"staging array" in built_lib.ogs_last_error_string()
        # a field that fits goes on to the usual refusals (a host-only handle)
        assert built_lib.ogs_gather_scatter_host_noalloc(h, v.ctypes.data, 1, 1, 0, 0, None) == _lib.OGS_EINVAL
        assert b"host-only" in built_lib.ogs_last_error_string()
    finally:
        built_lib.ogs_free(h)


def test_python_mirror_raises(built_lib):
    ids = np.array([1, 2, 1, 3], np.int64)
    with pytest.raises(_lib.OgsError) as e:
        ogs.ogs_t().Setup(4, ids.copy(), None, ogs.Unsigned, ogs.Auto, True)
    assert e.value.status == _lib.OGS_EINVAL
    g = ogs.ogs_t().Setup(4, ids.copy(), host_only=True)
    assert not g.gather_defined  # two members of group 1 are positive
    assert (g.N, g.NlocalT, g.Ngather) == (4, 3, 3)


def test_batch_tuner_cache_key(built_lib):
    """The tuner caches per (value type, SM count, k range, histogram of
    log2(warp tiles) over the entries): the order of the entries and sizes
    within one power of two do not change the key; the type, the SM count,
    the k range and the size classes do."""
    def key(type_, sms, recs, ks):
        k = C.c_uint64()
        r = np.asarray(recs, np.int64)
        kk = np.asarray(ks, np.int32)
        assert built_lib.ogs_batch_tune_key(type_, sms, r.size, r.ctypes.data, kk.ctypes.data, C.byref(k)) == \
            _lib.OGS_OK
        return k.value
    base = key(1, 152, [10, 300, 5000], [1, 2, 4])
    assert key(1, 152, [5000, 10, 300], [4, 1, 2]) == base      # order
    assert key(1, 152, [11, 260, 4100], [2, 1, 4]) == base      # same powers of two, same k range
    assert key(0, 152, [10, 300, 5000], [1, 2, 4]) != base      # type
    assert key(1, 148, [10, 300, 5000], [1, 2, 4]) != base      # SM count
    assert key(1, 152, [10, 300, 5000], [1, 2, 8]) != base      # k range
    assert key(1, 152, [10, 300, 9000], [1, 2, 4]) != base      # a size class
    assert key(1, 152, [10, 300, 5000, 5000], [1, 2, 4, 4]) != base  # how many per class
    assert built_lib.ogs_batch_tune_key(1, 152, 2, None, None, C.byref(C.c_uint64())) == _lib.OGS_EINVAL
