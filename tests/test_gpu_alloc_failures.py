"""Allocation failures, injected on the host: ogs_debug_fail_alloc(n) makes
the library's n-th device or page-locked allocation from now fail as if the
memory were exhausted.  Every call that allocates must then return
OGS_ENOMEM, free what it took (the library's allocation ledger is back where
it was), and leave the objects it was given usable.  No GPU memory is
actually exhausted and no kernel faults.  The reference has no such paths:
LIBP_ABORT terminates (include/utils.hpp:57-76)."""
import ctypes as C

import numpy as np
import pytest

from dawgs_gb300 import _lib, mesh, ogs
from helpers import same_bits, values

pytestmark = pytest.mark.gpu


def held(L):
    v = [C.c_int64() for _ in range(4)]
    assert L.ogs_debug_allocations(*[C.byref(x) for x in v]) == _lib.OGS_OK
    return tuple(x.value for x in v)


def each_failure(L, call, undo, limit=64, keeps=False):
    """call() with its 1st, 2nd, ... allocation failing, until it succeeds;
    each failure must give OGS_ENOMEM and leave the ledger unchanged, and
    undo() after the success must release everything again (unless the call
    `keeps` what it allocated).  Returns how many allocations it made."""
    base = held(L)
    for n in range(1, limit + 1):
        assert L.ogs_debug_fail_alloc(n) == _lib.OGS_OK
        try:
            st = call()
        finally:
            L.ogs_debug_fail_alloc(0)
        if st == _lib.OGS_OK:
            undo()
            if not keeps:
                assert held(L) == base
            return n - 1
        assert st == _lib.OGS_ENOMEM, (n, st, L.ogs_last_error_string())
        assert held(L) == base, (n, held(L), base)
    raise AssertionError("the call never succeeded")


@pytest.mark.parametrize("flags", [_lib.SETUP_DEVICE_MAPS, _lib.SETUP_HOST_MAPS])
def test_setup_frees_everything_on_allocation_failure(cuda, flags):
    L = _lib.lib()
    ids = mesh.box_ids(8, 7, 6, 3)
    h = C.c_void_p()

    def call():
        return L.ogs_setup_ex(C.byref(h), ids.size, ids.copy().ctypes.data, 0, 0, flags)
    n = each_failure(L, call, lambda: L.ogs_free(h))
    assert n >= 1  # the maps' arena at least (the device path also allocates its scratch)


def test_reserve_host_then_host_calls_allocate_nothing(cuda, oracle_mod):
    L = _lib.lib()
    ids = mesh.box_ids(8, 8, 8, 3)
    sids = ids.copy()
    g = ogs.ogs_t().Setup(sids.size, sids, None, ogs.Signed, ogs.Auto, True)  # Gather is well defined
    h = g.handle
    stream = None
    # a failed reservation returns OGS_ENOMEM and frees what it took
    n = each_failure(L, lambda: L.ogs_reserve_host(h, 3, 1), lambda: None, keeps=True)
    assert n >= 1
    assert L.ogs_reserve_host(h, 3, 1) == _lib.OGS_OK
    before = held(L)
    ref = oracle_mod.OracleOgs(ids.copy(), "signed", unique=True)
    # with the next allocation armed to fail, every _host call no larger than
    # the reservation succeeds: none of them allocates
    L.ogs_debug_fail_alloc(1)
    try:
        for k, dt in ((3, np.float64), (1, np.float64), (2, np.float32), (3, np.int64)):
            v = values(k * ids.size, dt, "add", seed=40 + k)
            want = ref.gather_scatter(v.copy(), k, "add", "sym")
            got = v.copy()
            st = L.ogs_gather_scatter_host(h, got.ctypes.data, k, int(ogs._type_of(got)), 0, 0, stream)
            assert st == _lib.OGS_OK, L.ogs_last_error_string()
            assert same_bits(got, want)
        gv = np.zeros(3 * g.Ngather)
        v = values(3 * ids.size, np.float64, "add", seed=50)
        assert L.ogs_gather_host(h, gv.ctypes.data, v.ctypes.data, 3, 1, 0, 0, stream) == _lib.OGS_OK
        out = np.zeros_like(v)
        assert L.ogs_scatter_host(h, out.ctypes.data, gv.ctypes.data, 3, 1, 0, stream) == _lib.OGS_OK
        assert same_bits(out, ref.gather_scatter(v.copy(), 3, "add", "sym"))
    finally:
        L.ogs_debug_fail_alloc(0)
    assert held(L) == before
    g.Free()


def test_host_call_without_reservation_fails_cleanly_and_recovers(cuda, oracle_mod):
    L = _lib.lib()
    ids = mesh.box_ids(6, 6, 6, 3)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    base = held(L)
    v = values(ids.size, np.float64, "add", seed=61)
    x = v.copy()
    L.ogs_debug_fail_alloc(1)
    try:
        st = L.ogs_gather_scatter_host(g.handle, x.ctypes.data, 1, 1, 0, 0, None)
    finally:
        L.ogs_debug_fail_alloc(0)
    assert st == _lib.OGS_ENOMEM
    assert b"staging" in L.ogs_last_error_string()
    assert held(L) == base
    assert same_bits(x, v)  # the field was not touched
    assert L.ogs_gather_scatter_host(g.handle, x.ctypes.data, 1, 1, 0, 0, None) == _lib.OGS_OK
    assert same_bits(x, oracle_mod.OracleOgs(ids.copy(), "unsigned").gather_scatter(v.copy(), 1, "add", "sym"))
    g.Free()


def test_batch_and_server_creation_free_everything_on_failure(cuda):
    import torch
    L = _lib.lib()
    ids = mesh.box_ids(4, 4, 4, 2)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    field = torch.zeros(ids.size, dtype=torch.float64, device="cuda")
    arr = (_lib.OgsBatchEntry * 2)(_lib.OgsBatchEntry(g.handle, field.data_ptr(), 1, 0, 0, 0),
                                   _lib.OgsBatchEntry(g.handle, field.data_ptr() + 8 * 0, 1, 0, 0, 0))
    b = C.c_void_p()
    each_failure(L, lambda: L.ogs_batch_create(C.byref(b), 1, arr, 1, 0), lambda: L.ogs_batch_free(b))
    cfg = _lib.OgsServerConfig(64 << 20, 64, 16)
    s = C.c_void_p()
    n = each_failure(L, lambda: L.ogs_server_create(C.byref(s), C.byref(cfg)), lambda: L.ogs_server_free(s))
    assert n >= 2  # the field pool and at least one launch table
    g.Free()
