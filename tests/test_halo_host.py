"""halo_t at one rank through the C ABI, without a GPU: Setup checks that
every id group has exactly one positive member (the reference's LIBP_ABORT,
ogsSetup.cpp:286-288), the halo has no rows, and Exchange / Combine leave the
vector alone while still calling the caller's exchange (start, then finish),
as the reference's exchange object runs at one rank (ogsHalo.cpp:39-143)."""
import ctypes as C

import numpy as np
import pytest

from dawgs_gb300 import _lib, mesh, ogs


def unique_ids():
    ids = mesh.box_ids(4, 3, 2, 2)
    seen, out = set(), ids.copy()
    for n, b in enumerate(ids):
        if b in seen:
            out[n] = -b
        seen.add(b)
    return out


def test_one_rank_halo_has_no_rows_and_runs_the_exchange(built_lib):
    ids = unique_ids()
    h = ogs.halo_t().Setup(ids.size, ids)
    assert (h.N, h.NhaloP, h.NhaloT, h.Nhalo, h.gathered_halo) == (ids.size, 0, 0, 0, False)
    calls = []
    h.set_exchange(lambda buf, k, t, tr, st: calls.append(("start", k, t, tr)),
                   lambda buf, k, t, tr, st: calls.append(("finish", k, t, tr)))
    v = np.arange(3 * ids.size, dtype=np.float64)
    h.Exchange(v, 3)
    h.Combine(v, 3)
    assert np.array_equal(v, np.arange(3 * ids.size, dtype=np.float64))
    assert calls == [("start", 3, 1, 1), ("finish", 3, 1, 1), ("start", 3, 1, 2), ("finish", 3, 1, 2)]
    assert h.reserve(3) == 0  # no rows, no buffer
    h.Free()


def test_halo_setup_rejects_ids_without_one_positive_member(built_lib):
    L = _lib.lib()
    h = C.c_void_p()
    ids = np.array([1, 2, 1, -3, -3], np.int64)  # id 1 twice positive, id 3 never
    assert L.ogs_halo_setup(C.byref(h), ids.size, ids.ctypes.data, 0, 0) == _lib.OGS_EINVAL
    assert b"positive Ids for baseId" in L.ogs_last_error_string()
    ids = np.array([1, -1, 2, 0, -2], np.int64)
    assert L.ogs_halo_setup(C.byref(h), ids.size, ids.ctypes.data, 0, 0) == _lib.OGS_OK
    assert L.ogs_halo_free(h) == _lib.OGS_OK
    assert L.ogs_halo_setup(C.byref(h), 3, ids.ctypes.data, 9, 0) == _lib.OGS_EINVAL  # method


def test_halo_from_gather_counts(built_lib):
    L = _lib.lib()
    h = C.c_void_p()
    assert L.ogs_halo_setup_from_gather(C.byref(h), 10, 3, 5, 7) == _lib.OGS_OK
    c = _lib.OgsHaloCounts()
    assert L.ogs_halo_get_counts(h, C.byref(c)) == _lib.OGS_OK
    assert (c.N, c.NlocalT, c.NhaloP, c.NhaloT, c.Nhalo, c.Nrecv, c.gathered) == (15, 10, 3, 5, 2, 7, 1)
    L.ogs_halo_free(h)
    assert L.ogs_halo_setup_from_gather(C.byref(h), 10, 6, 5, 0) == _lib.OGS_EINVAL  # NhaloP > NhaloT
    with pytest.raises(_lib.OgsError):
        g = ogs.ogs_t().Setup(4, np.array([1, 2, 1, 3], np.int64), host_only=True)  # ill-defined gather
        ogs.halo_t().SetupFromGather(g)
