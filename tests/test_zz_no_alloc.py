"""ogs_gather_scatter_host_noalloc, the host-buffer GatherScatter for callers
that cannot let a library allocate device memory while they run (it stages
the field in a fixed device array instead of a cudaMalloc'd buffer).  Called
through the C ABI twice in a row, it must give exactly what
ogs_gather_scatter_host gives for the same inputs: every type, Add and Max,
every transpose on a Signed handle, interleaved k, and rows above degree 8.
It must refuse what ogs_gather_scatter_host refuses.  This file sorts last
so that a run stopping at the first failure has already run every other
test."""
import ctypes as C

import numpy as np
import pytest

from dawgs_gb300 import _lib, mesh
from helpers import first_diff, random_ids, same_bits, signed_ids, values

pytestmark = pytest.mark.gpu

TYPE_CODE = {np.float32: 0, np.float64: 1, np.int32: 2, np.int64: 3}
OP_CODE = {"add": 0, "max": 2}
TRANS_CODE = {"sym": 0, "notrans": 1, "trans": 2}


def _setup(L, ids, kind=0, unique=0):
    h = C.c_void_p()
    assert L.ogs_setup(C.byref(h), ids.size, ids.ctypes.data, kind, 0, unique, 0) == _lib.OGS_OK, \
        L.ogs_last_error_string()
    return h


def _stream():
    import torch
    return torch.cuda.current_stream().cuda_stream


def _compare_twice(L, h, cases):
    """Each case through ogs_gather_scatter_host, then every case again through
    the no-allocation entry point, twice in a row."""
    stream = _stream()
    wants, inputs = [], []
    for dtype, k, op, trans, n, seed in cases:
        v = values(k * n, dtype, op, seed=seed)
        w = v.copy()
        st = L.ogs_gather_scatter_host(h, w.ctypes.data, k, TYPE_CODE[dtype], OP_CODE[op], TRANS_CODE[trans], stream)
        assert st == _lib.OGS_OK, L.ogs_last_error_string()
        inputs.append(v)
        wants.append(w)
    for _ in range(2):
        for (dtype, k, op, trans, _, _), v, want in zip(cases, inputs, wants):
            got = v.copy()
            st = L.ogs_gather_scatter_host_noalloc(h, got.ctypes.data, k, TYPE_CODE[dtype], OP_CODE[op],
                                                   TRANS_CODE[trans], stream)
            assert st == _lib.OGS_OK, L.ogs_last_error_string()
            assert same_bits(got, want), (np.dtype(dtype).name, k, op, trans, first_diff(got, want))


def test_noalloc_matches_host_entry_point_twice(cuda):
    L = _lib.lib()
    ids = mesh.box_ids(10, 10, 10, 3)
    h = _setup(L, ids)
    try:
        _compare_twice(L, h, [(np.float64, 1, "add", "sym", ids.size, 501),
                              (np.float64, 3, "add", "sym", ids.size, 502)])
    finally:
        L.ogs_free(h)


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32, np.int64])
def test_noalloc_signed_every_type_op_and_transpose(cuda, dtype):
    L = _lib.lib()
    ids = signed_ids(mesh.box_ids(6, 5, 4, 3), seed=7)
    h = _setup(L, ids, kind=1)
    try:
        cases = [(dtype, k, op, trans, ids.size, 600 + 7 * j)
                 for j, (k, op, trans) in enumerate((k, op, t) for k in (1, 2) for op in ("add", "max")
                                                    for t in ("sym", "notrans", "trans"))]
        _compare_twice(L, h, cases)
    finally:
        L.ogs_free(h)


def test_noalloc_rows_above_degree_eight(cuda):
    """Rows of up to a few hundred members run on the general-tile kernel."""
    L = _lib.lib()
    ids = random_ids(20000, 150, seed=31, zero_frac=0.05)
    h = _setup(L, ids)
    try:
        _compare_twice(L, h, [(np.float64, 1, "add", "sym", ids.size, 701),
                              (np.float32, 3, "max", "sym", ids.size, 702),
                              (np.int64, 1, "add", "sym", ids.size, 703)])
    finally:
        L.ogs_free(h)


def test_noalloc_refuses_what_the_host_entry_point_refuses(cuda):
    L = _lib.lib()
    v = np.zeros(64, np.float64)
    # a handle from ogs_gslib_setup keeps gslib's member order and fold rules
    ids = np.repeat(np.arange(1, 33, dtype=np.int64), 2)
    g = C.c_void_p()
    assert L.ogs_gslib_setup(C.byref(g), ids.ctypes.data, ids.size, 0) == _lib.OGS_OK
    try:
        assert L.ogs_gather_scatter_host_noalloc(g, v.ctypes.data, 1, 1, 0, 0, None) == _lib.OGS_EINVAL
        assert b"ogs_gslib_setup" in L.ogs_last_error_string()
    finally:
        L.ogs_free(g)
    # caller maps in which local node 0 sits in two rows
    rs = np.array([0, 2, 4], np.int32)
    ci = np.array([0, 1, 0, 2], np.int32)
    m = C.c_void_p()
    assert L.ogs_setup_maps(C.byref(m), 64, 2, 2, None, None, rs.ctypes.data, ci.ctypes.data, 0) == _lib.OGS_OK
    try:
        assert L.ogs_gather_scatter_host_noalloc(m, v.ctypes.data, 1, 1, 0, 0, None) == _lib.OGS_EINVAL
        assert b"two rows" in L.ogs_last_error_string()
    finally:
        L.ogs_free(m)


def test_noalloc_rejects_fields_beyond_its_array(cuda):
    L = _lib.lib()
    ids = mesh.box_ids(24, 24, 24, 7)  # 7,077,888 nodes: 56.6 MB of fp64 > 32 MiB
    h = _setup(L, ids)
    try:
        v = np.zeros(ids.size)
        assert L.ogs_gather_scatter_host_noalloc(h, v.ctypes.data, 1, 1, 0, 0, None) == _lib.OGS_ERANGE
        assert b"staging array" in L.ogs_last_error_string()
    finally:
        L.ogs_free(h)
