"""ogs_gather_scatter_host_noalloc, the host-buffer GatherScatter for callers
that cannot let a library allocate device memory while they run (it stages
the field in a fixed device array instead of a cudaMalloc'd buffer).  Called
through the C ABI twice in a row, it must give exactly what
ogs_gather_scatter_host gives for the same inputs.  This file sorts last so
that a run stopping at the first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from dawgs_gb300 import _lib, mesh
from helpers import first_diff, same_bits, values

pytestmark = pytest.mark.gpu


def _setup(L, ids):
    h = C.c_void_p()
    assert L.ogs_setup(C.byref(h), ids.size, ids.ctypes.data, 0, 0, 0, 0) == _lib.OGS_OK
    return h


def test_noalloc_matches_host_entry_point_twice(cuda):
    import torch
    L = _lib.lib()
    ids = mesh.box_ids(10, 10, 10, 3)
    h = _setup(L, ids)
    stream = torch.cuda.current_stream().cuda_stream
    try:
        cases = [(np.float64, 1, 501), (np.float64, 3, 502)]
        wants, inputs = [], []
        for dtype, k, seed in cases:  # the existing entry point first
            v = values(k * ids.size, dtype, "add", seed=seed)
            w = v.copy()
            assert L.ogs_gather_scatter_host(h, w.ctypes.data, k, 1, 0, 0, stream) == _lib.OGS_OK
            inputs.append(v)
            wants.append(w)
        for (dtype, k, _), v, want in zip(cases, inputs, wants):  # then two no-allocation calls in a row
            got = v.copy()
            st = L.ogs_gather_scatter_host_noalloc(h, got.ctypes.data, k, 1, 0, 0, stream)
            assert st == _lib.OGS_OK, L.ogs_last_error_string()
            assert same_bits(got, want), (k, first_diff(got, want))
    finally:
        L.ogs_free(h)


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
