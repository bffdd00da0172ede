"""Maps built on the GPU (sort and scans, ogs_dsetup.cu) equal the host
setup's hash-table maps and the oracle's: counts, rowStarts/colIds of the N
and T maps, the layout built from them, ids rewritten by `unique`, and the
GatherScatter results (ogsSetup.cpp:69-190, 333-433, 569-776)."""
import numpy as np
import pytest
import torch

from dawgs_gb300 import _lib, mesh, ogs
from helpers import random_ids, same_bits, signed_ids, values

pytestmark = pytest.mark.gpu

CASES = {
    "c1_box": lambda: mesh.box_ids(10, 10, 10, 3),
    "box_p1": lambda: mesh.box_ids(7, 5, 3, 1),
    "box_permuted": lambda: mesh.permute_elements(mesh.box_ids(6, 5, 4, 4), 4, seed=2),
    "random_multiplicity": lambda: random_ids(20000, 1500, seed=4, zero_frac=0.05),
    "high_degree": lambda: random_ids(5000, 7, seed=8),
    "all_zero": lambda: np.zeros(100, np.int64),
    "empty": lambda: np.zeros(0, np.int64),
    "single": lambda: np.array([42], np.int64),
    "one_zero_then_ids": lambda: np.array([0, 5, 5, 0, 7], np.int64),
    "huge_ids": lambda: np.array([2 ** 62, -(2 ** 62), 3, 2 ** 40, 3, -(2 ** 40), 2 ** 63 - 1], np.int64),
    "partial_32bit": lambda: (random_ids(3000, 400, seed=3) * (2 ** 31 + 11)),
}


def _setup(ids, kind, unique, maps):
    b = ids.copy()
    g = ogs.ogs_t().Setup(b.size, b, None, ogs.Signed if kind == "signed" else ogs.Unsigned,
                          ogs.Auto, unique, maps=maps)
    return g, b


def _same_handle(gd, gh):
    for attr in ("N", "NlocalP", "NlocalT", "Ngather", "NgatherGlobal", "nnzT", "nnzN",
                 "gather_defined", "max_degree"):
        assert getattr(gd, attr) == getattr(gh, attr), attr
    for x, y in zip(gd.maps(), gh.maps()):
        assert np.array_equal(x, y)
    assert gd.layout_stats() == gh.layout_stats()


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("kind,unique", [("unsigned", False), ("signed", False), ("signed", True)])
def test_device_maps_equal_host_and_oracle(cuda, oracle_mod, name, kind, unique):
    ids = CASES[name]()
    if kind == "signed" and ids.size:
        ids = signed_ids(ids, seed=6)
    gd, idd = _setup(ids, kind, unique, "device")
    gh, idh = _setup(ids, kind, unique, "host")
    _same_handle(gd, gh)
    assert np.array_equal(idd, idh)
    a = ids.copy()
    ref = oracle_mod.OracleOgs(a, kind, unique)
    for x, y in zip(gd.maps(), ref.maps()):
        assert np.array_equal(x, y)
    assert np.array_equal(idd, a)


def test_device_maps_bad_id(cuda):
    ids = np.array([1, np.iinfo(np.int64).min, 2], np.int64)
    with pytest.raises(ogs.OgsError) as e:
        _setup(ids, "signed", False, "device")
    assert e.value.status == _lib.OGS_ERANGE


@pytest.mark.parametrize("kind", ["unsigned", "signed"])
def test_device_maps_full_size_gather_scatter(cuda, oracle_mod, kind):
    """24^3 p=7 (7.1M local nodes) and a permuted 32x32x16 p=5 mesh: device and
    host maps give the same handle and bit-identical GatherScatter results; the
    default setup (no maps flag) takes the device path at this size."""
    for ids in (mesh.box_ids(24, 24, 24, 7), mesh.permute_elements(mesh.box_ids(32, 32, 16, 5), 5, seed=2024)):
        if kind == "signed":
            ids = signed_ids(ids, seed=11)
        gd, _ = _setup(ids, kind, False, None)
        gh, _ = _setup(ids, kind, False, "host")
        _same_handle(gd, gh)
        v = values(ids.size, np.float64, "add", seed=5)
        outs = []
        for g in (gd, gh):
            d = torch.from_numpy(v.copy()).cuda()
            g.GatherScatter(d, 1, ogs.Add, ogs.Sym)
            torch.cuda.synchronize()
            outs.append(d.cpu().numpy())
        assert same_bits(outs[0], outs[1])
