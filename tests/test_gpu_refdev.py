"""The device baseline (refdev/okl_equiv.cu: the reference's OKL gatherScatter
algorithm with its 512-member row blocks, ogsKernels.okl:32-81 and
ogsOperator.cpp:447-512) gives the library's results bit for bit: both fold
each row from the op identity over its members in ascending order."""
import numpy as np
import pytest
import torch

from dawgs_gb300 import mesh, ogs
from helpers import random_ids, same_bits, values

pytestmark = pytest.mark.gpu

TC = {np.float32: 0, np.float64: 1, np.int32: 2, np.int64: 3}
OPC = {"add": 0, "mul": 1, "max": 2, "min": 3}


@pytest.fixture(scope="module")
def refdev_mod(cuda):
    import refdev
    refdev.build()
    return refdev


@pytest.mark.parametrize("mname,make", [
    ("box_10x10x10_p3", lambda: mesh.box_ids(10, 10, 10, 3)),
    ("box_permuted_p5", lambda: mesh.permute_elements(mesh.box_ids(8, 6, 5, 5), 5, seed=4)),
    ("random_deg1_to_40", lambda: random_ids(30000, 2500, seed=7, zero_frac=0.05)),
])
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64], ids=lambda t: np.dtype(t).name)
@pytest.mark.parametrize("op", ["add", "max"])
def test_refdev_matches_library(refdev_mod, mname, make, dtype, op):
    ids = make()
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    rd = refdev_mod.RefDevOgs(g)
    for k in (1, 3):
        v = values(k * ids.size, dtype, op, seed=13 + k)
        a = torch.from_numpy(v.copy()).cuda()
        b = torch.from_numpy(v.copy()).cuda()
        g.GatherScatter(a, k, ogs.Op[op.capitalize()], ogs.Sym)
        assert rd.gather_scatter(b.data_ptr(), k, TC[dtype], OPC[op]) == 0
        torch.cuda.synchronize()
        assert same_bits(a.cpu().numpy(), b.cpu().numpy()), (mname, k)


def test_refdev_refuses_rows_above_512(refdev_mod):
    ids = np.concatenate([np.full(600, 5, np.int64), np.arange(10, 20, dtype=np.int64)])
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    with pytest.raises(RuntimeError):
        refdev_mod.RefDevOgs(g)
