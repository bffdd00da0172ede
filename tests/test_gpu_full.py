"""Full-size single-mesh runs: the 24^3 degree sweep (p=1..7 against the oracle
bit for bit; p=15, 56.6M local nodes, through size-independent properties)."""
import numpy as np
import pytest
import torch

from dawgs_gb300 import mesh, ogs
from helpers import first_diff, same_bits, values

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6, 7])
def test_sweep_24cubed_fp64_add_matches_oracle(cuda, oracle_mod, p):
    ids = mesh.box_ids(24, 24, 24, p)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    ref = oracle_mod.OracleOgs(ids.copy(), "unsigned")
    v = values(ids.size, np.float64, "add", seed=p)
    d = dev(v)
    g.GatherScatter(d, 1, ogs.Add, ogs.Sym)
    got = d.cpu().numpy()
    want = ref.gather_scatter(v.copy(), 1, "add", "sym")
    assert same_bits(got, want), first_diff(got, want)


def test_c2_all_ops_and_types(cuda, oracle_mod):
    """24^3 p=7: fp32 Add, int32/int64 Min/Max (U[-2^30,2^30)), Gather(Trans) and
    Scatter(NoTrans) on the signed unique handle, fused GS on the unsigned one."""
    ids = mesh.box_ids(24, 24, 24, 7)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    ref = oracle_mod.OracleOgs(ids.copy(), "unsigned")
    for dtype, op in ((np.float32, "add"), (np.int32, "min"), (np.int32, "max"),
                      (np.int64, "min"), (np.int64, "max"), (np.float64, "mul")):
        v = values(ids.size, dtype, op, seed=5)
        d = dev(v)
        g.GatherScatter(d, 1, ogs.Op[op.capitalize()], ogs.Sym)
        got = d.cpu().numpy()
        assert same_bits(got, ref.gather_scatter(v.copy(), 1, op, "sym")), (dtype, op)
    ua, ub = ids.copy(), ids.copy()
    sg = ogs.ogs_t().Setup(ua.size, ua, None, ogs.Signed, ogs.Auto, True)
    sref = oracle_mod.OracleOgs(ub, "signed", unique=True)
    v = values(ids.size, np.float64, "add", seed=9)
    gv = torch.zeros(sg.Ngather, dtype=torch.float64, device="cuda")
    sg.Gather(gv, dev(v), 1, ogs.Add, ogs.Trans)
    want = np.zeros(sref.Ngather)
    sref.gather(want, v, 1, "add", "trans")
    assert same_bits(gv.cpu().numpy(), want)
    out = torch.zeros(ids.size, dtype=torch.float64, device="cuda")
    sg.Scatter(out, gv, 1, ogs.NoTrans)
    assert same_bits(out.cpu().numpy(), sref.scatter(np.zeros(ids.size), want, 1, "notrans"))
    # Gather then Scatter equals the fused GatherScatter (dawgsMain.cpp:399-405)
    assert same_bits(out.cpu().numpy(), ref.gather_scatter(v.copy(), 1, "add", "sym"))


def test_p15_properties(cuda):
    """56.6M local nodes: GS is idempotent for Max/Min, exact under scaling by 2
    for Add, and Gather then Scatter equals the fused call."""
    ids = mesh.box_ids(24, 24, 24, 15)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    assert g.N == 56623104
    v = dev(values(ids.size, np.float64, "add", seed=15))
    once = v.clone()
    g.GatherScatter(once, 1, ogs.Max, ogs.Sym)
    twice = once.clone()
    g.GatherScatter(twice, 1, ogs.Max, ogs.Sym)
    assert torch.equal(once, twice)
    a = v.clone()
    g.GatherScatter(a, 1, ogs.Add, ogs.Sym)
    b = v * 2
    g.GatherScatter(b, 1, ogs.Add, ogs.Sym)
    assert torch.equal(a * 2, b)
    # every node of a row holds the same value: the max over a row equals each member
    assert torch.equal(once >= v, torch.ones_like(v, dtype=torch.bool))
    sa = ids.copy()
    sg = ogs.ogs_t().Setup(sa.size, sa, None, ogs.Signed, ogs.Auto, True)
    gv = torch.zeros(sg.Ngather, dtype=torch.float64, device="cuda")
    sg.Gather(gv, v, 1, ogs.Add, ogs.Trans)
    out = torch.empty_like(v)
    sg.Scatter(out, gv, 1, ogs.NoTrans)
    assert torch.equal(out, a)
