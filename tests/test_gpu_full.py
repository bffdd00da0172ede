"""Full-size single-mesh runs: the 24^3 degree sweep p=1..15 against the
oracle bit for bit (fp64 Add GatherScatter at every p; fp32 Add and int64 Max
at p=11 and p=15; Gather (Trans) and Scatter (NoTrans) on the Signed unique
handle at p=7 and p=15), plus size-independent properties at p=15 (56.6M
local nodes).

The contract is the reference host operator's: each row folds from the op
identity over its members in ascending local index (ogsOperator.cpp:311-360)
and rows are numbered by first appearance (ogsSetup.cpp:406-433)."""
import numpy as np
import pytest
import torch

from dawgs_gb300 import mesh, ogs
from helpers import first_diff, same_bits, values

pytestmark = pytest.mark.gpu


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


_BOX = {}


def box(oracle_mod, p):
    """(ids, library handle, oracle handle) of the 24^3 box at degree p, one at a time."""
    if p not in _BOX:
        _BOX.clear()
        ids = mesh.box_ids(24, 24, 24, p)
        _BOX[p] = (ids, ogs.ogs_t().Setup(ids.size, ids.copy()), oracle_mod.OracleOgs(ids.copy(), "unsigned"))
    return _BOX[p]


def check_gs(g, ref, n, dtype, op, seed):
    v = values(n, dtype, op, seed=seed)
    d = dev(v)
    g.GatherScatter(d, 1, ogs.Op[op.capitalize()], ogs.Sym)
    got = d.cpu().numpy()
    del d
    want = ref.gather_scatter(v, 1, op, "sym")
    assert same_bits(got, want), (np.dtype(dtype).name, op, first_diff(got, want))


@pytest.mark.parametrize("p", list(range(1, 16)))
def test_sweep_24cubed_fp64_add_matches_oracle(cuda, oracle_mod, p):
    ids, g, ref = box(oracle_mod, p)
    check_gs(g, ref, ids.size, np.float64, "add", p)


@pytest.mark.parametrize("p", [11, 15])
@pytest.mark.parametrize("dtype,op", [(np.float32, "add"), (np.int64, "max")])
def test_sweep_24cubed_other_types_match_oracle(cuda, oracle_mod, p, dtype, op):
    ids, g, ref = box(oracle_mod, p)
    check_gs(g, ref, ids.size, dtype, op, 100 + p)


def test_c2_all_ops_and_types(cuda, oracle_mod):
    """24^3 p=7: fp32 Add, int32/int64 Min/Max (U[-2^30,2^30)), Gather(Trans) and
    Scatter(NoTrans) on the signed unique handle, fused GS on the unsigned one."""
    ids, g, ref = box(oracle_mod, 7)
    for dtype, op in ((np.float32, "add"), (np.int32, "min"), (np.int32, "max"),
                      (np.int64, "min"), (np.int64, "max"), (np.float64, "mul")):
        check_gs(g, ref, ids.size, dtype, op, 5)
    check_signed_gather_scatter(oracle_mod, ids, ref, seed=9)


def check_signed_gather_scatter(oracle_mod, ids, ref, seed):
    ua, ub = ids.copy(), ids.copy()
    sg = ogs.ogs_t().Setup(ua.size, ua, None, ogs.Signed, ogs.Auto, True)
    sref = oracle_mod.OracleOgs(ub, "signed", unique=True)
    v = values(ids.size, np.float64, "add", seed=seed)
    gv = torch.zeros(sg.Ngather, dtype=torch.float64, device="cuda")
    sg.Gather(gv, dev(v), 1, ogs.Add, ogs.Trans)
    want = np.zeros(sref.Ngather)
    sref.gather(want, v, 1, "add", "trans")
    got = gv.cpu().numpy()
    assert same_bits(got, want), first_diff(got, want)
    out = torch.zeros(ids.size, dtype=torch.float64, device="cuda")
    sg.Scatter(out, gv, 1, ogs.NoTrans)
    got = out.cpu().numpy()
    want_s = sref.scatter(np.zeros(ids.size), want, 1, "notrans")
    assert same_bits(got, want_s), first_diff(got, want_s)
    # Gather then Scatter equals the fused GatherScatter (dawgsMain.cpp:399-405)
    fused = ref.gather_scatter(v.copy(), 1, "add", "sym")
    assert same_bits(got, fused), first_diff(got, fused)
    sg.Free()


def test_p15_gather_scatter_signed_match_oracle(cuda, oracle_mod):
    ids, _, ref = box(oracle_mod, 15)
    check_signed_gather_scatter(oracle_mod, ids, ref, seed=151)


def test_p15_properties(cuda, oracle_mod):
    """56.6M local nodes: GS is idempotent for Max/Min, exact under scaling by 2
    for Add, and Gather then Scatter equals the fused call."""
    ids, g, _ = box(oracle_mod, 15)
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
    del once, twice, b
    sa = ids.copy()
    sg = ogs.ogs_t().Setup(sa.size, sa, None, ogs.Signed, ogs.Auto, True)
    gv = torch.zeros(sg.Ngather, dtype=torch.float64, device="cuda")
    sg.Gather(gv, v, 1, ogs.Add, ogs.Trans)
    out = torch.empty_like(v)
    sg.Scatter(out, gv, 1, ogs.NoTrans)
    assert torch.equal(out, a)
    sg.Free()
