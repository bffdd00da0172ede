"""Seeded random cases through every entry point, against the oracle.

Each case draws an id list (size 1..6000, 1..n groups, some zeros, some
negated), a kind, k, a value type, an op and a transpose, and checks bit for
bit: device GatherScatter, host-buffer GatherScatter, Gather and Scatter on
the Signed unique handle of the same ids, and a batched launch over three
such handles.  The draws cover degrees 1..~60 (general tiles), empty meshes
of one node, k of 1, 2, 3 and 5, and every pattern the kernels specialise
(plain and masked builds, register and cp.async pipelines)."""
import numpy as np
import pytest
import torch

from dawgs_gb300 import mesh, ogs
from helpers import first_diff, same_bits, values

pytestmark = pytest.mark.gpu

TYPES = [np.float64, np.float32, np.int64, np.int32]
OPS = ["add", "mul", "max", "min"]
TRANS = {"sym": ogs.Sym, "notrans": ogs.NoTrans, "trans": ogs.Trans}
_TORCH = {np.float32: torch.float32, np.float64: torch.float64, np.int32: torch.int32, np.int64: torch.int64}


def draw(seed):
    r = mesh.splitmix64(np.arange(16, dtype=np.uint64) + np.uint64(1000 * seed + 7))
    n = 1 + int(r[0] % np.uint64(6000))
    groups = 1 + int(r[1] % np.uint64(n))
    ids = mesh.uniform_values(n, np.int64, 1, groups + 1, seed)
    zero = mesh.uniform_values(n, np.int64, 0, 10, seed + 1) == 0
    ids[zero] = 0
    signed = bool(r[2] % np.uint64(2))
    if signed:
        neg = mesh.uniform_values(n, np.int64, 0, 4, seed + 2) == 0
        ids = np.where(neg, -ids, ids)
    k = [1, 2, 3, 5][int(r[3] % np.uint64(4))]
    dtype = TYPES[int(r[4] % np.uint64(4))]
    op = OPS[int(r[5] % np.uint64(4))]
    trans = list(TRANS)[int(r[6] % np.uint64(3))] if signed else "sym"
    return ids, signed, k, dtype, op, trans


@pytest.mark.parametrize("seed", range(40))
def test_random_case_every_entry_point(cuda, oracle_mod, seed):
    ids, signed, k, dtype, op, trans = draw(seed)
    kind = "signed" if signed else "unsigned"
    g = ogs.ogs_t().Setup(ids.size, ids.copy(), None, ogs.Signed if signed else ogs.Unsigned)
    ref = oracle_mod.OracleOgs(ids.copy(), kind)
    v = values(k * ids.size, dtype, op, seed=seed)
    want = ref.gather_scatter(v.copy(), k, op, trans)
    d = torch.from_numpy(v.copy()).cuda()
    g.GatherScatter(d, k, ogs.Op[op.capitalize()], TRANS[trans])
    torch.cuda.synchronize()
    got = d.cpu().numpy()
    assert same_bits(got, want), ("device", first_diff(got, want))
    h = torch.from_numpy(v.copy()).pin_memory()
    g.GatherScatter(h, k, ogs.Op[op.capitalize()], TRANS[trans])
    assert same_bits(h.numpy(), want), ("host", first_diff(h.numpy(), want))

    # Gather (Trans, NoTrans) and Scatter on the Signed unique handle of the same ids
    ua, ub = np.abs(ids), np.abs(ids)
    gu = ogs.ogs_t().Setup(ua.size, ua, None, ogs.Signed, ogs.Auto, True)
    refu = oracle_mod.OracleOgs(ub, "signed", unique=True)
    for tname in ("trans", "notrans"):
        gw = np.zeros(k * refu.Ngather, dtype)
        refu.gather(gw, v, k, op, tname)
        dgv = torch.zeros(k * gu.Ngather, dtype=_TORCH[dtype], device="cuda")
        gu.Gather(dgv, torch.from_numpy(v.copy()).cuda(), k, ogs.Op[op.capitalize()], TRANS[tname])
        torch.cuda.synchronize()
        assert same_bits(dgv.cpu().numpy(), gw), ("gather", tname)
        v0 = values(k * ids.size, dtype, "add", seed=seed + 100)
        dv = torch.from_numpy(v0.copy()).cuda()
        gu.Scatter(dv, torch.from_numpy(gw).cuda(), k, TRANS[tname])
        torch.cuda.synchronize()
        assert same_bits(dv.cpu().numpy(), refu.scatter(v0.copy(), gw, k, tname)), ("scatter", tname)


@pytest.mark.parametrize("seed", range(12))
def test_random_batches(cuda, oracle_mod, seed):
    """Three random handles of one value type in one batched launch."""
    entries, wants, fields = [], [], []
    dtype = TYPES[seed % 4]
    for j in range(3):
        ids, signed, k, _, op, trans = draw(100 + 3 * seed + j)
        kind = "signed" if signed else "unsigned"
        g = ogs.ogs_t().Setup(ids.size, ids.copy(), None, ogs.Signed if signed else ogs.Unsigned)
        ref = oracle_mod.OracleOgs(ids.copy(), kind)
        v = values(k * ids.size, dtype, op, seed=seed * 10 + j)
        wants.append(ref.gather_scatter(v.copy(), k, op, trans))
        d = torch.from_numpy(v.copy()).cuda()
        fields.append(d)
        entries.append((g, d, k, ogs.Op[op.capitalize()], TRANS[trans]))
    b = ogs.ogs_batch_t(entries)
    b.GatherScatter()
    torch.cuda.synchronize()
    for d, w in zip(fields, wants):
        got = d.cpu().numpy()
        assert same_bits(got, w), first_diff(got, w)
