"""Emulated multi-rank GatherScatter on the GPU (dawgs_gb300/ranks.py): every
rank's gatherLocal, gatherHalo and postmpi are library operators built from
maps (ogs_setup_maps), the send buffers are packed and the exchange is done
by ogs_extract, and postmpi's Gather runs in place.  The fields equal the
oracle's restatement of the reference's multi-rank fold order bit for bit, and
the single-rank result of the whole mesh exactly for integer types and
Max/Min (within rounding for floating-point Add and Mul, whose order the rank
split changes)."""
import numpy as np
import pytest
import torch

import oracle
from dawgs_gb300 import mesh, ogs, ranks
from helpers import first_diff, same_bits, values
from oracle import ranks as oranks

pytestmark = pytest.mark.gpu

PARTS = [((6, 5, 4, 3), 2, "slabs"), ((6, 5, 4, 3), 3, "random"), ((5, 4, 4, 2), 4, "random"),
         ((8, 4, 4, 2), 8, "slabs"), ((4, 4, 3, 1), 5, "random")]


@pytest.fixture(scope="module")
def setups(cuda):
    out = {}
    for box, R, how in PARTS:
        parts = oranks.partition_box(*box, R, how=how, seed=17)
        out[(box, R, how)] = (parts, ranks.ranks_ogs_t(parts))
    return out


@pytest.mark.parametrize("key", PARTS, ids=lambda p: f"{p[0]}-{p[1]}-{p[2]}")
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64], ids=lambda t: np.dtype(t).name)
@pytest.mark.parametrize("op", ["add", "mul", "max", "min"])
def test_ranks_match_oracle(setups, oracle_mod, key, dtype, op):
    parts, rk = setups[key]
    for k in (1, 3):
        vs = [values(k * p.size, dtype, op, seed=40 + i + 7 * k) for i, p in enumerate(parts)]
        want = oranks.ranks_gather_scatter(parts, vs, k, op)
        ds = [torch.from_numpy(v.copy()).cuda() for v in vs]
        rk.GatherScatter(ds, k, ogs.Op[op.capitalize()])
        torch.cuda.synchronize()
        for r, (d, w) in enumerate(zip(ds, want)):
            got = d.cpu().numpy()
            assert same_bits(got, w), (key, k, r, first_diff(got, w))
        if np.dtype(dtype).kind == "i" or op in ("max", "min"):
            # the rank split does not change exact folds: whole-mesh single-rank result
            g = np.concatenate(parts)
            single = oracle.OracleOgs(g.copy(), "unsigned").gather_scatter(np.concatenate(vs), k, op, "sym")
            assert same_bits(np.concatenate([d.cpu().numpy() for d in ds]), single)


MODES = [("signed", "sym", "add"), ("signed", "notrans", "add"), ("signed", "trans", "mul"),
         ("signed", "notrans", "max"), ("halo", "notrans", "add"), ("halo", "trans", "add")]
_T = {"sym": ogs.Sym, "notrans": ogs.NoTrans, "trans": ogs.Trans}


@pytest.mark.parametrize("key", PARTS[:4], ids=lambda p: f"{p[0]}-{p[1]}-{p[2]}")
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int64], ids=lambda t: np.dtype(t).name)
@pytest.mark.parametrize("kind,trans,op", MODES)
def test_signed_and_halo_ranks_match_oracle(cuda, oracle_mod, key, dtype, kind, trans, op):
    """ogs_t GatherScatter on Signed ranks and halo_t Exchange (NoTrans) /
    Combine (Trans) on Halo ranks."""
    box, R, how = key
    parts = oranks.signed_parts(oranks.partition_box(*box, R, how=how, seed=17), 5, kind)
    rk = ranks.ranks_ogs_t(parts, ranks.SIGNED if kind == "signed" else ranks.HALO)
    for k in (1, 2):
        vs = [values(k * p.size, dtype, op, seed=70 + i + 3 * k) for i, p in enumerate(parts)]
        want = oranks.ranks_gather_scatter(parts, vs, k, op, kind, trans)
        ds = [torch.from_numpy(v.copy()).cuda() for v in vs]
        if kind == "signed":
            rk.GatherScatter(ds, k, ogs.Op[op.capitalize()], _T[trans])
        elif trans == "notrans":
            rk.Exchange(ds, k)
        else:
            rk.Combine(ds, k)
        torch.cuda.synchronize()
        for r, (d, w) in enumerate(zip(ds, want)):
            got = d.cpu().numpy()
            assert same_bits(got, w), (key, kind, trans, k, r, first_diff(got, w))


def test_ranks_float_add_close_to_single_rank(setups, oracle_mod):
    parts, rk = setups[((5, 4, 4, 2), 4, "random")]
    vs = [values(p.size, np.float64, "add", seed=3 + i) for i, p in enumerate(parts)]
    ds = [torch.from_numpy(v.copy()).cuda() for v in vs]
    rk.GatherScatter(ds, 1, ogs.Add)
    single = oracle.OracleOgs(np.concatenate(parts), "unsigned").gather_scatter(np.concatenate(vs), 1, "add", "sym")
    got = np.concatenate([d.cpu().numpy() for d in ds])
    assert np.allclose(got, single, rtol=1e-13, atol=1e-15)  # fp64 Add, fold order changed by the split


def test_ranks_larger_mesh_start_finish(oracle_mod, cuda):
    """12^3 p=4 over 8 ranks (random elements), Start and Finish called apart."""
    parts = oranks.partition_box(12, 12, 12, 4, 8, how="random", seed=5)
    rk = ranks.ranks_ogs_t(parts)
    vs = [values(p.size, np.float64, "add", seed=60 + i) for i, p in enumerate(parts)]
    want = oranks.ranks_gather_scatter(parts, vs, 1, "add")
    ds = [torch.from_numpy(v.copy()).cuda() for v in vs]
    rk.GatherScatterStart(ds, 1, ogs.Add)
    rk.GatherScatterFinish(ds, 1, ogs.Add)
    torch.cuda.synchronize()
    for d, w in zip(ds, want):
        assert same_bits(d.cpu().numpy(), w)


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64], ids=lambda t: np.dtype(t).name)
def test_extract(cuda, dtype):
    rng = np.random.default_rng(1)
    for k in (1, 3):
        q = values(1000 * k, dtype, "add", seed=2)
        ids = rng.integers(0, 1000, 777).astype(np.int32)
        out = torch.zeros(777 * k, dtype=torch.from_numpy(q).dtype, device="cuda")
        ogs.extract(out, torch.from_numpy(q).cuda(), torch.from_numpy(ids).cuda(), k)
        want = q.reshape(1000, k)[ids].reshape(-1)
        assert same_bits(out.cpu().numpy(), want)


def test_operator_with_shared_column_refuses_writes(cuda):
    g = ogs.ogs_t().SetupMaps(4, [0, 2, 4], [0, 1, 1, 3])   # local node 1 in two rows
    v = torch.ones(4, dtype=torch.float64, device="cuda")
    gv = torch.zeros(2, dtype=torch.float64, device="cuda")
    g.Gather(gv, v, 1, ogs.Add, ogs.Trans)
    torch.cuda.synchronize()
    assert gv.cpu().tolist() == [2.0, 2.0]
    with pytest.raises(ogs.OgsError):
        g.GatherScatter(v, 1, ogs.Add, ogs.Sym)
    with pytest.raises(ogs.OgsError):
        g.Scatter(v, gv, 1, ogs.Trans)


@pytest.mark.parametrize("op,ident", [("add", 0.0), ("max", -np.finfo(np.float64).max)])
def test_operator_empty_rows_gather_identity(cuda, op, ident):
    g = ogs.ogs_t().SetupMaps(4, [0, 2, 2, 3, 3], [0, 2, 1])  # rows 1 and 3 empty
    v = torch.tensor([1.0, 2.0, 3.0, 4.0], dtype=torch.float64, device="cuda")
    gv = torch.full((4,), 7.0, dtype=torch.float64, device="cuda")
    g.Gather(gv, v, 1, ogs.Op[op.capitalize()], ogs.Trans)
    torch.cuda.synchronize()
    first = 4.0 if op == "add" else 3.0
    assert gv.cpu().tolist() == [first, ident, 2.0, ident]
    g.GatherScatter(v, 1, ogs.Op[op.capitalize()], ogs.Sym)  # empty rows write nothing
    torch.cuda.synchronize()
    assert v.cpu().tolist() == [first, 2.0, first, 4.0]


@pytest.mark.parametrize("key", PARTS[:4], ids=lambda p: f"{p[0]}-{p[1]}-{p[2]}")
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int64], ids=lambda t: np.dtype(t).name)
@pytest.mark.parametrize("kind", ["signed", "unsigned"])
@pytest.mark.parametrize("trans", ["notrans", "trans"])
def test_gathered_halo_matches_oracle(cuda, oracle_mod, key, dtype, kind, trans):
    """halo_t made from a gather: Exchange (NoTrans) and Combine (Trans) on
    gathered vectors [local rows | halo rows]."""
    box, R, how = key
    parts = oranks.partition_box(*box, R, how=how, seed=17)
    if kind == "signed":
        parts = oranks.signed_parts(parts, 5, "halo")
    rk = ranks.ranks_ogs_t(parts, ranks.SIGNED if kind == "signed" else ranks.UNSIGNED)
    for k in (1, 3):
        gvs = [values(n * k, dtype, "add", seed=90 + i + k) for i, n in enumerate(rk.gathered_sizes())]
        want = oranks.gathered_exchange(parts, gvs, k, kind, trans)
        ds = [torch.from_numpy(g.copy()).cuda() for g in gvs]
        (rk.GatheredExchange if trans == "notrans" else rk.GatheredCombine)(ds, k)
        torch.cuda.synchronize()
        for r, (d, w) in enumerate(zip(ds, want)):
            got = d.cpu().numpy()
            assert same_bits(got, w), (key, kind, trans, k, r, first_diff(got, w))


@pytest.mark.parametrize("key", PARTS[:4], ids=lambda p: f"{p[0]}-{p[1]}-{p[2]}")
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32], ids=lambda t: np.dtype(t).name)
@pytest.mark.parametrize("trans", ["trans", "notrans", "sym"])
def test_ranks_gather_and_scatter_match_oracle(cuda, oracle_mod, key, dtype, trans):
    """Multi-rank ogs_t Gather (Trans exchanges) and Scatter (NoTrans
    exchanges) on a Signed setup with one positive copy per id."""
    box, R, how = key
    parts = oranks.signed_parts(oranks.partition_box(*box, R, how=how, seed=17), 5, "halo")
    rk = ranks.ranks_ogs_t(parts, ranks.SIGNED)
    assert rk.gather_defined()
    T = {"trans": ogs.Trans, "notrans": ogs.NoTrans, "sym": ogs.Sym}[trans]
    for k in (1, 2):
        for op in ("add", "max"):
            vs = [values(p.size * k, dtype, op, seed=110 + i + k) for i, p in enumerate(parts)]
            want = oranks.ranks_gather(parts, vs, k, op, trans)
            gds = [torch.zeros(n * k, dtype=torch.from_numpy(vs[0]).dtype, device="cuda")
                   for n in rk.gather_sizes(T)]
            rk.Gather(gds, [torch.from_numpy(v).cuda() for v in vs], k, ogs.Op[op.capitalize()], T)
            torch.cuda.synchronize()
            for r, (d, w) in enumerate(zip(gds, want)):
                got = d.cpu().numpy()
                assert same_bits(got, w), ("gather", key, trans, op, k, r, first_diff(got, w))
        gvs = [values(n * k, dtype, "add", seed=130 + i + k) for i, n in enumerate(rk.gather_sizes(T))]
        v0 = [values(p.size * k, dtype, "add", seed=150 + i) for i, p in enumerate(parts)]
        want = oranks.ranks_scatter(parts, v0, gvs, k, trans)
        ds = [torch.from_numpy(v.copy()).cuda() for v in v0]
        rk.Scatter(ds, [torch.from_numpy(g).cuda() for g in gvs], k, T)
        torch.cuda.synchronize()
        for r, (d, w) in enumerate(zip(ds, want)):
            got = d.cpu().numpy()
            assert same_bits(got, w), ("scatter", key, trans, k, r, first_diff(got, w))


def test_ranks_gather_refused_when_not_defined(cuda):
    parts = oranks.partition_box(4, 4, 3, 2, 2, how="slabs")  # Unsigned: every copy positive
    rk = ranks.ranks_ogs_t(parts, ranks.UNSIGNED)
    assert not rk.gather_defined()
    with pytest.raises(ValueError):
        rk.Gather([torch.zeros(1, device="cuda")] * 2, [torch.zeros(p.size, device="cuda") for p in parts], 1)

