"""Batched gather-scatter: many meshes of uneven size, degree, k and op in one
persistent launch give, entry by entry, exactly the oracle's result -- the
same as one plain call per mesh -- with and without CUDA-graph replay, after
tuning, and after re-pointing the entries at new fields."""
import numpy as np
import pytest
import torch

from dawgs_gb300 import mesh, ogs
from helpers import first_diff, random_ids, same_bits, signed_ids, values

pytestmark = pytest.mark.gpu

OPS = [ogs.Add, ogs.Mul, ogs.Max, ogs.Min]
OPN = {ogs.Add: "add", ogs.Mul: "mul", ogs.Max: "max", ogs.Min: "min"}
TRN = {ogs.Sym: "sym", ogs.NoTrans: "notrans", ogs.Trans: "trans"}


def build_mix(oracle_mod, count, seed, dtype, signed=False, general=False, ks=(1, 2, 3, 4)):
    out = []
    for j, (nx, ny, nz, p) in enumerate(mesh.mesh_mix(count, seed, lo=1, hi=6, pmax=5)):
        ids = mesh.box_ids(nx, ny, nz, p)
        if general and j % 5 == 0:
            ids = np.concatenate([ids, random_ids(3000, 60, seed=j) + 10 ** 7])
        kind = ogs.Unsigned
        if signed and j % 2:
            ids = signed_ids(ids, seed=j)
            kind = ogs.Signed
        g = ogs.ogs_t().Setup(ids.size, ids.copy(), None, kind)
        ref = oracle_mod.OracleOgs(ids.copy(), "signed" if kind == ogs.Signed else "unsigned")
        k = ks[j % len(ks)]
        op = OPS[j % 4]
        trans = [ogs.Sym, ogs.NoTrans, ogs.Trans][j % 3] if kind == ogs.Signed else ogs.Sym
        v = values(k * ids.size, dtype, OPN[op], seed=100 + j)
        out.append((g, ref, v, k, op, trans))
    return out


def check(mix, fields):
    for (g, ref, v, k, op, trans), d in zip(mix, fields):
        want = ref.gather_scatter(v.copy(), k, OPN[op], TRN[trans])
        got = d.cpu().numpy()
        assert same_bits(got, want), (g.N, k, OPN[op], first_diff(got, want))


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64], ids=lambda t: np.dtype(t).name)
def test_batch_matches_oracle_per_entry(cuda, oracle_mod, dtype):
    mix = build_mix(oracle_mod, 24, seed=7, dtype=dtype, signed=True, general=True)
    fields = [torch.from_numpy(v.copy()).cuda() for (_, _, v, _, _, _) in mix]
    b = ogs.ogs_batch_t([(g, d, k, op, trans) for (g, _, _, k, op, trans), d in zip(mix, fields)])
    assert b.items > 0
    b.GatherScatter()
    torch.cuda.synchronize()
    check(mix, fields)


def test_batch_graph_tune_and_new_fields(cuda, oracle_mod):
    mix = build_mix(oracle_mod, 40, seed=11, dtype=np.float64)
    fields = [torch.from_numpy(v.copy()).cuda() for (_, _, v, _, _, _) in mix]
    b = ogs.ogs_batch_t([(g, d, k, op, trans) for (g, _, _, k, op, trans), d in zip(mix, fields)], graph=True)
    cfg = b.tune(use_cache=False)
    assert cfg["block"] in (128, 256) and cfg["ctas_per_sm"] >= 1 and cfg["ms"] > 0 and not cfg["from_cache"]
    for d, (_, _, v, _, _, _) in zip(fields, mix):  # the tuner timed on scratch copies
        assert same_bits(d.cpu().numpy(), v)
    assert b.tune()["from_cache"]  # the same key again
    b.GatherScatter()  # captures
    torch.cuda.synchronize()
    check(mix, fields)
    for d, (_, _, v, _, _, _) in zip(fields, mix):
        d.copy_(torch.from_numpy(v))
    b.GatherScatter()  # replays
    torch.cuda.synchronize()
    check(mix, fields)
    fresh = [torch.from_numpy(v.copy()).cuda() for (_, _, v, _, _, _) in mix]
    b.set_fields(fresh)
    b.GatherScatter()
    torch.cuda.synchronize()
    check(mix, fresh)


def test_batch_of_one_equals_plain_call(cuda, oracle_mod):
    ids = mesh.box_ids(12, 10, 8, 5)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    v = values(2 * ids.size, np.float64, "add", seed=3)
    a = torch.from_numpy(v.copy()).cuda()
    c = torch.from_numpy(v.copy()).cuda()
    ogs.ogs_batch_t([(g, a, 2, ogs.Add, ogs.Sym)]).GatherScatter()
    g.GatherScatter(c, 2, ogs.Add, ogs.Sym)
    torch.cuda.synchronize()
    assert torch.equal(a, c)


@pytest.mark.parametrize("cfg", [dict(), dict(block=128, ctas_per_sm=3), dict(occupancy=3, ctas_per_sm=6),
                                 dict(block=128, occupancy=3, ctas_per_sm=5),
                                 dict(pipeline=1), dict(pipeline=1, occupancy=3, ctas_per_sm=2),
                                 dict(solo_items=1, solo_streams=3), dict(solo_items=40, solo_streams=8, ctas_per_sm=1)],
                         ids=["default", "block128", "occ3", "block128-occ3", "ring", "ring-occ3", "all-solo", "mixed"])
@pytest.mark.parametrize("signed", [True, False], ids=["masked", "plain"])
def test_batch_configurations_give_the_same_results(cuda, oracle_mod, cfg, signed):
    """Every configuration the tuner may choose -- block size, CTAs per SM,
    entries run alone on the single-mesh kernel over parallel graph branches
    -- gives each entry the oracle's result, for a batch with Signed entries
    (masks and store modes) and for an all-Sym Unsigned batch (the kernels
    built without those branches)."""
    mix = build_mix(oracle_mod, 30, seed=13, dtype=np.float64, signed=signed, general=True)
    fields = [torch.from_numpy(v.copy()).cuda() for (_, _, v, _, _, _) in mix]
    b = ogs.ogs_batch_t([(g, d, k, op, trans) for (g, _, _, k, op, trans), d in zip(mix, fields)], graph=True)
    b.set_config(**cfg)
    got = b.config
    for key, val in cfg.items():
        assert got[key] == val
    for _ in range(2):  # capture, then replay
        for d, (_, _, v, _, _, _) in zip(fields, mix):
            d.copy_(torch.from_numpy(v))
        b.GatherScatter()
        torch.cuda.synchronize()
        check(mix, fields)


@pytest.mark.parametrize("cfg", [dict(), dict(occupancy=3, ctas_per_sm=3), dict(pipeline=1),
                                 dict(pipeline=1, occupancy=3, ctas_per_sm=2)],
                         ids=["register", "register-occ3", "ring", "ring-occ3"])
@pytest.mark.parametrize("dtype", [np.float64, np.int32], ids=lambda t: np.dtype(t).name)
def test_batch_larger_k(cuda, oracle_mod, cfg, dtype):
    """Entries with k = 5, 7, 13 and 33 beside k = 1 and 2: each record's 32
    row lanes x k components are split over its k items, by the entry's
    multiply-high divisor (k < 11585) in both pipelines."""
    mix = build_mix(oracle_mod, 12, seed=17, dtype=dtype, signed=True, ks=(5, 1, 7, 13, 2, 33))
    fields = [torch.from_numpy(v.copy()).cuda() for (_, _, v, _, _, _) in mix]
    b = ogs.ogs_batch_t([(g, d, k, op, trans) for (g, _, _, k, op, trans), d in zip(mix, fields)])
    b.set_config(**cfg)
    b.GatherScatter()
    torch.cuda.synchronize()
    check(mix, fields)
