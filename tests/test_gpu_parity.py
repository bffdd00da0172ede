"""Parity of the sm_103a kernels (through the C ABI) with the CPU oracle.

Bit-exact for every type and op: rows are folded from the identity over their
members in ascending local index, the reference host order
(ogsOperator.cpp:60-97, 206-238, 311-360), so fp32/fp64 Add/Mul agree to the
last bit and no tolerance is used anywhere in this file.
"""
import numpy as np
import pytest
import torch

from dawgs_gb300 import mesh, ogs
from helpers import OPS, TRANS, TYPES, first_diff, random_ids, same_bits, signed_ids, values

pytestmark = pytest.mark.gpu

MESHES = {
    "box_10x10x10_p3": lambda: mesh.box_ids(10, 10, 10, 3),
    "box_permuted_p4": lambda: mesh.permute_elements(mesh.box_ids(5, 4, 3, 4), 4, seed=3),
    "random_deg1_to_40": lambda: random_ids(30000, 2500, seed=7, zero_frac=0.05),
    "mixed_degrees": lambda: np.concatenate([random_ids(4000, 4000, seed=1),      # mostly 1-3
                                             random_ids(3000, 500, seed=2) + 10 ** 6,  # ~6
                                             random_ids(2000, 3, seed=3) + 2 * 10 ** 6]),  # ~700
}
KIND_IDS = {"unsigned": lambda ids: ids, "signed": lambda ids: signed_ids(ids, seed=9)}

_TORCH = {np.float32: torch.float32, np.float64: torch.float64, np.int32: torch.int32, np.int64: torch.int64}


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def from_dev(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.fixture(scope="module")
def handles(cuda, oracle_mod):
    out = {}
    for mname, make in MESHES.items():
        base = make()
        for kind, flag in KIND_IDS.items():
            ids = flag(base)
            g = ogs.ogs_t().Setup(ids.size, ids.copy(), None,
                                  ogs.Signed if kind == "signed" else ogs.Unsigned)
            out[(mname, kind)] = (g, oracle_mod.OracleOgs(ids.copy(), kind), ids)
    return out


@pytest.mark.parametrize("mname", list(MESHES))
@pytest.mark.parametrize("kind", list(KIND_IDS))
@pytest.mark.parametrize("dtype", TYPES, ids=lambda t: np.dtype(t).name)
@pytest.mark.parametrize("op", OPS)
def test_gather_scatter_matches_oracle(handles, mname, kind, dtype, op):
    g, ref, ids = handles[(mname, kind)]
    for trans in TRANS:
        for k in (1, 3):
            v = values(k * ids.size, dtype, op, seed=31 + k)
            want = ref.gather_scatter(v.copy(), k, op, trans)
            d = to_dev(v)
            g.GatherScatter(d, k, ogs.Op[op.capitalize()], ogs.Transpose[
                {"sym": "Sym", "notrans": "NoTrans", "trans": "Trans"}[trans]])
            got = from_dev(d)
            assert same_bits(got, want), (trans, k, first_diff(got, want))


@pytest.mark.parametrize("mname", list(MESHES))
@pytest.mark.parametrize("dtype", TYPES, ids=lambda t: np.dtype(t).name)
@pytest.mark.parametrize("op", OPS)
def test_gather_and_scatter_unique_handle(cuda, oracle_mod, mname, dtype, op):
    """Signed unique handle, as dawgs' PerformanceTest/CorrectnessTest use it
    (dawgsMain.cpp:169-176, 399-413): Gather(Trans|NoTrans|Sym), Scatter(all)."""
    base = MESHES[mname]()
    ids_a, ids_b = base.copy(), base.copy()
    g = ogs.ogs_t().Setup(ids_a.size, ids_a, None, ogs.Signed, ogs.Auto, True)
    ref = oracle_mod.OracleOgs(ids_b, "signed", unique=True)
    assert np.array_equal(ids_a, ids_b) and g.gather_defined
    for k in (1, 2):
        v = values(k * base.size, dtype, op, seed=41)
        for trans, T in (("trans", ogs.Trans), ("notrans", ogs.NoTrans), ("sym", ogs.Sym)):
            want = np.zeros(k * ref.Ngather, dtype)
            ref.gather(want, v, k, op, trans)
            dgv = torch.zeros(k * g.Ngather, dtype=_TORCH[dtype], device="cuda")
            g.Gather(dgv, to_dev(v), k, ogs.Op[op.capitalize()], T)
            got = from_dev(dgv)
            assert same_bits(got, want), ("gather", trans, k, first_diff(got, want))
            # Scatter the gathered vector back over a fresh local vector.
            v0 = values(k * base.size, dtype, "add", seed=43)
            swant = ref.scatter(v0.copy(), want, k, trans)
            dv = to_dev(v0)
            g.Scatter(dv, to_dev(want), k, T)
            sgot = from_dev(dv)
            assert same_bits(sgot, swant), ("scatter", trans, k, first_diff(sgot, swant))


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int64], ids=lambda t: np.dtype(t).name)
@pytest.mark.parametrize("nf", [2, 8, 19])
def test_many_layout_matches_per_array_oracle(cuda, oracle_mod, dtype, nf):
    """k separate arrays in one call equal k single-array gather-scatters
    (gslib gs_many semantics, gs.c:1354); 19 arrays exercise the 16-array split."""
    ids = mesh.permute_elements(mesh.box_ids(6, 5, 4, 3), 3, seed=5)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    ref = oracle_mod.OracleOgs(ids.copy(), "unsigned")
    for op in ("add", "mul", "max"):
        vs = [values(ids.size, dtype, op, seed=50 + j) for j in range(nf)]
        ds = [to_dev(x) for x in vs]
        g.GatherScatterMany(ds, ogs.Op[op.capitalize()], ogs.Sym)
        for x, dx in zip(vs, ds):
            want = ref.gather_scatter(x.copy(), 1, op, "sym")
            assert same_bits(from_dev(dx), want)


@pytest.mark.parametrize("k", [2, 3, 5, 7, 8, 13, 33])
def test_interleaved_k_every_mode(cuda, oracle_mod, k):
    """Interleaved k > 1: a tile's 32 row lanes x k components are split over
    its k warp items, so a thread's row lane and component depend on k (powers
    of two and not, k > 32).  GatherScatter on Unsigned and Signed handles
    (every transpose), Gather and Scatter of every type on a Signed unique
    handle."""
    base = mesh.permute_elements(mesh.box_ids(6, 5, 4, 3), 3, seed=11)
    for kind in ("unsigned", "signed"):
        ids = base if kind == "unsigned" else signed_ids(base, seed=12)
        g = ogs.ogs_t().Setup(ids.size, ids.copy(), None, ogs.Signed if kind == "signed" else ogs.Unsigned)
        ref = oracle_mod.OracleOgs(ids.copy(), kind)
        for dtype, op in ((np.float64, "add"), (np.int32, "max"), (np.float32, "mul")):
            for trans in TRANS:
                v = values(k * ids.size, dtype, op, seed=40 + k)
                d = to_dev(v)
                g.GatherScatter(d, k, ogs.Op[op.capitalize()], ogs.Transpose[
                    {"sym": "Sym", "notrans": "NoTrans", "trans": "Trans"}[trans]])
                want = ref.gather_scatter(v.copy(), k, op, trans)
                assert same_bits(from_dev(d), want), (kind, dtype, op, trans, first_diff(from_dev(d), want))
    ids_a, ids_b = base.copy(), base.copy()
    g = ogs.ogs_t().Setup(ids_a.size, ids_a, None, ogs.Signed, ogs.Auto, True)
    ref = oracle_mod.OracleOgs(ids_b, "signed", unique=True)
    for dtype, op in ((np.float64, "add"), (np.int32, "max"), (np.float32, "mul"), (np.int64, "min")):
        v = values(k * base.size, dtype, op, seed=60 + k)
        for trans, T in (("trans", ogs.Trans), ("notrans", ogs.NoTrans)):
            want = np.zeros(k * g.Ngather, dtype)
            ref.gather(want, v, k, op, trans)
            dgv = torch.zeros(k * g.Ngather, dtype=_TORCH[dtype], device="cuda")
            g.Gather(dgv, to_dev(v), k, ogs.Op[op.capitalize()], T)
            assert same_bits(from_dev(dgv), want), ("gather", dtype, op, trans)
            v0 = values(k * base.size, dtype, "add", seed=61 + k)
            dv = to_dev(v0)
            g.Scatter(dv, to_dev(want), k, T)
            assert same_bits(from_dev(dv), ref.scatter(v0.copy(), want, k, trans)), ("scatter", dtype, trans)


@pytest.mark.parametrize("k", [11584, 11585, 12001])
def test_interleaved_k_at_the_divisor_limit(cuda, oracle_mod, k):
    """The row lane of a thread is (32j + t) / k by a multiply-high for
    k < 11585 and by a division above: both sides of that limit, for
    GatherScatter (every transpose, Signed), Gather and Scatter (Signed
    unique) and the batched kernel, on a small mesh."""
    base = mesh.box_ids(2, 2, 1, 2)
    ids = signed_ids(base, seed=14)
    g = ogs.ogs_t().Setup(ids.size, ids.copy(), None, ogs.Signed)
    ref = oracle_mod.OracleOgs(ids.copy(), "signed")
    for trans in TRANS:
        v = values(k * ids.size, np.float64, "add", seed=k)
        d = to_dev(v)
        g.GatherScatter(d, k, ogs.Add, ogs.Transpose[{"sym": "Sym", "notrans": "NoTrans", "trans": "Trans"}[trans]])
        want = ref.gather_scatter(v.copy(), k, "add", trans)
        assert same_bits(from_dev(d), want), (trans, first_diff(from_dev(d), want))
    # Gather and Scatter (the register pipeline) on a Signed unique handle
    ids_a, ids_b = base.copy(), base.copy()
    gq = ogs.ogs_t().Setup(ids_a.size, ids_a, None, ogs.Signed, ogs.Auto, True)
    refq = oracle_mod.OracleOgs(ids_b, "signed", unique=True)
    v = values(k * base.size, np.float64, "add", seed=k + 2)
    for trans, T in (("trans", ogs.Trans), ("notrans", ogs.NoTrans)):
        want = np.zeros(k * gq.Ngather, np.float64)
        refq.gather(want, v, k, "add", trans)
        dgv = torch.zeros(k * gq.Ngather, dtype=torch.float64, device="cuda")
        gq.Gather(dgv, to_dev(v), k, ogs.Add, T)
        assert same_bits(from_dev(dgv), want), ("gather", trans)
        v0 = values(k * base.size, np.float64, "add", seed=k + 3)
        dv = to_dev(v0)
        gq.Scatter(dv, to_dev(want), k, T)
        assert same_bits(from_dev(dv), refq.scatter(v0.copy(), want, k, trans)), ("scatter", trans)
    gu = ogs.ogs_t().Setup(base.size, base.copy())
    refu = oracle_mod.OracleOgs(base.copy(), "unsigned")
    v = values(k * base.size, np.float64, "max", seed=k + 1)
    d = to_dev(v)
    b = ogs.ogs_batch_t([(gu, d, k, ogs.Max, ogs.Sym)])
    b.GatherScatter()
    torch.cuda.synchronize()
    assert same_bits(from_dev(d), refu.gather_scatter(v.copy(), k, "max", "sym"))


def test_c3_irregular_multifield(cuda, oracle_mod):
    """32x32x16 p=5 with a seeded element permutation; k=3 interleaved and k=8
    separate arrays; fp64/fp32 Add (U[-1,1]) and Mul (U[0.5,2])."""
    ids = mesh.permute_elements(mesh.box_ids(32, 32, 16, 5), 5, seed=2024)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    ref = oracle_mod.OracleOgs(ids.copy(), "unsigned")
    assert g.N == 3538944 and g.NgatherGlobal == 2099601
    for dtype in (np.float64, np.float32):
        for op in ("add", "mul"):
            v = values(3 * ids.size, dtype, op, seed=7)
            d = to_dev(v)
            g.GatherScatter(d, 3, ogs.Op[op.capitalize()], ogs.Sym)
            assert same_bits(from_dev(d), ref.gather_scatter(v.copy(), 3, op, "sym"))
            vs = [values(ids.size, dtype, op, seed=70 + j) for j in range(8)]
            ds = [to_dev(x) for x in vs]
            g.GatherScatterMany(ds, ogs.Op[op.capitalize()], ogs.Sym)
            for x, dx in zip(vs, ds):
                assert same_bits(from_dev(dx), ref.gather_scatter(x.copy(), 1, op, "sym"))


def test_host_buffer_entry_points(cuda, oracle_mod):
    """memory<T> overloads: host buffers in, host buffers out, GPU in between."""
    base = mesh.box_ids(6, 6, 6, 3)
    ids_a, ids_b = base.copy(), base.copy()
    g = ogs.ogs_t().Setup(ids_a.size, ids_a, None, ogs.Signed, ogs.Auto, True)
    ref = oracle_mod.OracleOgs(ids_b, "signed", unique=True)
    for dtype in TYPES:
        v = values(base.size, dtype, "add", seed=3)
        a = g.GatherScatter(v.copy(), 1, ogs.Add, ogs.Sym)
        assert same_bits(a, ref.gather_scatter(v.copy(), 1, "add", "sym"))
        gv = np.zeros(g.Ngather, dtype)
        g.Gather(gv, v, 1, ogs.Add, ogs.Trans)
        want = np.zeros(ref.Ngather, dtype)
        ref.gather(want, v, 1, "add", "trans")
        assert same_bits(gv, want)
        out = values(base.size, dtype, "add", seed=4)
        g.Scatter(out, gv, 1, ogs.NoTrans)
        assert same_bits(out, ref.scatter(values(base.size, dtype, "add", seed=4), want, 1, "notrans"))
    pinned = torch.from_numpy(values(base.size, np.float64, "add", seed=5)).pin_memory()
    want = ref.gather_scatter(pinned.numpy().copy(), 1, "add", "sym")
    g.GatherScatter(pinned, 1, ogs.Add, ogs.Sym)
    assert same_bits(pinned.numpy(), want)


def test_side_stream_and_repeatability(cuda, oracle_mod):
    ids = mesh.box_ids(8, 7, 6, 4)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    ref = oracle_mod.OracleOgs(ids.copy(), "unsigned")
    v = values(ids.size, np.float64, "add", seed=77)
    want = ref.gather_scatter(v.copy(), 1, "add", "sym")
    s = torch.cuda.Stream()
    outs = []
    for _ in range(3):
        d = to_dev(v)
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            g.GatherScatter(d, 1, ogs.Add, ogs.Sym, stream=s)
        s.synchronize()
        outs.append(d.cpu().numpy())
    for o in outs:
        assert same_bits(o, want)


def test_host_pipeline_graph_replay_and_cache(cuda, oracle_mod):
    """The host-buffer call captures its copy/compute pipeline once per buffer
    and parameters and replays it: repeated calls on one buffer, calls that
    rotate through more buffers than the cache keeps, and changing k or op all
    give the oracle's result."""
    ids = mesh.box_ids(12, 10, 9, 4)  # enough tiles for a multi-slice pipeline
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    assert len(g.layout_stats()["phases"]) > 1
    ref = oracle_mod.OracleOgs(ids.copy(), "unsigned")
    buf = torch.empty(2 * ids.size, dtype=torch.float64).pin_memory()
    for rep in range(3):
        v = values(ids.size, np.float64, "add", seed=60 + rep)
        buf[: ids.size].copy_(torch.from_numpy(v))
        g.GatherScatter(buf[: ids.size], 1, ogs.Add, ogs.Sym)
        assert same_bits(buf[: ids.size].numpy(), ref.gather_scatter(v.copy(), 1, "add", "sym"))
    v2 = values(2 * ids.size, np.float64, "max", seed=70)
    buf.copy_(torch.from_numpy(v2))
    g.GatherScatter(buf, 2, ogs.Max, ogs.Sym)
    assert same_bits(buf.numpy(), ref.gather_scatter(v2.copy(), 2, "max", "sym"))
    bufs = [torch.from_numpy(values(ids.size, np.float64, "add", seed=80 + j)).pin_memory() for j in range(6)]
    for _ in range(2):
        for j, b in enumerate(bufs):
            v = values(ids.size, np.float64, "add", seed=80 + j)
            b.copy_(torch.from_numpy(v))
            g.GatherScatter(b, 1, ogs.Add, ogs.Sym)
            assert same_bits(b.numpy(), ref.gather_scatter(v.copy(), 1, "add", "sym"))


def _zero_block(ids):
    ids = ids.copy()
    a = int(ids.size * 0.3)
    ids[a:a + ids.size // 5] = 0
    return ids


@pytest.mark.parametrize("zero_block", [False, True])
def test_host_gather_and_scatter_pipelines(cuda, oracle_mod, zero_block):
    """Host-buffer Gather and Scatter on a Signed unique handle with a
    four-slice pipeline (page-locked buffers): gathered rows go out as the
    slices that write them finish, and the Scatter's rows come in ahead of
    the slices that read them.  With a block of zero ids the Scatter leaves
    those entries alone, so the field also comes in."""
    base = mesh.box_ids(16, 14, 12, 4)
    if zero_block:
        base = _zero_block(base)
    sids = signed_ids(base, seed=21)
    a = sids.copy()
    g = ogs.ogs_t().Setup(a.size, a, None, ogs.Signed, ogs.Auto, True)
    assert len(g.layout_stats()["phases"]) >= 2
    ref = oracle_mod.OracleOgs(sids.copy(), "signed", True)
    for dtype, op, k in ((np.float64, "add", 1), (np.float32, "max", 1), (np.int64, "min", 1), (np.float64, "add", 3)):
        for trans, T in (("trans", ogs.Trans), ("notrans", ogs.NoTrans), ("sym", ogs.Sym)):
            v = values(k * base.size, dtype, op, seed=31)
            hv = torch.from_numpy(v.copy()).pin_memory()
            hgv = torch.zeros(k * g.Ngather, dtype=hv.dtype).pin_memory()
            g.Gather(hgv, hv, k, ogs.Op[op.capitalize()], T)
            want = ref.gather(np.zeros(k * g.Ngather, dtype), v.copy(), k, op, trans)
            assert same_bits(hgv.numpy(), want), (dtype, op, k, trans)
            out = torch.from_numpy(values(k * base.size, dtype, op, seed=32)).pin_memory()
            g.Scatter(out, hgv, k, T)
            assert same_bits(out.numpy(), ref.scatter(values(k * base.size, dtype, op, seed=32), want.copy(), k,
                                                      trans)), (dtype, op, k, trans)
