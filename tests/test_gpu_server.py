"""Served gather-scatter: a stream of requests over resident meshes, admitted
against an HBM budget and batched while others run, gives for every request
exactly the result of that request run alone (ogs_gather_scatter_host) and of
the oracle."""
import numpy as np
import pytest
import torch

from dawgs_gb300 import mesh, ogs
from helpers import first_diff, random_ids, same_bits, signed_ids, values

pytestmark = pytest.mark.gpu

OPN = {ogs.Add: "add", ogs.Mul: "mul", ogs.Max: "max", ogs.Min: "min"}
TRN = {ogs.Sym: "sym", ogs.NoTrans: "notrans", ogs.Trans: "trans"}
DT = [np.float64, np.float32, np.int64, np.int32]


def make_meshes(oracle_mod, n, seed, general=False):
    out = []
    for j, (nx, ny, nz, p) in enumerate(mesh.mesh_mix(n, seed, lo=1, hi=7, pmax=5)):
        ids = mesh.box_ids(nx, ny, nz, p)
        if general and j % 2 == 0:
            # rows of up to ~40 members: the general-tile launch beside the batch
            ids = np.concatenate([ids, random_ids(2000, 60, seed=j) + 10 ** 7])
        kind = ogs.Unsigned
        if j % 3 == 2:
            ids = signed_ids(ids, seed=j)
            kind = ogs.Signed
        g = ogs.ogs_t().Setup(ids.size, ids.copy(), None, kind)
        out.append((g, oracle_mod.OracleOgs(ids.copy(), "signed" if kind == ogs.Signed else "unsigned"), kind))
    return out


def make_requests(meshes, count, seed):
    rng = mesh.uniform_values(4 * count, np.int64, 0, 1 << 30, seed)
    reqs = []
    for i in range(count):
        m = int(rng[4 * i] % len(meshes))
        g, ref, kind = meshes[m]
        dt = DT[int(rng[4 * i + 1] % 4)]
        k = 1 + int(rng[4 * i + 2] % 8)
        op = [ogs.Add, ogs.Add, ogs.Min, ogs.Max, ogs.Mul][int(rng[4 * i + 3] % 5)]
        trans = [ogs.Sym, ogs.NoTrans, ogs.Trans][i % 3] if kind == ogs.Signed else ogs.Sym
        v = values(k * g.N, dt, OPN[op], seed=1000 + i)
        reqs.append((m, v, k, op, trans))
    return reqs


def run(server, meshes, reqs):
    ids = {}
    host = []
    for m, v, k, op, trans in reqs:
        h = torch.from_numpy(v.copy()).pin_memory()
        host.append(h)
    for (m, v, k, op, trans), h in zip(reqs, host):
        rid = server.submit(m, h, k, op, trans)
        ids[rid] = h
    server.drain()
    return host


@pytest.mark.parametrize("budget_mb,general", [(4096, False), (1, False), (4096, True)],
                         ids=["4096MB", "1MB", "4096MB-general-rows"])
def test_served_results_equal_alone_and_oracle(cuda, oracle_mod, budget_mb, general):
    meshes = make_meshes(oracle_mod, 6, seed=3, general=general)
    server = ogs.ogs_server_t(field_budget_bytes=budget_mb << 20, max_inflight=64, max_batch=32)
    mids = [server.add_mesh(g) for g, _, _ in meshes]
    assert mids == list(range(len(meshes)))
    reqs = make_requests(meshes, 160, seed=9)
    big = max(meshes[m][0].N * k * v.dtype.itemsize for m, v, k, _, _ in reqs)
    assert big <= budget_mb << 20
    host = run(server, meshes, reqs)
    for (m, v, k, op, trans), h in zip(reqs, host):
        g, ref, _ = meshes[m]
        alone = v.copy()
        g.GatherScatter(alone, k, op, trans)  # host-buffer path, one request on its own
        got = h.numpy()
        assert same_bits(got, alone), (m, k, OPN[op], TRN[trans], first_diff(got, alone))
        want = ref.gather_scatter(v.copy(), k, OPN[op], TRN[trans])
        assert same_bits(got, want)
    a, d = server.times(0, len(reqs))
    assert np.all(d >= a)
    launches, batched = server.counters()
    assert batched == len(reqs) and 1 <= launches <= len(reqs)
    server.Free()


def test_server_rejects_bad_requests(cuda):
    ids = mesh.box_ids(3, 3, 3, 2)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    server = ogs.ogs_server_t(field_budget_bytes=1 << 20, max_inflight=4, max_batch=4)
    m = server.add_mesh(g)
    from dawgs_gb300 import _lib
    with pytest.raises(_lib.OgsError):
        server.submit(m + 5, np.zeros(ids.size), 1)
    with pytest.raises(_lib.OgsError) as e:
        server.submit(m, np.zeros(ids.size * 1000), 1000)  # larger than the whole budget
    assert e.value.status == _lib.OGS_ERANGE
    server.Free()


def _pinned(v):
    return torch.from_numpy(v.copy()).pin_memory()


def _wait_state(server, rid, want, limit_s=10.0):
    t0 = server.clock()
    while server.state(rid) != want:
        assert server.clock() - t0 < limit_s, f"request {rid} never reached state {want}"


def test_request_arriving_while_a_batch_runs_overlaps_it(cuda, oracle_mod):
    """Continuous batching: a small request submitted while a large one is on
    the GPU is launched before the large one retires, finishes first (its
    copies do not queue behind the large field's), and both results equal
    the requests run alone."""
    big_ids = mesh.box_ids(24, 24, 24, 5)   # 2,985,984 nodes x k=8 fp64: 191 MB each way
    small_ids = mesh.box_ids(4, 4, 4, 2)
    gb = ogs.ogs_t().Setup(big_ids.size, big_ids.copy())
    gs = ogs.ogs_t().Setup(small_ids.size, small_ids.copy())
    server = ogs.ogs_server_t(field_budget_bytes=1 << 30, max_inflight=16, max_batch=8)
    mb, ms = server.add_mesh(gb), server.add_mesh(gs)
    vb = values(8 * gb.N, np.float64, "add", seed=71)
    vs = values(2 * gs.N, np.float64, "max", seed=72)
    hb, hs = _pinned(vb), _pinned(vs)
    rb = server.submit(mb, hb, 8)
    _wait_state(server, rb, server.ADMITTED)
    rs = server.submit(ms, hs, 2, ogs.Max)
    server.wait(rs)
    server.wait(rb)
    a, launched, done = server.times(0, 2, launched=True)
    assert launched[1] < done[0], "the later request waited for the running batch to retire"
    assert done[1] < done[0], "the small request finished after the large one"
    for g, v, h, k, op in ((gb, vb, hb, 8, ogs.Add), (gs, vs, hs, 2, ogs.Max)):
        alone = v.copy()
        g.GatherScatter(alone, k, op, ogs.Sym)
        assert same_bits(h.numpy(), alone)
    ref = oracle_mod.OracleOgs(small_ids.copy(), "unsigned")
    assert same_bits(hs.numpy(), ref.gather_scatter(vs.copy(), 2, "max", "sym"))
    server.Free()


def test_admission_lets_small_requests_pass_one_that_does_not_fit(cuda):
    """With the budget held by one large field, a second large request waits;
    a small request submitted after it is admitted and launched first."""
    big_ids = mesh.box_ids(24, 24, 24, 4)   # 1,728,000 nodes x k=4 fp64 = 55.3 MB
    small_ids = mesh.box_ids(3, 3, 3, 2)
    gb = ogs.ogs_t().Setup(big_ids.size, big_ids.copy())
    gs = ogs.ogs_t().Setup(small_ids.size, small_ids.copy())
    big_bytes = 4 * 8 * gb.N
    server = ogs.ogs_server_t(field_budget_bytes=big_bytes + (4 << 20), max_inflight=16, max_batch=8)
    mb, ms = server.add_mesh(gb), server.add_mesh(gs)
    vb1, vb2 = values(4 * gb.N, np.float64, "add", seed=81), values(4 * gb.N, np.float64, "add", seed=82)
    vs = values(gs.N, np.float64, "add", seed=83)
    h1, h2, h3 = _pinned(vb1), _pinned(vb2), _pinned(vs)
    r1 = server.submit(mb, h1, 4)
    r2 = server.submit(mb, h2, 4)
    r3 = server.submit(ms, h3, 1)
    server.drain()
    a, launched, done = server.times(0, 3, launched=True)
    assert launched[2] < launched[1], "the small request waited behind the large one that did not fit"
    for g, v, h, k in ((gb, vb1, h1, 4), (gb, vb2, h2, 4), (gs, vs, h3, 1)):
        alone = v.copy()
        g.GatherScatter(alone, k, ogs.Add, ogs.Sym)
        assert same_bits(h.numpy(), alone)
    assert [server.state(r) for r in (r1, r2, r3)] == [server.DONE] * 3
    server.Free()


def test_cancel_pending_request_and_bounded_wait(cuda):
    """A request that cannot be admitted yet can be withdrawn (its field is
    never touched); a bounded wait on a running request returns OGS_ETIMEOUT
    and the request still completes."""
    from dawgs_gb300 import _lib
    big_ids = mesh.box_ids(24, 24, 24, 5)
    gb = ogs.ogs_t().Setup(big_ids.size, big_ids.copy())
    big_bytes = 8 * 8 * gb.N
    server = ogs.ogs_server_t(field_budget_bytes=big_bytes, max_inflight=16, max_batch=8)
    m = server.add_mesh(gb)
    v1, v2 = values(8 * gb.N, np.float64, "add", seed=91), values(8 * gb.N, np.float64, "add", seed=92)
    h1, h2 = _pinned(v1), _pinned(v2)
    r1 = server.submit(m, h1, 8)
    r2 = server.submit(m, h2, 8)   # the budget holds one of the two
    assert server.cancel(r2) is True
    assert server.state(r2) == server.CANCELLED
    with pytest.raises(_lib.OgsError) as e:
        server.wait(r1, timeout=0.0)
    assert e.value.status == _lib.OGS_ETIMEOUT
    server.wait(r1, timeout=60.0)
    server.wait(r2)          # a cancelled request is final
    assert server.cancel(r1) is False
    server.drain()
    assert same_bits(h2.numpy(), v2)  # never ran
    alone = v1.copy()
    gb.GatherScatter(alone, 8, ogs.Add, ogs.Sym)
    assert same_bits(h1.numpy(), alone)
    _, launched, done = server.times(0, 2, launched=True)
    assert launched[1] == -1 and done[1] == -1
    server.Free()
