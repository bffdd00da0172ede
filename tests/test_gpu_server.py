"""Served gather-scatter: a stream of requests over resident meshes, admitted
against an HBM budget and batched while others run, gives for every request
exactly the result of that request run alone (ogs_gather_scatter_host) and of
the oracle."""
import numpy as np
import pytest
import torch

from dawgs_gb300 import mesh, ogs
from helpers import first_diff, same_bits, signed_ids, values

pytestmark = pytest.mark.gpu

OPN = {ogs.Add: "add", ogs.Mul: "mul", ogs.Max: "max", ogs.Min: "min"}
TRN = {ogs.Sym: "sym", ogs.NoTrans: "notrans", ogs.Trans: "trans"}
DT = [np.float64, np.float32, np.int64, np.int32]


def make_meshes(oracle_mod, n, seed):
    out = []
    for j, (nx, ny, nz, p) in enumerate(mesh.mesh_mix(n, seed, lo=1, hi=7, pmax=5)):
        ids = mesh.box_ids(nx, ny, nz, p)
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


@pytest.mark.parametrize("budget_mb", [4096, 1])
def test_served_results_equal_alone_and_oracle(cuda, oracle_mod, budget_mb):
    meshes = make_meshes(oracle_mod, 6, seed=3)
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
