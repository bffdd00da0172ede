"""One handle used from several streams and several host threads at once.

A handle is immutable after setup, so device-buffer calls on it may run
concurrently (the reference's static kernel tables and data stream,
ogsBase.hpp:64 and ogsUtils.cpp:39-43, allow no such use).  Every result
must still equal the oracle's bit for bit (ogsOperator.cpp:60-97, 206-238,
311-360)."""
import threading

import numpy as np
import pytest
import torch

from dawgs_gb300 import mesh, ogs
from helpers import same_bits, signed_ids, values

pytestmark = pytest.mark.gpu

TORCH = {np.float32: torch.float32, np.float64: torch.float64, np.int32: torch.int32, np.int64: torch.int64}
OPS = {"add": ogs.Add, "mul": ogs.Mul, "max": ogs.Max, "min": ogs.Min}


def _cases(n):
    """(dtype, op, k) for each concurrent call."""
    out = []
    for i in range(n):
        dt = [np.float64, np.float32, np.int64, np.int32][i % 4]
        op = ["add", "max", "min", "mul"][(i // 4) % 4]
        out.append((dt, op, 1 + i % 3))
    return out


def test_many_streams_one_handle(cuda, oracle_mod):
    ids = mesh.permute_elements(mesh.box_ids(10, 9, 8, 5), 5, seed=31)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    ref = oracle_mod.OracleOgs(ids.copy(), "unsigned")
    cases = _cases(16)
    host = [values(k * ids.size, dt, op, seed=500 + i) for i, (dt, op, k) in enumerate(cases)]
    devs = [torch.from_numpy(h.copy()).cuda() for h in host]
    streams = [torch.cuda.Stream() for _ in range(8)]
    torch.cuda.synchronize()
    for i, ((dt, op, k), d) in enumerate(zip(cases, devs)):
        s = streams[i % len(streams)]
        with torch.cuda.stream(s):
            # two calls back to back on each field: the second folds the first's result
            g.GatherScatter(d, k, OPS[op], ogs.Sym, stream=s)
            g.GatherScatter(d, k, OPS[op], ogs.Sym, stream=s)
    torch.cuda.synchronize()
    for i, ((dt, op, k), d) in enumerate(zip(cases, devs)):
        want = ref.gather_scatter(ref.gather_scatter(host[i].copy(), k, op, "sym"), k, op, "sym")
        assert same_bits(d.cpu().numpy(), want), (i, dt, op, k)


def test_threads_share_one_handle(cuda, oracle_mod):
    """Host threads, each with its own stream, call Gather, Scatter and
    GatherScatter on one Signed unique handle at the same time."""
    base = mesh.box_ids(9, 8, 7, 4)
    sids = signed_ids(base, seed=12)
    g = ogs.ogs_t().Setup(sids.size, sids.copy(), None, ogs.Signed, ogs.Auto, True)
    ref = oracle_mod.OracleOgs(sids.copy(), "signed", True)
    nthreads, reps = 6, 5
    dts = [np.float64, np.int64, np.float32]
    # expected results first (the oracle runs on this thread only)
    want = {}
    for t in range(nthreads):
        dt = dts[t % 3]
        for r in range(reps):
            v = values(base.size, dt, "add", seed=1000 * t + r)
            wgv = ref.gather(np.zeros(g.Ngather, dt), v.copy(), 1, "add", "trans")
            want[t, r] = (v, wgv, ref.gather_scatter(v.copy(), 1, "add", "sym"),
                          ref.scatter(values(base.size, dt, "add", seed=77 + t), wgv.copy(), 1, "notrans"))
    errors = []

    def work(t):
        try:
            s = torch.cuda.Stream()
            dt = dts[t % 3]
            for r in range(reps):
                v, want_gv, want_v, want_out = want[t, r]
                d = torch.from_numpy(v.copy()).cuda()
                gv = torch.zeros(g.Ngather, dtype=TORCH[dt], device="cuda")
                out = torch.from_numpy(values(base.size, dt, "add", seed=77 + t)).cuda()
                torch.cuda.synchronize()
                with torch.cuda.stream(s):
                    g.Gather(gv, d, 1, ogs.Add, ogs.Trans, stream=s)
                    g.GatherScatter(d, 1, ogs.Add, ogs.Sym, stream=s)
                    g.Scatter(out, gv, 1, ogs.NoTrans, stream=s)
                s.synchronize()
                if not same_bits(gv.cpu().numpy(), want_gv):
                    errors.append((t, r, "gather"))
                if not same_bits(d.cpu().numpy(), want_v):
                    errors.append((t, r, "gather_scatter"))
                if not same_bits(out.cpu().numpy(), want_out):
                    errors.append((t, r, "scatter"))
        except Exception as e:  # noqa: BLE001 -- reported below
            errors.append((t, repr(e)))

    th = [threading.Thread(target=work, args=(t,)) for t in range(nthreads)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    assert not errors, errors
