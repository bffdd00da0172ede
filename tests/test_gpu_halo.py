"""halo_t through the C ABI on emulated ranks: each rank's halo is an
ogs_halo made from its gatherHalo maps (or from its gathered vector's
counts), and the caller's exchange -- the MPI step, here the all-to-all
emulated on one GPU: send packing by ogs_extract in `start`, the receive
gather and the postmpi fold (ogsAllToAll.cpp:255-331) in `finish` -- is
passed in as callbacks.  Every rank runs its Start before any Finish, as MPI
ranks would.  Results equal the oracle's restatement of the reference's
multi-rank Exchange / Combine (ogsHalo.cpp:39-359) bit for bit."""
import numpy as np
import pytest
import torch

from dawgs_gb300 import _lib, ogs, ranks
from helpers import first_diff, same_bits, values
from oracle import ranks as oranks

pytestmark = pytest.mark.gpu

PARTS = [((6, 5, 4, 3), 2, "slabs"), ((6, 5, 4, 3), 3, "random"), ((5, 4, 4, 2), 4, "random"),
         ((8, 4, 4, 2), 8, "slabs")]
TS = {0: 4, 1: 8, 2: 4, 3: 8}


class AllToAll:
    """The emulated exchange of every rank's halo buffer (one send buffer for
    all ranks; rank r's received entries land after its NhaloT rows)."""

    def __init__(self, rk, which, dtype, k):
        self.rk, self.which, self.k = rk, which, k
        off, self.send_ids, self.recv_src = rk.plan[which]
        self.off = off
        self.send = torch.empty(max(int(off[-1]), 1) * k, dtype=dtype, device="cuda")
        self.L = _lib.lib()

    def start(self, r):
        def f(buf, k, t, trans, stream):
            ns = self.send_ids[r].numel()
            if ns:
                return self.L.ogs_extract(ns, k, t, self.send_ids[r].data_ptr(), buf,
                                          self.send.data_ptr() + int(self.off[r]) * k * TS[t], stream)
            return 0
        return f

    def finish(self, j):
        def f(buf, k, t, trans, stream):
            m = self.rk.maps[j]
            nh = m["nhalo"]
            nrecv = self.recv_src[j].numel()
            st = 0
            if nrecv:
                st = self.L.ogs_extract(nrecv, k, t, self.recv_src[j].data_ptr(), self.send.data_ptr(),
                                        buf + nh * k * TS[t], stream)
            post = self.rk.postN[j] if self.which == "N" else self.rk.postT[j]
            if not st and nh:
                st = self.L.ogs_gather(post.handle, buf, buf, k, t, 0, 2, stream)
            return st
        return f


def recv_rows(rk, j):
    return max(rk.maps[j]["postT_cols"], rk.maps[j]["postN_cols"]) - rk.maps[j]["nhalo"]


@pytest.mark.parametrize("key", PARTS, ids=lambda p: f"{p[0]}-{p[1]}-{p[2]}")
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int64], ids=lambda t: np.dtype(t).name)
@pytest.mark.parametrize("trans", ["notrans", "trans"])
def test_halo_c_abi_matches_oracle(cuda, oracle_mod, key, dtype, trans):
    box, R, how = key
    parts = oranks.signed_parts(oranks.partition_box(*box, R, how=how, seed=17), 5, "halo")
    rk = ranks.ranks_ogs_t(parts, ranks.HALO)
    halos = []
    for j, m in enumerate(rk.maps):
        rsT, ciT, rsN, ciN = m["halo"]
        halos.append(ogs.halo_t().SetupMaps(m["N"], m["nhaloP"], rsT, ciT, rsN, ciN, Nrecv=recv_rows(rk, j)))
        assert halos[-1].NhaloT == m["nhalo"] and halos[-1].Nhalo == m["nhalo"] - m["nhaloP"]
    for k in (1, 3):
        vs = [values(k * p.size, dtype, "add", seed=70 + i + 3 * k) for i, p in enumerate(parts)]
        want = oranks.ranks_gather_scatter(parts, vs, k, "add", "halo", trans)
        ds = [torch.from_numpy(v.copy()).cuda() for v in vs]
        x = AllToAll(rk, "N" if trans == "notrans" else "T", ds[0].dtype, k)
        for j, h in enumerate(halos):
            h.set_exchange(x.start(j), x.finish(j))
        for j, h in enumerate(halos):  # every rank starts ...
            (h.ExchangeStart if trans == "notrans" else h.CombineStart)(ds[j], k)
        for j, h in enumerate(halos):  # ... before any finishes
            (h.ExchangeFinish if trans == "notrans" else h.CombineFinish)(ds[j], k)
        torch.cuda.synchronize()
        for r, (d, w) in enumerate(zip(ds, want)):
            got = d.cpu().numpy()
            assert same_bits(got, w), (key, trans, k, r, first_diff(got, w))


@pytest.mark.parametrize("key", PARTS[:3], ids=lambda p: f"{p[0]}-{p[1]}-{p[2]}")
@pytest.mark.parametrize("kind", ["signed", "unsigned"])
@pytest.mark.parametrize("trans", ["notrans", "trans"])
def test_gathered_halo_c_abi_matches_oracle(cuda, oracle_mod, key, kind, trans):
    """halo_t made from a gather (SetupFromGather): the halo rows are copied
    out of and back into gathered vectors [local rows | halo rows]."""
    box, R, how = key
    parts = oranks.partition_box(*box, R, how=how, seed=17)
    if kind == "signed":
        parts = oranks.signed_parts(parts, 5, "halo")
    rk = ranks.ranks_ogs_t(parts, ranks.SIGNED if kind == "signed" else ranks.UNSIGNED)
    halos = [ogs.halo_t().SetupFromGather(NlocalT=m["nlocal"], NhaloP=m["nhaloP"], NhaloT=m["nhalo"],
                                          Nrecv=recv_rows(rk, j)) for j, m in enumerate(rk.maps)]
    k = 2
    gvs = [values(n * k, np.float64, "add", seed=90 + i) for i, n in enumerate(rk.gathered_sizes())]
    want = oranks.gathered_exchange(parts, gvs, k, kind, trans)
    ds = [torch.from_numpy(g.copy()).cuda() for g in gvs]
    x = AllToAll(rk, "N" if trans == "notrans" else "T", ds[0].dtype, k)
    for j, h in enumerate(halos):
        h.set_exchange(x.start(j), x.finish(j))
    for j, h in enumerate(halos):
        (h.ExchangeStart if trans == "notrans" else h.CombineStart)(ds[j], k)
    for j, h in enumerate(halos):
        (h.ExchangeFinish if trans == "notrans" else h.CombineFinish)(ds[j], k)
    torch.cuda.synchronize()
    for r, (d, w) in enumerate(zip(ds, want)):
        got = d.cpu().numpy()
        assert same_bits(got, w), (key, kind, trans, r, first_diff(got, w))


def test_halo_reserved_buffer_is_reused(cuda, oracle_mod):
    """The buffer ogs_halo_reserve returns is the one the exchange is given,
    and Start/Finish reuse it (no allocation per call)."""
    parts = oranks.signed_parts(oranks.partition_box(6, 5, 4, 3, 2, how="slabs", seed=17), 5, "halo")
    rk = ranks.ranks_ogs_t(parts, ranks.HALO)
    halos = []
    for j, m in enumerate(rk.maps):
        rsT, ciT, rsN, ciN = m["halo"]
        halos.append(ogs.halo_t().SetupMaps(m["N"], m["nhaloP"], rsT, ciT, rsN, ciN, Nrecv=recv_rows(rk, j)))
    k = 2
    bufs = [h.reserve(k, np.float64) for h in halos]
    assert all(b != 0 for b in bufs)
    vs = [values(k * p.size, np.float64, "add", seed=120 + i) for i, p in enumerate(parts)]
    want = oranks.ranks_gather_scatter(parts, vs, k, "add", "halo", "notrans")
    ds = [torch.from_numpy(v.copy()).cuda() for v in vs]
    x = AllToAll(rk, "N", ds[0].dtype, k)
    seen = []
    for j, h in enumerate(halos):
        st, fi = x.start(j), x.finish(j)
        h.set_exchange(lambda buf, *a, st=st: (seen.append(buf), st(buf, *a))[1], fi)
    for j, h in enumerate(halos):
        h.ExchangeStart(ds[j], k)
    assert seen == bufs
    assert [h.reserve(k, np.float64) for h in halos] == bufs
    for j, h in enumerate(halos):
        h.ExchangeFinish(ds[j], k)
    torch.cuda.synchronize()
    for d, w in zip(ds, want):
        assert same_bits(d.cpu().numpy(), w)


@pytest.mark.parametrize("combine", [False, True])
def test_halo_host_vector_is_staged_through_the_device(cuda, combine):
    """Host vectors: the field goes to the device, the halo steps and the
    exchange run there, and the field comes back.  A gathered halo (5 local
    rows, 4 halo rows of which 2 owned) with an exchange that writes known
    values into the rows it receives (Exchange: rows 2..3, Combine: rows 0..1
    of the halo buffer)."""
    L = _lib.lib()
    k, nl, nhp, nht = 2, 5, 2, 4
    h = ogs.halo_t().SetupFromGather(NlocalT=nl, NhaloP=nhp, NhaloT=nht)
    const = torch.tensor([100.0, 101.0, 102.0, 103.0], dtype=torch.float64, device="cuda")
    rows = torch.tensor([0, 1], dtype=torch.int32, device="cuda")
    seen = {}

    def finish(buf, kk, t, trans, stream):
        seen["start_rows"] = None
        at = 0 if trans == 2 else nhp
        return L.ogs_extract(2, kk, t, rows.data_ptr(), const.data_ptr(), buf + at * kk * 8, stream)
    h.set_exchange(None, finish)
    v = np.arange((nl + nht) * k, dtype=np.float64)
    want = v.copy()
    if combine:
        h.Combine(v, k)
        want[nl * k:(nl + nhp) * k] = const.cpu().numpy()
    else:
        h.Exchange(v, k)
        want[(nl + nhp) * k:(nl + nht) * k] = const.cpu().numpy()
    assert same_bits(v, want)
    h.Free()
