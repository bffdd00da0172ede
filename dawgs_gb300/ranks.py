"""Several ranks of the reference's multi-rank gather-scatter, emulated in one
process on one GPU: the device half of the path a multi-rank caller runs.

At several ranks the reference splits each rank's rows into local rows (ids on
this rank only) and halo rows (ids shared with other ranks), and an ogs_t
GatherScatter becomes (libs/ogs/ogs.cpp:39-123, ogsAllToAll.cpp:126-175):

  Start:  halo Gather    haloBuf[h] = fold of the rank's members of halo row h
          extract        sendBuf[n] = haloBuf[sendIds[n]]      (ogsKernels.okl:167-177)
          exchange       all-to-all of the send buffers into each rank's
                         receive region haloBuf[Nhalo:]          (MPI in the reference)
  Finish: local GatherScatter over the local rows (overlapping the exchange)
          postmpi Gather haloBuf[h] = fold(haloBuf[h], received partials of h)
          halo Scatter   the members of halo row h get haloBuf[h]

A halo_t (kind Halo, libs/ogs/ogsHalo.cpp:39-359) runs the same halo steps
without local rows: Exchange with Add/NoTrans (the owner's value goes to
every copy), Combine with Add/Trans (every copy's value is summed into the
owner's).  NoTrans gathers the N members (positive ids) and sends only from
ranks that hold one; Trans and Sym gather all members; the Scatter writes the
T members (NoTrans, Sym) or the N members (Trans) (ogsOperator.cpp:60-360).

Here every rank's operators are library handles built from maps
(ogs_setup_maps), the packing is ogs_extract, and the exchange -- the network
step of the reference -- is one more ogs_extract per rank, gathering its
receive region from the concatenated send buffers of all ranks.  The maps
follow the reference's construction (ogsSetup.cpp:333-566
ConstructSharedNodes, 569-846 Local*Setup; ogsAllToAll.cpp:178-331):

* rows by first appearance on the rank, in four classes numbered apart:
  local rows with a positive member, then the other local rows; halo rows with
  a positive member on this rank, then the other halo rows;
* members in ascending local index; N members: ids > 0 (Signed), all members
  of a halo row whose group's positive id is on this rank (Halo), all
  (Unsigned);
* a rank sends each halo row to every other holder of its id, ordered by
  (destination, row); the N sends are the rows with a positive member;
* a rank receives from the source ranks in ascending order;
* postmpi T row h = [h, its received T entries]; postmpi N row h = [h if the
  row has a positive member, its received N entries], over a compact N receive
  region.  The library wants an N map inside the T map, so the two postmpi maps
  are two operators here.

A halo row therefore folds the rank's own partial first, then the other
ranks' partials by ascending rank -- the reference's order.  The reference
distributes ids by |id| % size and sorts across ranks to find the shared ones;
with all ranks in one process one pass over all ranks' ids finds them.
"""
from __future__ import annotations

import numpy as np

from . import ogs

UNSIGNED, SIGNED, HALO = int(ogs.Unsigned), int(ogs.Signed), int(ogs.Halo)


def _distinct(x):
    """Sorted distinct values (sort-based: faster than np.unique's hash path
    on millions of ids)."""
    s = np.sort(x)
    if s.size == 0:
        return s
    return s[np.concatenate(([True], s[1:] != s[:-1]))]


def _csr(rows_of_members, nrows, keep=None):
    """CSR map with members of each row in ascending local index:
    rows_of_members[n] = row of local node n, or -1; keep: optional mask."""
    sel = rows_of_members >= 0
    if keep is not None:
        sel &= keep
    n = np.nonzero(sel)[0]
    r = rows_of_members[n]
    order = np.argsort(r, kind="stable")  # stable: members stay in ascending local index
    counts = np.bincount(r, minlength=nrows)
    starts = np.zeros(nrows + 1, np.int64)
    np.cumsum(counts, out=starts[1:])
    return starts.astype(np.int32), n[order].astype(np.int32)


def _number_rows(first, positive, members):
    """The groups `members` (indices into uniq) split into positive and other
    groups, each in order of first appearance: rows are numbered positive
    groups first (ogsSetup.cpp:406-433)."""
    pos = members[positive[members]]
    neg = members[~positive[members]]
    pos = pos[np.argsort(first[pos], kind="stable")]
    neg = neg[np.argsort(first[neg], kind="stable")]
    return pos, neg


def build_rank_maps(ids_list, kind=UNSIGNED):
    """Per-rank maps of the emulated multi-rank setup (see the module text).

    Each rank's dict: N, nlocal, nlocalP, local (rsT, ciT, rsN, ciN), nhalo,
    nhaloP, halo (rsT, ciT, rsN, ciN), halo_ids, send_T, send_N (halo rows in
    send order), send_counts_T/N[R], recv_rows_T/N, postT (rs, ci) over
    nhalo + len(recv_rows_T) columns, postN (rs, ci) over nhalo +
    len(recv_rows_N) columns."""
    if kind not in (UNSIGNED, SIGNED, HALO):
        raise ValueError("kind must be Unsigned, Signed or Halo")
    R = len(ids_list)
    ids_list = [np.asarray(x, dtype=np.int64) for x in ids_list]
    absids = [np.abs(x) for x in ids_list]
    per_rank = [_distinct(a[a != 0]) for a in absids]
    allids = np.concatenate(per_rank) if per_rank else np.zeros(0, np.int64)
    ids_u, nranks = np.unique(allids, return_counts=True)
    shared_ids = ids_u[nranks > 1]
    if kind == HALO:
        # every id group needs exactly one positive id over all ranks (ogsSetup.cpp:293-296)
        pos_all = np.concatenate([x[x > 0] for x in ids_list]) if R else np.zeros(0, np.int64)
        u = _distinct(pos_all)
        c = np.searchsorted(np.sort(pos_all), u, side="right") - np.searchsorted(np.sort(pos_all), u, side="left")
        cnt = np.zeros(ids_u.size, np.int64)
        cnt[np.searchsorted(ids_u, u)] = c
        bad = ids_u[cnt != 1]
        if bad.size:
            raise ValueError(f"Halo setup: id {int(bad[0])} has {int(cnt[cnt != 1][0])} positive copies, not 1")
    out = []
    for r in range(R):
        a, x = absids[r], ids_list[r]
        nz = np.nonzero(a)[0]
        uniq, first = np.unique(a[nz], return_index=True)
        first = nz[first]
        node_uniq = np.full(a.size, -1, np.int64)
        node_uniq[nz] = np.searchsorted(uniq, a[nz])
        is_sh = np.isin(uniq, shared_ids)
        has_pos = np.zeros(uniq.size, bool)
        if kind == UNSIGNED:
            has_pos[:] = True
        else:
            has_pos[node_uniq[nz][x[nz] > 0]] = True
        loc_p, loc_n = _number_rows(first, has_pos, np.nonzero(~is_sh)[0])
        hal_p, hal_n = _number_rows(first, has_pos, np.nonzero(is_sh)[0])
        if kind == HALO:
            loc_p = loc_p[:0]
            loc_n = loc_n[:0]
        row_of = np.full(uniq.size, -1, np.int64)
        row_of[np.concatenate([loc_p, loc_n])] = np.arange(loc_p.size + loc_n.size)
        row_of[np.concatenate([hal_p, hal_n])] = np.arange(hal_p.size + hal_n.size)
        rows_local = np.full(a.size, -1, np.int64)
        rows_halo = np.full(a.size, -1, np.int64)
        member_sh = np.zeros(a.size, bool)
        member_sh[nz] = is_sh[node_uniq[nz]]
        if kind != HALO:
            m = ~member_sh
            m[a == 0] = False
            rows_local[m] = row_of[node_uniq[m]]
        rows_halo[member_sh] = row_of[node_uniq[member_sh]]
        # N members
        if kind == UNSIGNED:
            nmem = a != 0
        elif kind == SIGNED:
            nmem = x > 0
        else:  # Halo: every member of a row whose positive id is on this rank
            nmem = np.zeros(a.size, bool)
            nmem[nz] = has_pos[node_uniq[nz]]
        nl, nh = loc_p.size + loc_n.size, hal_p.size + hal_n.size
        local = _csr(rows_local, nl) + _csr(rows_local, nl, nmem)
        halo = _csr(rows_halo, nh) + _csr(rows_halo, nh, nmem)
        order_h = np.concatenate([hal_p, hal_n])
        out.append({"N": int(a.size), "nlocal": int(nl), "nlocalP": int(loc_p.size), "local": local,
                    "nhalo": int(nh), "nhaloP": int(hal_p.size), "halo": halo,
                    "halo_ids": uniq[order_h], "halo_pos": has_pos[order_h]})
    # exchange: rank r sends halo row h (id b) to every other holder j,
    # ordered by (j, h); N sends are the rows with a positive member
    B = np.concatenate([m["halo_ids"] for m in out]) if R else np.zeros(0, np.int64)
    RK = np.concatenate([np.full(m["nhalo"], r, np.int64) for r, m in enumerate(out)]) if R else B
    H = np.concatenate([np.arange(m["nhalo"]) for m in out]) if R else B
    P = np.concatenate([m["halo_pos"] for m in out]) if R else np.zeros(0, bool)
    o = np.lexsort((RK, B))
    B, RK, H, P = B[o], RK[o], H[o], P[o]
    n = B.size
    newgrp = np.ones(n, bool)
    newgrp[1:] = B[1:] != B[:-1]
    gid = np.cumsum(newgrp) - 1
    gstart = np.nonzero(newgrp)[0]
    gsize = np.diff(np.append(gstart, n))
    per = gsize[gid]                                   # group size of each holder entry
    i_idx = np.repeat(np.arange(n), per)               # every (holder, holder) pair of a group
    base = np.repeat(np.cumsum(per) - per, per)
    j_idx = gstart[gid[i_idx]] + (np.arange(i_idx.size) - base)
    keep = i_idx != j_idx
    i_idx, j_idx = i_idx[keep], j_idx[keep]
    src, dst, hs, hd, ps = RK[i_idx], RK[j_idx], H[i_idx], H[j_idx], P[i_idx]
    so = np.lexsort((hs, dst, src))                    # send order: source, destination, source row
    for r in range(R):
        sel = so[src[so] == r]
        m = out[r]
        m["send_T"] = hs[sel].astype(np.int32)
        m["send_N"] = hs[sel][ps[sel]].astype(np.int32)
        m["send_counts_T"] = np.bincount(dst[sel], minlength=R).astype(np.int64)
        m["send_counts_N"] = np.bincount(dst[sel][ps[sel]], minlength=R).astype(np.int64)
    ro = np.lexsort((hs, src, dst))                    # receive order: destination, source, source row
    for j in range(R):
        sel = ro[dst[ro] == j]
        m = out[j]
        m["recv_rows_T"] = hd[sel].astype(np.int64)
        m["recv_rows_N"] = hd[sel][ps[sel]].astype(np.int64)
        nh, nhp = m["nhalo"], m["nhaloP"]
        m["postT"] = _csr(np.concatenate([np.arange(nh), m["recv_rows_T"]]), nh)
        m["postN"] = _csr(np.concatenate([np.arange(nhp), np.full(nh - nhp, -1), m["recv_rows_N"]]), nh)
        m["postT_cols"] = nh + m["recv_rows_T"].size
        m["postN_cols"] = nh + m["recv_rows_N"].size
    return out


class ranks_ogs_t:
    """ogs_t GatherScatter (kind Unsigned or Signed) and halo_t
    Exchange/Combine (kind Halo) over R emulated ranks on one device.

    ids_list: one int64 id array per rank.  Fields: one device tensor per rank
    (k interleaved components), all of one dtype."""

    def __init__(self, ids_list, kind=UNSIGNED):
        import torch
        self.R = len(ids_list)
        self.kind = int(kind)
        self._ids = [np.asarray(x, dtype=np.int64) for x in ids_list]
        self.maps = build_rank_maps(ids_list, self.kind)
        self.local, self.halo, self.postT, self.postN = [], [], [], []
        for m in self.maps:
            sgn = self.kind != UNSIGNED
            rsT, ciT, rsN, ciN = m["local"]
            self.local.append(ogs.ogs_t().SetupMaps(m["N"], rsT, ciT, rsN if sgn else None,
                                                    ciN if sgn else None, NrowsN=m["nlocalP"]))
            rsT, ciT, rsN, ciN = m["halo"]
            self.halo.append(ogs.ogs_t().SetupMaps(m["N"], rsT, ciT, rsN if sgn else None,
                                                   ciN if sgn else None, NrowsN=m["nhaloP"]))
            self.postT.append(ogs.ogs_t().SetupMaps(m["postT_cols"], *m["postT"]))
            self.postN.append(ogs.ogs_t().SetupMaps(m["postN_cols"], *m["postN"]))
        dev = torch.device("cuda", torch.cuda.current_device())
        self.dev = dev
        self.plan = {}
        for which in ("T", "N"):
            off = np.zeros(self.R + 1, np.int64)
            np.cumsum([m["send_" + which].size for m in self.maps], out=off[1:])
            send_ids = [torch.from_numpy(m["send_" + which]).to(dev) for m in self.maps]
            recv_src = []
            for j in range(self.R):
                src = []
                for r in range(self.R):
                    cnts = self.maps[r]["send_counts_" + which]
                    before = int(cnts[:j].sum())
                    src.append(off[r] + before + np.arange(int(cnts[j])))
                recv_src.append(torch.from_numpy(np.concatenate(src).astype(np.int32)).to(dev))
            self.plan[which] = (off, send_ids, recv_src)
        self._bufs = {}

    def _buffers(self, dtype, k):
        import torch
        key = (dtype, k)
        if key not in self._bufs:
            nsend = max(int(self.plan["T"][0][-1]), 1)
            send = torch.empty(nsend * k, dtype=dtype, device=self.dev)
            bufs = [torch.empty(max(m["postT_cols"], m["postN_cols"], 1) * k, dtype=dtype, device=self.dev)
                    for m in self.maps]
            self._bufs[key] = (send, bufs)
        return self._bufs[key]

    # -- the steps; every rank runs on its own stream, forked from and joined
    # back to the caller's stream, so the ranks' small launches overlap --
    def _streams(self):
        import torch
        if not hasattr(self, "_rank_streams"):
            self._rank_streams = [torch.cuda.Stream(self.dev) for _ in range(self.R)]
        return self._rank_streams

    def _fork(self, stream):
        import torch
        main = stream if stream is not None else torch.cuda.current_stream(self.dev)
        ev = torch.cuda.Event()
        ev.record(main)
        for s in self._streams():
            s.wait_event(ev)
        return main

    def _join(self, main):
        import torch
        for s in self._streams():
            ev = torch.cuda.Event()
            ev.record(s)
            main.wait_event(ev)

    def _sends(self, vs, k, op, trans, which):
        """Halo Gather and send packing on every rank's stream; returns one
        event per rank."""
        import torch
        off, send_ids, _ = self.plan[which]
        send, bufs = self._buffers(vs[0].dtype, k)
        done = []
        for r, (m, s) in enumerate(zip(self.maps, self._streams())):
            nh = m["nhalo"]
            if nh:
                self.halo[r].Gather(bufs[r][: nh * k], vs[r], k, op, trans, stream=s)
            ns = send_ids[r].numel()
            if ns:
                ogs.extract(send[off[r] * k:(off[r] + ns) * k], bufs[r], send_ids[r], k, stream=s)
            ev = torch.cuda.Event()
            ev.record(s)
            done.append(ev)
        return done

    def _recv(self, j, k, which, sent, s, dtype):
        """Rank j's receive region, once every rank's send buffer is packed."""
        _, _, recv_src = self.plan[which]
        send, bufs = self._buffers(dtype, k)
        for ev in sent:
            s.wait_event(ev)
        nrecv = recv_src[j].numel()
        if nrecv:
            nh = self.maps[j]["nhalo"]
            ogs.extract(bufs[j][nh * k:(nh + nrecv) * k], send, recv_src[j], k, stream=s)

    def _post_scatter(self, j, vs, k, op, trans, which, s):
        _, bufs = self._buffers(vs[0].dtype, k)
        m = self.maps[j]
        nh = m["nhalo"]
        if not nh:
            return
        post, cols = (self.postN[j], m["postN_cols"]) if which == "N" else (self.postT[j], m["postT_cols"])
        post.Gather(bufs[j][: nh * k], bufs[j][: cols * k], k, op, ogs.Trans, stream=s)
        self.halo[j].Scatter(vs[j], bufs[j][: nh * k], k, trans, stream=s)

    def _local(self, vs, k, op, trans):
        for r, s in enumerate(self._streams()):
            if self.local[r].NlocalT:
                self.local[r].GatherScatter(vs[r], k, op, trans, stream=s)

    def _which(self, trans):
        return "N" if int(trans) == int(ogs.NoTrans) else "T"

    def _start(self, vs, k, op, trans, stream):
        which = self._which(trans)
        main = self._fork(stream)
        sent = self._sends(vs, k, op, trans, which)
        for j, s in enumerate(self._streams()):
            self._recv(j, k, which, sent, s, vs[0].dtype)
        self._join(main)

    def _finish(self, vs, k, op, trans, stream, local):
        which = self._which(trans)
        main = self._fork(stream)
        if local:
            self._local(vs, k, op, trans)
        for j, s in enumerate(self._streams()):
            self._post_scatter(j, vs, k, op, trans, which, s)
        self._join(main)

    def _whole(self, vs, k, op, trans, stream, local):
        """Start and Finish in one pass: each rank's local GatherScatter runs
        while the other ranks still pack their sends (the overlap the
        reference's Start/Finish split is for)."""
        which = self._which(trans)
        main = self._fork(stream)
        sent = self._sends(vs, k, op, trans, which)
        if local:
            self._local(vs, k, op, trans)
        for j, s in enumerate(self._streams()):
            self._recv(j, k, which, sent, s, vs[0].dtype)
            self._post_scatter(j, vs, k, op, trans, which, s)
        self._join(main)

    # -- ogs_t (ogs.cpp:39-123) --
    def _need_gs(self):
        if self.kind == HALO:
            raise ValueError("GatherScatter needs an Unsigned or Signed setup")

    def GatherScatterStart(self, vs, k, op=ogs.Add, trans=ogs.Sym, stream=None):
        """Halo Gather, send packing, exchange."""
        self._need_gs()
        self._start(vs, k, op, trans, stream)

    def GatherScatterFinish(self, vs, k, op=ogs.Add, trans=ogs.Sym, stream=None):
        """Local GatherScatter, postmpi Gather, halo Scatter."""
        self._finish(vs, k, op, trans, stream, local=True)

    def GatherScatter(self, vs, k, op=ogs.Add, trans=ogs.Sym, stream=None):
        self._need_gs()
        self._whole(vs, k, op, trans, stream, local=True)
        return vs

    # -- halo_t (ogsHalo.cpp:39-359, not gathered) --
    def _need_halo(self):
        if self.kind != HALO:
            raise ValueError("Exchange and Combine need a Halo setup")

    def ExchangeStart(self, vs, k, stream=None):
        self._need_halo()
        self._start(vs, k, ogs.Add, ogs.NoTrans, stream)

    def ExchangeFinish(self, vs, k, stream=None):
        self._finish(vs, k, ogs.Add, ogs.NoTrans, stream, local=False)

    def Exchange(self, vs, k, stream=None):
        self._need_halo()
        self._whole(vs, k, ogs.Add, ogs.NoTrans, stream, local=False)
        return vs

    def CombineStart(self, vs, k, stream=None):
        self._need_halo()
        self._start(vs, k, ogs.Add, ogs.Trans, stream)

    def CombineFinish(self, vs, k, stream=None):
        self._finish(vs, k, ogs.Add, ogs.Trans, stream, local=False)

    def Combine(self, vs, k, stream=None):
        self._need_halo()
        self._whole(vs, k, ogs.Add, ogs.Trans, stream, local=False)
        return vs

    # -- ogs_t Gather and Scatter (ogs.cpp:202-298, 392-488): gathered
    # vectors are [local rows | halo rows]; only Trans Gather and NoTrans
    # Scatter exchange --
    def gather_defined(self):
        """Every id has exactly one positive copy over all ranks (ogsSetup.cpp:276-282)."""
        if not hasattr(self, "_gdef"):
            ids = np.concatenate([np.asarray(x, np.int64) for x in self._ids]) if self.R else np.zeros(0, np.int64)
            a = np.abs(ids[ids != 0])
            allu = _distinct(a)
            pos = np.sort(ids[ids > 0])
            cnt = np.searchsorted(pos, allu, side="right") - np.searchsorted(pos, allu, side="left")
            self._gdef = bool(self.kind == SIGNED and np.all(cnt == 1))
        return self._gdef

    def gather_sizes(self, trans=ogs.Trans):
        """Rows of each rank's gathered vector: NlocalT + NhaloP (NhaloT for Sym)."""
        sym = int(trans) == int(ogs.Sym)
        return [m["nlocal"] + (m["nhalo"] if sym else m["nhaloP"]) for m in self.maps]

    def _need_gather(self):
        if not self.gather_defined():
            raise ValueError("Gather operation not well-defined.")  # ogsSetup.cpp:861-864

    def Gather(self, gvs, vs, k, op=ogs.Add, trans=ogs.Trans, stream=None):
        import torch
        self._need_gather()
        t = int(trans)
        main = self._fork(stream)
        if t == int(ogs.Trans):
            sent = self._sends(vs, k, op, trans, "T")
        for r, (m, s) in enumerate(zip(self.maps, self._streams())):
            nl = m["nlocal"]
            if nl:
                self.local[r].Gather(gvs[r][: nl * k], vs[r], k, op, trans, stream=s)
            if t != int(ogs.Trans) and m["nhalo"]:
                rows = m["nhalo"] if t == int(ogs.Sym) else m["nhaloP"]
                if rows:
                    self.halo[r].Gather(gvs[r][nl * k:(nl + rows) * k], vs[r], k, op, trans, stream=s)
        if t == int(ogs.Trans):
            _, bufs = self._buffers(vs[0].dtype, k)
            for j, (m, s) in enumerate(zip(self.maps, self._streams())):
                self._recv(j, k, "T", sent, s, vs[0].dtype)
                nl, nh, nhp = m["nlocal"], m["nhalo"], m["nhaloP"]
                if not nh:
                    continue
                self.postT[j].Gather(bufs[j][: nh * k], bufs[j][: m["postT_cols"] * k], k, op, ogs.Trans,
                                     stream=s)
                if nhp:
                    with torch.cuda.stream(s):
                        gvs[j][nl * k:(nl + nhp) * k].copy_(bufs[j][: nhp * k])
        self._join(main)
        return gvs

    def Scatter(self, vs, gvs, k, trans=ogs.NoTrans, stream=None):
        import torch
        self._need_gather()
        t = int(trans)
        main = self._fork(stream)
        if t == int(ogs.NoTrans):
            off, send_ids, _ = self.plan["N"]
            send, bufs = self._buffers(vs[0].dtype, k)
            sent = []
            for r, (m, s) in enumerate(zip(self.maps, self._streams())):
                nl, nhp = m["nlocal"], m["nhaloP"]
                with torch.cuda.stream(s):
                    if nhp:
                        bufs[r][: nhp * k].copy_(gvs[r][nl * k:(nl + nhp) * k])
                ns = send_ids[r].numel()
                if ns:
                    ogs.extract(send[off[r] * k:(off[r] + ns) * k], bufs[r], send_ids[r], k, stream=s)
                ev = torch.cuda.Event()
                ev.record(s)
                sent.append(ev)
        for r, (m, s) in enumerate(zip(self.maps, self._streams())):
            nl = m["nlocal"]
            if nl:
                self.local[r].Scatter(vs[r], gvs[r][: nl * k], k, trans, stream=s)
            # Trans reads halo rows [0, NhaloP), Sym [0, NhaloT), after the local rows
            rows = m["nhalo"] if t == int(ogs.Sym) else m["nhaloP"]
            if t != int(ogs.NoTrans) and rows:
                self.halo[r].Scatter(vs[r], gvs[r][nl * k:(nl + rows) * k], k, trans, stream=s)
        if t == int(ogs.NoTrans):
            for j, (m, s) in enumerate(zip(self.maps, self._streams())):
                self._recv(j, k, "N", sent, s, vs[0].dtype)
                self._post_scatter(j, vs, k, ogs.Add, ogs.NoTrans, "N", s)
        self._join(main)
        return vs

    # -- halo_t made from a gather (halo_t::SetupFromGather, ogsSetup.cpp:888-
    # 913; the gathered_halo branches of ogsHalo.cpp:39-359): the vectors are
    # gathered ones, [local rows | halo rows, those with a positive member
    # first], and the halo rows are copied instead of gathered --
    def gathered_sizes(self):
        """(NlocalT + NhaloT) rows of each rank's gathered vector."""
        return [m["nlocal"] + m["nhalo"] for m in self.maps]

    def _gathered(self, gvs, k, trans, stream):
        import torch
        if self.kind == HALO:
            raise ValueError("a gathered halo comes from an Unsigned or Signed setup")
        which = self._which(trans)
        off, send_ids, recv_src = self.plan[which]
        send, bufs = self._buffers(gvs[0].dtype, k)
        main = self._fork(stream)
        sent = []
        for r, (m, s) in enumerate(zip(self.maps, self._streams())):
            nl, nh, nhp = m["nlocal"], m["nhalo"], m["nhaloP"]
            rows = nhp if which == "N" else nh  # NoTrans sends the owned rows, Trans all halo rows
            with torch.cuda.stream(s):
                if rows:
                    bufs[r][: rows * k].copy_(gvs[r][nl * k:(nl + rows) * k])
            ns = send_ids[r].numel()
            if ns:
                ogs.extract(send[off[r] * k:(off[r] + ns) * k], bufs[r], send_ids[r], k, stream=s)
            ev = torch.cuda.Event()
            ev.record(s)
            sent.append(ev)
        for j, (m, s) in enumerate(zip(self.maps, self._streams())):
            self._recv(j, k, which, sent, s, gvs[0].dtype)
            nl, nh, nhp = m["nlocal"], m["nhalo"], m["nhaloP"]
            if not nh:
                continue
            post, cols = (self.postN[j], m["postN_cols"]) if which == "N" else (self.postT[j], m["postT_cols"])
            post.Gather(bufs[j][: nh * k], bufs[j][: cols * k], k, ogs.Add, ogs.Trans, stream=s)
            with torch.cuda.stream(s):
                if which == "N":  # the owners' values into the rows this rank does not own
                    if nh > nhp:
                        gvs[j][(nl + nhp) * k:(nl + nh) * k].copy_(bufs[j][nhp * k:nh * k])
                elif nhp:  # the combined values into the owned rows
                    gvs[j][nl * k:(nl + nhp) * k].copy_(bufs[j][: nhp * k])
        self._join(main)
        return gvs

    def GatheredExchange(self, gvs, k, stream=None):
        """Every copy of a halo row gets its owner's value (Add, NoTrans)."""
        return self._gathered(gvs, k, ogs.NoTrans, stream)

    def GatheredCombine(self, gvs, k, stream=None):
        """The owner's copy of a halo row gets the sum over all copies (Add, Trans)."""
        return self._gathered(gvs, k, ogs.Trans, stream)


__all__ = ["build_rank_maps", "ranks_ogs_t", "UNSIGNED", "SIGNED", "HALO"]
