"""Several ranks of the reference's multi-rank gather-scatter, emulated in one
process on one GPU: the device half of the path a multi-rank caller runs.

At several ranks the reference splits each rank's rows into local rows (ids on
this rank only) and halo rows (ids shared with other ranks), and a
GatherScatter becomes (libs/ogs/ogs.cpp:39-123, ogsAllToAll.cpp:126-175):

  Start:  halo Gather   haloBuf[h] = fold of the rank's members of halo row h
          extract       sendBuf[n] = haloBuf[sendIds[n]]       (ogsKernels.okl:167-177)
          exchange      all-to-all of the send buffers into each rank's
                        receive region haloBuf[Nhalo:]           (MPI in the reference)
  Finish: local GatherScatter over the local rows (overlapping the exchange)
          postmpi Gather haloBuf[h] = fold(haloBuf[h], received partials of h)
          halo Scatter  every member of halo row h gets haloBuf[h]

Here every rank's operators are library handles built from maps
(ogs_setup_maps), the packing is ogs_extract, and the exchange -- a network
step in the reference -- is one more ogs_extract per rank that gathers its
receive region from the concatenated send buffers of all ranks.  The maps
follow the reference's construction for Unsigned handles
(ogsSetup.cpp:333-566 ConstructSharedNodes, 686-776 LocalUnsignedSetup;
ogsAllToAll.cpp:178-331): rows numbered by first appearance on the rank, local
and halo rows separately; members in ascending local index; each rank sends
its halo rows to every other rank holding the same id, ordered by
(destination rank, row); a rank receives from the source ranks in ascending
order; postmpi row h lists h itself, then its received entries in receive
order.  So a halo row folds the rank's own partial first, then the other
ranks' partials by ascending rank -- the reference's order.

The reference distributes ids to ranks by |id| % size and sorts across ranks
to find shared ids; with all ranks in one process the shared ids come from one
pass over all ranks' ids instead.  Only Unsigned handles are emulated.
"""
from __future__ import annotations

import numpy as np

from . import ogs


def _csr(rows_of_members, nrows):
    """T map with members of each row in ascending local index:
    rows_of_members[n] = row of local node n, or -1."""
    n = np.nonzero(rows_of_members >= 0)[0]
    r = rows_of_members[n]
    order = np.argsort(r, kind="stable")  # stable: members stay in ascending local index
    counts = np.bincount(r, minlength=nrows)
    starts = np.zeros(nrows + 1, np.int64)
    np.cumsum(counts, out=starts[1:])
    return starts.astype(np.int32), n[order].astype(np.int32)


def build_rank_maps(ids_list):
    """Per-rank maps of the emulated multi-rank Unsigned setup.

    Returns a list of dicts (one per rank) with: N, local (rowStarts, colIds),
    halo (rowStarts, colIds), halo_ids (|id| of each halo row), send_ids
    (halo rows in send order), send_counts[R], recv_counts[R], recv_rows
    (the local halo row of each received entry, receive order), post
    (rowStarts, colIds) over [halo rows | received entries]."""
    R = len(ids_list)
    absids = [np.abs(np.asarray(x, dtype=np.int64)) for x in ids_list]
    # ranks holding each id
    per_rank = [np.unique(a[a != 0]) for a in absids]
    allids = np.concatenate(per_rank) if per_rank else np.zeros(0, np.int64)
    ids_u, nranks = np.unique(allids, return_counts=True)
    shared_ids = ids_u[nranks > 1]
    out = []
    for r, a in enumerate(absids):
        nz = np.nonzero(a)[0]
        uniq, first = np.unique(a[nz], return_index=True)
        first = nz[first]
        is_sh = np.isin(uniq, shared_ids)
        # rows by first appearance, local and halo rows separately (ogsSetup.cpp:406-433)
        loc = np.nonzero(~is_sh)[0]
        hal = np.nonzero(is_sh)[0]
        loc = loc[np.argsort(first[loc], kind="stable")]
        hal = hal[np.argsort(first[hal], kind="stable")]
        row_of_uniq = np.empty(uniq.size, np.int64)
        row_of_uniq[loc] = np.arange(loc.size)
        row_of_uniq[hal] = np.arange(hal.size)
        node_uniq = np.searchsorted(uniq, a[nz])
        rows_local = np.full(a.size, -1, np.int64)
        rows_halo = np.full(a.size, -1, np.int64)
        m_loc = ~is_sh[node_uniq]
        rows_local[nz[m_loc]] = row_of_uniq[node_uniq[m_loc]]
        rows_halo[nz[~m_loc]] = row_of_uniq[node_uniq[~m_loc]]
        out.append({"N": int(a.size), "local": _csr(rows_local, loc.size), "halo": _csr(rows_halo, hal.size),
                    "halo_ids": uniq[hal], "nhalo": int(hal.size)})
    # exchange: rank r sends halo row h (id b) to every other rank j holding b,
    # ordered by (j, h) (ogsAllToAll.cpp:185-245)
    holders = {}
    for r, m in enumerate(out):
        for h, b in enumerate(m["halo_ids"]):
            holders.setdefault(int(b), []).append((r, h))
    sends = [[[] for _ in range(R)] for _ in range(R)]  # sends[r][j] = [(h_r, h_j)]
    for b, lst in holders.items():
        for r, hr in lst:
            for j, hj in lst:
                if j != r:
                    sends[r][j].append((hr, hj))
    for r in range(R):
        send_ids, counts = [], []
        for j in range(R):
            sends[r][j].sort()
            send_ids += [hr for hr, _ in sends[r][j]]
            counts.append(len(sends[r][j]))
        out[r]["send_ids"] = np.asarray(send_ids, np.int32)
        out[r]["send_counts"] = np.asarray(counts, np.int64)
    # receive order: source ranks ascending, each source in its send order
    for j in range(R):
        recv_rows, recv_src = [], []
        for r in range(R):
            recv_rows += [hj for _, hj in sends[r][j]]
        m = out[j]
        m["recv_rows"] = np.asarray(recv_rows, np.int64)
        m["recv_counts"] = np.asarray([len(sends[r][j]) for r in range(R)], np.int64)
        nh = m["nhalo"]
        # postmpi: row h = [h, Nhalo + p for received p of row h, in receive order]
        rows = np.concatenate([np.arange(nh), m["recv_rows"]])
        m["post"] = _csr(rows, nh)
        m["post_cols"] = nh + len(recv_rows)
    return out


class ranks_ogs_t:
    """GatherScatter over R emulated ranks on one device.

    ids_list: one int64 id array per rank.  Fields: one device tensor per rank
    (k interleaved components), all of one dtype."""

    def __init__(self, ids_list):
        import torch
        self.R = len(ids_list)
        self.maps = build_rank_maps(ids_list)
        self.local, self.halo, self.post = [], [], []
        for m in self.maps:
            self.local.append(ogs.ogs_t().SetupMaps(m["N"], *m["local"]))
            self.halo.append(ogs.ogs_t().SetupMaps(m["N"], *m["halo"]))
            self.post.append(ogs.ogs_t().SetupMaps(m["post_cols"], *m["post"]))
        # send buffers of all ranks, concatenated; each rank's receive region
        # gathers from it (the exchange)
        self.send_off = np.zeros(self.R + 1, np.int64)
        np.cumsum([m["send_ids"].size for m in self.maps], out=self.send_off[1:])
        dev = torch.device("cuda", torch.cuda.current_device())
        self.d_send_ids = [torch.from_numpy(m["send_ids"]).to(dev) for m in self.maps]
        recv_src = []
        for j, m in enumerate(self.maps):
            src = []
            for r in range(self.R):
                # position of (r -> j) entries inside r's send list
                before = int(self.maps[r]["send_counts"][:j].sum())
                cnt = int(self.maps[r]["send_counts"][j])
                src.append(self.send_off[r] + before + np.arange(cnt))
            recv_src.append(torch.from_numpy(np.concatenate(src).astype(np.int32)
                                             if src else np.zeros(0, np.int32)).to(dev))
        self.d_recv_src = recv_src
        self._bufs = {}

    def _buffers(self, dtype, k):
        import torch
        key = (dtype, k)
        if key not in self._bufs:
            dev = self.d_send_ids[0].device if self.R else None
            send = torch.empty(max(int(self.send_off[-1]) * k, 1), dtype=dtype, device=dev)
            bufs = [torch.empty(max(m["post_cols"] * k, 1), dtype=dtype, device=dev) for m in self.maps]
            self._bufs[key] = (send, bufs)
        return self._bufs[key]

    def GatherScatterStart(self, vs, k, op, stream=None):
        """Halo Gather, extract into the send buffers, exchange."""
        send, bufs = self._buffers(vs[0].dtype, k)
        for r, m in enumerate(self.maps):
            nh = m["nhalo"]
            if nh:
                self.halo[r].Gather(bufs[r][: nh * k], vs[r], k, op, ogs.Trans, stream=stream)
            ns = m["send_ids"].size
            if ns:
                ogs.extract(send[self.send_off[r] * k:(self.send_off[r] + ns) * k], bufs[r], self.d_send_ids[r],
                            k, stream=stream)
        for j, m in enumerate(self.maps):
            nrecv = self.d_recv_src[j].numel()
            if nrecv:
                nh = m["nhalo"]
                ogs.extract(bufs[j][nh * k:(nh + nrecv) * k], send, self.d_recv_src[j], k, stream=stream)

    def GatherScatterFinish(self, vs, k, op, stream=None):
        """Local GatherScatter, postmpi Gather (in place), halo Scatter."""
        _, bufs = self._buffers(vs[0].dtype, k)
        for r, m in enumerate(self.maps):
            if self.local[r].NlocalT:
                self.local[r].GatherScatter(vs[r], k, op, ogs.Sym, stream=stream)
            nh = m["nhalo"]
            if nh:
                self.post[r].Gather(bufs[r][: nh * k], bufs[r][: m["post_cols"] * k], k, op, ogs.Trans,
                                    stream=stream)
                self.halo[r].Scatter(vs[r], bufs[r][: nh * k], k, ogs.Trans, stream=stream)

    def GatherScatter(self, vs, k, op=ogs.Add, stream=None):
        self.GatherScatterStart(vs, k, op, stream)
        self.GatherScatterFinish(vs, k, op, stream)
        return vs


__all__ = ["build_rank_maps", "ranks_ogs_t"]
