"""Oracle for the emulated multi-rank gather-scatter (test infrastructure).

Computes, from the global picture alone, what the reference's multi-rank
GatherScatter (ogs_t, kinds Unsigned and Signed; libs/ogs/ogs.cpp:39-123 with
the all-to-all exchange of ogsAllToAll.cpp:126-175) and halo_t
Exchange/Combine (kind Halo; ogsHalo.cpp:39-359) leave on each rank:

* an id held by one rank (not for Halo, which leaves such ids alone): the
  single-rank operation over that rank's members (ogsOperator.cpp:60-360);
* an id held by several ranks: each holder folds its gather members -- N
  members (positive ids) for NoTrans, all members otherwise -- into a partial
  (gatherHalo Gather, ogs.cpp:59); it then folds, from the op identity, its own
  partial (for NoTrans only if it has an N member) followed by the partials of
  the other senders in ascending rank (for NoTrans only holders with an N
  member send, ogsAllToAll.cpp:232-241; postmpi rows list the own entry, then
  received entries in receive order, 270-331), and writes the result to its
  N members (Trans) or all members (NoTrans, Sym) (gatherHalo Scatter,
  ogs.cpp:120).  Holders of one id can therefore differ in the last bit for
  floating-point Add and Mul, as in the reference.
* N members: ids > 0 (Signed); all members on the rank holding the id's one
  positive copy and none elsewhere (Halo, ogsSetup.cpp:790-800); all
  (Unsigned).

Every fold runs through the C oracle (OracleOgs), so the op semantics are the
oracle's.  This module computes the expected fields; it builds no maps.
"""
from __future__ import annotations

import numpy as np

from . import OracleOgs


def _identity(dtype, op):
    dt = np.dtype(dtype)
    big = np.finfo(dt).max if dt.kind == "f" else np.iinfo(dt).max
    return {"add": dt.type(0), "mul": dt.type(1), "max": dt.type(-big), "min": dt.type(big)}[op]


def _rows_by_first_appearance(ids):
    """Distinct nonzero |ids| in order of first appearance (the oracle's row order)."""
    a = np.abs(ids)
    nz = np.nonzero(a)[0]
    u, first = np.unique(a[nz], return_index=True)
    return u[np.argsort(first, kind="stable")]


def ranks_gather_scatter(ids_list, vs, k, op, kind="unsigned", trans="sym"):
    """Expected fields after a multi-rank GatherScatter (kind "unsigned" or
    "signed"), or a halo Exchange (kind "halo", op "add", trans "notrans") or
    Combine (kind "halo", op "add", trans "trans").  ids_list: int64 id arrays
    per rank; vs: numpy field arrays per rank (k interleaved components)."""
    idsl = [np.asarray(x, dtype=np.int64) for x in ids_list]
    absids = [np.abs(x) for x in idsl]
    holders = {}
    for r, a in enumerate(absids):
        for b in np.unique(a[a != 0]):
            holders.setdefault(int(b), []).append(r)
    shared = np.asarray(sorted(b for b, h in holders.items() if len(h) > 1), np.int64)
    owner = {}
    if kind == "halo":
        for r, x in enumerate(idsl):
            for b in np.unique(x[x > 0]):
                owner[int(b)] = r
    dtype = vs[0].dtype
    notrans, tr = trans == "notrans", trans == "trans"

    def nmask(r):
        """N members of rank r."""
        x, a = idsl[r], absids[r]
        if kind == "unsigned":
            return a != 0
        if kind == "signed":
            return x > 0
        return np.array([owner.get(int(b), -1) == r for b in a], bool) & (a != 0)

    out = [v.copy() for v in vs]
    if kind != "halo":
        for r, (x, a) in enumerate(zip(idsl, absids)):
            loc = np.where(np.isin(a, shared), 0, x if kind == "signed" else a)
            OracleOgs(loc, kind).gather_scatter(out[r], k, op, trans)
    # partials of the shared ids: fold over the gather members
    partial = []
    for r, a in enumerate(absids):
        sh = np.isin(a, shared)
        gmem = sh & (nmask(r) if notrans else True)
        ih = np.where(gmem, a, 0)
        rows = _rows_by_first_appearance(ih)
        p = {}
        if rows.size:
            gv = np.zeros(rows.size * k, dtype)
            OracleOgs(ih.copy(), "unsigned").gather(gv, vs[r], k, op, "trans")
            for i, b in enumerate(rows):
                p[int(b)] = gv[i * k:(i + 1) * k]
        partial.append(p)
    ident = np.full(k, _identity(dtype, op), dtype)
    for j, a in enumerate(absids):
        sh = np.isin(a, shared)
        mine = [int(b) for b in _rows_by_first_appearance(np.where(sh, a, 0))]
        if not mine:
            continue
        cid, vals, empty = [], [], set()
        for b in mine:
            seq = ([j] if b in partial[j] else []) + [s for s in holders[b] if s != j and b in partial[s]]
            if not seq:
                empty.add(b)
            for s in seq:
                cid.append(b)
                vals.append(partial[s][b])
        val = {b: ident for b in empty}
        if cid:
            uniq_order = [b for b in mine if b not in empty]
            gv = np.zeros(len(uniq_order) * k, dtype)
            OracleOgs(np.asarray(cid, np.int64), "unsigned").gather(gv, np.concatenate(vals).astype(dtype), k, op,
                                                                    "trans")
            for i, b in enumerate(uniq_order):
                val[b] = gv[i * k:(i + 1) * k]
        smem = sh & (nmask(j) if tr else True)
        x = out[j]
        for n in np.nonzero(smem)[0]:
            x[n * k:(n + 1) * k] = val[int(a[n])]
    return out


def partition_box(nx, ny, nz, p, R, how="slabs", seed=0):
    """Ids of an nx*ny*nz box of degree-p hexes split over R ranks by element:
    "slabs" (contiguous element ranges in the box's element order, like
    MakeIds' rank grid along z, dawgsMain.cpp:58-105) or "random" (each
    element to a rank drawn from a seeded generator).  Returns per-rank id
    arrays, each element's nodes contiguous in element order."""
    from dawgs_gb300 import mesh
    ids = mesh.box_ids(nx, ny, nz, p)
    npe = (p + 1) ** 3
    ne = nx * ny * nz
    if how == "slabs":
        owner = (np.arange(ne) * R) // max(ne, 1)
    else:
        owner = (mesh.splitmix64(np.arange(ne, dtype=np.uint64) + np.uint64(seed)) % np.uint64(R)).astype(np.int64)
    el = ids.reshape(ne, npe)
    return [el[owner == r].reshape(-1).copy() for r in range(R)]


def signed_parts(parts, seed, kind):
    """Signs for a partition.  "signed": each entry negative with probability
    1/2 (a seeded generator).  "halo": each id's one positive copy on the
    lowest rank holding it, at its first local occurrence there, every other
    copy negative (ogsSetup.cpp:293-296 needs exactly one)."""
    from dawgs_gb300 import mesh
    out = []
    if kind == "signed":
        for r, p in enumerate(parts):
            flip = (mesh.splitmix64(np.arange(p.size, dtype=np.uint64) + np.uint64(seed + 1000 * r)) & np.uint64(1))
            out.append(np.where(flip.astype(bool), -p, p))
        return out
    seen = set()
    for p in parts:
        q = -np.abs(p)
        for n in range(p.size):
            b = int(abs(p[n]))
            if b and b not in seen:
                seen.add(b)
                q[n] = b
        out.append(q)
    return out


def gathered_rows(ids_list, kind):
    """Each rank's gathered-vector rows by id: (local ids in row order, halo
    ids in row order, number of halo rows with a positive member).  Rows by
    first appearance on the rank, in four classes numbered apart: local rows
    with a positive member, the other local rows, halo rows with a positive
    member, the other halo rows (ogsSetup.cpp:406-433)."""
    idsl = [np.asarray(x, dtype=np.int64) for x in ids_list]
    absids = [np.abs(x) for x in idsl]
    holders = {}
    for r, a in enumerate(absids):
        for b in np.unique(a[a != 0]):
            holders.setdefault(int(b), []).append(r)
    out = []
    for x, a in zip(idsl, absids):
        order = _rows_by_first_appearance(a)
        pos = set(int(b) for b in np.unique(a[x > 0])) if kind == "signed" else set(int(b) for b in order)
        loc = [int(b) for b in order if len(holders[int(b)]) == 1]
        hal = [int(b) for b in order if len(holders[int(b)]) > 1]
        loc = [b for b in loc if b in pos] + [b for b in loc if b not in pos]
        halp = [b for b in hal if b in pos]
        out.append((loc, halp + [b for b in hal if b not in pos], len(halp)))
    return out, holders


def gathered_exchange(ids_list, gvs, k, kind, trans):
    """Expected gathered vectors after a halo_t made from a gather runs
    Exchange (trans "notrans": each copy of a halo row not owned on its rank
    gets identity + the owners' values, ogsHalo.cpp:55-146) or Combine (trans
    "trans": each owned copy gets identity + its own value + the other copies'
    values by ascending rank, ogsHalo.cpp:203-290).  gvs: per rank
    [local rows | halo rows] * k."""
    rows, holders = gathered_rows(ids_list, kind)
    dtype = gvs[0].dtype
    where = []  # per rank: halo id -> (row in the gathered vector, owned)
    for loc, hal, nhp in rows:
        where.append({b: (len(loc) + h, h < nhp) for h, b in enumerate(hal)})
    out = [g.copy() for g in gvs]
    ident = np.full(k, _identity(dtype, "add"), dtype)
    for j, (loc, hal, nhp) in enumerate(rows):
        todo = [b for b in hal if (not where[j][b][1]) == (trans == "notrans")]
        cid, vals, empty = [], [], set()
        for b in todo:
            if trans == "notrans":
                seq = [s for s in holders[b] if s != j and where[s][b][1]]
            else:
                seq = [j] + [s for s in holders[b] if s != j]
            if not seq:
                empty.add(b)
            for s in seq:
                row = where[s][b][0]
                cid.append(b)
                vals.append(gvs[s][row * k:(row + 1) * k])
        val = {b: ident for b in empty}
        if cid:
            order = [b for b in todo if b not in empty]
            gv = np.zeros(len(order) * k, dtype)
            OracleOgs(np.asarray(cid, np.int64), "unsigned").gather(gv, np.concatenate(vals).astype(dtype), k,
                                                                    "add", "trans")
            for i, b in enumerate(order):
                val[b] = gv[i * k:(i + 1) * k]
        for b in todo:
            row = where[j][b][0]
            out[j][row * k:(row + 1) * k] = val[b]
    return out


def _fold_lists(lists, k, op, dtype):
    """fold from the op identity over each list of k-vectors, in list order
    (through OracleOgs: entries of row i carry id i + 1, rows in order)."""
    out = [None] * len(lists)
    cid, vals = [], []
    for i, lst in enumerate(lists):
        if not lst:
            out[i] = np.full(k, _identity(dtype, op), dtype)
        for x in lst:
            cid.append(i + 1)
            vals.append(x)
    if cid:
        present = [i for i, lst in enumerate(lists) if lst]
        gv = np.zeros(len(present) * k, dtype)
        OracleOgs(np.asarray(cid, np.int64), "unsigned").gather(gv, np.concatenate(vals).astype(dtype), k, op,
                                                                "trans")
        for n, i in enumerate(present):
            out[i] = gv[n * k:(n + 1) * k]
    return out


def _members(ids_list):
    """Per rank: |id| -> (all members, positive members), ascending local index."""
    out = []
    for x in ids_list:
        x = np.asarray(x, np.int64)
        m = {}
        for n in np.nonzero(x)[0]:
            b = int(abs(x[n]))
            t, p = m.setdefault(b, ([], []))
            t.append(int(n))
            if x[n] > 0:
                p.append(int(n))
        out.append(m)
    return out


def ranks_gather(ids_list, vs, k, op, trans):
    """Expected gathered vectors of a multi-rank Signed ogs_t Gather
    (ogs.cpp:202-298): [local rows | halo rows with a positive member (all
    halo rows for Sym)]; local rows and NoTrans/Sym halo rows fold this
    rank's members (N members for NoTrans), Trans halo rows fold this rank's
    partial and then the other holders' partials by ascending rank."""
    rows, holders = gathered_rows(ids_list, "signed")
    mem = _members(ids_list)
    dtype = vs[0].dtype
    sel = (lambda b, r: mem[r][b][1]) if trans == "notrans" else (lambda b, r: mem[r][b][0])
    out = []
    for r, (loc, hal, nhp) in enumerate(rows):
        v = vs[r]
        val = lambda n: v[n * k:(n + 1) * k]
        lists = [[val(n) for n in sel(b, r)] for b in loc]
        hrows = hal if trans == "sym" else hal[:nhp]
        if trans == "trans":
            for b in hrows:
                seq = [r] + [s for s in holders[b] if s != r]
                lists.append([_fold_lists([[vs[s][n * k:(n + 1) * k] for n in mem[s][b][0]]], k, op, dtype)[0]
                              for s in seq])
        else:
            lists += [[val(n) for n in sel(b, r)] for b in hrows]
        folded = _fold_lists(lists, k, op, dtype)
        out.append(np.concatenate(folded) if folded else np.zeros(0, dtype))
    return out


def ranks_scatter(ids_list, vs, gvs, k, trans):
    """Expected local vectors after a multi-rank Signed ogs_t Scatter
    (ogs.cpp:392-488) of gathered vectors [local rows | halo rows]: Trans
    writes each row's value to its positive members, NoTrans and Sym to all
    members; NoTrans halo rows take, from the op identity (Add), the value of
    the rank holding the positive copy (exchanged)."""
    rows, holders = gathered_rows(ids_list, "signed")
    mem = _members(ids_list)
    dtype = vs[0].dtype
    where = [{b: (len(loc) + h) for h, b in enumerate(hal)} for loc, hal, _ in rows]
    owner = {b: r for r, (loc, hal, nhp) in enumerate(rows) for b in hal[:nhp]}
    out = [v.copy() for v in vs]
    for r, (loc, hal, nhp) in enumerate(rows):
        g = gvs[r]
        tgt = (lambda b: mem[r][b][1]) if trans == "trans" else (lambda b: mem[r][b][0])
        for i, b in enumerate(loc):
            for n in tgt(b):
                out[r][n * k:(n + 1) * k] = g[i * k:(i + 1) * k]
        if trans == "notrans":
            lists = []
            for b in hal:
                o = owner.get(b)
                lists.append([] if o is None else [gvs[o][where[o][b] * k:(where[o][b] + 1) * k]])
            vals = _fold_lists(lists, k, "add", dtype)
            for b, x in zip(hal, vals):
                for n in mem[r][b][0]:
                    out[r][n * k:(n + 1) * k] = x
        else:
            for h, b in enumerate(hal if trans == "sym" else hal[:nhp]):
                row = len(loc) + h
                for n in tgt(b):
                    out[r][n * k:(n + 1) * k] = g[row * k:(row + 1) * k]
    return out
