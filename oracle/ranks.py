"""Oracle for the emulated multi-rank GatherScatter (test infrastructure).

Computes, from the global picture alone, what the reference's multi-rank
Unsigned GatherScatter leaves on each rank (libs/ogs/ogs.cpp:39-123 with the
all-to-all exchange of ogsAllToAll.cpp:126-175):

* an id held by one rank: that rank's ordinary fold over its members in
  ascending local index (ogsOperator.cpp:311-360);
* an id held by several ranks: each holder first folds its own members
  (gatherHalo Gather, ogs.cpp:59), then folds, from the op identity, its own
  partial followed by the other holders' partials in ascending rank (postmpi:
  row h lists h first, then received entries in receive order, and entries
  arrive ordered by source rank, ogsAllToAll.cpp:270-331), and writes that
  to all its members (gatherHalo Scatter, ogs.cpp:120).  Holders of one id
  can therefore differ in the last bit for floating-point Add and Mul, as in
  the reference.

Every fold runs through the C oracle (OracleOgs), so the op semantics are the
oracle's.  This module computes the expected fields; it builds no maps.
"""
from __future__ import annotations

import numpy as np

from . import OracleOgs


def _rows_by_first_appearance(ids):
    """Distinct nonzero |ids| in order of first appearance (the oracle's row order)."""
    a = np.abs(ids)
    nz = np.nonzero(a)[0]
    u, first = np.unique(a[nz], return_index=True)
    return u[np.argsort(first, kind="stable")]


def ranks_gather_scatter(ids_list, vs, k, op):
    """Expected fields after a multi-rank GatherScatter (Sym).  ids_list: int64
    id arrays per rank; vs: numpy field arrays per rank (k interleaved
    components, same dtype); op: "add" | "mul" | "max" | "min"."""
    R = len(ids_list)
    absids = [np.abs(np.asarray(x, dtype=np.int64)) for x in ids_list]
    holders = {}
    for r, a in enumerate(absids):
        for b in np.unique(a[a != 0]):
            holders.setdefault(int(b), []).append(r)
    shared = np.asarray(sorted(b for b, h in holders.items() if len(h) > 1), np.int64)
    dtype = vs[0].dtype
    out, partial = [], []
    for r, a in enumerate(absids):
        sh = np.isin(a, shared)
        x = vs[r].copy()
        # local rows: ordinary single-rank fold, shared ids left out
        OracleOgs(np.where(sh, 0, a), "unsigned").gather_scatter(x, k, op, "sym")
        out.append(x)
        # halo partials: Gather over the shared ids of this rank
        ih = np.where(sh, a, 0)
        rows = _rows_by_first_appearance(ih)
        p = {}
        if rows.size:
            gv = np.zeros(rows.size * k, dtype)
            OracleOgs(ih.copy(), "unsigned").gather(gv, vs[r], k, op, "trans")
            for i, b in enumerate(rows):
                p[int(b)] = gv[i * k:(i + 1) * k]
        partial.append(p)
    for r, a in enumerate(absids):
        mine = [int(b) for b in _rows_by_first_appearance(np.where(np.isin(a, shared), a, 0))]
        if not mine:
            continue
        # each id's entries in fold order: own partial, then the other holders by rank
        cid, vals = [], []
        for b in mine:
            for s in [r] + [s for s in holders[b] if s != r]:
                cid.append(b)
                vals.append(partial[s][b])
        cid = np.asarray(cid, np.int64)
        w = np.concatenate(vals).astype(dtype)
        gv = np.zeros(len(mine) * k, dtype)
        OracleOgs(cid.copy(), "unsigned").gather(gv, w, k, op, "trans")
        val = {b: gv[i * k:(i + 1) * k] for i, b in enumerate(mine)}
        x = out[r]
        for n in np.nonzero(np.isin(a, shared))[0]:
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
