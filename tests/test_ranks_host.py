"""The emulated multi-rank maps (dawgs_gb300/ranks.py) on the CPU: a scalar
executor runs the reference's multi-rank GatherScatter steps over them (halo
Gather, extract, all-to-all, local GatherScatter, postmpi Gather, halo
Scatter; ogs.cpp:39-123, ogsAllToAll.cpp:126-175) and must give the oracle's
fields bit for bit; ogs_setup_maps accepts every map and rejects bad ones."""
import ctypes as C

import numpy as np
import pytest

from dawgs_gb300 import _lib, ogs, ranks
from helpers import values
from oracle import ranks as oranks


def _fold(vals, op, dt):
    if dt.kind == "f":
        big = np.finfo(dt).max
    else:
        big = np.iinfo(dt).max
    a = {"add": dt.type(0), "mul": dt.type(1), "max": dt.type(-big), "min": dt.type(big)}[op]
    with np.errstate(over="ignore", invalid="ignore"):
        for b in vals:
            if op == "add":
                a = dt.type(a + b)
            elif op == "mul":
                a = dt.type(a * b)
            elif op == "max":
                a = b if b > a else a
            else:
                a = b if b < a else a
    return a


def _fold_rows(rs, ci, rows, src, k, op, dt):
    out = {}
    for r in rows:
        out[r] = np.array([_fold([src[m * k + c] for m in ci[rs[r]:rs[r + 1]]], op, dt) for c in range(k)], dt)
    return out


def _op_gather(maps4, nrowsN, src, gv, k, op, dt, trans):
    """ogsOperator Gather (ogsOperator.cpp:60-97): NoTrans folds the N members
    of rows < NrowsN, otherwise the T members of every row."""
    rsT, ciT, rsN, ciN = maps4
    rs, ci, rows = (rsN, ciN, range(nrowsN)) if trans == "notrans" else (rsT, ciT, range(len(rsT) - 1))
    for r, val in _fold_rows(rs, ci, rows, src, k, op, dt).items():
        gv[r * k:(r + 1) * k] = val


def _op_scatter(maps4, nrowsN, dst, gv, k, trans):
    """ogsOperator Scatter (ogsOperator.cpp:206-238): Trans writes the N
    members of rows < NrowsN, otherwise the T members of every row."""
    rsT, ciT, rsN, ciN = maps4
    rs, ci, rows = (rsN, ciN, range(nrowsN)) if trans == "trans" else (rsT, ciT, range(len(rsT) - 1))
    for r in rows:
        for m in ci[rs[r]:rs[r + 1]]:
            dst[m * k:(m + 1) * k] = gv[r * k:(r + 1) * k]


def _op_gs(maps4, v, k, op, dt, trans):
    """ogsOperator GatherScatter (ogsOperator.cpp:311-360): gather N members
    for NoTrans, T otherwise; write N members for Trans, T otherwise; every row."""
    rsT, ciT, rsN, ciN = maps4
    g = (rsN, ciN) if trans == "notrans" else (rsT, ciT)
    s = (rsN, ciN) if trans == "trans" else (rsT, ciT)
    vals = _fold_rows(*g, range(len(rsT) - 1), v, k, op, dt)
    for r, val in vals.items():
        for m in s[1][s[0][r]:s[0][r + 1]]:
            v[m * k:(m + 1) * k] = val


def cpu_emulate(maps, vs, k, op, trans="sym", halo_only=False):
    """The reference's multi-rank steps over the emulated maps, one scalar at a time."""
    dt = vs[0].dtype
    R = len(maps)
    which = "N" if trans == "notrans" else "T"
    vs = [v.copy() for v in vs]
    bufs, sends = [], []
    for m, v in zip(maps, vs):
        hb = np.zeros(max(m["postT_cols"], m["postN_cols"]) * k, dt)
        _op_gather(m["halo"], m["nhaloP"], v, hb, k, op, dt, trans)
        bufs.append(hb)
        ids = m["send_" + which]
        sends.append(np.concatenate([hb[h * k:(h + 1) * k] for h in ids]) if ids.size else np.zeros(0, dt))
    for j, m in enumerate(maps):
        parts = []
        for r in range(R):
            cnt = maps[r]["send_counts_" + which]
            before = int(cnt[:j].sum()) * k
            parts.append(sends[r][before:before + int(cnt[j]) * k])
        recv = np.concatenate(parts)
        bufs[j][m["nhalo"] * k:m["nhalo"] * k + recv.size] = recv
    for m, v, hb in zip(maps, vs, bufs):
        if not halo_only:
            _op_gs(m["local"], v, k, op, dt, trans)
        nh = m["nhalo"]
        post = m["post" + which]
        out = hb.copy()
        for r, val in _fold_rows(*post, range(nh), hb, k, op, dt).items():
            out[r * k:(r + 1) * k] = val
        _op_scatter(m["halo"], m["nhaloP"], v, out[: nh * k], k, trans)
    return vs


CASES = [((4, 3, 2, 2), 2, "slabs"), ((4, 3, 2, 2), 3, "random"), ((3, 3, 3, 1), 4, "random"),
         ((5, 2, 2, 2), 5, "slabs")]
KINDS = {"unsigned": ranks.UNSIGNED, "signed": ranks.SIGNED, "halo": ranks.HALO}


# (kind, transpose, op): ogs_t GatherScatter for Unsigned/Signed; halo_t
# Exchange (NoTrans) and Combine (Trans) always add
MODES = [("unsigned", "sym", "add"), ("unsigned", "sym", "max"), ("signed", "sym", "add"),
         ("signed", "notrans", "add"), ("signed", "trans", "max"), ("signed", "notrans", "min"),
         ("halo", "notrans", "add"), ("halo", "trans", "add")]


@pytest.mark.parametrize("box,R,how", CASES)
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32], ids=lambda t: np.dtype(t).name)
@pytest.mark.parametrize("kind,trans,op", MODES)
def test_emulated_ranks_match_oracle(oracle_mod, box, R, how, dtype, kind, trans, op):
    parts = oranks.partition_box(*box, R, how=how, seed=9)
    if kind != "unsigned":
        parts = oranks.signed_parts(parts, 4, kind)
    maps = ranks.build_rank_maps(parts, KINDS[kind])
    for k in (1, 2):
        vs = [values(k * p.size, dtype, op, seed=20 + i) for i, p in enumerate(parts)]
        got = cpu_emulate(maps, vs, k, op, trans, halo_only=kind == "halo")
        want = oranks.ranks_gather_scatter(parts, vs, k, op, kind, trans)
        for g, w in zip(got, want):
            assert g.tobytes() == w.tobytes(), (box, R, how, k)


def test_maps_are_consistent():
    parts = oranks.partition_box(6, 4, 3, 2, 4, how="random", seed=3)
    maps = ranks.build_rank_maps(parts)
    for j, m in enumerate(maps):
        # every halo row receives one entry from every other holder of its id
        holders = sum(np.isin(m["halo_ids"], np.abs(p)).astype(int) for i, p in enumerate(parts) if i != j)
        assert np.array_equal(np.bincount(m["recv_rows_T"], minlength=m["nhalo"]), holders)
        assert sum(int(maps[r]["send_counts_T"][j]) for r in range(len(maps))) == m["recv_rows_T"].size
        # every local node is in exactly one local or halo row
        cols = np.concatenate([m["local"][1], m["halo"][1]])
        assert np.array_equal(np.sort(cols), np.arange(m["N"]))
        # the library accepts each operator's maps (host-only handles)
        for N, maps4 in ((m["N"], m["local"]), (m["N"], m["halo"])):
            g = ogs.ogs_t().SetupMaps(N, *maps4[:2], host_only=True)
            assert g.NlocalT == maps4[0].size - 1 and g.nnzT == maps4[1].size
        for N, (rs, ci) in ((m["postT_cols"], m["postT"]), (m["postN_cols"], m["postN"])):
            ogs.ogs_t().SetupMaps(N, rs, ci, host_only=True)


def test_signed_and_halo_maps_accepted():
    parts = oranks.partition_box(5, 4, 3, 2, 3, how="random", seed=8)
    for kind in ("signed", "halo"):
        sp = oranks.signed_parts(parts, 2, kind)
        for m in ranks.build_rank_maps(sp, KINDS[kind]):
            for N, maps4, nP in ((m["N"], m["local"], m["nlocalP"]), (m["N"], m["halo"], m["nhaloP"])):
                g = ogs.ogs_t().SetupMaps(N, maps4[0], maps4[1], maps4[2], maps4[3], NrowsN=nP, host_only=True)
                assert g.NlocalP == nP and g.nnzN == maps4[3].size


def test_halo_needs_one_positive_copy():
    parts = oranks.partition_box(3, 2, 2, 1, 2, how="slabs")
    with pytest.raises(ValueError):
        ranks.build_rank_maps(parts, ranks.HALO)  # every copy positive


def test_setup_maps_rejects_bad_maps(built_lib):
    h = C.c_void_p()

    def setup(N, rsT, ciT, rsN=None, ciN=None, NrowsN=None):
        rsT = np.asarray(rsT, np.int32)
        ciT = np.asarray(ciT, np.int32)
        a = [C.byref(h), N, NrowsN if NrowsN is not None else rsT.size - 1, rsT.size - 1]
        if rsN is None:
            a += [None, None]
        else:
            rsN = np.asarray(rsN, np.int32)
            ciN = np.asarray(ciN, np.int32)
            a += [rsN.ctypes.data, ciN.ctypes.data if ciN.size else None]
        a += [rsT.ctypes.data, ciT.ctypes.data if ciT.size else None, _lib.SETUP_HOST_ONLY]
        return built_lib.ogs_setup_maps(*a)

    assert setup(4, [0, 2, 4], [0, 1, 2, 3]) == _lib.OGS_OK
    built_lib.ogs_free(h)
    assert setup(4, [0, 2, 4], [0, 1, 2, 9]) == _lib.OGS_ERANGE          # column outside [0, N)
    assert setup(4, [0, 3, 2], [0, 1, 2, 3]) == _lib.OGS_EINVAL          # rowStarts decreases
    assert setup(4, [1, 2, 4], [0, 1, 2, 3]) == _lib.OGS_EINVAL          # rowStarts[0] != 0
    assert setup(4, [0, 2, 4], [0, 1, 2, 3], [0, 1, 2], [1, 3]) == _lib.OGS_OK    # N rows subsequences
    built_lib.ogs_free(h)
    assert setup(4, [0, 2, 4], [0, 1, 2, 3], [0, 1, 2], [1, 0]) == _lib.OGS_EINVAL  # N member not in T row
    assert setup(4, [0, 2, 4], [0, 1, 2, 3], [0, 1, 2], [1, 3], NrowsN=1) == _lib.OGS_EINVAL  # row >= NrowsN
    assert b"NrowsN" in built_lib.ogs_last_error_string()
    assert setup(4, [0, 2, 4], [0, 1, 2, 3], [0, 1, 1], [1], NrowsN=1) == _lib.OGS_OK
    built_lib.ogs_free(h)


def test_setup_maps_with_empty_rows():
    """Rows without members (postmpi N rows with nothing received) are valid:
    they go to the general bucket."""
    rs = np.array([0, 2, 2, 3, 3, 3], np.int32)  # rows 1, 3 and 4 empty
    ci = np.array([0, 2, 1], np.int32)
    g = ogs.ogs_t().SetupMaps(4, rs, ci, host_only=True)
    st = g.layout_stats()
    assert g.NlocalT == 5 and st["rows_general"] == 3


def cpu_gathered(maps, gvs, k, trans):
    """Gathered-halo Exchange / Combine over the emulated maps, scalar by scalar."""
    dt = gvs[0].dtype
    R = len(maps)
    which = "N" if trans == "notrans" else "T"
    gvs = [g.copy() for g in gvs]
    bufs, sends = [], []
    for m, g in zip(maps, gvs):
        nl, nh, nhp = m["nlocal"], m["nhalo"], m["nhaloP"]
        hb = np.zeros(max(m["postT_cols"], m["postN_cols"]) * k, dt)
        rows = nhp if which == "N" else nh
        hb[: rows * k] = g[nl * k:(nl + rows) * k]
        bufs.append(hb)
        ids = m["send_" + which]
        sends.append(np.concatenate([hb[h * k:(h + 1) * k] for h in ids]) if ids.size else np.zeros(0, dt))
    for j, m in enumerate(maps):
        parts = []
        for r in range(R):
            cnt = maps[r]["send_counts_" + which]
            before = int(cnt[:j].sum()) * k
            parts.append(sends[r][before:before + int(cnt[j]) * k])
        recv = np.concatenate(parts)
        bufs[j][m["nhalo"] * k:m["nhalo"] * k + recv.size] = recv
    for m, g, hb in zip(maps, gvs, bufs):
        nl, nh, nhp = m["nlocal"], m["nhalo"], m["nhaloP"]
        out = hb.copy()
        for r, val in _fold_rows(*m["post" + which], range(nh), hb, k, "add", dt).items():
            out[r * k:(r + 1) * k] = val
        if which == "N":
            g[(nl + nhp) * k:(nl + nh) * k] = out[nhp * k:nh * k]
        else:
            g[nl * k:(nl + nhp) * k] = out[: nhp * k]
    return gvs


@pytest.mark.parametrize("box,R,how", CASES)
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32], ids=lambda t: np.dtype(t).name)
@pytest.mark.parametrize("kind", ["signed", "unsigned"])
@pytest.mark.parametrize("trans", ["notrans", "trans"])
def test_gathered_halo_matches_oracle(oracle_mod, box, R, how, dtype, kind, trans):
    parts = oranks.partition_box(*box, R, how=how, seed=9)
    if kind == "signed":
        parts = oranks.signed_parts(parts, 4, "halo")  # one positive copy per id: the gather is defined
    maps = ranks.build_rank_maps(parts, KINDS[kind])
    rows, _ = oranks.gathered_rows(parts, kind)
    for m, (loc, hal, nhp) in zip(maps, rows):  # the two numberings agree
        assert (m["nlocal"], m["nhalo"], m["nhaloP"]) == (len(loc), len(hal), nhp)
        assert [int(b) for b in m["halo_ids"]] == hal
    for k in (1, 2):
        gvs = [values((m["nlocal"] + m["nhalo"]) * k, dtype, "add", seed=30 + i) for i, m in enumerate(maps)]
        got = cpu_gathered(maps, gvs, k, trans)
        want = oranks.gathered_exchange(parts, gvs, k, kind, trans)
        for g, w in zip(got, want):
            assert g.tobytes() == w.tobytes(), (box, R, how, k)

