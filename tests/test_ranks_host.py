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


def _gather(rs, ci, src, k, op, dt):
    out = np.zeros((len(rs) - 1) * k, dt)
    for r in range(len(rs) - 1):
        for c in range(k):
            out[r * k + c] = _fold([src[m * k + c] for m in ci[rs[r]:rs[r + 1]]], op, dt)
    return out


def _scatter(rs, ci, dst, gv, k):
    for r in range(len(rs) - 1):
        for m in ci[rs[r]:rs[r + 1]]:
            dst[m * k:(m + 1) * k] = gv[r * k:(r + 1) * k]


def cpu_emulate(maps, vs, k, op):
    dt = vs[0].dtype
    R = len(maps)
    vs = [v.copy() for v in vs]
    bufs, sends = [], []
    for m, v in zip(maps, vs):
        hb = np.zeros(m["post_cols"] * k, dt)
        hb[: m["nhalo"] * k] = _gather(*m["halo"], v, k, op, dt)
        bufs.append(hb)
        sends.append(np.concatenate([hb[h * k:(h + 1) * k] for h in m["send_ids"]]) if m["send_ids"].size
                     else np.zeros(0, dt))
    for j, m in enumerate(maps):
        parts = []
        for r in range(R):
            before = int(maps[r]["send_counts"][:j].sum()) * k
            parts.append(sends[r][before:before + int(maps[r]["send_counts"][j]) * k])
        recv = np.concatenate(parts) if parts else np.zeros(0, dt)
        bufs[j][m["nhalo"] * k:] = recv
    for m, v, hb in zip(maps, vs, bufs):
        rs, ci = m["local"]
        _scatter(rs, ci, v, _gather(rs, ci, v, k, op, dt), k)
        hb[: m["nhalo"] * k] = _gather(*m["post"], hb, k, op, dt)
        _scatter(*m["halo"], v, hb[: m["nhalo"] * k], k)
    return vs


CASES = [((4, 3, 2, 2), 2, "slabs"), ((4, 3, 2, 2), 3, "random"), ((3, 3, 3, 1), 4, "random"),
         ((5, 2, 2, 2), 5, "slabs")]


@pytest.mark.parametrize("box,R,how", CASES)
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32], ids=lambda t: np.dtype(t).name)
@pytest.mark.parametrize("op", ["add", "max"])
def test_emulated_ranks_match_oracle(oracle_mod, box, R, how, dtype, op):
    parts = oranks.partition_box(*box, R, how=how, seed=9)
    maps = ranks.build_rank_maps(parts)
    for k in (1, 2):
        vs = [values(k * p.size, dtype, op, seed=20 + i) for i, p in enumerate(parts)]
        got = cpu_emulate(maps, vs, k, op)
        want = oranks.ranks_gather_scatter(parts, vs, k, op)
        for g, w in zip(got, want):
            assert g.tobytes() == w.tobytes(), (box, R, how, k)


def test_maps_are_consistent():
    parts = oranks.partition_box(6, 4, 3, 2, 4, how="random", seed=3)
    maps = ranks.build_rank_maps(parts)
    for j, m in enumerate(maps):
        # every halo row receives one entry from every other holder of its id
        holders = sum(np.isin(m["halo_ids"], np.abs(p)).astype(int) for i, p in enumerate(parts) if i != j)
        assert np.array_equal(np.bincount(m["recv_rows"], minlength=m["nhalo"]), holders)
        assert int(m["recv_counts"].sum()) == m["recv_rows"].size
        assert sum(int(maps[r]["send_counts"][j]) for r in range(len(maps))) == m["recv_rows"].size
        # every local node is in exactly one local or halo row
        cols = np.concatenate([m["local"][1], m["halo"][1]])
        assert np.array_equal(np.sort(cols), np.arange(m["N"]))
        # the library accepts each operator's maps (host-only handles)
        for N, (rs, ci) in ((m["N"], m["local"]), (m["N"], m["halo"]), (m["post_cols"], m["post"])):
            g = ogs.ogs_t().SetupMaps(N, rs, ci, host_only=True)
            assert g.NlocalT == rs.size - 1 and g.nnzT == ci.size


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
