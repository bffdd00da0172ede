"""Pin the CPU oracle (oracle/ogs_oracle.c) to the reference.

1. Against tests/golden/golden.json, which gslib -- the reference's own
   checker, 3rdParty/gslib, built from the reference tree -- produced
   (tests/golden/make_golden.py), including gs_test.c's known answers.
2. Against gslib live, on more cases, when oracle/_ref/libgsref.so exists.

gslib and host ogs fold each id group in the same order (primary then the
others ascending, gs_local.c:58-72; ogs starts from the identity, which is
exact for 0+x and 1*x), so results agree bit for bit.  Two documented
differences are excluded: gslib leaves degree-1 entries untouched where ogs
computes identity-op-x (visible only for -0.0, NaN and, for Max, values at or
below -max), and for transpose=1 gslib writes id groups with no unflagged
member where ogs skips them (ogsOperator.cpp:321-326).
"""
import base64
import hashlib
import json
import os

import numpy as np
import pytest

from dawgs_gb300 import mesh
from helpers import OPS, TYPES, first_diff, random_ids, same_bits, signed_ids, values

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("case", [c for c in GOLD["cases"] if c["kind"] == "unsigned"],
                         ids=lambda c: f"{c['dtype']}-{c['op']}-{c['layout']}")
def test_oracle_matches_gslib_golden_unsigned(oracle_mod, case):
    nx, ny, nz, p = case["mesh"]
    ids = mesh.box_ids(nx, ny, nz, p)
    h = oracle_mod.OracleOgs(ids.copy(), "unsigned")
    k, dt, op = case["k"], np.dtype(case["dtype"]), case["op"]
    if case["layout"] == "many":
        vs = [values(ids.size, dt, op, case["seed"] + j) for j in range(k)]
        assert sha(np.concatenate(vs)) == case["input_sha256"], "input generator drifted"
        for x in vs:
            h.gather_scatter(x, 1, op, "sym")
        out = np.concatenate(vs)
    else:
        v = values(k * ids.size, dt, op, case["seed"])
        assert sha(v) == case["input_sha256"], "input generator drifted"
        out = h.gather_scatter(v, k, op, "sym")
    assert sha(out) == case["output_sha256"]


@pytest.mark.parametrize("case", [c for c in GOLD["cases"] if c["kind"] == "signed"],
                         ids=lambda c: f"{c['dtype']}-{c['op']}-{c['trans']}")
def test_oracle_matches_gslib_golden_signed(oracle_mod, case):
    nx, ny, nz, p = case["mesh"]
    sids = signed_ids(mesh.box_ids(nx, ny, nz, p), case["flag_seed"])
    h = oracle_mod.OracleOgs(sids.copy(), "signed")
    dt, op = np.dtype(case["dtype"]), case["op"]
    v = values(sids.size, dt, op, case["seed"])
    assert sha(v) == case["input_sha256"]
    ref = np.frombuffer(base64.b64decode(case["output_b64"]), dtype=dt)
    out = h.gather_scatter(v.copy(), 1, op, case["trans"])
    absid = np.abs(sids)
    has_pos = np.zeros(absid.max() + 1, bool)
    has_pos[absid[sids > 0]] = True
    keep = has_pos[absid]
    # Groups with no unflagged member follow ogs's own rule, not gslib's:
    # Trans leaves them untouched (ogsOperator.cpp:321-326, NrowsN rows only);
    # NoTrans writes the op identity (ogsOperator.cpp:333-339), which for integer
    # Max is -max where gslib uses INT_MIN/LLONG_MIN (gs_defs.h:48-52).
    if case["trans"] == "trans":
        assert same_bits(out[~keep], v[~keep])
    else:
        ident = {"add": 0, "mul": 1, "max": -np.finfo(dt).max if dt.kind == "f" else -np.iinfo(dt).max,
                 "min": np.finfo(dt).max if dt.kind == "f" else np.iinfo(dt).max}[op]
        assert same_bits(out[~keep], np.full((~keep).sum(), ident, dt))
    if case["trans"] == "trans" and dt.kind == "f" and op in ("add", "mul"):
        # With flags and transpose=1 gslib folds the unflagged members
        # before the flagged ones; ogs folds in ascending local index.
        # Same terms, another order: relative tolerance 1e-14 (fp64).
        np.testing.assert_allclose(out[keep], ref[keep], rtol=1e-14, atol=1e-14)
        return
    assert same_bits(out[keep], ref[keep]), first_diff(out[keep], ref[keep])


def test_oracle_gs_test_kats(oracle_mod):
    kat = GOLD["gs_test_kats"]
    ids = np.array(kat["ids"], np.int64)
    h = oracle_mod.OracleOgs(ids.copy(), "signed")
    assert h.gather_scatter(np.ones(5), 1, "add", "notrans").tolist() == kat["transpose0"]
    assert h.gather_scatter(np.ones(5), 1, "add", "trans").tolist() == kat["transpose1"]
    h1 = oracle_mod.OracleOgs(np.array([1], np.int64), "unsigned")
    assert h1.gather_scatter(np.ones(1), 1, "add", "sym").tolist() == kat["chain_gs"]
    assert h1.gather_scatter(np.array([1.0, 2.0]), 2, "add", "sym").tolist() == kat["chain_vec"]


def _gsref():
    import oracle
    if not oracle.gsref_available():
        pytest.skip("gslib from the reference tree is not built here")
    return oracle


@pytest.mark.parametrize("dtype", TYPES)
@pytest.mark.parametrize("op", OPS)
def test_oracle_matches_gslib_live_irregular(oracle_mod, dtype, op):
    """Random ids with multiplicities up to ~30 and zeros, permuted box meshes."""
    o = _gsref()
    for seed, ids in [(1, random_ids(5000, 900, seed=3, zero_frac=0.1)),
                      (2, mesh.permute_elements(mesh.box_ids(5, 4, 3, 3), 3, seed=9))]:
        h = o.OracleOgs(ids.copy(), "unsigned")
        g = o.GsRef(ids)
        for k in (1, 3):
            v = values(k * ids.size, dtype, op, seed)
            a = h.gather_scatter(v.copy(), k, op, "sym")
            b = g.gs_vec(v.copy(), k, op, 0) if k > 1 else g.gs(v.copy(), op, 0)
            assert same_bits(a, b), first_diff(a, b)


def test_oracle_row_order_contract(oracle_mod):
    """Rows by first appearance, positive groups first, colIds ascending
    (ogsSetup.cpp:406-433, 637-663): checked on a hand-made id list."""
    ids = np.array([5, -7, 5, 0, 9, -9, 7, -3, -3, 2], np.int64)
    h = oracle_mod.OracleOgs(ids.copy(), "signed")
    rsT, ciT, rsN, ciN = h.maps()
    # groups by first appearance: 5(pos), 7(pos via index 6), 9(pos), 3(neg only), 2(pos)
    # positive rows first: 5 -> 0, 7 -> 1, 9 -> 2, 2 -> 3; then 3 -> 4
    assert h.NlocalP == 4 and h.NlocalT == 5
    assert rsT.tolist() == [0, 2, 4, 6, 7, 9]
    assert ciT.tolist() == [0, 2, 1, 6, 4, 5, 9, 7, 8]
    assert rsN.tolist() == [0, 2, 3, 4, 5, 5]
    assert ciN.tolist() == [0, 2, 6, 4, 9]
    assert not h.gather_defined  # group 5 has two positive members
    u = ids.copy()
    hu = oracle_mod.OracleOgs(u, "signed", unique=True)
    assert hu.gather_defined and hu.NlocalP == hu.NlocalT == 5
    # lowest local index of each group keeps the positive id
    assert u.tolist() == [5, 7, -5, 0, 9, -9, -7, 3, -3, 2]
