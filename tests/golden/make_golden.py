"""Generate tests/golden/golden.json from the reference's own gather-scatter
checker, gslib (3rdParty/gslib of paranumal/dawgs, built by `make -C oracle
ref` into oracle/_ref/libgsref.so), and record the known-answer tests of
3rdParty/gslib/tests/gs_test.c:64-104 at one rank.

Run here, where the reference tree exists:

    python tests/golden/make_golden.py

Inputs are not stored: they are regenerated from dawgs_gb300.mesh with the
seeds below (a counter-based splitmix64 stream, identical on every machine),
and a digest of each input is stored so that generator drift is detected.
Outputs are stored as sha256 digests (large cases) or base64 bytes (small).
"""
from __future__ import annotations

import base64
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from dawgs_gb300 import mesh  # noqa: E402
import oracle  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")

TYPES = ["float32", "float64", "int32", "int64"]
OPS = ["add", "mul", "max", "min"]


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def b64(a: np.ndarray) -> str:
    return base64.b64encode(np.ascontiguousarray(a).tobytes()).decode()


def values(n, dtype, op, seed):
    """Field values by op, the distributions of the benchmark configurations."""
    dt = np.dtype(dtype)
    if dt.kind == "f":
        return mesh.uniform_values(n, dt, 0.5, 2.0, seed) if op == "mul" else \
            mesh.uniform_values(n, dt, -1.0, 1.0, seed)
    if op == "mul":
        return mesh.uniform_values(n, dt, -3, 4, seed)
    return mesh.uniform_values(n, dt, -(2 ** 30), 2 ** 30, seed)


def signed_ids(ids, seed):
    r = mesh.uniform_values(ids.size, np.int64, 0, 4, seed)
    return np.where(r == 0, -ids, ids).astype(np.int64)


def main():
    oracle.build(ref=True)
    gold = {"generator": "tests/golden/make_golden.py", "source": "gslib (3rdParty/gslib) via oracle/_ref",
            "cases": []}

    # C1: 10^3 hexes, p=3, Unsigned (all ids positive): gs / gs_vec / gs_many, every type and op.
    ids = mesh.box_ids(10, 10, 10, 3)
    g = oracle.GsRef(ids)
    for t in TYPES:
        for op in OPS:
            v = values(ids.size, t, op, seed=11)
            out = g.gs(v.copy(), op, 0)
            gold["cases"].append({"mesh": [10, 10, 10, 3], "kind": "unsigned", "layout": "k1", "k": 1,
                                  "dtype": t, "op": op, "seed": 11, "trans": "sym",
                                  "input_sha256": digest(v), "output_sha256": digest(out)})
            v3 = values(3 * ids.size, t, op, seed=12)
            out3 = g.gs_vec(v3.copy(), 3, op, 0)
            gold["cases"].append({"mesh": [10, 10, 10, 3], "kind": "unsigned", "layout": "vec", "k": 3,
                                  "dtype": t, "op": op, "seed": 12, "trans": "sym",
                                  "input_sha256": digest(v3), "output_sha256": digest(out3)})
        vs = [values(ids.size, t, "add", seed=13 + j) for j in range(2)]
        outs = g.gs_many([x.copy() for x in vs], "add", 0)
        gold["cases"].append({"mesh": [10, 10, 10, 3], "kind": "unsigned", "layout": "many", "k": 2,
                              "dtype": t, "op": "add", "seed": 13, "trans": "sym",
                              "input_sha256": digest(np.concatenate(vs)),
                              "output_sha256": digest(np.concatenate(outs))})

    # Signed ids (about a quarter flagged) on a small box: gs transpose 0 and 1,
    # stored in full.  transpose=0 is ogs NoTrans; transpose=1 is ogs Trans except
    # for groups with no unflagged member, which gslib writes and ogs leaves alone
    # (ogsOperator.cpp:321-326 runs Trans over the NrowsN positive rows only).
    ids = mesh.box_ids(4, 3, 2, 2)
    sids = signed_ids(ids, seed=5)
    g = oracle.GsRef(sids)
    for t in ["float64", "int64"]:
        for op in OPS:
            v = values(ids.size, t, op, seed=21)
            for tp in (0, 1):
                out = g.gs(v.copy(), op, tp)
                gold["cases"].append({"mesh": [4, 3, 2, 2], "kind": "signed", "flag_seed": 5,
                                      "layout": "k1", "k": 1, "dtype": t, "op": op, "seed": 21,
                                      "trans": "notrans" if tp == 0 else "trans",
                                      "input_sha256": digest(v), "output_b64": b64(out)})

    # gs_test.c:24-60 at np=1: ids {-11, -1, 1, 1, 1}, all values 1.
    kat_ids = np.array([-11, -1, 1, 1, 1], np.int64)
    g = oracle.GsRef(kat_ids)
    kat = {"ids": kat_ids.tolist()}
    for tp in (0, 1):
        out = g.gs(np.ones(5, np.float64), "add", tp)
        kat[f"transpose{tp}"] = out.tolist()
    # gs_test.c:62-104 at np=1: one id {1}; answer 1 for gs, (1,2) for gs_vec and gs_many.
    g1 = oracle.GsRef(np.array([1], np.int64))
    kat["chain_gs"] = g1.gs(np.ones(1), "add", 0).tolist()
    kat["chain_vec"] = g1.gs_vec(np.array([1.0, 2.0]), 2, "add", 0).tolist()
    kat["chain_many"] = [x.tolist() for x in g1.gs_many([np.ones(1), 2 * np.ones(1)], "add", 0)]
    gold["gs_test_kats"] = kat

    with open(OUT, "w") as f:
        json.dump(gold, f, indent=1)
    print(f"wrote {OUT}: {len(gold['cases'])} cases")


if __name__ == "__main__":
    main()
