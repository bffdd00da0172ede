"""A checked build of the library (-DOGS_CHECK_BOUNDS=1: every column and
row id a kernel loads is compared with the handle's node and row counts
before any value is read or written through it) runs the operators on
regular, permuted, signed, high-degree, empty-row and device-built maps, the
host-buffer, no-alloc and gslib entry points, and finds no id out of range;
its results equal the oracle's bit for bit (ogsOperator.cpp:60-97, 206-238,
311-360).  The build goes to a temporary directory and runs in a child
process, so the default library of the other tests is untouched."""
import json
import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent('''
    import ctypes as C, json, sys
    import numpy as np, torch
    import oracle
    from dawgs_gb300 import _lib, mesh, ogs
    from helpers import random_ids, same_bits, signed_ids, values

    L = _lib.lib()
    out = {}
    TORCH = {np.float32: torch.float32, np.float64: torch.float64, np.int32: torch.int32, np.int64: torch.int64}
    OPS = {"add": ogs.Add, "mul": ogs.Mul, "max": ogs.Max, "min": ogs.Min}
    TR = {"sym": ogs.Sym, "notrans": ogs.NoTrans, "trans": ogs.Trans}

    def record(name, g, same):
        torch.cuda.synchronize()
        out[name] = [g.checked_id_errors(), bool(same)]

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()

    # unsigned box and permuted box: every type and op, k = 1 and 3, and 2 separate arrays
    for mname, ids in (("box", mesh.box_ids(10, 9, 8, 3)),
                       ("perm", mesh.permute_elements(mesh.box_ids(7, 6, 5, 4), 4, seed=3))):
        g = ogs.ogs_t().Setup(ids.size, ids.copy())
        ref = oracle.OracleOgs(ids.copy(), "unsigned")
        ok = True
        for dt in (np.float64, np.float32, np.int64, np.int32):
            for op in OPS:
                for k in (1, 3):
                    v = values(k * ids.size, dt, op, seed=k)
                    d = dev(v)
                    g.GatherScatter(d, k, OPS[op], ogs.Sym)
                    ok &= same_bits(d.cpu().numpy(), ref.gather_scatter(v.copy(), k, op, "sym"))
            vs = [values(ids.size, dt, "add", seed=20 + j) for j in range(2)]
            ds = [dev(v) for v in vs]
            g.GatherScatterMany(ds, ogs.Add, ogs.Sym)
            for d, v in zip(ds, vs):
                ok &= same_bits(d.cpu().numpy(), ref.gather_scatter(v.copy(), 1, "add", "sym"))
        record(mname, g, ok)

    # signed unique handles (N masks, row ids): Gather, Scatter, GatherScatter, every transpose;
    # the high-degree case has rows above degree 8 (the general kernel)
    for mname, base in (("signed_box", mesh.box_ids(8, 7, 6, 3)), ("high_degree", random_ids(6000, 40, seed=9))):
        sids = signed_ids(base, seed=4)
        a = sids.copy()
        g = ogs.ogs_t().Setup(a.size, a, None, ogs.Signed, ogs.Auto, True)
        ref = oracle.OracleOgs(sids.copy(), "signed", True)
        ok = True
        for tr in TR:
            v = values(base.size, np.float64, "add", seed=5)
            d = dev(v)
            g.GatherScatter(d, 1, ogs.Add, TR[tr])
            ok &= same_bits(d.cpu().numpy(), ref.gather_scatter(v.copy(), 1, "add", tr))
            if tr == "sym":
                continue
            gv = torch.zeros(g.Ngather, dtype=torch.float64, device="cuda")
            g.Gather(gv, dev(v), 1, ogs.Add, TR[tr])
            want_gv = ref.gather(np.zeros(g.Ngather), v.copy(), 1, "add", tr)
            ok &= same_bits(gv.cpu().numpy(), want_gv)
            d = dev(v)
            g.Scatter(d, gv, 1, TR[tr])
            ok &= same_bits(d.cpu().numpy(), ref.scatter(v.copy(), want_gv.copy(), 1, tr))
        record(mname, g, ok)

    # maps built on the GPU (N >= 65,536), and the host-buffer pipeline over several slices
    ids = mesh.box_ids(14, 12, 10, 4)
    g = ogs.ogs_t().Setup(ids.size, ids.copy())
    ref = oracle.OracleOgs(ids.copy(), "unsigned")
    v = values(ids.size, np.float64, "add", seed=7)
    d = dev(v)
    g.GatherScatter(d, 1, ogs.Add, ogs.Sym)
    want = ref.gather_scatter(v.copy(), 1, "add", "sym")
    ok = same_bits(d.cpu().numpy(), want)
    pinned = torch.from_numpy(v.copy()).pin_memory()
    g.GatherScatter(pinned, 1, ogs.Add, ogs.Sym)
    ok &= same_bits(pinned.numpy(), want)
    record("device_maps_and_host_pipeline", g, ok)

    # the no-alloc host entry point
    small = mesh.box_ids(6, 6, 6, 3)
    g = ogs.ogs_t().Setup(small.size, small.copy())
    v = values(small.size, np.float64, "max", seed=8)
    h = v.copy()
    _lib.check(L.ogs_gather_scatter_host_noalloc(g.handle, h.ctypes.data, 1, 1, int(ogs.Max), 0, None))
    record("noalloc", g, same_bits(h, oracle.OracleOgs(small.copy(), "unsigned").gather_scatter(v.copy(), 1, "max", "sym")))

    # operators from caller maps with empty rows (postmpi-style), gathered in place
    rsT = np.array([0, 2, 2, 5, 5], np.int32)
    ciT = np.array([0, 3, 1, 2, 4], np.int32)
    g = ogs.ogs_t().SetupMaps(5, rsT, ciT)
    x = dev(np.arange(5, dtype=np.float64) + 1.0)
    gv = torch.full((4,), -1.0, dtype=torch.float64, device="cuda")
    g.Gather(gv, x, 1, ogs.Add, ogs.Trans)
    record("maps_with_empty_rows", g, same_bits(gv.cpu().numpy(), np.array([5.0, 0.0, 10.0, 0.0])))

    # gslib entry points (gs, gs_vec, gs_many): ids checked, results covered by the gslib tests
    gl = ogs.gslib_t(signed_ids(mesh.box_ids(5, 5, 4, 2), seed=2))
    u = dev(values(gl.n * 2, np.float64, "add", seed=3))
    gl.gs(u[: gl.n], ogs.Add, 0)
    gl.gs_vec(u, 2, ogs.Add, 1)
    gl.gs_many([u[: gl.n], u[gl.n:]], ogs.Min, 0)
    torch.cuda.synchronize()
    n = C.c_uint64()
    _lib.check(L.ogs_checked_id_errors(gl._h, C.byref(n)))
    out["gslib"] = [n.value, True]
    print(json.dumps(out))
''')


def test_checked_build_finds_no_id_out_of_range(cuda, oracle_mod, tmp_path):
    from dawgs_gb300 import build
    lib = str(tmp_path / "libdawgs_ogs_checked.so")
    build.build(extra=["-DOGS_CHECK_BOUNDS=1"], build_dir=str(tmp_path / "obj"), lib=lib)
    env = dict(os.environ, DAWGS_OGS_LIB=lib,
               PYTHONPATH=os.pathsep.join([ROOT, os.path.join(ROOT, "tests"), os.environ.get("PYTHONPATH", "")]))
    r = subprocess.run([sys.executable, "-c", CHILD], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert len(res) == 8, res
    for name, (errors, same) in res.items():
        assert errors == 0, (name, errors)
        assert same, name
