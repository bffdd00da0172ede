"""NVTX ranges: the library marks setup (and its map and layout builds), the
host-buffer calls, batch calls and server batches on the host timeline.
tests/nvtx/nvtx_probe.c is an NVTX injection library that logs every push and
pop; each check runs in a child process, since NVTX loads its injection once
per process, at the first range."""
import os
import shutil
import subprocess
import sys
import textwrap

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def cuda_include():
    for root in (os.environ.get("CUDA_HOME"), os.path.dirname(os.path.dirname(shutil.which("nvcc") or "")),
                 "/usr/local/cuda"):
        if root and os.path.exists(os.path.join(root, "include", "nvtx3", "nvToolsExt.h")):
            return os.path.join(root, "include")
    return None


@pytest.fixture(scope="module")
def probe(tmp_path_factory, built_lib):
    inc = cuda_include()
    if inc is None or shutil.which("gcc") is None:
        pytest.skip("no gcc or NVTX headers")
    so = str(tmp_path_factory.mktemp("nvtx") / "nvtx_probe.so")
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-I" + inc, "-o", so,
                    os.path.join(HERE, "nvtx", "nvtx_probe.c")], check=True)
    return so


def run_logged(probe, tmp_path, code):
    log = str(tmp_path / "nvtx.log")
    env = dict(os.environ, NVTX_INJECTION64_PATH=probe, OGS_NVTX_LOG=log, PYTHONPATH=ROOT)
    out = subprocess.run([sys.executable, "-c", textwrap.dedent(code)], env=env, cwd=ROOT,
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = open(log).read().splitlines() if os.path.exists(log) else []
    depth = 0
    for ln in lines:  # every push is popped, never below zero
        depth += 1 if ln.startswith("push ") else -1
        assert depth >= 0
    assert depth == 0
    return [ln[5:] for ln in lines if ln.startswith("push ")]


def test_setup_ranges_nest(probe, tmp_path):
    """On any machine: ogs_setup with the maps built on the host pushes its
    range and, inside it, the host map and layout builds (a machine without a
    GPU then refuses the upload, after the ranges closed)."""
    names = run_logged(probe, tmp_path, """
        import ctypes as C
        from dawgs_gb300 import _lib, mesh
        L = _lib.lib()
        ids = mesh.box_ids(3, 3, 3, 2)
        h = C.c_void_p()
        L.ogs_setup(C.byref(h), ids.size, ids.ctypes.data, 0, 0, 0, 0)
    """)
    assert names[:3] == ["ogs_setup", "ogs_setup: maps on the host", "ogs_setup: layout on the host"], names


@pytest.mark.gpu
def test_call_batch_and_server_ranges(cuda, probe, tmp_path):
    names = run_logged(probe, tmp_path, """
        import numpy as np, torch
        from dawgs_gb300 import mesh, ogs
        ids = mesh.box_ids(12, 12, 12, 3)  # above the size that builds maps on the GPU
        g = ogs.ogs_t().Setup(ids.size, ids.copy())
        v = torch.from_numpy(mesh.uniform_values(ids.size, np.float64, -1.0, 1.0, seed=1)).pin_memory()
        g.GatherScatter(v, 1, ogs.Add, ogs.Sym)
        d = v.cuda()
        b = ogs.ogs_batch_t([(g, d, 1, ogs.Add, ogs.Sym)])
        b.GatherScatter()
        srv = ogs.ogs_server_t(field_budget_bytes=1 << 28, max_inflight=64, max_batch=16)
        srv.add_mesh(g)
        srv.wait(srv.submit(0, v, 1, ogs.Add))
        srv.Free()
        torch.cuda.synchronize()
    """)
    for want in ("ogs_setup", "ogs_setup: maps on the GPU", "ogs_gather_scatter_host", "ogs_batch_gather_scatter",
                 "ogs_server: small-field batch"):
        assert want in names, (want, names)
