"""The C++ drop-in header (include/ogs.hpp) compiled into a caller written
like dawgs' CorrectnessTest and run on the GPU."""
import os
import subprocess

import pytest

from dawgs_gb300 import build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_cpp_caller(cuda, tmp_path):
    exe = str(tmp_path / "test_ogs_api")
    cmd = [build.nvcc(), "-std=c++17", "-O2", "-I", build.INCLUDE,
           os.path.join(HERE, "cpp", "test_ogs_api.cpp"), "-o", exe,
           "-L", build.LIBDIR, "-ldawgs_ogs", "-Xlinker", f"-rpath,{build.LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASSED" in r.stdout and r.stdout.count("(bit-exact)") == 5
