"""include/ogs.hpp and include/ogs_c.h compile warning-free, as C++17 and
(the C header) as C99, and a caller written like dawgs' CorrectnessTest links
against the library -- without a GPU (running it is tests/test_gpu_cpp_api.py)."""
import os
import shutil
import subprocess

import pytest

from dawgs_gb300 import build

HERE = os.path.dirname(os.path.abspath(__file__))


def _cuda_root():
    return os.path.dirname(os.path.dirname(build.nvcc()))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_cpp_caller_compiles_and_links(built_lib, tmp_path):
    exe = str(tmp_path / "test_ogs_api")
    cuda = _cuda_root()
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", build.INCLUDE,
           "-I", os.path.join(cuda, "include"), os.path.join(HERE, "cpp", "test_ogs_api.cpp"), "-o", exe,
           "-L", build.LIBDIR, "-ldawgs_ogs", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           f"-Wl,-rpath,{build.LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_c_header_is_c99(tmp_path):
    src = tmp_path / "use.c"
    src.write_text('#include "ogs_c.h"\nint main(void) { ogs_handle h = 0; return ogs_free(h) == OGS_OK ? 0 : 1; }\n')
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", build.INCLUDE, "-c",
                        str(src), "-o", str(tmp_path / "use.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
