"""In-tree build of libdawgs_ogs.so for sm_103a with nvcc (no cmake, no torch
extension machinery: the library's interface is plain C).

    python -m dawgs_gb300.build [--force] [--verbose]

Each translation unit compiles in parallel into dawgs_gb300/_build/; the shared
library lands in dawgs_gb300/lib/.  A unit is rebuilt when it or any header is
newer than its object.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libdawgs_ogs.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3",
          "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libdawgs_ogs.so")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith((".h", ".hpp"))]
    return hs


def _obj(src):
    return os.path.join(BUILD, os.path.basename(src) + ".o")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose, extra):
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", src, "-o", _obj(src)]
    if src.endswith(".cu") and verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, r.returncode, r.stdout + r.stderr, cmd


def build(force: bool = False, verbose: bool = False, extra=(), build_dir=None, lib=None) -> str:
    """Compile and link; `extra` nvcc flags, `build_dir`/`lib` redirect the
    objects and the library (e.g. a variant built with other -D settings)."""
    global BUILD, LIB
    saved = BUILD, LIB
    if build_dir:
        BUILD = build_dir
    if lib:
        LIB = lib
    try:
        return _build(force, verbose, extra)
    finally:
        BUILD, LIB = saved


def _build(force, verbose, extra):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    hs = headers()
    srcs = sources()
    todo = [s for s in srcs if force or _stale(_obj(s), [s, *hs])]
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            for src, rc, out, cmd in ex.map(lambda s: _compile(s, verbose, list(extra)), todo):
                if verbose or rc:
                    sys.stderr.write(out)
                if rc:
                    raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{' '.join(cmd)}\n{out}")
    objs = [_obj(s) for s in srcs]
    if force or todo or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs,
               "-Xlinker", "--no-undefined"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))


if __name__ == "__main__":
    main()
