"""Builds libopenpiv_gb300.so (sm_103a) in-tree.

Every CUDA translation unit is compiled by nvcc for sm_103a only, in
parallel; the C ABI layer is compiled as host C++17; all are linked into
``lib/libopenpiv_gb300.so`` with the static CUDA runtime.  Incremental: a
translation unit is rebuilt only when it or a header changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(HERE, "lib", "libopenpiv_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build openpiv-gb300")


def _headers() -> list[str]:
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(src: str, obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + deps)


def _compile(args: list[str]) -> tuple[list[str], int, str]:
    r = subprocess.run(args, capture_output=True, text=True)
    return args, r.returncode, r.stdout + r.stderr


def build(verbose: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    deps = _headers()
    common = ["-std=c++17", "-O3", "-I", INCLUDE, "-I", CSRC]
    jobs = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(src, obj, deps):
            jobs.append([nvcc] + ARCH + common + ["-lineinfo", "-Xcompiler", "-fPIC",
                                                  "-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(src, obj, deps):
            jobs.append([nvcc] + common + ["-Xcompiler", "-fPIC,-Wall", "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            for args, rc, out in ex.map(_compile, jobs):
                if verbose or rc != 0:
                    sys.stderr.write(" ".join(args) + "\n" + out)
                if rc != 0:
                    raise RuntimeError(f"compilation failed: {args[-3]}")
    if jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        args = [nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs
        _, rc, out = _compile(args)
        if rc != 0:
            sys.stderr.write(out)
            raise RuntimeError("link failed")
    build_examples()
    return LIB


def build_examples() -> list[str]:
    """The C++ example programs (examples/*.cpp) against the library."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("a C++ compiler is required to build the examples")
    exes = []
    for src in sorted(glob.glob(os.path.join(HERE, "examples", "*.cpp"))):
        exe = os.path.join(HERE, "lib", os.path.splitext(os.path.basename(src))[0])
        deps = [src, LIB, os.path.join(HERE, "cpp", "openpiv_gb300.hpp"),
                os.path.join(INCLUDE, "openpiv_gb300.h")]
        if not os.path.exists(exe) or any(os.path.getmtime(d) > os.path.getmtime(exe) for d in deps):
            args = [cxx, "-std=c++17", "-O2", "-Wall", "-I", INCLUDE, "-I", os.path.join(HERE, "cpp"),
                    src, "-L", os.path.dirname(LIB), "-lopenpiv_gb300",
                    "-Wl,-rpath,$ORIGIN", "-o", exe]
            _, rc, out = _compile(args)
            if rc != 0:
                sys.stderr.write(out)
                raise RuntimeError(f"example build failed: {src}")
        exes.append(exe)
    return exes


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
