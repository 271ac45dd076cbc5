"""The reference-typed drop-in header (openpiv-cxx_gb300/cpp/openpiv_gpu.h),
host side: the process example's per-window loop with the correlator
swapped to openpiv::gpu::FFT (tests/cpp/process_dropin.cpp) compiles and
links against the reference's own core types -- with the reference's
find_peaks / fit_simple_gaussian / generate_cartesian_grid and with the
gpu:: ones -- and against the test-only stand-in types; without a GPU the
harness stops with the library's error instead of computing anything on
the CPU.  The GPU runs are in test_gpu_dropin.py."""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "openpiv-cxx_gb300")
REFERENCE = os.environ.get("OPENPIV_REFERENCE", "/root/reference")
HARNESS = os.path.join(HERE, "cpp", "process_dropin.cpp")


def build_harness(out, reference=None, gpu_peaks=False):
    """Compiles the drop-in harness; `reference`: the reference's source tree
    (its own headers and core/{size,rect,util}.cpp), else the stand-in types."""
    args = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
            "-I", os.path.join(PKG, "cpp"), "-I", os.path.join(HERE, "cpp")]
    srcs = [HARNESS]
    if reference is not None:
        import torch

        torch_inc = os.path.join(os.path.dirname(torch.__file__), "include")   # fmt, header-only
        args += ["-DOPIV_WITH_REFERENCE", "-I", os.path.join(reference, "openpiv"),
                 "-idirafter", torch_inc, "-DFMT_HEADER_ONLY", "-D_USE_MATH_DEFINES", "-pthread"]
        if gpu_peaks:
            args.append("-DOPIV_GPU_PEAKS")
        srcs += [os.path.join(reference, "openpiv", "core", f) for f in ("size.cpp", "rect.cpp", "util.cpp")]
    lib = os.path.join(PKG, "lib")
    args += srcs + ["-L", lib, "-lopenpiv_gb300", "-Wl,-rpath," + lib, "-o", str(out)]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return str(out)


@pytest.mark.parametrize("gpu_peaks", [False, True])
def test_harness_builds_against_reference_types(lib, tmp_path, gpu_peaks):
    if not os.path.isdir(os.path.join(REFERENCE, "openpiv")):
        pytest.skip("reference sources not on this machine")
    pytest.importorskip("torch")
    exe = build_harness(tmp_path / "process_dropin_ref", REFERENCE, gpu_peaks)
    assert os.path.exists(exe)


def test_harness_builds_against_standin_and_needs_a_gpu(lib, tmp_path):
    torch = pytest.importorskip("torch")
    exe = build_harness(tmp_path / "process_dropin")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: the runs are in test_gpu_dropin.py")
    a = np.zeros((64, 64), np.uint8)
    fa = tmp_path / "a.u8"
    a.tofile(fa)
    r = subprocess.run([exe, "64", "64", str(fa), str(fa), "32", "0.5", "complex", "0"],
                       capture_output=True, text=True)
    # the first correlation throws the library's error: no CPU fallback
    assert r.returncode != 0
    assert "device" in r.stderr
