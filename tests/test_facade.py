"""The C++17 facade (openpiv-cxx_gb300/cpp/openpiv_gb300.hpp) compiled into a
host program: reference names, grid known answers, error messages, peaks
and the Gaussian fit.  No GPU."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "openpiv-cxx_gb300")


def test_facade_host_parts(lib, tmp_path):
    exe = tmp_path / "test_facade"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(PKG, "cpp"), os.path.join(HERE, "cpp", "test_facade.cpp"),
                    "-L", os.path.join(PKG, "lib"), "-lopenpiv_gb300",
                    "-Wl,-rpath," + os.path.join(PKG, "lib"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "ok"
