"""The exact pass decides which of several equal-valued peaks comes first by
replaying the introsort that std::sort uses (csrc/sort_order.h).  This
compiles that header into a host program and checks it against std::sort
itself on tie-heavy candidate lists."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "openpiv-cxx_gb300", "csrc")


def test_sort_order_matches_std_sort(tmp_path):
    exe = tmp_path / "test_sort_order"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", CSRC,
                    os.path.join(HERE, "cpp", "test_sort_order.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")
