"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "openpiv-cxx_gb300")
# the reference sources (read-only), where this machine has them
REFERENCE = os.environ.get("OPENPIV_REFERENCE", "/root/reference")
for p in (PKG, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib():
    """The built libopenpiv_gb300.so (built on first use)."""
    import opiv_gb300

    if not os.path.exists(opiv_gb300.lib_path()):
        sys.path.insert(0, PKG)
        import build as pkg_build

        pkg_build.build()
    return opiv_gb300.load()


@pytest.fixture(scope="session")
def orc():
    """The oracle's CPU restatement (parity build)."""
    from oracle import oracle

    if not oracle.available("port"):
        oracle.build(ref=False)
    return oracle.get("port")


@pytest.fixture(scope="session")
def ref_lib():
    """The reference compiled from its own sources, where this machine has it."""
    from oracle import oracle

    if not oracle.available("ref"):
        if os.path.isdir(os.path.join(REFERENCE, "openpiv")):
            subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REFERENCE}"],
                           check=True)
        else:
            pytest.skip("reference sources not on this machine")
    return oracle.get("ref")
