"""Test configuration: the `gpu` marker and import paths.

CPU tests (`-m "not gpu"`) check the oracle against the golden fixtures and
known answers, the host-side set-up code, and that libhe4g.so loads and
exports every entry point of include/he4g.h. GPU tests (`-m gpu`) run the
sm_103a library through its C ABI against the oracle.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "4hetddft-isotropic_gb300")
for p in (ROOT, PKG_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def he4gpu_mod():
    import he4gpu
    he4gpu.abi.load()
    return he4gpu
