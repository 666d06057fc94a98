"""Test configuration: the `gpu` marker and import paths.

Tests marked ``gpu`` need a GB300 and run the library's CUDA kernels through
the C ABI; everything else runs on a CPU-only machine (oracle vs golden
fixtures, host-side logic, the shared library's exported symbols).
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "lennard-jones-cuda_gb300"), os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def ljlib():
    import ljgb
    return ljgb.load()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ljgb_mod(ljlib):
    import ljgb
    return ljgb
