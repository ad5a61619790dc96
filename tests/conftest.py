"""Shared test setup: build the libraries once, expose both front ends.

Tests marked ``gpu`` need a CUDA device and call the product through its
C-ABI (libapic_gpu.so); everything else runs on the CPU (the oracle, host
logic, the ABI's exported symbols).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "apic-fluid-simulation_gb300")
TESTS = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, PKG, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gpu_lib():
    from apic_gb300 import build
    build.build()
    import apic_gb300
    lib = apic_gb300.load_library()
    return lib


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def has_gpu(gpu_lib):
    import apic_gb300
    return apic_gb300.device_count() > 0
