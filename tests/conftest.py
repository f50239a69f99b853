"""pytest configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a CUDA device and the built libpirgpu.so; the rest
run on any host (the CPU oracle, the host-side logic, the ABI surface)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests"), os.path.join(ROOT, "lala-pc_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libpirgpu.so")
    config.addinivalue_line("markers", "slow: long-running CPU check")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def gpu_ctx_factory():
    import pirgpu
    return pirgpu.Context
