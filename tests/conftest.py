"""Shared test configuration.

Tests marked ``gpu`` need a CUDA device and the built libvfps; everything
else runs on the CPU (oracle checks, host logic, C-ABI symbol checks).
"""
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(ROOT, "tests", "golden",
                           "reference_tests.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def gpu_ctx():
    """CUDA context of libvfps on device 0 (built in-tree first)."""
    from inovesa_gb300.build import build
    build()
    from inovesa_gb300 import vfps
    ctx = vfps.Context(0)
    yield ctx
    ctx.synchronize()
    assert ctx.device_status() == 0
