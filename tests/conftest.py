"""Shared pytest configuration.

Tests marked ``gpu`` need a GB300 (sm_103a) and the built CUDA library; the
rest run on any CPU host.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(autouse=True)
def no_silent_device_timeout(request):
    """After every GPU test that used the library: no kernel wait of a
    device-pointer call gave up unreported (ugemm_check raises if one did)."""
    yield
    if request.node.get_closest_marker("gpu") is None:
        return
    ug = sys.modules.get("ugemm_gb300")
    if ug is None or ug._lib is None:
        return
    import torch
    if torch.cuda.is_available():
        ug.check()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    path = os.path.join(ROOT, "tests", "golden", "ugemm_golden.npz")
    return np.load(path)
