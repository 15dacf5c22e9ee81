"""Pytest configuration: the `gpu` marker and shared fixtures.

Tests marked `gpu` run the CUDA library on cuda:0; everything else runs on the
CPU (oracle against the golden fixtures, host logic, the C ABI's exports).
"""

from __future__ import annotations

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def pytest_collection_modifyitems(config, items):
    try:
        import torch  # noqa: PLC0415

        has_gpu = torch.cuda.is_available()
    except Exception:  # noqa: BLE001
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle  # noqa: PLC0415

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu():
    """Initialises the library on cuda:0 once per session."""
    import torch  # noqa: PLC0415

    from ragnar_gb300 import capi  # noqa: PLC0415

    capi.check(capi.lib().rg_init(0))
    return torch.device("cuda:0")
