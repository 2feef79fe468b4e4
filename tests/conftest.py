import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libqsfgpu.so")
    config.addinivalue_line("markers", "slow: runs a full-size configuration")


def pytest_collection_modifyitems(config, items):
    # keep the no-allocation entry point test last in collection order
    items.sort(key=lambda it: 1 if os.path.basename(str(it.fspath)).startswith("test_zz") else 0)
