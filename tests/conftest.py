import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")
    config.addinivalue_line("markers", "slow: long CPU run, enabled with TEA_SLOW=1")


def pytest_collection_modifyitems(config, items):
    if os.environ.get("TEA_SLOW"):
        return
    skip = pytest.mark.skip(reason="long run; set TEA_SLOW=1")
    for item in items:
        if "slow" in item.keywords:
            item.add_marker(skip)
