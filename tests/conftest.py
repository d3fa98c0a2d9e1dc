import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


def pytest_collection_modifyitems(config, items):
    if os.environ.get("TL_RUN_SLOW"):
        return
    skip = pytest.mark.skip(reason="slow CPU test; set TL_RUN_SLOW=1")
    for it in items:
        if "slow" in it.keywords and "gpu" not in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "reference_benchmarks.json")) as f:
        return json.load(f)
