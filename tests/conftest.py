import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmfgb.so")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "reference_bk5.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden13():
    """Outputs of the reference's serial BK1 / BK3 (tests/golden/make_golden.py)."""
    import json
    with open(os.path.join(ROOT, "tests", "golden", "reference_bk1_bk3.json")) as f:
        return json.load(f)
