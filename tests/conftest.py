import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(setname):
    import json
    with open(os.path.join(GOLDEN, setname + ".json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def engine():
    import cuspx_gb300
    eng = cuspx_gb300.Engine(0)
    yield eng
    eng.close()
