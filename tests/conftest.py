import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GB300)")


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN


def fixture_model(name):
    from kmos_gb300 import model as M
    return M.load_json(os.path.join(GOLDEN, "models", name + ".json"))
