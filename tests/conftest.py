import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


def _load(name):
    return json.loads((GOLDEN / name).read_text())


@pytest.fixture(scope="session")
def golden_encodings():
    return _load("encodings.json")


@pytest.fixture(scope="session")
def golden_patterns():
    return _load("site_patterns.json")


@pytest.fixture(scope="session")
def golden_transition():
    return _load("transition.json")


@pytest.fixture(scope="session")
def golden_likelihood():
    return _load("likelihood.json")


def gpu_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False
