import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


@pytest.fixture(scope="session")
def goldens():
    return json.loads((ROOT / "tests" / "golden" / "goldens.json").read_text())


@pytest.fixture(scope="session")
def qb():
    import __graft_entry__ as ge
    return ge.load_package()


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    o.lib()
    return o
