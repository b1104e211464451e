import json
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and runs the CUDA kernels")


@pytest.fixture(scope="session")
def golden():
    return json.loads((ROOT / "tests/golden/domino_ref_cases.json").read_text())


@pytest.fixture(scope="session")
def rt():
    import randomtilingspublic_gb300 as m

    if not m.LIB_PATH.exists():
        from randomtilingspublic_gb300 import build

        build.build()
    m.lib()
    return m


@pytest.fixture(scope="session")
def orc():
    from tests import oracle_py

    oracle_py.lib()
    return oracle_py
