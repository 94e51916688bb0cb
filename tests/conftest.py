import gzip
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the native kernels")


def golden_bytes(name: str) -> bytes:
    with gzip.open(os.path.join(GOLDEN, name + ".gz"), "rb") as f:
        return f.read()


@pytest.fixture(scope="session")
def scene_main_bytes():
    return golden_bytes("scene_main.bin")


@pytest.fixture(scope="session")
def scene_stress_bytes():
    return golden_bytes("scene_stress.bin")


@pytest.fixture(scope="session")
def golden_main():
    import json
    return json.load(open(os.path.join(GOLDEN, "golden_scen_main.json")))


@pytest.fixture(scope="session")
def golden_stress():
    import json
    return json.load(open(os.path.join(GOLDEN, "golden_scen_stress.json")))


@pytest.fixture(scope="session")
def scene_holdout_bytes():
    return golden_bytes("scene_holdout.bin")


@pytest.fixture(scope="session")
def golden_holdout():
    import json
    return json.load(open(os.path.join(GOLDEN, "golden_scen_holdout.json")))
