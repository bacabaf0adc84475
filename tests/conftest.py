import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(pathlib.Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103a GPU and runs the CUDA library")
    config.addinivalue_line("markers", "slow: large workloads")


@pytest.fixture(scope="session")
def built_library():
    from mrustsc_gb300 import build

    return build.build()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o

    o.build()
    return o
