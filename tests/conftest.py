import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "freefem-sources_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libffgpu.so")
    config.addinivalue_line("markers", "slow: larger parity sizes")


@pytest.fixture(scope="session", autouse=True)
def _built_oracle():
    import ffo
    ffo.build()
    yield
