import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU and the built CUDA library")


@pytest.fixture(scope="session")
def built_lib():
    from spectrum_gb300 import build
    return build.build()
