import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libuslam.so")


@pytest.fixture(scope="session")
def brief_pattern():
    from uni_slam_gb300 import pattern

    return pattern.load()
