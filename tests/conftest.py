"""Shared test configuration.

Tests marked ``gpu`` need a CUDA device and the in-tree native library; the
rest run on CPU (oracle against golden vectors, host logic, the C-ABI
library's exported symbols).
"""

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built native library")


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN
