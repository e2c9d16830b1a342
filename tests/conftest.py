"""Shared pytest configuration: the ``gpu`` marker and import paths."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests", "golden"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")


import numpy as _np  # noqa: E402
import pytest as _pytest  # noqa: E402

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


@_pytest.fixture
def golden():
    def load(name):
        return _np.load(os.path.join(GOLDEN_DIR, name + ".npz"))

    return load
