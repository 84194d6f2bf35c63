"""Shared pytest configuration: the ``gpu`` marker and common fixtures."""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GB300 device (sm_103) and the built library"
    )
    config.addinivalue_line("markers", "slow: CPU test taking tens of seconds")


class _Golden:
    """Lazy view of one golden .npz archive keyed as 'case/array'."""

    def __init__(self, path):
        self._data = np.load(path)

    def case(self, name):
        prefix = name + "/"
        return {k[len(prefix):]: self._data[k] for k in self._data.files
                if k.startswith(prefix)}

    def __getitem__(self, key):
        return self._data[key]

    @property
    def files(self):
        return self._data.files


@pytest.fixture(scope="session")
def ref_goldens():
    return _Golden(os.path.join(GOLDEN, "reference_goldens.npz"))


@pytest.fixture(scope="session")
def workloads():
    return _Golden(os.path.join(GOLDEN, "workloads.npz"))


@pytest.fixture(scope="session")
def cuda_lib():
    """Built native library on a CUDA device (GPU tests only)."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    from gstools_gb300 import build, _native

    build.build()
    return _native.load()
