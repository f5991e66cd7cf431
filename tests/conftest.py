import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, 'double-batched-fft-library_gb300')
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300, sm_103a)')


def _ensure_built():
    import build as pkg_build  # double-batched-fft-library_gb300/build.py

    pkg_build.build()


@pytest.fixture(scope='session')
def bb():
    """The bbfft_gb300 binding with the library built in-tree."""
    _ensure_built()
    import bbfft_gb300

    bbfft_gb300.lib()
    return bbfft_gb300


@pytest.fixture(scope='session')
def po():
    from oracle import pyoracle

    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope='session')
def torch_cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail('GPU test run without a CUDA device')
    return torch
