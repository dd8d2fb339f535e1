import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libskewt_gb300.so")
    # temporary files of the tests stay inside the checkout (pytest empties this folder per run)
    if not config.option.basetemp:
        config.option.basetemp = os.path.join(ROOT, ".pytest_tmp")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load the CUDA library; skip when no GPU is visible."""
    if not has_gpu():
        pytest.skip("no CUDA device")
    from skewtcloudsim_gb300 import build, _lib
    build.build()
    return _lib.load()
