import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(autouse=True, scope="session")
def _models_on_torch_stream():
    """GPU tests make their inputs with torch kernels on torch's current stream;
    every model runs on that stream, so its kernels are ordered after them."""
    try:
        import torch
    except ImportError:
        yield
        return
    if torch.cuda.is_available():
        import moris_gb300 as mg
        mg.set_default_stream(lambda: torch.cuda.current_stream().cuda_stream)
    yield
