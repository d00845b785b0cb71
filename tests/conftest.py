import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library, loaded (GPU tests)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from svox2_gb300 import _lib
    return _lib.load()
