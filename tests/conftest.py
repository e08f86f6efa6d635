import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fuzzy-ellipses_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def cuda_device():
    """The CUDA device for -m gpu tests. Fails (does not skip) without a GPU or the native
    library, so a GPU run can never pass on a fallback."""
    import torch

    import fuzzy_ellipses

    if not torch.cuda.is_available():
        pytest.fail("gpu test requested but torch.cuda.is_available() is False")
    fuzzy_ellipses.load_native()
    return torch.device("cuda:0")
