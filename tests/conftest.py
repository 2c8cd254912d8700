import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("", "oracle", "gvdb-voxels_gb300", "tests"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI of libgbvdb.so)")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load libgbvdb.so; GPU tests fail loudly without it."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but CUDA is not available")
    import build_lib
    import gbvdb

    build_lib.build()
    return gbvdb.load()
