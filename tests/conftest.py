import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "knn-toolbox_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) and the built CUDA library")


@pytest.fixture(scope="session")
def engine():
    """The CUDA engine, built in-tree; GPU tests fail loudly if it is missing."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without CUDA")
    import cuknns
    cuknns.lib()
    return cuknns


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O
