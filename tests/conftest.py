import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "cornerstone-octree_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a); parity of the CUDA path vs the oracle")


@pytest.fixture(scope="session")
def cs():
    """The CUDA binding; GPU tests fail loudly if the library is missing."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import cstone_gb300

    return cstone_gb300


@pytest.fixture(scope="session")
def O():
    import oracle

    oracle.build()
    return oracle
