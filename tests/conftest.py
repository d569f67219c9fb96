import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def built():
    """Build the native libraries (host builder + CUDA library) and the oracle once per session."""
    from gpugi_gb300 import build as b
    b.build_all()
    import oracle.build as ob
    ob.build()
    return True


@pytest.fixture(scope="session")
def cuda_ctx(built):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from gpugi_gb300 import cuda
    ctx = cuda.Context(0)
    yield ctx
    ctx.close()
