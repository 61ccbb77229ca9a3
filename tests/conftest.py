import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def cuda_ctx():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from imps_cpp_tools_gb300 import Context
    ctx = Context(0)
    ctx.set_stream(torch.cuda.current_stream())
    yield ctx
    torch.cuda.synchronize()
