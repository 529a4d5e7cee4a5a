import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def gpu_ctx():
    """One simit_gb300 context for the GPU tests; its stream is made torch's
    current stream so that test tensors are ordered with the C ABI's kernels."""
    import torch
    from simit_gb300.runtime import Context
    c = Context(0)
    prev = torch.cuda.current_stream()
    torch.cuda.set_stream(c.torch_stream)
    yield c
    torch.cuda.synchronize()
    torch.cuda.set_stream(prev)
    c.close()
