import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gctx():
    """A library context on cuda:0.  GPU tests fail (not skip) without a device: the
    CUDA path is the only path."""
    import torch

    from shamrock_gb300 import _lib

    assert torch.cuda.is_available(), "GPU test run without a CUDA device"
    torch.cuda.init()
    ctx = _lib.Context(0)
    yield ctx
    ctx.close()


@pytest.fixture(scope="session")
def golden():
    import json

    def load(name):
        with open(os.path.join(ROOT, "tests", "golden", name)) as f:
            return json.load(f)

    return load
