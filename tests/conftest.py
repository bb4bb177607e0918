import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def gpu_ctx():
    from ochre_gb300 import GpuContext
    ctx = GpuContext(0)
    yield ctx
    ctx.close()


@pytest.fixture(scope="session")
def gpu_ctx_chain():
    """A context forced onto the general kernel chain (no fused path)."""
    from ochre_gb300 import GpuContext
    ctx = GpuContext(0, chain_only=True)
    yield ctx
    ctx.close()


@pytest.fixture(params=["fused", "chain"])
def any_ctx(request):
    return request.getfixturevalue("gpu_ctx" if request.param == "fused" else "gpu_ctx_chain")


@pytest.fixture(autouse=True)
def _quiet_numpy():
    with np.errstate(all="ignore"):
        yield
