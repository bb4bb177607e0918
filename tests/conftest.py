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


@pytest.fixture(scope="session")
def gpu_ctx_chain_rows():
    """The general chain with the one-warp-per-tile-row coverage kernel forced
    (the default picks it only when there are many tile rows)."""
    from ochre_gb300 import GpuContext, autotune
    ctx = GpuContext(0, chain_only=True)
    autotune.apply(ctx, {"chain_coverage_form": 2})
    yield ctx
    ctx.close()


@pytest.fixture(scope="session")
def gpu_ctx_chain_blocks():
    """The general chain with the block-form coverage kernel forced."""
    from ochre_gb300 import GpuContext, autotune
    ctx = GpuContext(0, chain_only=True)
    autotune.apply(ctx, {"chain_coverage_form": 1})
    yield ctx
    ctx.close()


@pytest.fixture(params=["fused", "chain", "chain_rows", "chain_blocks"])
def any_ctx(request):
    return request.getfixturevalue({"fused": "gpu_ctx", "chain": "gpu_ctx_chain", "chain_rows": "gpu_ctx_chain_rows",
                                    "chain_blocks": "gpu_ctx_chain_blocks"}[request.param])


@pytest.fixture(autouse=True)
def _quiet_numpy():
    with np.errstate(all="ignore"):
        yield
