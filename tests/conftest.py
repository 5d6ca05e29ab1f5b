import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def product_lib():
    from j3d_gb300 import build
    build.build()
    from j3d_gb300 import _ffi
    return _ffi.lib()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle.oracle as O
    O.build()
    O.lib()
    return O


@pytest.fixture(scope="session")
def gpu_ctx(product_lib):
    if not _has_gpu():
        pytest.skip("no CUDA GPU")
    from j3d_gb300 import Context
    ctx = Context(0)
    yield ctx
    ctx.close()


@pytest.fixture(params=["trace", "raster"])
def primary(request, gpu_ctx):
    """Runs a frame test once with traced and once with rasterised primary
    hits (the context's mode is restored to automatic afterwards)."""
    from j3d_gb300 import PRIMARY_AUTO, PRIMARY_RASTER, PRIMARY_TRACE
    gpu_ctx.set_primary_mode(PRIMARY_TRACE if request.param == "trace" else PRIMARY_RASTER)
    yield request.param
    gpu_ctx.set_primary_mode(PRIMARY_AUTO)
