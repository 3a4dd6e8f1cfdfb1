import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "madsdp.jl_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_lib():
    """Build libmadsdp_gpu.so if it is missing or stale (nvcc cross-compiles)."""
    import build as build_mod  # madsdp.jl_gb300/build.py
    return build_mod.build()


@pytest.fixture(scope="session")
def gpu_ctx(built_lib):
    import torch  # noqa: F401  (first CUDA user in the process)
    import madsdp_gpu
    if madsdp_gpu._lib.load().msdp_device_count() < 1:
        pytest.skip("no CUDA device")
    return madsdp_gpu.default_context()
