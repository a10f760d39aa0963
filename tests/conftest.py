"""Shared test setup: import paths, the `gpu` marker, library builds."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "smoothedparticles.jl_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def sph_lib():
    """libsphgpu.so, built in-tree if missing (nvcc cross-compiles without a GPU)."""
    from sphgpu import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from sphgpu.build import build_library
        build_library()
    return _lib.load()


@pytest.fixture(scope="session")
def gpu(sph_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return sph_lib
