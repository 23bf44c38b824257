"""Shared test setup: import paths, the `gpu` marker, library fixtures."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT / "fluid-toy_gb300", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu() -> bool:
    try:
        import ctypes
        rt = None
        for name in ("libcudart.so", "libcudart.so.13", "libcuda.so.1"):
            try:
                rt = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if rt is None:
            return False
        n = ctypes.c_int(0)
        if hasattr(rt, "cudaGetDeviceCount"):
            return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
        if rt.cuInit(0) != 0:
            return False
        return rt.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def fslib():
    """libfluidsph.so, built in-tree if stale."""
    from fluidsph import abi
    from fluidsph.build import build_library
    build_library()
    return abi.load()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle
