"""The C-ABI library loads, exports every symbol include/fluidsph.h declares,
and reports errors (never aborts) — no GPU compute is called here."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "fluidsph.h"


def test_library_exports_every_header_symbol(fslib):
    from fluidsph import abi
    declared = abi.exported_symbols(HEADER)
    assert len(declared) >= 30
    missing = [s for s in declared if not hasattr(fslib, s)]
    assert not missing, missing
    # the ctypes binding covers exactly the declared functions
    assert sorted(abi.SIGNATURES) == declared


def test_abi_version(fslib):
    from fluidsph import abi
    assert fslib.fs_abi_version() == abi.FS_ABI_VERSION


def test_struct_sizes_match_reference_layouts():
    from fluidsph import abi
    for t, n in abi.STRUCT_SIZES.items():
        assert C.sizeof(t) == n
    assert abi.GpuContainerGeometry.wall_stiffness.offset == 112
    assert abi.GpuRigidBody.rot_row0.offset == 48
    assert abi.GpuMouseForce.direction.offset == 32


def test_create_rejects_bad_arguments(fslib):
    from fluidsph import abi, params as P
    sph = P.sph_params_3d(0.08, 1.0, 8000.0, 35, 0.45, 15, 6.5, 0.305, 0.008, 1)
    geom = P.container_geometry(1, 1, 0, 1)
    parts = np.zeros((1, 16), np.float32)
    h = C.c_void_p()
    # wrong ABI version is refused before any device work
    rc = fslib.fs_create(parts.ctypes.data, 1, C.byref(sph), C.byref(geom), 0, None, 0, 0,
                         0xDEAD, C.byref(h))
    assert rc == -2 and b"ABI" in fslib.fs_last_error()
    rc = fslib.fs_create(None, 1, C.byref(sph), C.byref(geom), 0, None, 0, 0,
                         abi.FS_ABI_VERSION, C.byref(h))
    assert rc == -1
    bad = P.sph_params_3d(0.0, 1.0, 8000.0, 35, 0.45, 15, 6.5, 0.305, 0.008, 1)
    rc = fslib.fs_create(parts.ctypes.data, 1, C.byref(bad), C.byref(geom), 0, None, 0, 0,
                         abi.FS_ABI_VERSION, C.byref(h))
    assert rc == -1
    assert fslib.fs_step(None, 1) == -1
    assert fslib.fs_destroy(None) == 0
    # the batched loss call checks its handle before any device work
    losses = (C.c_double * 2)()
    assert fslib.fs_adj_splat_mse_losses(None, 2, None, None, None, None, 0, losses) == -1
    assert b"null handle" in fslib.fs_last_error()


def test_create_without_gpu_reports_no_device(fslib):
    from conftest import HAS_GPU
    if HAS_GPU:
        pytest.skip("a GPU is present")
    from fluidsph import abi, params as P
    sph = P.sph_params_3d(0.08, 1.0, 8000.0, 35, 0.45, 15, 6.5, 0.305, 0.008, 1)
    geom = P.container_geometry(1, 1, 0, 1)
    parts = np.zeros((1, 16), np.float32)
    h = C.c_void_p()
    rc = fslib.fs_create(parts.ctypes.data, 1, C.byref(sph), C.byref(geom), 0, None, 0, 0,
                         abi.FS_ABI_VERSION, C.byref(h))
    assert rc == -6 and not h.value


def test_python_mirror_raises_without_library(tmp_path):
    from fluidsph import abi
    saved = abi._lib
    abi._lib = None
    try:
        with pytest.raises(FileNotFoundError):
            abi.load(tmp_path / "missing.so")
    finally:
        abi._lib = saved
