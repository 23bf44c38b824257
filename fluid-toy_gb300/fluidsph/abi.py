"""ctypes binding of libfluidsph.so (include/fluidsph.h).

The structs are the reference's ``#[repr(C)]`` POD structs
(src/simulation/particle.rs, src/state/simulation.rs, src/state/interaction.rs,
src/state/rigid_body.rs, src/simulation/sph_3d_grid.rs). Particles cross the
boundary as ``numpy.float32`` arrays of shape (N, 16), one row per 64-byte
``SphParticle3D`` record; the column layout is given by the ``COL_*`` slices.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import LIB_PATH

FS_ABI_VERSION = 0x00010057
FS_OK = 0
FS_STAGE_COUNT = 10
FS_STAT_COUNT = 6
STAGE_NAMES = ("clear", "hash", "scan", "reorder", "density", "xsph", "force_predict",
               "pcisph_solve", "finalize_integrate", "step")

# SphParticle3D columns (particle.rs:8-17)
COL_POS = slice(0, 3)
COL_PAD0 = 3
COL_VEL = slice(4, 7)
COL_PAD1 = 7
COL_FORCE = slice(8, 11)
COL_DENSITY = 11
COL_NEAR = 12
COL_NORMAL = slice(13, 16)


class GpuSphParams3D(C.Structure):
    _fields_ = [("kernel_radius", C.c_float), ("kernel_radius_sq", C.c_float),
                ("kernel_radius_pow5", C.c_float), ("kernel_radius_pow6", C.c_float),
                ("kernel_radius_pow9", C.c_float), ("mass", C.c_float),
                ("rest_density", C.c_float), ("stiffness", C.c_float),
                ("near_stiffness", C.c_float), ("viscosity", C.c_float), ("dt", C.c_float),
                ("num_particles", C.c_uint32), ("surface_tension", C.c_float),
                ("pcisph_delta", C.c_float), ("xsph_epsilon", C.c_float),
                ("_padding_st", C.c_float)]


class GpuContainerGeometry(C.Structure):
    _fields_ = [("half_width", C.c_float), ("half_height", C.c_float),
                ("half_depth", C.c_float), ("center_y", C.c_float),
                ("forward_row0", C.c_float * 4), ("forward_row1", C.c_float * 4),
                ("forward_row2", C.c_float * 4), ("inverse_row0", C.c_float * 4),
                ("inverse_row1", C.c_float * 4), ("inverse_row2", C.c_float * 4),
                ("wall_stiffness", C.c_float), ("damping", C.c_float),
                ("clip_enabled", C.c_uint32), ("clip_margin", C.c_float)]


class GpuGravity(C.Structure):
    _fields_ = [("direction", C.c_float * 3), ("_padding", C.c_float)]


class GpuMouseForce(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("radius", C.c_float), ("strength", C.c_float),
                ("is_active", C.c_uint32), ("mode", C.c_uint32), ("_pad", C.c_float),
                ("direction", C.c_float * 3), ("_pad2", C.c_float)]


class GpuRigidBody(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("half_extent", C.c_float),
                ("velocity", C.c_float * 3), ("is_active", C.c_uint32),
                ("stiffness", C.c_float), ("shape", C.c_uint32), ("_pad1", C.c_float),
                ("_pad2", C.c_float), ("rot_row0", C.c_float * 4), ("rot_row1", C.c_float * 4),
                ("rot_row2", C.c_float * 4)]


class GpuRigidBodyAccum(C.Structure):
    _fields_ = [("force_x", C.c_int32), ("force_y", C.c_int32), ("force_z", C.c_int32),
                ("contact_count", C.c_uint32), ("torque_x", C.c_int32),
                ("torque_y", C.c_int32), ("torque_z", C.c_int32), ("_pad", C.c_uint32)]

    def as_tuple(self):
        return (self.force_x, self.force_y, self.force_z, self.contact_count,
                self.torque_x, self.torque_y, self.torque_z)


class FsRigidBodyState(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("half_extent", C.c_float),
                ("velocity", C.c_float * 3), ("density", C.c_float),
                ("orientation", C.c_float * 4), ("angular_velocity", C.c_float * 3),
                ("shape", C.c_uint32), ("enabled", C.c_uint32), ("held", C.c_uint32),
                ("wall_stiffness", C.c_float), ("_pad", C.c_uint32)]


class FsKernelForms(C.Structure):
    _fields_ = [("density_loads", C.c_uint32), ("solve_loads", C.c_uint32),
                ("xsph_loads", C.c_uint32), ("decided", C.c_uint32), ("bucket", C.c_uint32),
                ("ms", (C.c_float * 5) * 3)]


class FsKernelFormsEntry(C.Structure):
    _fields_ = [("device", C.c_uint32), ("bucket", C.c_uint32), ("many_scenes", C.c_uint32),
                ("iterations", C.c_uint32), ("density_loads", C.c_uint32),
                ("solve_loads", C.c_uint32), ("xsph_loads", C.c_uint32), ("_pad", C.c_uint32),
                ("ms", (C.c_float * 5) * 3)]


class GpuGridParams(C.Structure):
    _fields_ = [("grid_size_x", C.c_uint32), ("grid_size_y", C.c_uint32),
                ("grid_size_z", C.c_uint32), ("total_cells", C.c_uint32),
                ("cell_size", C.c_float), ("inv_cell_size", C.c_float),
                ("grid_origin_x", C.c_float), ("grid_origin_y", C.c_float),
                ("grid_origin_z", C.c_float), ("num_particles", C.c_uint32),
                ("_padding", C.c_uint32 * 2)]


class GpuMcGridParams(C.Structure):
    _fields_ = [("grid_min", C.c_float * 3), ("grid_size", C.c_uint32),
                ("grid_max", C.c_float * 3), ("cell_size", C.c_float),
                ("kernel_radius", C.c_float), ("iso_value", C.c_float),
                ("num_particles", C.c_uint32), ("max_vertices", C.c_uint32)]


class GpuSprayParams(C.Structure):
    _fields_ = [("min_speed", C.c_float), ("emission_rate", C.c_float), ("lifetime", C.c_float),
                ("lifetime_variation", C.c_float), ("drag", C.c_float),
                ("speed_multiplier", C.c_float), ("velocity_jitter", C.c_float),
                ("dt", C.c_float), ("max_particles", C.c_uint32),
                ("num_sph_particles", C.c_uint32), ("frame_count", C.c_uint32),
                ("gravity_y", C.c_float), ("k_trapped_air", C.c_float),
                ("k_wave_crest", C.c_float), ("ta_limit", C.c_float),
                ("bubble_buoyancy", C.c_float), ("bubble_drag", C.c_float),
                ("wc_limit", C.c_float), ("_pad", C.c_float * 2)]


# GpuSprayParticle as numpy rows of 12 float32 (kind is a uint32 bit pattern)
SPRAY_DTYPE = np.dtype([("pos", "<f4", 3), ("lifetime", "<f4"), ("vel", "<f4", 3),
                        ("max_lifetime", "<f4"), ("kind", "<u4"), ("age", "<f4"),
                        ("pad", "<f4", 2)])


class FsDevicePointers(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in (
        "pos", "vel", "force", "sorted_pos", "sorted_vel", "sorted_density", "sorted_normal",
        "cell_counts", "cell_starts", "cell_begin", "particle_cell_indices", "sorted_to_orig",
        "stream")]


class FsSceneInfo(C.Structure):
    _fields_ = [("particle_offset", C.c_uint32), ("num_particles", C.c_uint32),
                ("active_particles", C.c_uint32), ("sorted_offset", C.c_uint32),
                ("cell_offset", C.c_uint32), ("total_cells", C.c_uint32),
                ("_pad", C.c_uint32 * 2), ("grid", GpuGridParams)]


STRUCT_SIZES = {
    GpuSphParams3D: 64, GpuContainerGeometry: 128, GpuGravity: 16, GpuMouseForce: 48,
    GpuRigidBody: 96, GpuRigidBodyAccum: 32, GpuGridParams: 48, FsSceneInfo: 80,
    GpuMcGridParams: 48, FsRigidBodyState: 80, GpuSprayParams: 80, FsKernelForms: 80,
    FsKernelFormsEntry: 92,
}
for _t, _n in STRUCT_SIZES.items():
    assert C.sizeof(_t) == _n, (_t.__name__, C.sizeof(_t))

_P = C.POINTER
_vp = C.c_void_p
_u32 = C.c_uint32
_f = C.c_float

# name -> (restype, argtypes); exactly the functions include/fluidsph.h declares
SIGNATURES = {
    "fs_last_error": (C.c_char_p, []),
    "fs_abi_version": (_u32, []),
    "fs_compute_rest_density": (_f, [_f, _f]),
    "fs_compute_pcisph_delta": (_f, [_f, _f, _f, _f]),
    "fs_sph_params_3d": (C.c_int, [_f, _f, _f, _f, _f, _f, _f, _f, _f, _u32,
                                   _P(GpuSphParams3D)]),
    "fs_container_geometry": (C.c_int, [_f, _f, _f, _f, _f, _f, _f, _f, _u32, _f,
                                        _P(GpuContainerGeometry)]),
    "fs_quat_to_rotation_rows": (C.c_int, [_P(_f), _P(_f)]),
    "fs_grid_params_for": (C.c_int, [_f, _u32, _P(GpuGridParams)]),
    "fs_rigid_body_to_gpu": (C.c_int, [_P(FsRigidBodyState), _P(GpuRigidBody)]),
    "fs_integrate_rigid_body": (C.c_int, [_P(FsRigidBodyState), _P(GpuContainerGeometry), _f,
                                          _u32, _P(_f), _P(GpuRigidBodyAccum)]),
    "fs_clamp_rigid_body": (C.c_int, [_P(FsRigidBodyState), _P(GpuContainerGeometry), C.c_int]),
    "fs_rigid_coupling_set_state": (C.c_int, [_vp, _u32, _P(FsRigidBodyState)]),
    "fs_rigid_coupling_get_state": (C.c_int, [_vp, _u32, _P(FsRigidBodyState)]),
    "fs_frames": (C.c_int, [_vp, _u32, _u32]),
    "fs_mc_grid_params": (C.c_int, [_P(_f), _P(_f), _u32, _f, _f, _u32, _P(GpuMcGridParams)]),
    "fs_create": (C.c_int, [_vp, _u32, _P(GpuSphParams3D), _P(GpuContainerGeometry), _u32,
                            _vp, _u32, C.c_int, _u32, _P(_vp)]),
    "fs_destroy": (C.c_int, [_vp]),
    "fs_step": (C.c_int, [_vp, _u32]),
    "fs_prepare_steps": (C.c_int, [_vp, _u32]),
    "fs_update_sph_params": (C.c_int, [_vp, _P(GpuSphParams3D)]),
    "fs_update_container_geometry": (C.c_int, [_vp, _P(GpuContainerGeometry)]),
    "fs_update_mouse_force": (C.c_int, [_vp, _P(GpuMouseForce)]),
    "fs_update_gravity": (C.c_int, [_vp, _P(GpuGravity)]),
    "fs_update_rigid_body": (C.c_int, [_vp, _P(GpuRigidBody)]),
    "fs_set_pcisph_iterations": (C.c_int, [_vp, _u32]),
    "fs_clear_rigid_body_accum": (C.c_int, [_vp]),
    "fs_read_rigid_body_accum": (C.c_int, [_vp, _P(GpuRigidBodyAccum)]),
    "fs_num_particles": (C.c_int, [_vp, _P(_u32)]),
    "fs_grid_params": (C.c_int, [_vp, _P(GpuGridParams)]),
    "fs_spawn_particles": (C.c_int, [_vp, _P(_f), _u32, _f, _P(_u32)]),
    "fs_spawn_positions": (C.c_int, [_P(C.c_float), _u32, C.c_float, _u32, _u32, _vp, _P(_u32)]),
    "fs_download_particles": (C.c_int, [_vp, _vp, _u32]),
    "fs_download_sorted": (C.c_int, [_vp, _vp, _u32]),
    "fs_download_cells": (C.c_int, [_vp, _vp, _vp, _u32]),
    "fs_download_index_maps": (C.c_int, [_vp, _vp, _vp, _u32]),
    "fs_upload_particles": (C.c_int, [_vp, _vp, _u32]),
    "fs_density_splat": (C.c_int, [_vp, _u32, _P(GpuMcGridParams), _P(GpuContainerGeometry),
                                   _vp, C.c_int]),
    "fs_device_pointers": (C.c_int, [_vp, _P(FsDevicePointers)]),
    "fs_set_stream": (C.c_int, [_vp, _vp]),
    "fs_sync": (C.c_int, [_vp]),
    "fs_enable_stage_timing": (C.c_int, [_vp, C.c_int]),
    "fs_stage_times": (C.c_int, [_vp, _P(C.c_double), _P(_u32), C.c_int]),
    "fs_neighbor_stats": (C.c_int, [_vp, _P(C.c_uint64), C.c_int]),
    "fs_prefix_scan_noalloc": (C.c_int, [_vp, _vp, _u32, _vp, _vp]),
    "fs_export_particles_aos": (C.c_int, [_vp, _u32, C.c_int, _vp, _u32]),
    "fs_load_batching": (C.c_int, [_vp, _P(C.c_int), _P(C.c_int)]),
    "fs_kernel_forms": (C.c_int, [_vp, _vp]),
    "fs_set_kernel_forms": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int]),
    "fs_kernel_forms_table": (C.c_int, [_vp, _u32, _P(_u32)]),
    "fs_selftest_arithmetic": (C.c_int, [C.c_int, _P(C.c_ulonglong)]),
    "fs_selftest_scan_wait": (C.c_int, [_vp, C.c_int, _vp]),
    "fs_selftest_fp32_rate": (C.c_int, [C.c_int, _P(C.c_double)]),
    "fs_batch_create": (C.c_int, [_vp, _P(_u32), _u32, _vp, _vp, _vp, _u32, C.c_int, _u32,
                                  _P(_vp)]),
    "fs_batch_num_scenes": (C.c_int, [_vp, _P(_u32)]),
    "fs_batch_scene_info": (C.c_int, [_vp, _u32, _P(FsSceneInfo)]),
    "fs_batch_update_scene": (C.c_int, [_vp, _u32, _P(GpuSphParams3D), _P(GpuContainerGeometry),
                                        _P(GpuGravity), _P(GpuMouseForce), _P(GpuRigidBody)]),
    "fs_batch_read_rigid_body_accum": (C.c_int, [_vp, _vp, _u32]),
    "fs_batch_download_scene": (C.c_int, [_vp, _u32, _vp, _u32]),
    "fs_batch_download_scene_sorted": (C.c_int, [_vp, _u32, _vp, _u32]),
    "fs_batch_download_scene_cells": (C.c_int, [_vp, _u32, _vp, _vp, _u32]),
    "fs_batch_download_scene_index_maps": (C.c_int, [_vp, _u32, _vp, _vp, _u32]),
    "fs_batch_upload_scene": (C.c_int, [_vp, _u32, _vp, _u32]),
    "fs_spray_create": (C.c_int, [_vp, _u32, _u32, _P(_vp)]),
    "fs_spray_destroy": (C.c_int, [_vp]),
    "fs_spray_step": (C.c_int, [_vp, _P(GpuSprayParams)]),
    "fs_spray_reset": (C.c_int, [_vp]),
    "fs_spray_stats": (C.c_int, [_vp, _P(_u32)]),
    "fs_spray_limits": (C.c_int, [_vp, _P(_f), _P(_u32)]),
    "fs_spray_download": (C.c_int, [_vp, _vp, _u32]),
    "fs_spray_device_buffer": (C.c_int, [_vp, _P(_vp)]),
    "fs_adj_create": (C.c_int, [_vp, _u32, _P(_vp)]),
    "fs_adj_destroy": (C.c_int, [_vp]),
    "fs_adj_forward": (C.c_int, [_vp, _u32]),
    "fs_adj_set_tape_budget": (C.c_int, [_vp, C.c_uint64]),
    "fs_adj_tape_info": (C.c_int, [_vp, _P(_u32), _P(C.c_uint64)]),
    "fs_adj_set_cotangents": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "fs_adj_splat_mse_loss": (C.c_int, [_vp, _u32, _P(GpuMcGridParams), _P(GpuContainerGeometry),
                                        _vp, C.c_int, _P(C.c_double)]),
    "fs_adj_splat_mse_losses": (C.c_int, [_vp, _u32, _P(_u32), _P(GpuMcGridParams),
                                          _P(GpuContainerGeometry), _P(_vp), C.c_int,
                                          _P(C.c_double)]),
    "fs_adj_backward": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp]),
    "fs_adj_param_gradients": (C.c_int, [_vp, _vp, _u32]),
    "fs_adj_final_splat": (C.c_int, [_vp, _u32, _P(GpuMcGridParams), _P(GpuContainerGeometry),
                                     _vp, C.c_int]),
}
FS_BATCH_MAX_SCENES = 65535
FS_NOALLOC_SCAN_MAX_CELLS = 1 << 26
FS_ADJ_NUM_PARAMS = 5

_lib = None


class FluidSphError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"fluidsph error {code}: {message}")
        self.code = code


def load(path: Path | str | None = None):
    """Load libfluidsph.so (built by fluidsph.build). Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(
            f"{p} is missing: build it with fluidsph.build.build_library() "
            "(there is no CPU fallback for the SPH step)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.fs_abi_version() != FS_ABI_VERSION:
        raise FluidSphError(-2, "library ABI version differs from this binding")
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != FS_OK:
        msg = _lib.fs_last_error().decode() if _lib is not None else "library not loaded"
        raise FluidSphError(rc, msg)


def exported_symbols(header: Path) -> list[str]:
    """Function names declared in a C header (``fs_*(`` declarations)."""
    import re
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fs_[a-z0-9_]+)\s*\(", text)))


def as_particles(arr: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(arr, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] != 16:
        raise ValueError("particles must be an (N, 16) float32 array of SphParticle3D rows")
    return a
