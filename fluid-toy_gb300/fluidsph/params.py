"""Parameter-struct builders over the library's host helpers, restating the
reference's state builders (src/state/simulation.rs:139-184, 315-480;
src/state/rigid_body.rs:131-146, 188-205; src/state/interaction.rs:113-128).
These run on the host only and need no GPU.
"""
from __future__ import annotations

import ctypes as C

from . import abi
from .abi import (GpuContainerGeometry, GpuGravity, GpuGridParams, GpuMouseForce, GpuRigidBody,
                  GpuSphParams3D, check)


def compute_rest_density(h: float, mass: float) -> float:
    return float(abi.load().fs_compute_rest_density(h, mass))


def compute_pcisph_delta(h: float, mass: float, rest_density: float, dt: float) -> float:
    return float(abi.load().fs_compute_pcisph_delta(h, mass, rest_density, dt))


def sph_params_3d(kernel_radius: float, mass: float, rest_density: float | None,
                  stiffness: float, near_stiffness: float, viscosity: float,
                  surface_tension: float, xsph_epsilon: float, dt: float,
                  num_particles: int) -> GpuSphParams3D:
    """SphConfig::to_gpu_params_3d. ``rest_density=None`` derives it from h and
    mass like the reference (compute_rest_density)."""
    lib = abi.load()
    if rest_density is None:
        rest_density = lib.fs_compute_rest_density(kernel_radius, mass)
    p = GpuSphParams3D()
    check(lib.fs_sph_params_3d(kernel_radius, mass, rest_density, stiffness, near_stiffness,
                               viscosity, surface_tension, xsph_epsilon, dt, int(num_particles),
                               C.byref(p)))
    return p


def container_geometry(width: float, depth: float, floor_y: float, height: float,
                       tilt_x: float = 0.0, tilt_z: float = 0.0, wall_stiffness: float = 200.0,
                       damping: float = 0.55, clip_enabled: bool = False,
                       clip_margin: float = 0.0) -> GpuContainerGeometry:
    """ContainerConfig::to_gpu_geometry (rotation R = Rz * Rx)."""
    g = GpuContainerGeometry()
    check(abi.load().fs_container_geometry(width, depth, floor_y, height, tilt_x, tilt_z,
                                           wall_stiffness, damping, 1 if clip_enabled else 0,
                                           clip_margin, C.byref(g)))
    return g


def gravity(gy: float = -9.8, gx: float = 0.0, gz: float = 0.0) -> GpuGravity:
    g = GpuGravity()
    g.direction[:] = [gx, gy, gz]
    return g


def mouse_force(position=(0.0, 0.0, 0.0), radius: float = 0.5, strength: float = 30.0,
                active: bool = False, mode: int = 0, direction=(0.0, 0.0, -1.0)) -> GpuMouseForce:
    """GpuMouseForce (defaults = GpuMouseForce::default())."""
    m = GpuMouseForce()
    m.position[:] = list(position)
    m.radius = radius
    m.strength = strength
    m.is_active = 1 if active else 0
    m.mode = int(mode)
    m.direction[:] = list(direction)
    return m


def rigid_body(position=(0.0, 0.0, 0.0), half_extent: float = 0.15, velocity=(0.0, 0.0, 0.0),
               active: bool = False, stiffness: float = 200.0, shape: int = 0,
               orientation=(0.0, 0.0, 0.0, 1.0)) -> GpuRigidBody:
    """RigidBodyConfig::to_gpu_rigid_body (stiffness = wall_stiffness there)."""
    b = GpuRigidBody()
    b.position[:] = list(position)
    b.half_extent = half_extent
    b.velocity[:] = list(velocity)
    b.is_active = 1 if active else 0
    b.stiffness = stiffness
    b.shape = int(shape)
    rows = (C.c_float * 12)()
    q = (C.c_float * 4)(*orientation)
    check(abi.load().fs_quat_to_rotation_rows(q, rows))
    b.rot_row0[:] = rows[0:4]
    b.rot_row1[:] = rows[4:8]
    b.rot_row2[:] = rows[8:12]
    return b


def grid_params_for(kernel_radius: float, num_particles: int) -> GpuGridParams:
    g = GpuGridParams()
    check(abi.load().fs_grid_params_for(kernel_radius, int(num_particles), C.byref(g)))
    return g


def mc_grid_params(grid_min, grid_max, grid_size: int, kernel_radius: float,
                   iso_value: float = 0.0, num_particles: int = 0):
    """MarchingCubesRenderer::update_params (marching_cubes.rs:2099-2113)."""
    from .abi import GpuMcGridParams
    out = GpuMcGridParams()
    lo = (C.c_float * 3)(*[float(v) for v in grid_min])
    hi = (C.c_float * 3)(*[float(v) for v in grid_max])
    check(abi.load().fs_mc_grid_params(lo, hi, int(grid_size), float(kernel_radius),
                                       float(iso_value), int(num_particles), C.byref(out)))
    return out


def rigid_body_state(position=(0.0, 0.2, 0.0), half_extent: float = 0.15, shape: int = 0,
                     density: float = 300.0, velocity=(0.0, 0.0, 0.0),
                     orientation=(0.0, 0.0, 0.0, 1.0), angular_velocity=(0.0, 0.0, 0.0),
                     enabled: bool = True, held: bool = False, wall_stiffness: float = 200.0):
    """FsRigidBodyState (RigidBodyConfig, src/state/rigid_body.rs:86-128)."""
    from .abi import FsRigidBodyState
    s = FsRigidBodyState()
    s.position[:] = list(position)
    s.half_extent = half_extent
    s.shape = int(shape)
    s.density = density
    s.velocity[:] = list(velocity)
    s.orientation[:] = list(orientation)
    s.angular_velocity[:] = list(angular_velocity)
    s.enabled = 1 if enabled else 0
    s.held = 1 if held else 0
    s.wall_stiffness = wall_stiffness
    return s


def rigid_body_to_gpu(state):
    """RigidBodyConfig::to_gpu_rigid_body (rigid_body.rs:131-146)."""
    out = GpuRigidBody()
    check(abi.load().fs_rigid_body_to_gpu(C.byref(state), C.byref(out)))
    return out


def integrate_rigid_body(state, container_geom, substep_dt: float, num_substeps: int, gravity,
                         accum) -> None:
    """integrate_rigid_body (rigid_body.rs:277-365), in place on `state`."""
    g = (C.c_float * 3)(*[float(v) for v in gravity])
    check(abi.load().fs_integrate_rigid_body(C.byref(state), C.byref(container_geom),
                                             float(substep_dt), int(num_substeps), g,
                                             C.byref(accum)))
