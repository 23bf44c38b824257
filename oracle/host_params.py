"""The reference's host-side parameter builders, restated in float32 numpy.

TEST INFRASTRUCTURE ONLY: used by tests/ (as a second, independent
restatement checked against the library's fs_* helpers and against the
mechanical translation of the Rust sources in oracle/_ref) and by bench.py's
reference arm, which builds its inputs with these functions so that it runs
without loading the product library.

Every operation is one IEEE float32 operation in the Rust source's order:
  compute_rest_density      src/state/simulation.rs:402-427
  compute_pcisph_delta      src/state/simulation.rs:429-480
  to_gpu_params_3d          src/state/simulation.rs:315-337
  rotation_matrices /
  to_gpu_geometry           src/state/simulation.rs:137-184
  quat_to_rotation_rows     src/state/rigid_body.rs:188-205
  to_gpu_rigid_body         src/state/rigid_body.rs:131-146
f32::powi(n) is binary exponentiation (LLVM's expansion of llvm.powi with a
constant exponent, and compiler-rt's __powisf2, agree for n > 0); f32::sin /
f32::cos are the C library's sinf / cosf, called here through ctypes so that
this restatement uses the same functions as compiled host code on the same
machine; iterator sums fold left from -0.0.
"""
from __future__ import annotations

import ctypes as C
import ctypes.util
import math

import numpy as np

f32 = np.float32
PI = f32(math.pi)  # std::f32::consts::PI

_libm = C.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.sinf.restype = C.c_float
_libm.sinf.argtypes = [C.c_float]
_libm.cosf.restype = C.c_float
_libm.cosf.argtypes = [C.c_float]


def sinf(x) -> np.float32:
    return f32(_libm.sinf(float(f32(x))))


def cosf(x) -> np.float32:
    return f32(_libm.cosf(float(f32(x))))


def powi(x, n: int) -> np.float32:
    """f32::powi for n >= 1: square-and-multiply from the lowest bit."""
    r, a = None, f32(x)
    while n:
        if n & 1:
            r = a if r is None else f32(r * a)
        n >>= 1
        if n:
            a = f32(a * a)
    return r


def compute_rest_density(h, mass) -> np.float32:
    """simulation.rs:402-427: poly6 sum over a lattice of spacing 0.6 h."""
    h, mass = f32(h), f32(mass)
    spacing = f32(h * f32(0.6))
    cells = int(np.ceil(f32(h / spacing))) + 1
    h2 = f32(h * h)
    scale = f32(f32(315.0) / f32(f32(f32(64.0) * PI) * powi(h, 9)))
    density = f32(0.0)
    for dz in range(-cells, cells + 1):
        for dy in range(-cells, cells + 1):
            for dx in range(-cells, cells + 1):
                ax = f32(f32(dx) * spacing)
                ay = f32(f32(dy) * spacing)
                az = f32(f32(dz) * spacing)
                r_sq = f32(f32(f32(ax * ax) + f32(ay * ay)) + f32(az * az))
                if r_sq < h2:
                    diff = f32(h2 - r_sq)
                    density = f32(density + f32(f32(f32(f32(mass * scale) * diff) * diff) * diff))
    return density


def compute_pcisph_delta(h, mass, rest_density, dt) -> np.float32:
    """simulation.rs:429-480: 0.2 / (beta (|sum grad|^2 + sum |grad|^2))."""
    h, mass, rest_density, dt = f32(h), f32(mass), f32(rest_density), f32(dt)
    spacing = f32(h * f32(0.6))
    cells = int(np.ceil(f32(h / spacing))) + 1
    sg = [f32(0.0), f32(0.0), f32(0.0)]
    sum_grad_sq = f32(0.0)
    h6 = powi(h, 6)
    hh = f32(h * h)
    for dz in range(-cells, cells + 1):
        for dy in range(-cells, cells + 1):
            for dx in range(-cells, cells + 1):
                if dx == 0 and dy == 0 and dz == 0:
                    continue
                rv = [f32(f32(dx) * spacing), f32(f32(dy) * spacing), f32(f32(dz) * spacing)]
                r_sq = f32(-0.0)
                for v in rv:
                    r_sq = f32(r_sq + f32(v * v))
                if r_sq < hh and r_sq > f32(1e-12):
                    r = f32(np.sqrt(r_sq))
                    hr = f32(h - r)
                    grad_mag = f32(f32(f32(f32(45.0) / f32(PI * h6)) * hr) * hr)
                    g = [f32(f32(grad_mag * v) / r) for v in rv]
                    for k in range(3):
                        sg[k] = f32(sg[k] + g[k])
                    sum_grad_sq = f32(sum_grad_sq + f32(f32(f32(g[0] * g[0]) + f32(g[1] * g[1]))
                                                        + f32(g[2] * g[2])))
    dot = f32(-0.0)
    for v in sg:
        dot = f32(dot + f32(v * v))
    beta = f32(f32(f32(f32(dt * dt) * mass) * mass) / f32(rest_density * rest_density))
    denom = f32(beta * f32(dot + sum_grad_sq))
    return f32(f32(0.2) / denom) if abs(denom) > f32(1e-10) else f32(0.0)


def sph_params_3d(kernel_radius, mass, rest_density, stiffness, near_stiffness, viscosity,
                  surface_tension, xsph_epsilon, dt, num_particles):
    """SphConfig::to_gpu_params_3d (simulation.rs:315-337); rest_density None
    derives it like the reference (compute_rest_density)."""
    from fluidsph.abi import GpuSphParams3D  # the struct layout only
    h = f32(kernel_radius)
    if rest_density is None:
        rest_density = compute_rest_density(h, mass)
    p = GpuSphParams3D()
    p.kernel_radius = h
    p.kernel_radius_sq = f32(h * h)
    p.kernel_radius_pow5 = powi(h, 5)
    p.kernel_radius_pow6 = powi(h, 6)
    p.kernel_radius_pow9 = powi(h, 9)
    p.mass = f32(mass)
    p.rest_density = f32(rest_density)
    p.stiffness = f32(stiffness)
    p.near_stiffness = f32(near_stiffness)
    p.viscosity = f32(viscosity)
    p.dt = f32(dt)
    p.num_particles = int(num_particles)
    p.surface_tension = f32(surface_tension)
    p.pcisph_delta = compute_pcisph_delta(h, mass, rest_density, dt)
    p.xsph_epsilon = f32(xsph_epsilon)
    p._padding_st = 0.0
    return p


def rotation_matrices(tilt_x, tilt_z):
    """ContainerConfig::rotation_matrices (simulation.rs:137-158): R = Rz Rx
    and its transpose, as rows of 4."""
    sx, cx = sinf(tilt_x), cosf(tilt_x)
    sz, cz = sinf(tilt_z), cosf(tilt_z)
    z = f32(0.0)
    fwd = [[cz, f32(f32(-sz) * cx), f32(sz * sx), z],
           [sz, f32(cz * cx), f32(f32(-cz) * sx), z],
           [z, sx, cx, z]]
    inv = [[cz, sz, z, z],
           [f32(f32(-sz) * cx), f32(cz * cx), sx, z],
           [f32(sz * sx), f32(f32(-cz) * sx), cx, z]]
    return fwd, inv


def container_geometry(width, depth, floor_y, height, tilt_x=0.0, tilt_z=0.0,
                       wall_stiffness=200.0, damping=0.55, clip_enabled=False, clip_margin=0.0):
    """ContainerConfig::to_gpu_geometry (simulation.rs:162-184)."""
    from fluidsph.abi import GpuContainerGeometry
    fwd, inv = rotation_matrices(tilt_x, tilt_z)
    g = GpuContainerGeometry()
    two = f32(2.0)
    g.half_width = f32(f32(width) / two)
    g.half_height = f32(f32(height) / two)
    g.half_depth = f32(f32(depth) / two)
    g.center_y = f32(f32(floor_y) + f32(f32(height) / two))
    for k, row in enumerate(fwd):
        getattr(g, f"forward_row{k}")[:] = [float(v) for v in row]
    for k, row in enumerate(inv):
        getattr(g, f"inverse_row{k}")[:] = [float(v) for v in row]
    g.wall_stiffness = f32(wall_stiffness)
    g.damping = f32(damping)
    g.clip_enabled = 1 if clip_enabled else 0
    g.clip_margin = f32(clip_margin)
    return g


def quat_to_rotation_rows(q):
    """rigid_body.rs:188-205: R_quat transposed (world -> body), rows of 4."""
    x, y, z, w = (f32(v) for v in q)
    xx, yy, zz = f32(x * x), f32(y * y), f32(z * z)
    xy, xz, yz = f32(x * y), f32(x * z), f32(y * z)
    wx, wy, wz = f32(w * x), f32(w * y), f32(w * z)
    one, two, zero = f32(1.0), f32(2.0), f32(0.0)
    return [[f32(one - f32(two * f32(yy + zz))), f32(two * f32(xy + wz)),
             f32(two * f32(xz - wy)), zero],
            [f32(two * f32(xy - wz)), f32(one - f32(two * f32(xx + zz))),
             f32(two * f32(yz + wx)), zero],
            [f32(two * f32(xz + wy)), f32(two * f32(yz - wx)),
             f32(one - f32(two * f32(xx + yy))), zero]]


def gravity(gy=-9.8, gx=0.0, gz=0.0):
    from fluidsph.abi import GpuGravity
    g = GpuGravity()
    g.direction[:] = [gx, gy, gz]
    return g


def rigid_body(position=(0.0, 0.0, 0.0), half_extent=0.15, velocity=(0.0, 0.0, 0.0),
               active=False, stiffness=200.0, shape=0, orientation=(0.0, 0.0, 0.0, 1.0)):
    """RigidBodyConfig::to_gpu_rigid_body (rigid_body.rs:131-146)."""
    from fluidsph.abi import GpuRigidBody
    b = GpuRigidBody()
    b.position[:] = list(position)
    b.half_extent = half_extent
    b.velocity[:] = list(velocity)
    b.is_active = 1 if active else 0
    b.stiffness = stiffness
    b.shape = int(shape)
    rows = quat_to_rotation_rows(orientation)
    b.rot_row0[:] = [float(v) for v in rows[0]]
    b.rot_row1[:] = [float(v) for v in rows[1]]
    b.rot_row2[:] = [float(v) for v in rows[2]]
    return b
