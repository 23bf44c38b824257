"""Seeded synthetic scenes for the SPH step (the workloads' inputs).

The reference seeds its lattice jitter from the wall clock
(src/simulation/particle.rs:54-55, 64-76), so its inputs are not reproducible;
these generators replace it with SplitMix64 streams.

Frame mapping: a box [0,Lx]x[0,Ly]x[0,Lz] becomes the reference container
with half extents L/2, floor_y = 0 (center_y = Ly/2), no tilt, and particles
shifted by (-Lx/2, 0, -Lz/2). A lattice block sits at the box's min corner
offset by one spacing (a dam break); every coordinate gets independent jitter
U[-0.002, 0.002].

Common parameters: h 0.08, rest density 8000 (set directly), mass 1,
near_stiffness 0.45, viscosity 15, surface_tension 6.5, wall_stiffness 250,
damping 0.55, dt 0.008, gravity (0,-9.81,0), xsph_epsilon 0.305, 4 PCISPH
iterations, stiffness 35 (read by no stage), pcisph_delta from
compute_pcisph_delta(0.08, 1, 8000, 0.008).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import params as P
from .abi import COL_POS, COL_VEL, GpuContainerGeometry, GpuGravity, GpuRigidBody, GpuSphParams3D

GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(seed: int, count: int) -> np.ndarray:
    """First `count` outputs of SplitMix64 seeded with `seed` (uint64)."""
    with np.errstate(over="ignore"):
        k = np.arange(1, count + 1, dtype=np.uint64)
        x = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + k * GOLDEN
        z = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform01(seed: int, count: int) -> np.ndarray:
    """Uniform doubles in [0, 1) from the top 53 bits of SplitMix64."""
    return (splitmix64(seed, count) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclass
class Common:
    h: float = 0.08
    rest_density: float = 8000.0
    mass: float = 1.0
    stiffness: float = 35.0
    near_stiffness: float = 0.45
    viscosity: float = 15.0
    surface_tension: float = 6.5
    wall_stiffness: float = 250.0
    damping: float = 0.55
    dt: float = 0.008
    gravity: float = -9.81
    xsph_epsilon: float = 0.305
    iterations: int = 4


@dataclass
class Scene:
    name: str
    particles: np.ndarray
    sph: GpuSphParams3D
    geom: GpuContainerGeometry
    gravity: GpuGravity
    rigid: GpuRigidBody | None
    iterations: int
    steps: int
    box: tuple
    info: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.particles)


def lattice_block(nx: int, ny: int, nz: int, box, spacing: float = 0.02, jitter: float = 0.002,
                  seed: int = 0) -> np.ndarray:
    """(N,16) SphParticle3D rows of an nx*ny*nz lattice at the box's min corner
    (offset one spacing), x fastest then z then y, in the container frame."""
    Lx, Ly, Lz = box
    iy, iz, ix = np.meshgrid(np.arange(ny), np.arange(nz), np.arange(nx), indexing="ij")
    ix, iy, iz = ix.ravel(), iy.ravel(), iz.ravel()
    n = ix.size
    u = uniform01(seed, 3 * n).reshape(n, 3)
    j = -jitter + 2.0 * jitter * u
    pos = np.empty((n, 3), np.float64)
    pos[:, 0] = (ix + 1) * spacing - Lx / 2.0 + j[:, 0]
    pos[:, 1] = (iy + 1) * spacing + j[:, 1]
    pos[:, 2] = (iz + 1) * spacing - Lz / 2.0 + j[:, 2]
    out = np.zeros((n, 16), np.float32)
    out[:, COL_POS] = pos.astype(np.float32)
    return out


def make_scene(name: str, particles: np.ndarray, box, c: Common | None = None, steps: int = 1,
               rigid: GpuRigidBody | None = None, tilt_x: float = 0.0, tilt_z: float = 0.0,
               info: dict | None = None, builders=None) -> Scene:
    """A scene over `particles`. `builders` supplies sph_params_3d,
    container_geometry and gravity with the signatures of fluidsph.params
    (the default, which evaluates them in this library); any module that
    restates the reference's builders bit for bit gives the same scene."""
    B = builders or P
    c = c or Common()
    Lx, Ly, Lz = box
    sph = B.sph_params_3d(c.h, c.mass, c.rest_density, c.stiffness, c.near_stiffness,
                          c.viscosity, c.surface_tension, c.xsph_epsilon, c.dt, len(particles))
    geom = B.container_geometry(Lx, Lz, 0.0, Ly, tilt_x, tilt_z, c.wall_stiffness, c.damping)
    return Scene(name, particles, sph, geom, B.gravity(c.gravity), rigid, c.iterations, steps,
                 tuple(box), info or {})


def config0(seed: int = 0, builders=None) -> Scene:
    """Plain dam break: 40x40x31 = 49,600 particles in a 1.6x1.2x0.8 box, 1000 steps."""
    box = (1.6, 1.2, 0.8)
    return make_scene("dam_break_49600", lattice_block(40, 40, 31, box, seed=seed), box, steps=1000,
                      builders=builders)


def config1(seed: int = 0, builders=None) -> Scene:
    """Plain at scale: 128x64x128 = 1,048,576 particles in a 4x2x3 box with a held
    sphere (radius 0.3, box centre (3.0,0.4,1.5) -> container (1.0,0.4,0.0)), 500 steps."""
    B = builders or P
    box = (4.0, 2.0, 3.0)
    c = Common()
    rb = B.rigid_body(position=(3.0 - box[0] / 2, 0.4, 1.5 - box[2] / 2), half_extent=0.3,
                      active=True, stiffness=c.wall_stiffness, shape=1)
    return make_scene("dam_break_1048576_sphere", lattice_block(128, 64, 128, box, seed=seed),
                      box, c, steps=500, rigid=rb, builders=builders)


def small_scene(nx: int = 10, ny: int = 8, nz: int = 6, box=(0.6, 0.5, 0.4), seed: int = 1,
                c: Common | None = None, **kw) -> Scene:
    """A few hundred particles for quick parity checks."""
    return make_scene(f"small_{nx}x{ny}x{nz}", lattice_block(nx, ny, nz, box, seed=seed), box,
                      c, **kw)


def fourier_velocity(pos: np.ndarray, seed: int, modes: int = 8, amplitude: float = 0.5,
                     box=(1.2, 1.0, 1.0)) -> np.ndarray:
    """Smooth random velocity field: sum of `modes` Fourier modes with random
    wave vectors (integer multiples of 2*pi/L), directions and phases, scaled
    so the largest speed is `amplitude`."""
    u = uniform01(seed, modes * 7).reshape(modes, 7)
    k = np.floor(1 + 3 * u[:, 0:3]) * (2 * np.pi / np.asarray(box))
    d = u[:, 3:6] - 0.5
    d /= np.linalg.norm(d, axis=1, keepdims=True) + 1e-12
    phase = 2 * np.pi * u[:, 6]
    v = np.zeros_like(pos, dtype=np.float64)
    for m in range(modes):
        v += np.sin(pos @ k[m] + phase[m])[:, None] * d[m][None, :]
    v *= amplitude / max(np.abs(v).max(), 1e-12)
    return v


def rollout_scene(nx: int, ny: int, nz: int, box, seed: int = 0, steps: int = 200,
                  name: str | None = None) -> Scene:
    """A lattice block with a smooth random initial velocity (8 Fourier
    modes, largest speed 0.5 m/s): the differentiable-rollout workload."""
    parts = lattice_block(nx, ny, nz, box, seed=seed)
    v = fourier_velocity(parts[:, COL_POS].astype(np.float64), seed + 1000, box=box)
    parts[:, COL_VEL] = v.astype(np.float32)
    return make_scene(name or f"rollout_{nx * ny * nz}", parts, box, steps=steps)


def config3(seed: int = 0) -> Scene:
    """Differentiable rollout: 32^3 = 32,768 particles in a 1.2x1x1 box with a
    smooth random initial velocity (8 Fourier modes, 0.5 m/s), 200 steps."""
    return rollout_scene(32, 32, 32, (1.2, 1.0, 1.0), seed, 200, "rollout_32768")


def config3_small(seed: int = 0) -> Scene:
    """The checking copy of the rollout: 2,048 particles (16x8x16), 20 steps."""
    return rollout_scene(16, 8, 16, (0.6, 0.5, 0.6), seed, 20, "rollout_2048")


def reference_physics_rollout(nx: int = 16, ny: int = 8, nz: int = 16, steps: int = 20,
                              seed: int = 0) -> Scene:
    """The rollout with the reference application's own default physics
    (SphConfig::default, src/state/simulation.rs:287-299: h 0.035, near
    stiffness 0.7, viscosity 0.7, surface tension 0.005, mass 1, wall
    stiffness 200; rest density from compute_rest_density; dt = 1/60/6 with
    the default 6 substeps) on a lattice at the spacing that rest density
    assumes (0.6 h), with the same smooth random initial velocity. Unlike the
    h = 0.08 / spacing 0.02 / surface tension 6.5 workloads, which start far
    from equilibrium and blow up within a few steps, this rollout stays smooth,
    so finite differences of its loss converge."""
    h = 0.035
    sp = 0.6 * h
    box = (0.5, 0.4, 0.5)
    parts = lattice_block(nx, ny, nz, box, spacing=sp, jitter=0.0005, seed=seed)
    v = fourier_velocity(parts[:, COL_POS].astype(np.float64), seed + 1000, box=box)
    parts[:, COL_VEL] = v.astype(np.float32)
    dt = 1.0 / 60.0 / 6.0
    rho0 = P.compute_rest_density(h, 1.0)
    sph = P.sph_params_3d(h, 1.0, rho0, 35.0, 0.7, 0.7, 0.005, 0.305, dt, len(parts))
    geom = P.container_geometry(box[0], box[2], 0.0, box[1], 0.0, 0.0, 200.0, 0.55)
    return Scene(f"reference_physics_rollout_{len(parts)}", parts, sph, geom, P.gravity(-9.81),
                 None, 4, steps, box)


def config4(seed: int = 0, num_scenes: int = 64, lo: int = 8192, hi: int = 32768,
            steps: int = 150) -> tuple[list, list]:
    """Batched parameter identification: `num_scenes` scenes set up as the
    batched ensemble (batch_scene) with counts log-uniform in [lo, hi], and per
    scene a hidden target: viscosity U[5, 25] and stiffness U[20, 50] (the
    surface tension keeps the scene's own value). The step reads no
    `stiffness` (src/state/simulation.rs:326 sets it; pressure strength is
    pcisph_delta, pcisph_solve.wgsl:178-179), so the hidden stiffness is
    carried into the live pressure parameter: the hidden pcisph_delta is the
    scene's delta times stiffness / 35 (35 = the configured stiffness).
    Returns (scenes, hidden)."""
    scs = [batch_scene(k, seed + 4_000, lo, hi, steps) for k in range(num_scenes)]
    hidden = []
    for k in range(num_scenes):
        u = uniform01(seed * 1_000_003 + 104_729 * (k + 1), 2)
        stiff = float(20.0 + 30.0 * u[1])
        hidden.append({"viscosity": float(5.0 + 20.0 * u[0]), "stiffness": stiff,
                       "pcisph_delta": float(np.float32(scs[k].sph.pcisph_delta * stiff / 35.0)),
                       "surface_tension": float(scs[k].sph.surface_tension)})
    return scs, hidden


def reference_physics_batch(num_scenes: int = 64, steps: int = 20, seed: int = 0) -> tuple:
    """Well-posed identification companion of config4: small rollouts with the
    reference app's default physics (reference_physics_rollout), lattices of
    8-12 x 6-8 x 8-12, each with a hidden viscosity U[0.35, 1.4] (the default
    is 0.7). Returns (scenes, hidden)."""
    scs, hidden = [], []
    for k in range(num_scenes):
        u = uniform01(seed * 1_000_003 + 31 * (k + 1), 4)
        nx, ny, nz = 8 + int(5 * u[0]), 6 + int(3 * u[1]), 8 + int(5 * u[2])
        sc = reference_physics_rollout(nx, ny, nz, steps, seed + k)
        scs.append(sc)
        hidden.append({"viscosity": float(0.35 + 1.05 * u[3]), "stiffness": float(sc.sph.stiffness),
                       "pcisph_delta": float(sc.sph.pcisph_delta),
                       "surface_tension": float(sc.sph.surface_tension)})
    return scs, hidden


def loss_grid(scene: Scene, grid_size: int = 64):
    """The MC grid of the rollout loss: grid_size^3 voxels over the scene's
    box (cell = largest extent / grid_size), splat radius h."""
    from . import params as Pm
    Lx, Ly, Lz = scene.box
    return Pm.mc_grid_params((-Lx / 2, 0.0, -Lz / 2), (Lx / 2, Ly, Lz / 2), grid_size,
                             scene.sph.kernel_radius)


def _to_container(parts: np.ndarray, geom: GpuContainerGeometry) -> np.ndarray:
    """Map positions given in the untilted container frame through the
    container's rotation about its centre (the local_to_world transform of
    container_common.wgsl), so a block at the local min corner stays inside a
    tilted box."""
    rows = np.array([list(geom.forward_row0)[:3], list(geom.forward_row1)[:3],
                     list(geom.forward_row2)[:3]], np.float64)
    local = parts[:, COL_POS].astype(np.float64)
    local[:, 1] -= geom.center_y
    world = local @ rows.T
    world[:, 1] += geom.center_y
    out = parts.copy()
    out[:, COL_POS] = world.astype(np.float32)
    return out


def batch_scene(k: int, seed: int = 0, lo: int = 2048, hi: int = 65536,
                steps: int = 200) -> Scene:
    """Scene k of the batched ensemble.

    count log-uniform in [lo, hi]; fill f ~ U[0.3, 0.6]; side lengths
    U[0.8, 2.0] rescaled so that count * 0.02^3 / V = f, redrawn (up to 32
    times) while a side leaves [0.8, 2.0], else clamped into it (small counts
    cannot reach the fill inside a 0.8 box: their effective fill is lower and
    is recorded in ``info``); viscosity U[5, 25], stiffness U[20, 50],
    surface_tension U[3, 10], tilt_x and tilt_z U[-15, 15] degrees. The block
    is a dam-break lattice at the box's min corner whose footprint covers
    f^(1/3) of the floor along x and z, filled x, z, then y up to `count`
    particles, then rotated with the container."""
    u = uniform01(seed * 1_000_003 + 7919 * (k + 1), 128)
    count = int(round(np.exp(np.log(lo) + u[0] * (np.log(hi) - np.log(lo)))))
    count = min(max(count, lo), hi)
    fill = 0.3 + 0.3 * u[1]
    target_v = count * 0.02 ** 3 / fill
    sides = None
    for a in range(32):
        L = 0.8 + 1.2 * u[2 + 3 * a: 5 + 3 * a]
        L = L * (target_v / np.prod(L)) ** (1.0 / 3.0)
        if np.all((L >= 0.8) & (L <= 2.0)):
            sides = L
            break
    clamped = sides is None
    if clamped:
        sides = np.clip(L, 0.8, 2.0)
    Lx, Ly, Lz = (float(np.float32(v)) for v in sides)
    eff_fill = count * 0.02 ** 3 / (Lx * Ly * Lz)
    g = min(eff_fill, 1.0) ** (1.0 / 3.0)
    max_x, max_z = int(Lx / 0.02) - 2, int(Lz / 0.02) - 2
    nx = min(max(int(g * Lx / 0.02), 1), max_x)
    nz = min(max(int(g * Lz / 0.02), 1), max_z)
    ny = -(-count // (nx * nz))
    if (ny + 1) * 0.02 > Ly - 0.02:
        nx, nz = max_x, max_z
        ny = -(-count // (nx * nz))
    c = Common(viscosity=float(5.0 + 20.0 * u[100]), stiffness=float(20.0 + 30.0 * u[101]),
               surface_tension=float(3.0 + 7.0 * u[102]))
    tilt_x = float(np.radians(-15.0 + 30.0 * u[103]))
    tilt_z = float(np.radians(-15.0 + 30.0 * u[104]))
    box = (Lx, Ly, Lz)
    parts = lattice_block(nx, ny, nz, box, seed=seed * 1_000_003 + 7919 * (k + 1) + 1)[:count]
    sc = make_scene(f"batch{k}_{count}", parts, box, c, steps=steps, tilt_x=tilt_x,
                    tilt_z=tilt_z, info={"fill": fill, "effective_fill": eff_fill,
                                         "clamped": clamped, "block": (nx, ny, nz)})
    sc.particles = _to_container(parts, sc.geom)
    return sc


def config2(seed: int = 0, num_scenes: int = 256, lo: int = 2048, hi: int = 65536,
            steps: int = 200) -> list:
    """Batched ensemble: `num_scenes` independent scenes (batch_scene)."""
    return [batch_scene(k, seed, lo, hi, steps) for k in range(num_scenes)]


CONFIGS = {0: config0, 1: config1, 3: config3}
