"""Whitewater (spray, foam, bubbles) over a simulation scene: the Python
mirror of the reference's SpraySystem (src/simulation/spray.rs) over
fs_spray_*. ``spray_params`` builds GpuSprayParams the way the reference app
does (app.rs:1048-1079) from SprayConfig::default (interaction.rs:67-89)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import SPRAY_DTYPE, GpuSprayParams, check


def spray_params(num_sph_particles: int, frame_dt: float, frame_count: int = 0,
                 gravity: float = 9.81, max_particles: int = 100_000, **overrides):
    """GpuSprayParams with SprayConfig's defaults; frame_dt = substep dt x substeps."""
    p = GpuSprayParams()
    p.min_speed, p.emission_rate, p.lifetime, p.lifetime_variation = 0.8, 30.0, 2.8, 0.5
    p.drag, p.speed_multiplier, p.velocity_jitter = 1.5, 0.85, 0.9
    p.dt = frame_dt
    p.max_particles = max_particles
    p.num_sph_particles = num_sph_particles
    p.frame_count = frame_count
    p.gravity_y = -gravity
    p.k_trapped_air, p.k_wave_crest = 1.25, 1.4
    p.ta_limit, p.wc_limit = 3.0, 1.0
    p.bubble_buoyancy, p.bubble_drag = 2.5, 0.6
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


class SpraySystem:
    def __init__(self, sim, max_particles: int = 100_000, scene: int = 0):
        self._lib = abi.load()
        self.max_particles = int(max_particles)
        h = C.c_void_p()
        check(self._lib.fs_spray_create(sim._h, int(scene), self.max_particles, C.byref(h)))
        self._h = h
        self.sim = sim
        sim._register(self)

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.fs_spray_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, params) -> None:
        check(self._lib.fs_spray_step(self._h, C.byref(params)))

    def reset(self) -> None:
        check(self._lib.fs_spray_reset(self._h))

    def read_stats(self) -> np.ndarray:
        out = (C.c_uint32 * 4)()
        check(self._lib.fs_spray_stats(self._h, out))
        return np.array(out, np.uint32)

    def auto_limits(self) -> tuple[tuple[float, float], int]:
        lim = (C.c_float * 2)()
        head = C.c_uint32()
        check(self._lib.fs_spray_limits(self._h, lim, C.byref(head)))
        return (lim[0], lim[1]), head.value

    def particles(self) -> np.ndarray:
        out = np.zeros(self.max_particles, SPRAY_DTYPE)
        check(self._lib.fs_spray_download(self._h, out.ctypes.data, self.max_particles))
        return out
