"""Flow statistics compared between the GPU rollout and the FP64 twin.

TEST INFRASTRUCTURE ONLY: used by tests/test_gpu_statistics.py and by
bench.py's configuration-0 statistics leg, as the checker.

Rollouts of the configured dam break are chaotic, so FP32 and FP64
trajectories separate particle by particle within tens of steps; the
comparison is between statistics of the flow, averaged over a window of
samples.
"""
from __future__ import annotations

import numpy as np

NAMES = ("total_mass", "mean_density_deviation", "mean_kinetic_energy", "v2_p50", "v2_p90",
         "v2_p99")


def flow_statistics(pos, vel, rho, rho0: float, mass: float, geom) -> np.ndarray:
    """(total mass, mean density deviation, mean |v|^2/2, |v|^2 p50/p90/p99).

    total mass sums m over particles whose state is finite and inside the
    container (in its local frame: world -> R^T (p - (0, center_y, 0))); the
    density deviation is rho / rho0 - 1 of the step's (gamma-corrected)
    density."""
    pos = np.asarray(pos, np.float64)
    vel = np.asarray(vel, np.float64)
    inv = np.array([list(geom.inverse_row0)[:3], list(geom.inverse_row1)[:3],
                    list(geom.inverse_row2)[:3]], np.float64)
    local = (pos - [0.0, geom.center_y, 0.0]) @ inv.T
    half = np.array([geom.half_width, geom.half_height, geom.half_depth]) * (1 + 1e-6)
    inside = np.isfinite(pos).all(1) & np.isfinite(vel).all(1) & (np.abs(local) <= half).all(1)
    v2 = (vel ** 2).sum(1)
    return np.array([mass * inside.sum(), np.mean(np.asarray(rho, np.float64) / rho0 - 1.0),
                     0.5 * v2.mean(), *np.quantile(v2, [0.5, 0.9, 0.99])])


def gpu_sample(sim, rho0: float, mass: float, geom) -> np.ndarray:
    p = sim.particles()
    s = sim.sorted_particles()
    return flow_statistics(p[:, 0:3], p[:, 4:7], s[:, 11], rho0, mass, geom)


def fp64_sample(o64, rho0: float, mass: float, geom) -> np.ndarray:
    q = o64.particles_f64()
    t = o64.particles_f64(sorted_=True)
    return flow_statistics(q[:, 0:3], q[:, 3:6], t[:, 9], rho0, mass, geom)
