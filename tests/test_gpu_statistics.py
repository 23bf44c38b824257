"""Multi-step statistics of the GPU rollout against the FP64 twin.

Rollouts of this workload are chaotic (the lattice starts at ~15x rest
density and settles at ~190x with speeds of ~100 m/s), so single trajectories
of the FP32 pipeline and of the FP64 twin separate within tens of steps, and
a per-particle comparison means nothing after that. What must agree are the
statistics of the flow. The band, for the 49,600-particle dam break
(configuration 0) over 200 steps:

* total mass (sum of m over particles with a finite state inside the
  container): equal;
* mean density deviation (rho / rho0 - 1), mean kinetic energy per unit mass
  (|v|^2 / 2) and the 50th / 90th / 99th percentiles of |v|^2, each averaged
  over the samples every 5 steps from step 105 to step 200: within
  STATS_BAND relative of the FP64 twin's.

The band is set from measurement: over steps 101-200 the FP32 pipeline (which
the GPU follows bit for bit) is within 0.63% of FP64 on every statistic,
and two FP64 runs whose initial positions differ by 1e-7 relative are
within 0.51% of each other (the chaotic spread itself)."""
import numpy as np
import pytest

from helpers import gpu_sim_for_scene

pytestmark = pytest.mark.gpu

STATS_BAND = 0.02
STEPS, FIRST, EVERY = 200, 105, 5


def test_config0_statistics_within_band_of_fp64(fslib, oracle_mod, capsys):
    from fluidsph import scenes
    from oracle.flow_stats import NAMES, fp64_sample, gpu_sample
    sc = scenes.config0()
    rho0, mass = float(sc.sph.rest_density), float(sc.sph.mass)
    sim = gpu_sim_for_scene(sc)
    o64 = oracle_mod.oracle_for_scene(sc, precision=64)
    g_samples, o_samples = [], []
    for k in range(1, STEPS + 1):
        sim.step(1)
        o64.step(1)
        if k >= FIRST and k % EVERY == 0:
            g_samples.append(gpu_sample(sim, rho0, mass, sc.geom))
            o_samples.append(fp64_sample(o64, rho0, mass, sc.geom))
    g = np.mean(g_samples, axis=0)
    o = np.mean(o_samples, axis=0)
    rel = np.abs(g - o) / np.abs(o)
    with capsys.disabled():
        print(f"\nconfig 0 statistics, steps {FIRST}-{STEPS} every {EVERY} (GPU FP32 | FP64 twin | "
              "relative difference):")
        for n, a, b, r in zip(NAMES, g, o, rel):
            print(f"  {n}: {a:.6g} | {b:.6g} | {r:.2e}")
    assert g[0] == o[0] == mass * sc.n  # every particle stays, finite, in the box
    assert (rel[1:] <= STATS_BAND).all(), dict(zip(NAMES, rel))
    sim.close()
