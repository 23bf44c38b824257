"""Headless runner: step one of the seeded workloads through the C ABI.

    python fluid-toy_gb300/fluidsph/run.py --config 1 --steps 12 [--graph]

Each step is one fs_step(sim, 1) call (one launch per kernel, the form that
profilers can address launch by launch) unless --graph replays them as one
captured graph. Prints the particle count, steps and wall time.
"""
from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

if __package__ in (None, ""):
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))

from fluidsph import scenes  # noqa: E402
from fluidsph.sim import SphSimulation3DGrid  # noqa: E402


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, default=0, choices=sorted(scenes.CONFIGS))
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--graph", action="store_true")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    sc = scenes.CONFIGS[a.config]()
    sim = SphSimulation3DGrid(sc.particles, sc.sph, sc.geom, device=a.device)
    sim.update_gravity(sc.gravity)
    sim.set_pcisph_iterations(sc.iterations)
    if sc.rigid is not None:
        sim.update_rigid_body(sc.rigid)
    t0 = time.perf_counter()
    if a.graph:
        sim.step(a.steps)
    else:
        for _ in range(a.steps):
            sim.step(1)
    sim.sync()
    print(f"{sc.name}: {sc.n} particles, {a.steps} steps, {time.perf_counter() - t0:.3f} s")
    sim.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
