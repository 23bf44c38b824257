"""Headless runner: step one of the seeded workloads through the C ABI.

    python fluid-toy_gb300/fluidsph/run.py --config 1 --steps 12 [--graph] [--warmup 20]
    python fluid-toy_gb300/fluidsph/run.py --batch --steps 10 --warmup 20
    python fluid-toy_gb300/fluidsph/run.py --identify --iterations 2

Each step is one fs_step(sim, 1) call (one launch per kernel, the form that
profilers can address launch by launch) unless --graph replays them as one
captured graph. Prints the particle count, steps and wall time. --warmup
steps run first (a simulation measures its neighbour passes' load depths on
its steps 8-17 and keeps the fastest from then on, unless its particle-count
bucket is already in the process-wide table); the measured steps run
inside the NVTX range `steps` (when torch is importable).

--lattice NX NY NZ replaces the configuration's lattice (same box, spacing and
parameters: e.g. 64 64 64 = 262,144 particles, a case small enough for
full-set profiles of the dam break); --forms D X S fixes the neighbour passes'
load depths (density, XSPH, solve; fs_set_kernel_forms) instead of tuning them.

--batch runs the 256-scene ensemble of scenes.config2 as one SphBatch3DGrid
(one launch per stage for all scenes) instead of a single scene.

--identify runs the batched parameter-identification workload instead (the
64 scenes of scenes.config4 as one batch, 150 steps, checkpoint every 15;
--scenes / --rollout-steps / --every shrink it for profiling):
per iteration a DifferentiableRollout forward, an MSE splat loss per scene
against zero targets and the backward, inside NVTX ranges named fwd<i> and
bwd<i> (when torch is importable) so a profiler can select one phase.
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


class _Ranges:
    """NVTX push/pop through torch when available, else no-ops."""

    def __init__(self):
        try:
            import torch
            self._nvtx = torch.cuda.nvtx
        except Exception:  # torch absent: no ranges
            self._nvtx = None

    def push(self, name: str) -> None:
        if self._nvtx is not None:
            self._nvtx.range_push(name)

    def pop(self) -> None:
        if self._nvtx is not None:
            self._nvtx.range_pop()


def identify(iterations: int, steps: int = 150, every: int = 15, num_scenes: int = 64,
             device: int = 0, forms=None) -> None:
    import numpy as np

    from fluidsph.adjoint import DifferentiableRollout
    from fluidsph.sim import SphBatch3DGrid

    scs, _ = scenes.config4(num_scenes=num_scenes, steps=steps)
    b = SphBatch3DGrid([s.particles for s in scs], [s.sph for s in scs], [s.geom for s in scs],
                       device=device)
    for k, s in enumerate(scs):
        b.update_scene(k, gravity=s.gravity)
    b.set_pcisph_iterations(scs[0].iterations)
    if forms is not None:
        # fixed depths (density, XSPH, solve), e.g. under a profiler, whose
        # serialised launches would skew the measurement
        b.set_kernel_forms(forms[0], forms[2], forms[1])
    else:
        # past the neighbour passes' load-depth measurement first, as the
        # bench does (its plain forward of the batch); the rollout starts from
        # the initial state again
        b.step(20)
        b.sync()
    f = b.kernel_forms()
    print(f"load depths: density {f['density_loads']}, xsph {f['xsph_loads']}, solve "
          f"{f['solve_loads']} ({f['decided']})", flush=True)
    grids = [scenes.loss_grid(s, 64) for s in scs]
    r = DifferentiableRollout(b, every)
    nv = _Ranges()
    targets = None
    for it in range(iterations):
        for k, s in enumerate(scs):
            b.upload_scene_particles(k, s.particles)
        b.sync()
        t0 = time.perf_counter()
        nv.push(f"fwd{it}")
        r.forward(steps)
        b.sync()
        nv.pop()
        t1 = time.perf_counter()
        if targets is None:
            targets = [np.zeros_like(r.final_splat(grids[k], scs[k].geom, scene=k))
                       for k in range(len(scs))]
        r.splat_mse_losses(grids, [s.geom for s in scs], targets)
        t2 = time.perf_counter()
        nv.push(f"bwd{it}")
        r.backward(scenes=len(scs))
        b.sync()
        nv.pop()
        t3 = time.perf_counter()
        print(f"identification iteration {it}: {sum(s.n for s in scs)} particles, forward "
              f"{1e3 * (t1 - t0) / steps:.3f} ms/step, loss {1e3 * (t2 - t1):.1f} ms, backward "
              f"{1e3 * (t3 - t2) / steps:.3f} ms/step", flush=True)
    r.close()
    b.close()


def run_steps(sim, steps: int, warmup: int, graph: bool) -> float:
    """Warm-up steps, then `steps` steps inside the NVTX range `steps`; returns
    the wall seconds of the measured steps."""
    if warmup:
        sim.step(warmup)
    sim.sync()
    nv = _Ranges()
    t0 = time.perf_counter()
    nv.push("steps")
    if graph:
        sim.step(steps)
    else:
        for _ in range(steps):
            sim.step(1)
    sim.sync()
    nv.pop()
    return time.perf_counter() - t0


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, default=0, choices=sorted(scenes.CONFIGS))
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--graph", action="store_true")
    ap.add_argument("--warmup", type=int, default=0)
    ap.add_argument("--batch", action="store_true", help="the 256-scene batched ensemble")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--identify", action="store_true")
    ap.add_argument("--iterations", type=int, default=2)
    ap.add_argument("--lattice", type=int, nargs=3, default=None,
                    help="NX NY NZ lattice in the configuration's box")
    ap.add_argument("--forms", type=int, nargs=3, default=None,
                    help="fixed load depths: density xsph solve")
    ap.add_argument("--scenes", type=int, default=64, help="--identify: scenes (the first n)")
    ap.add_argument("--rollout-steps", type=int, default=150, help="--identify: steps")
    ap.add_argument("--every", type=int, default=15, help="--identify: checkpoint interval")
    a = ap.parse_args(argv)
    if a.identify:
        identify(a.iterations, a.rollout_steps, a.every, a.scenes, device=a.device, forms=a.forms)
        return 0
    if a.batch:
        from fluidsph.sim import SphBatch3DGrid

        scs = scenes.config2()
        b = SphBatch3DGrid([s.particles for s in scs], [s.sph for s in scs],
                           [s.geom for s in scs], device=a.device)
        for k, s in enumerate(scs):
            b.update_scene(k, gravity=s.gravity)
        b.set_pcisph_iterations(scs[0].iterations)
        secs = run_steps(b, a.steps, a.warmup, a.graph)
        print(f"batched ensemble: {len(scs)} scenes, {sum(s.n for s in scs)} particles, "
              f"{a.steps} steps, {secs:.3f} s")
        b.close()
        return 0
    sc = scenes.CONFIGS[a.config]()
    if a.lattice:
        nx, ny, nz = a.lattice
        sc.particles = scenes.lattice_block(nx, ny, nz, sc.box)
        sc.sph.num_particles = len(sc.particles)
        sc.name = f"{sc.name}_lattice_{nx}x{ny}x{nz}"
    sim = SphSimulation3DGrid(sc.particles, sc.sph, sc.geom, device=a.device)
    sim.update_gravity(sc.gravity)
    sim.set_pcisph_iterations(sc.iterations)
    if sc.rigid is not None:
        sim.update_rigid_body(sc.rigid)
    if a.forms:
        sim.set_kernel_forms(a.forms[0], a.forms[2], a.forms[1])
    secs = run_steps(sim, a.steps, a.warmup, a.graph)
    print(f"{sc.name}: {sc.n} particles, {a.steps} steps, {secs:.3f} s")
    sim.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
