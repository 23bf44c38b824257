"""Generate the golden fixtures of the SPH step from the reference's own shaders.

The reference has no tests or golden data for this path, and its WGSL needs
wgpu and a GPU adapter, which this machine does not have. oracle/build_ref.py
translates the reference's step shaders (src/shaders/*.wgsl) mechanically to
C++ and drives them with the dispatch sequence of SphSimulation3DGrid::step();
this script runs that translation on seeded scenes and records its outputs.

Run here, where the reference tree exists:
    python tests/golden/make_golden.py
Writes tests/golden/step_fixtures.npz and tests/golden/manifest.json.

Small cases are stored in full; for the 49,600-particle cases the fixture
holds SHA-256 digests of every output buffer (floats canonicalised: -0 -> +0,
every NaN -> one quiet NaN) plus a strided sample of particles.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
for p in (ROOT / "fluid-toy_gb300", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

HERE = Path(__file__).resolve().parent
FULL_LIMIT = 1000  # particles: store arrays in full up to this
SAMPLE_STRIDE = 97


def canon(a: np.ndarray) -> np.ndarray:
    a = np.array(a, copy=True)
    if a.dtype.kind == "f":
        a[a == 0] = 0
        a[np.isnan(a)] = np.float32("nan")
    return np.ascontiguousarray(a)


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(canon(a).tobytes()).hexdigest()


def build_case(name: str):
    """Scene + settings of a fixture case (deterministic from code + seed)."""
    from fluidsph import params as P
    from fluidsph import scenes

    mouse = None
    sdf = None
    if name == "small_default":
        sc = scenes.small_scene(seed=1)
        steps = 3
    elif name == "small_rigid_sphere_vortex_tilt":
        sc = scenes.small_scene(nx=12, ny=10, nz=8, seed=2)
        sc.geom = P.container_geometry(0.6, 0.4, 0.0, 0.5, 0.15, -0.1, 250.0, 0.55)
        sc.rigid = P.rigid_body(position=(0.0, 0.1, 0.0), half_extent=0.08, active=True,
                                stiffness=250.0, shape=1, velocity=(0.05, 0.0, -0.1))
        mouse = P.mouse_force(position=(0.05, 0.12, 0.0), radius=0.2, strength=40.0, active=True,
                              mode=2, direction=(0.2, -0.1, -1.0))
        sc.iterations = 3
        steps = 2
    elif name.startswith("small_shape"):
        shape = int(name[-1])
        sc = scenes.small_scene(nx=14, ny=10, nz=10, seed=10 + shape)
        sc.rigid = P.rigid_body(position=(0.0, 0.12, 0.0), half_extent=0.1, active=True,
                                stiffness=250.0, shape=shape, velocity=(0.1, -0.2, 0.05),
                                orientation=(0.1, 0.2, 0.3, 0.927))
        if shape == 4:
            r = 16
            c = (np.arange(r) + 0.5) / r * 2 - 1
            z, y, x = np.meshgrid(c, c, c, indexing="ij")
            sdf = (np.sqrt(x * x + y * y + z * z) - 0.8).astype(np.float32)
        steps = 2
    elif name == "small_mouse_modes":
        sc = scenes.small_scene(seed=5)
        steps = 5
        mouse = "all"
    elif name == "small_outside_xsph_off":
        sc = scenes.small_scene(seed=2)
        sc.sph.xsph_epsilon = 0.0
        sc.particles[:4, 0:3] = [[2.5, 0.1, 0.0], [-3.0, 0.2, 0.1], [0.0, 4.0, 0.0],
                                 [0.1, 0.1, 2.3]]
        steps = 2
    elif name == "dam_break_49600_step1":
        sc = scenes.config0()
        steps = 1
    elif name == "dam_break_49600_step8":
        sc = scenes.config0()
        steps = 8
    else:
        raise KeyError(name)
    return sc, steps, mouse, sdf


CASES = ["small_default", "small_rigid_sphere_vortex_tilt", "small_mouse_modes", "small_shape0", "small_shape2",
         "small_shape3", "small_shape4", "small_outside_xsph_off", "dam_break_49600_step1",
         "dam_break_49600_step8"]


def run_case(name: str, make_sim):
    """Run one case with `make_sim(scene, sdf) -> sim` (oracle, reference or GPU
    wrapper with the reference's method names); return the outputs."""
    from fluidsph import params as P
    sc, steps, mouse, sdf = build_case(name)
    sim = make_sim(sc, sdf)
    if mouse is not None and mouse != "all":
        sim.update_mouse_force(mouse)
    sim.clear_rigid_body_accum()
    for k in range(steps):
        if mouse == "all":
            sim.update_mouse_force(P.mouse_force(position=(0.0, 0.1, 0.0), radius=0.3,
                                                 strength=40.0, active=True, mode=k % 5,
                                                 direction=(0.3, -0.2, -1.0)))
        sim.step(1)
    counts, starts = sim.cells()
    ci, so = sim.index_maps()
    acc = sim.read_rigid_body_accum()
    acc = acc.as_tuple() if hasattr(acc, "as_tuple") else tuple(acc)
    return {"particles": sim.particles(), "sorted": sim.sorted_particles(), "counts": counts,
            "starts": starts, "cell_indices": ci, "sorted_to_orig": so,
            "accum": np.asarray(acc, np.int64)}


def main() -> None:
    from oracle import oracle
    ref = oracle.load_ref()
    if ref is None:
        raise SystemExit("the reference translation (oracle/_ref) is not available")

    def make_ref(sc, sdf):
        return oracle.oracle_for_scene(sc, lib=ref, sdf=sdf)

    arrays = {}
    manifest = {"generator": "tests/golden/make_golden.py",
                "source": "reference WGSL step shaders translated by oracle/wgsl2cpp.py, "
                          "driven by oracle/ref_driver.cpp",
                "cases": {}}
    for name in CASES:
        out = run_case(name, make_ref)
        n = len(out["particles"])
        entry = {"n": n, "digests": {k: digest(v) for k, v in out.items()},
                 "accum": out["accum"].tolist()}
        if n <= FULL_LIMIT:
            for k, v in out.items():
                arrays[f"{name}/{k}"] = canon(v)
            entry["stored"] = "full"
        else:
            idx = np.arange(0, n, SAMPLE_STRIDE)
            arrays[f"{name}/particles_sample"] = canon(out["particles"][idx])
            arrays[f"{name}/sorted_sample"] = canon(out["sorted"][idx])
            entry["stored"] = f"digests + every {SAMPLE_STRIDE}th particle"
        manifest["cases"][name] = entry
        print(f"{name}: n={n} accum={entry['accum']}")
    np.savez_compressed(HERE / "step_fixtures.npz", **arrays)
    (HERE / "manifest.json").write_text(json.dumps(manifest, indent=1) + "\n")


if __name__ == "__main__":
    main()
