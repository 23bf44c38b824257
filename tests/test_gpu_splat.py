"""GPU parity of the marching-cubes density pass (fs_density_splat,
mc_density.wgsl:130-231, isotropic path) against the FP32 oracle: bit-exact
fields on the same sorted state, for the reference's grid bounds, a wider
splat radius, clipping against a tilted box and grids reaching past the SPH
grid; host and device outputs; a batch scene against its plain simulation."""
import numpy as np
import pytest

from helpers import assert_same_floats, gpu_sim_for_scene

pytestmark = pytest.mark.gpu


def _cases(sc):
    from fluidsph import params as P
    Lx, Ly, Lz = sc.box
    m = 0.08 + 0.05  # kernel radius x scale + 0.05 (app.rs:1480)
    lo = (-Lx / 2 - m, -m, -Lz / 2 - m)
    hi = (Lx / 2 + m, Ly + m, Lz / 2 + m)
    clip = P.container_geometry(Lx, Lz, 0.0, Ly, 0.03, -0.04, 250.0, 0.55, clip_enabled=True,
                                clip_margin=0.02)
    return [(P.mc_grid_params(lo, hi, 32, 0.08), sc.geom),
            (P.mc_grid_params(lo, hi, 27, 0.08 * 1.7), clip),
            (P.mc_grid_params((-2.5, -2.5, -2.5), (2.5, 2.5, 2.5), 40, 0.08), clip)]


@pytest.fixture(scope="module")
def scenes_mod():
    from fluidsph import scenes
    return scenes


def test_splat_matches_oracle_small(scenes_mod, oracle_mod):
    sc = scenes_mod.small_scene(nx=12, ny=9, nz=8, seed=4)
    sim = gpu_sim_for_scene(sc)
    orc = oracle_mod.oracle_for_scene(sc)
    sim.step(3)
    orc.step(3)
    for mc, geom in _cases(sc):
        g = sim.density_splat(mc, geom)
        o = orc.density_splat(mc, geom).astype(np.float32)
        assert_same_floats(g, o, f"splat gs={mc.grid_size} h={mc.kernel_radius}")
        assert (g > 0).any()


def test_splat_dam_break_49600(scenes_mod, oracle_mod):
    from fluidsph import params as P
    sc = scenes_mod.config0()
    sim = gpu_sim_for_scene(sc)
    orc = oracle_mod.oracle_for_scene(sc)
    sim.step(3)
    orc.step(3)
    Lx, Ly, Lz = sc.box
    mc = P.mc_grid_params((-Lx / 2 - 0.13, -0.13, -Lz / 2 - 0.13),
                          (Lx / 2 + 0.13, Ly + 0.13, Lz / 2 + 0.13), 64, 0.08)
    g = sim.density_splat(mc, sc.geom)
    o = orc.density_splat(mc, sc.geom).astype(np.float32)
    assert_same_floats(g, o, "splat config 0")
    assert (g > 0).sum() > 10000


def test_splat_device_output_and_batch(scenes_mod):
    import torch
    from fluidsph.sim import SphBatch3DGrid
    scs = scenes_mod.config2(seed=2, num_scenes=3, lo=500, hi=3000, steps=2)
    b = SphBatch3DGrid([s.particles for s in scs], [s.sph for s in scs], [s.geom for s in scs])
    sims = [gpu_sim_for_scene(s) for s in scs]
    for k, s in enumerate(scs):
        b.update_scene(k, gravity=s.gravity)
    b.set_pcisph_iterations(scs[0].iterations)
    b.step(2)
    for sim in sims:
        sim.step(2)
    for k, s in enumerate(scs):
        for mc, geom in _cases(s)[:2]:
            ref = sims[k].density_splat(mc, geom)
            gs = mc.grid_size
            dev = torch.full((gs, gs, gs), 7.0, dtype=torch.float32, device="cuda")
            b.density_splat(mc, geom, scene=k, out_device_ptr=dev.data_ptr())
            b.sync()
            assert_same_floats(dev.cpu().numpy(), ref, f"scene {k} device splat")
            assert_same_floats(b.density_splat(mc, geom, scene=k), ref, f"scene {k} host splat")
