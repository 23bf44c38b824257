"""GPU parity of the batched form (fs_batch_*): every scene of a batch against
a plain simulation built from the same inputs, bit for bit in every buffer
(cell counts and starts, index maps, sorted records, canonical state, rigid
body accumulators), and against the FP32 oracle for a few scenes. The full
256-scene ensemble is checked through the same per-scene equality on a
sample of scenes."""
import numpy as np
import pytest

from helpers import assert_same_floats, check_grid_invariants, gpu_sim_for_scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sc():
    from fluidsph import scenes
    return scenes


def _batch_for(scenes, sdf=None, mouse=None):
    from fluidsph.sim import SphBatch3DGrid
    b = SphBatch3DGrid([s.particles for s in scenes], [s.sph for s in scenes],
                       [s.geom for s in scenes], sdf=sdf)
    for k, s in enumerate(scenes):
        b.update_scene(k, gravity=s.gravity, rigid_body=s.rigid,
                       mouse=None if mouse is None else mouse.get(k))
    b.set_pcisph_iterations(scenes[0].iterations)
    b.clear_rigid_body_accum()
    return b


def _plain_for(scene, sdf=None, mouse=None):
    sim = gpu_sim_for_scene(scene, sdf=sdf)
    if mouse is not None:
        sim.update_mouse_force(mouse)
    sim.clear_rigid_body_accum()
    return sim


def _compare_scene(b, k, sim, what):
    counts_b, starts_b = b.scene_cells(k)
    counts_p, starts_p = sim.cells()
    np.testing.assert_array_equal(counts_b, counts_p, err_msg=f"{what} cell_counts")
    np.testing.assert_array_equal(starts_b, starts_p, err_msg=f"{what} cell_starts")
    n_act = b.scene_info(k).active_particles
    ci_b, so_b = b.scene_index_maps(k)
    ci_p, so_p = sim.index_maps()
    np.testing.assert_array_equal(ci_b, ci_p[:n_act], err_msg=f"{what} particle_cell_indices")
    np.testing.assert_array_equal(so_b, so_p[:n_act], err_msg=f"{what} sorted_to_orig")
    check_grid_invariants(counts_b, starts_b, ci_b, so_b, n_act)
    sb, sp = b.scene_sorted_particles(k), sim.sorted_particles(n_act)
    assert_same_floats(sb, sp, f"{what} sorted records")
    pb, pp = b.scene_particles(k), sim.particles()
    assert_same_floats(pb, pp, f"{what} canonical records")


def _mixed(sc, num=6, seed=3):
    """Small scenes of uneven sizes with different parameters and tilts, a
    rigid body of each analytic shape, tilted gravity on one scene and mouse
    forces on two."""
    from fluidsph import params as P
    scenes = sc.config2(seed=seed, num_scenes=num, lo=300, hi=4000, steps=4)
    for k, s in enumerate(scenes):
        if k % 2 == 0:
            s.rigid = P.rigid_body(position=(0.05, 0.15, -0.05), half_extent=0.12,
                                   active=True, stiffness=250.0, shape=(k // 2) % 4)
    scenes[1].gravity = P.gravity(-9.0, gx=2.0, gz=-1.0)
    mouse = {2: P.mouse_force(position=(0.0, 0.1, 0.0), radius=0.3, strength=40.0,
                              active=True, mode=1),
             3: P.mouse_force(position=(-0.1, 0.2, 0.1), radius=0.4, strength=30.0,
                              active=True, mode=2, direction=(0.0, 1.0, 0.0))}
    return scenes, mouse


def test_batch_matches_plain_scenes(sc):
    scenes, mouse = _mixed(sc)
    b = _batch_for(scenes, mouse=mouse)
    sims = [_plain_for(s, mouse=mouse.get(k)) for k, s in enumerate(scenes)]
    assert b.num_scenes() == len(scenes)
    assert b.num_particles() == sum(s.n for s in scenes)
    for step_call in (1, 1, 3):  # single steps, then a graph-replayed run
        b.step(step_call)
        for sim in sims:
            sim.step(step_call)
        for k, sim in enumerate(sims):
            _compare_scene(b, k, sim, f"scene {k} after +{step_call}")
    acc_b = b.read_rigid_body_accums()
    for k, sim in enumerate(sims):
        assert acc_b[k].as_tuple() == sim.read_rigid_body_accum().as_tuple(), f"scene {k} accum"
    assert any(a.contact_count for a in acc_b), "no scene touched its rigid body"


def test_batch_scene_info_layout(sc):
    scenes, _ = _mixed(sc, num=5, seed=11)
    b = _batch_for(scenes)
    p = c = s_off = 0
    for k, s in enumerate(scenes):
        info = b.scene_info(k)
        assert (info.particle_offset, info.num_particles) == (p, s.n)
        assert (info.active_particles, info.sorted_offset, info.cell_offset) == (s.n, s_off, c)
        assert info.grid.total_cells == info.total_cells
        p += s.n
        s_off += s.n
        c += info.total_cells


def test_batch_partial_active_counts(sc):
    """num_particles below a scene's count leaves its tail untouched and moves
    the later scenes' slots; results still equal the plain simulations."""
    scenes, _ = _mixed(sc, num=4, seed=5)
    b = _batch_for(scenes)
    sims = [_plain_for(s) for s in scenes]
    import copy
    p1 = copy.copy(scenes[1].sph)
    p1.num_particles = scenes[1].n - 37
    b.update_scene(1, sph_params=p1)
    sims[1].update_sph_params(p1)
    assert b.scene_info(1).active_particles == scenes[1].n - 37
    assert b.scene_info(2).sorted_offset == scenes[0].n + scenes[1].n - 37
    b.step(2)
    for sim in sims:
        sim.step(2)
    for k, sim in enumerate(sims):
        _compare_scene(b, k, sim, f"scene {k}")
    # the inactive tail of scene 1 is exactly its input
    tail = b.scene_particles(1)[-37:]
    assert_same_floats(tail, scenes[1].particles[-37:], "inactive tail")


def test_batch_against_oracle(sc, oracle_mod):
    scenes, mouse = _mixed(sc, num=3, seed=8)
    b = _batch_for(scenes, mouse=mouse)
    b.step(2)
    for k, s in enumerate(scenes):
        orc = oracle_mod.OracleSim(s.particles, s.sph, s.geom)
        orc.update_gravity(s.gravity)
        orc.set_pcisph_iterations(s.iterations)
        if s.rigid is not None:
            orc.update_rigid_body(s.rigid)
        if k in mouse:
            orc.update_mouse_force(mouse[k])
        orc.step(1)
        orc.step(1)
        assert_same_floats(b.scene_particles(k), orc.particles(), f"scene {k} vs oracle")
        counts_b, starts_b = b.scene_cells(k)
        counts_o, starts_o = orc.cells()
        np.testing.assert_array_equal(counts_b, counts_o)
        np.testing.assert_array_equal(starts_b, starts_o)


def test_batch_rejects_plain_per_scene_calls(sc):
    from fluidsph import params as P
    from fluidsph.abi import FluidSphError
    scenes, _ = _mixed(sc, num=2, seed=9)
    b = _batch_for(scenes)
    with pytest.raises(FluidSphError) as e:
        b.update_gravity(P.gravity(-9.81))
    assert e.value.code == -7
    with pytest.raises(FluidSphError):
        b.spawn_particles((0.0, 0.5, 0.0), 10, 0.05)
    with pytest.raises(FluidSphError) as e:
        b.scene_particles(2)
    assert e.value.code == -1


def test_full_ensemble_sampled_scenes(sc):
    """The 256-scene ensemble: scenes sampled across the count range evolve
    exactly like their plain simulations."""
    scenes = sc.config2(steps=3)
    b = _batch_for(scenes)
    counts = np.array([s.n for s in scenes])
    pick = sorted({0, 1, int(np.argmax(counts)), int(np.argmin(counts)), len(scenes) - 1})
    sims = {k: _plain_for(scenes[k]) for k in pick}
    b.step(3)
    for k in pick:
        sims[k].step(3)
        _compare_scene(b, k, sims[k], f"ensemble scene {k} ({scenes[k].n} particles)")


def test_batch_coincident_particles(sc):
    """Scenes with groups of bit-identical positions (the density pass
    computes one per group and copies it), including the same coordinates in
    two scenes whose slots share a 32-slot warp at the scene boundary: each
    scene equals its plain simulation bit for bit."""
    import dataclasses
    rng = np.random.default_rng(7)
    scenes = []
    for k, (nx, ny, nz) in enumerate([(9, 7, 5), (8, 8, 6)]):
        s = sc.small_scene(nx, ny, nz, seed=20 + k)
        p = s.particles.copy()
        n = len(p)
        p[10:120:3, 0:3] = p[10, 0:3]
        for _ in range(30):
            src = int(rng.integers(0, n))
            p[rng.integers(0, n, size=int(rng.integers(1, 5))), 0:3] = p[src, 0:3]
        scenes.append(dataclasses.replace(s, particles=p))
    # the second scene's first particles at the first scene's group position
    scenes[1].particles[0:8, 0:3] = scenes[0].particles[10, 0:3]
    b = _batch_for(scenes)
    plains = [_plain_for(s) for s in scenes]
    for steps in (1, 13):
        b.step(steps)
        for sim in plains:
            sim.step(steps)
        for k, sim in enumerate(plains):
            _compare_scene(b, k, sim, f"scene {k} after {steps}")
    b.close()
    for sim in plains:
        sim.close()
