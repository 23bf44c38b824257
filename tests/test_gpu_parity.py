"""GPU parity: the sm_103a step through the C ABI against the FP32 oracle on
the same seeded inputs. The library keeps the shaders' evaluation order with
no fused multiply-add, so the bar is bit-exact for every buffer: cell ids,
counts, inclusive starts, both index maps, sorted density / near density /
normals, canonical positions, velocities and forces, and the fixed-point
rigid-body accumulator."""
import math

import numpy as np
import pytest

from helpers import assert_same_floats, check_grid_invariants, gpu_sim_for_scene, rel_err_stats

pytestmark = pytest.mark.gpu


def _compare(sim, orc, n, what=""):
    counts_g, starts_g = sim.cells()
    counts_o, starts_o = orc.cells()
    np.testing.assert_array_equal(counts_g, counts_o, err_msg=f"{what} cell_counts")
    np.testing.assert_array_equal(starts_g, starts_o, err_msg=f"{what} cell_starts")
    ci_g, so_g = sim.index_maps()
    ci_o, so_o = orc.index_maps()
    np.testing.assert_array_equal(ci_g, ci_o, err_msg=f"{what} particle_cell_indices")
    np.testing.assert_array_equal(so_g, so_o, err_msg=f"{what} sorted_to_orig")
    check_grid_invariants(counts_g, starts_g, ci_g, so_g, n)
    sg, so = sim.sorted_particles(), orc.sorted_particles()
    assert_same_floats(sg[:, 11], so[:, 11], f"{what} sorted density")
    assert_same_floats(sg[:, 12], so[:, 12], f"{what} sorted near_density")
    assert_same_floats(sg[:, 13:16], so[:, 13:16], f"{what} sorted normal")
    assert_same_floats(sg[:, 0:3], so[:, 0:3], f"{what} sorted position")
    assert_same_floats(sg[:, 4:7], so[:, 4:7], f"{what} sorted velocity")
    pg, po = sim.particles(), orc.particles()
    assert_same_floats(pg[:, 0:3], po[:, 0:3], f"{what} position")
    assert_same_floats(pg[:, 4:7], po[:, 4:7], f"{what} velocity")
    assert_same_floats(pg[:, 8:11], po[:, 8:11], f"{what} force (dv)")


def _run_pair(scene, steps, oracle_mod, sdf=None, mouse=None):
    sim = gpu_sim_for_scene(scene, sdf=sdf)
    orc = oracle_mod.OracleSim(scene.particles, scene.sph, scene.geom, sdf=sdf)
    orc.update_gravity(scene.gravity)
    orc.set_pcisph_iterations(scene.iterations)
    if scene.rigid is not None:
        orc.update_rigid_body(scene.rigid)
    if mouse is not None:
        sim.update_mouse_force(mouse)
        orc.update_mouse_force(mouse)
    sim.clear_rigid_body_accum()
    orc.clear_rigid_body_accum()
    for _ in range(steps):
        sim.step(1)
        orc.step(1)
    return sim, orc


@pytest.fixture(scope="module")
def sc():
    from fluidsph import scenes
    return scenes


def test_small_scene_one_step(fslib, oracle_mod, sc):
    scene = sc.small_scene()
    sim, orc = _run_pair(scene, 1, oracle_mod)
    _compare(sim, orc, scene.n, "small")


def test_config0_one_step_then_twenty(fslib, oracle_mod, sc):
    scene = sc.config0()
    sim, orc = _run_pair(scene, 1, oracle_mod)
    _compare(sim, orc, scene.n, "config0 step 1")
    for _ in range(19):
        sim.step(1)
        orc.step(1)
    _compare(sim, orc, scene.n, "config0 step 20")


def test_coincident_particles(fslib, oracle_mod, sc):
    """Groups of particles at bit-identical positions (the density pass
    computes one per group and copies it): groups inside one 32-slot warp,
    groups spanning warps and cells, and a large corner clump, stepped with
    every load depth of the neighbour passes (measured on steps 8-17)."""
    import dataclasses
    scene = sc.small_scene(12, 10, 8, seed=5)
    p = scene.particles.copy()
    n = len(p)
    rng = np.random.default_rng(11)
    # a large group at one particle's position
    p[40:240:2, 0:3] = p[40, 0:3]
    # many small groups of 2-6 members at random positions
    for _ in range(60):
        src = int(rng.integers(0, n))
        dst = rng.integers(0, n, size=int(rng.integers(1, 6)))
        p[dst, 0:3] = p[src, 0:3]
    scene = dataclasses.replace(scene, particles=p)
    sim, orc = _run_pair(scene, 1, oracle_mod)
    _compare(sim, orc, n, "coincident step 1")
    for _ in range(18):
        sim.step(1)
        orc.step(1)
    _compare(sim, orc, n, "coincident step 19")
    assert sim.load_batching()[1]


def test_big_cells(fslib, oracle_mod, sc):
    """Cells holding more than 512 particles (the reorder sorts them in
    chunks of 4096 and ranks across chunks) beside ordinary cells: just above
    the threshold, exactly one chunk, one chunk plus one particle, and three
    chunks, with the particles' indices shuffled so each cell's arrival order
    is random."""
    import copy
    import dataclasses

    from fluidsph.abi import COL_POS
    scene = sc.small_scene(12, 10, 8, seed=9)
    base = scene.particles
    h = float(scene.sph.kernel_radius)
    origin = -2.0 - h  # the reference grid's origin (bounds extent 2, one cell margin)
    rng = np.random.default_rng(17)
    lo, hi = base[:, COL_POS].min(axis=0), base[:, COL_POS].max(axis=0)
    rows = [base]
    # 4096 and 4097 particles alone in cells past the lattice's corners
    past = 1.5 * h / (hi - lo)
    for size, frac in ((513, 0.2), (4096, 1.0 + past), (4097, -past), (9000, 0.7)):
        k = np.floor((lo + frac * (hi - lo) - origin) / h)
        centre = origin + (k + 0.5) * h
        blk = np.repeat(base[:1], size, axis=0)
        blk[:, COL_POS] = (centre + rng.uniform(-0.3 * h, 0.3 * h, size=(size, 3))).astype(np.float32)
        rows.append(blk)
    p = np.concatenate(rows)
    p = p[rng.permutation(len(p))]
    sph = copy.copy(scene.sph)
    sph.num_particles = len(p)  # the dispatch count, as the reference's params carry it
    scene = dataclasses.replace(scene, particles=p, sph=sph)
    sim, orc = _run_pair(scene, 1, oracle_mod)
    counts, _ = sim.cells()
    assert (counts > 512).sum() == 4 and (counts == 4096).sum() == 1 and (counts == 4097).sum() == 1
    _compare(sim, orc, len(p), "big cells step 1")
    for _ in range(2):
        sim.step(1)
        orc.step(1)
    _compare(sim, orc, len(p), "big cells step 3")


def test_graph_replay_matches_single_steps(fslib, sc):
    scene = sc.small_scene(seed=3)
    a = gpu_sim_for_scene(scene)
    b = gpu_sim_for_scene(scene)
    a.step(6)
    for _ in range(6):
        b.step(1)
    assert_same_floats(a.particles(), b.particles(), "graph vs launches")


@pytest.mark.parametrize("shape", [0, 1, 2, 3, 4])
def test_rigid_body_shapes(fslib, oracle_mod, sc, shape):
    from fluidsph import params as P
    scene = sc.small_scene(nx=14, ny=10, nz=10, box=(0.6, 0.5, 0.4), seed=11)
    scene.rigid = P.rigid_body(position=(0.0, 0.12, 0.0), half_extent=0.1, active=True,
                               stiffness=250.0, shape=shape, velocity=(0.1, -0.2, 0.05),
                               orientation=(0.1, 0.2, 0.3, 0.927))
    sdf = None
    if shape == 4:
        # a sphere-like SDF on a 16^3 texture, in units of half_extent
        r = 16
        c = (np.arange(r) + 0.5) / r * 2 - 1
        z, y, x = np.meshgrid(c, c, c, indexing="ij")
        sdf = (np.sqrt(x * x + y * y + z * z) - 0.8).astype(np.float32)
    sim, orc = _run_pair(scene, 2, oracle_mod, sdf=sdf)
    _compare(sim, orc, scene.n, f"shape {shape}")
    acc_g = sim.read_rigid_body_accum().as_tuple()
    acc_o = orc.read_rigid_body_accum()
    assert acc_g == tuple(acc_o)
    assert acc_g[3] > 0, "expected contacts with the body"


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4])
def test_mouse_force_modes(fslib, oracle_mod, sc, mode):
    from fluidsph import params as P
    scene = sc.small_scene(seed=5)
    m = P.mouse_force(position=(0.0, 0.1, 0.0), radius=0.3, strength=40.0, active=True,
                      mode=mode, direction=(0.3, -0.2, -1.0))
    sim, orc = _run_pair(scene, 2, oracle_mod, mouse=m)
    _compare(sim, orc, scene.n, f"mouse mode {mode}")


def test_tilted_container_and_iterations(fslib, oracle_mod, sc):
    from fluidsph import params as P
    for k, tilt in ((1, 0.2), (2, -0.25), (5, 0.1)):
        scene = sc.small_scene(seed=9)
        scene.geom = P.container_geometry(0.6, 0.4, 0.0, 0.5, tilt, -tilt / 2, 250.0, 0.55)
        scene.iterations = k
        sim, orc = _run_pair(scene, 3, oracle_mod)
        _compare(sim, orc, scene.n, f"tilt {tilt} K={k}")


def test_xsph_off_and_outside_particles(fslib, oracle_mod, sc):
    scene = sc.small_scene(seed=2)
    scene.sph.xsph_epsilon = 0.0
    # particles beyond the +-2 grid: clamped in hashing, unclamped in lookups
    scene.particles[:4, 0:3] = [[2.5, 0.1, 0.0], [-3.0, 0.2, 0.1], [0.0, 4.0, 0.0],
                                [0.1, 0.1, 2.3]]
    sim, orc = _run_pair(scene, 2, oracle_mod)
    _compare(sim, orc, scene.n, "xsph off / outside")


def test_small_coordinates(fslib, oracle_mod, sc):
    """Positions with a coordinate 0 < |c| < 2^-34 switch the force pass to
    its checked direction numerators for that step, and pairs whose
    coordinate difference is below 2^-60 take the IEEE operations: a group of
    particles on the x = 0 and z = 0 planes and at tiny offsets from them
    (1e-30 .. 1e-12, both signs), within h of each other, then the same
    scene's later steps (the offsets grow out of the range)."""
    scene = sc.small_scene(seed=4)
    p = scene.particles
    n = scene.n
    rng = np.random.default_rng(3)
    centre = p[n // 2, 0:3].copy()
    tiny = np.array([0.0, 1e-30, -1e-30, 3e-25, -7e-20, 1e-19, -2e-18, 5e-15, 1e-12, -1e-12],
                    np.float32)
    k = 0
    for i in range(n // 2 - 40, n // 2 + 40, 2):
        p[i, 0] = tiny[k % len(tiny)]
        p[i, 2] = tiny[(k * 3 + 1) % len(tiny)]
        p[i, 1] = centre[1] + np.float32(0.01) * np.float32(rng.uniform(-1, 1))
        k += 1
    sim, orc = _run_pair(scene, 1, oracle_mod)
    _compare(sim, orc, n, "small coordinates step 1")
    for _ in range(4):
        sim.step(1)
        orc.step(1)
    _compare(sim, orc, n, "small coordinates step 5")


def test_cooperative_force(fslib, oracle_mod, sc):
    """A small, dense block (1,728 particles, hundreds of neighbours each):
    its heavy particles exceed the cooperative threshold, so their force pass
    runs a warp per particle (terms in parallel, sums in the walk's order);
    every buffer stays bit-exact against the oracle."""
    scene = sc.small_scene(12, 12, 12, box=(0.2, 0.2, 0.2), seed=6)
    sim, orc = _run_pair(scene, 3, oracle_mod)
    assert sim.neighbor_stats()["coop_force"] > 0
    _compare(sim, orc, scene.n, "cooperative force")


def test_empty_and_spawn(fslib, oracle_mod, sc):
    from fluidsph.sim import SphSimulation3DGrid
    scene = sc.make_scene("empty", np.zeros((0, 16), np.float32), (1, 1, 1))
    sim = SphSimulation3DGrid(scene.particles, scene.sph, scene.geom, max_particles=300)
    sim.step(2)
    assert sim.num_particles() == 0
    # spawn clips at capacity (sph_3d_grid.rs:1534-1569)
    assert sim.spawn_particles((0.0, 0.3, 0.0), 250, 0.05) == 250
    assert sim.spawn_particles((0.0, 0.3, 0.0), 100, 0.05) == 50
    assert sim.num_particles() == 300
    p = sim.particles()
    assert np.isfinite(p).all()
    # the records are fs_spawn_positions' (pinned to the reference's
    # spawn_particles by tests/test_ref_pin_host.py), byte for byte
    import ctypes as C
    want = np.zeros((300, 16), np.float32)
    got = C.c_uint32()
    pos = (C.c_float * 3)(0.0, 0.3, 0.0)
    assert fslib.fs_spawn_positions(pos, 250, C.c_float(0.05), 0, 300, want.ctypes.data,
                                    C.byref(got)) == 0 and got.value == 250
    assert fslib.fs_spawn_positions(pos, 100, C.c_float(0.05), 250, 300,
                                    want[250:].ctypes.data, C.byref(got)) == 0 and got.value == 50
    assert p.tobytes() == want.tobytes()
    # the spawned block then steps like any other input
    params = scene.sph
    params.num_particles = 300
    sim.update_sph_params(params)
    orc = oracle_mod.OracleSim(p, params, scene.geom)
    sim.step(1)
    orc.step(1)
    _compare(sim, orc, 300, "spawned")


def test_config1_full_size_one_step(fslib, oracle_mod, sc):
    """1,048,576 particles with the held sphere: every buffer bit-exact."""
    scene = sc.config1()
    sim, orc = _run_pair(scene, 1, oracle_mod)
    _compare(sim, orc, scene.n, "config1")
    assert sim.read_rigid_body_accum().as_tuple() == tuple(orc.read_rigid_body_accum())


def _fp64_twin(oracle_mod, scene):
    """The FP64 twin with the FP32 pipeline's discrete decisions: cells are
    hashed in FP32 arithmetic, so cell ids, candidate sets and slot order are
    the GPU's (they are checked bit-exact elsewhere) and only the precision of
    the continuous arithmetic differs. It also keeps, per particle, the sum of
    the magnitudes of the terms each pair sum adds."""
    o = oracle_mod.oracle_for_scene(scene, precision=64)
    o.set_cells_f32(True)
    o.track_terms(True)
    return o


def _vec_err(a, b, scale=None):
    """Per-particle |a - b| / |b| and, with `scale`, |a - b| / max(|b|, scale)."""
    d = np.linalg.norm(np.asarray(a, np.float64) - b, axis=1)
    m = np.linalg.norm(b, axis=1)
    rel = d / np.maximum(m, 1e-30)
    cond = None if scale is None else d / np.maximum(np.maximum(m, scale), 1e-30)
    return rel, cond, np.maximum(m, scale) / np.maximum(m, 1e-30) if scale is not None else None


def _summary(rel, cond=None, kappa=None, tol=1e-4):
    out = {"p50": float(np.quantile(rel, 0.5)), "p99": float(np.quantile(rel, 0.99)),
           "max": float(rel.max()), f"n_above_{tol:g}": int((rel > tol).sum())}
    if cond is not None:
        out["max_rel_to_term_magnitudes"] = float(cond.max())
        out["median_condition_number"] = float(np.median(kappa))
        bad = rel > tol
        if bad.any():
            out[f"min_condition_number_above_{tol:g}"] = float(kappa[bad].min())
    return out


def test_fp64_error_report(fslib, oracle_mod, sc, capsys):
    """The GPU's FP32 step against the FP64 twin after one step of config 0,
    per quantity, at the stated tolerances: density and near density 1e-5
    relative (every particle); position 1e-4 (every particle); velocity, the
    step's velocity change dv and the force pass's acceleration a_np 1e-4
    relative at p99 and, for every particle, 1e-4 relative to the magnitude
    of the terms summed. The last form is the conditioning-aware one: the
    lattice starts at ~15x rest density, so a particle's force is a sum of
    pair terms that cancel (median condition number ~50, up to ~1,300) and the
    plain relative error of a strongly cancelled sum measures the cancellation,
    not the arithmetic. The particles above 1e-4 plain relative error are
    counted and reported with their condition numbers."""
    scene = sc.config0()
    dt = float(scene.sph.dt)
    v0 = scene.particles[:, 4:7].astype(np.float64)
    sim = gpu_sim_for_scene(scene)
    sim.step(1)
    o64 = _fp64_twin(oracle_mod, scene)
    o64.step(1)
    ci_g, _ = sim.index_maps()
    ci_o, _ = o64.index_maps()
    np.testing.assert_array_equal(ci_g, ci_o)  # same discrete decisions
    sg = sim.sorted_particles()[ci_g]
    s64 = o64.particles_f64(sorted_=True)[ci_o]
    pg = sim.particles()
    p64 = o64.particles_f64()
    T = o64.term_magnitudes()
    sv = np.linalg.norm(v0, axis=1) + dt * (T[:, 0] + T[:, 1])  # velocity's summed terms
    vel = _vec_err(pg[:, 4:7], p64[:, 3:6], sv)
    dv = _vec_err(pg[:, 8:11], p64[:, 6:9], dt * (T[:, 0] + T[:, 1]))
    nrm = _vec_err(sg[:, 13:16], s64[:, 11:14], T[:, 2])
    pos = _vec_err(pg[:, 0:3], p64[:, 0:3])

    # a_np: with one PCISPH iteration (pressures all 0) from rest, the step's
    # velocity change is fl(dt * a_np) on both sides
    one = sc.config0()
    one.iterations = 1
    sim1 = gpu_sim_for_scene(one)
    sim1.step(1)
    o1 = _fp64_twin(oracle_mod, one)
    o1.step(1)
    T1 = o1.term_magnitudes()
    anp = _vec_err(sim1.particles()[:, 8:11] / dt, o1.particles_f64()[:, 6:9] / dt, T1[:, 0])
    rep = {
        "density": _summary(rel_err(sg[:, 11], s64[:, 9]), tol=1e-5),
        "near_density": _summary(rel_err(sg[:, 12], s64[:, 10]), tol=1e-5),
        "normal": _summary(*nrm),
        "force_a_np": _summary(*anp),
        "dv": _summary(*dv),
        "position": _summary(pos[0]),
        "velocity": _summary(*vel),
    }
    with capsys.disabled():
        print("\nFP64 relative error (GPU FP32 vs FP64 twin, config 0, 1 step):")
        for k, v in rep.items():
            print(f"  {k}: {v}")
    assert rep["density"]["max"] < 1e-5
    assert rep["near_density"]["max"] < 1e-5
    assert rep["position"]["max"] < 1e-4
    for q in ("velocity", "dv", "force_a_np"):
        assert rep[q]["p99"] < 1e-4, q
        assert rep[q]["max_rel_to_term_magnitudes"] < 1e-4, q
    assert rep["normal"]["max_rel_to_term_magnitudes"] < 1e-4
    sim.close()
    sim1.close()


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-30)
