"""CPU oracle checks (no GPU): grid-build invariants, hand-computable cases,
the reference's edge behaviours, and the FP32 restatement against its FP64
twin. Fixture-level pinning against the reference's own WGSL is in
test_golden.py."""
import math

import numpy as np
import pytest

from helpers import check_grid_invariants, rel_err_stats

f32 = np.float32


@pytest.fixture(scope="module")
def scenes_mod():
    from fluidsph import scenes
    return scenes


def _scene_with(scenes_mod, positions, box=(1.0, 1.0, 1.0), **kw):
    parts = np.zeros((len(positions), 16), np.float32)
    parts[:, 0:3] = np.asarray(positions, np.float32)
    return scenes_mod.make_scene("custom", parts, box, **kw)


def test_grid_build_invariants_config0(oracle_mod, scenes_mod):
    sc = scenes_mod.config0()
    o = oracle_mod.oracle_for_scene(sc)
    for st in (0, 1, 2):
        o.stage(st)
    counts, starts = o.cells()
    ci, so = o.index_maps()
    check_grid_invariants(counts, starts, ci, so, sc.n)
    # sorted records are exact copies of the canonical ones
    np.testing.assert_array_equal(o.sorted_particles()[ci], o.particles())


def test_cell_index_formula_and_clamp(oracle_mod, scenes_mod):
    # one particle far outside the +-2 grid is clamped into a boundary cell
    sc = _scene_with(scenes_mod, [[0.1, 0.2, 0.3], [5.0, -7.0, 0.0]])
    o = oracle_mod.oracle_for_scene(sc)
    o.stage(0)
    o.stage(1)
    counts, starts = o.cells()
    g = 52
    def cell(p):
        c = [min(max(int(math.floor(f32(f32(v) - f32(-2.08)) * f32(12.5))), 0), g - 1) for v in p]
        return c[0] + c[1] * g + c[2] * g * g
    assert counts[cell([0.1, 0.2, 0.3])] == 1
    assert counts[cell([5.0, -7.0, 0.0])] == 1
    assert cell([5.0, -7.0, 0.0]) == 51 + 0 * g + 26 * g * g


def test_outside_particle_sees_no_cells(oracle_mod, scenes_mod):
    # the density pass looks up the UNCLAMPED cell (sph_density_3d_grid.wgsl:
    # 122,134): a particle beyond the grid finds no valid cell, not even itself
    sc = _scene_with(scenes_mod, [[0.0, 0.5, 0.0], [3.0, 0.5, 0.0]])
    o = oracle_mod.oracle_for_scene(sc)
    for st in (0, 1, 2, 3):
        o.stage(st)
    s = o.sorted_particles()
    ci, _ = o.index_maps()
    assert s[ci[1], 11] == 0.0 and s[ci[1], 12] == 0.0
    assert s[ci[0], 11] > 0.0


def test_single_particle_density(oracle_mod, scenes_mod):
    sc = _scene_with(scenes_mod, [[0.0, 0.5, 0.0]])
    o = oracle_mod.oracle_for_scene(sc)
    for st in (0, 1, 2, 3):
        o.stage(st)
    s = o.sorted_particles()[0]
    p = sc.sph
    h = f32(p.kernel_radius)
    scale = f32(f32(315.0) / f32(f32(f32(64.0) * f32(3.14159265359)) * f32(p.kernel_radius_pow9)))
    d = f32(p.kernel_radius_sq)
    w0 = f32(f32(f32(scale * d) * d) * d)
    assert s[11] == f32(f32(1.0) * w0)  # gamma = 1 in the middle of a 1 m box
    sn = f32(f32(15.0) / f32(f32(3.14159265359) * f32(p.kernel_radius_pow6)))
    assert s[12] == f32(f32(f32(sn * h) * h) * h)
    assert (s[13:16] == 0).all()  # no neighbour: zero normal


def test_close_pair_uses_index_direction_and_separation(oracle_mod, scenes_mod):
    # r = 0.004 < 0.1 h: direction from sin/cos of the slot difference plus the
    # 200*(1 - r/min_dist) separation term (sph_force_3d_grid.wgsl:160-189)
    sc = _scene_with(scenes_mod, [[0.0, 0.5, 0.0], [0.004, 0.5, 0.0]], box=(1, 1, 1))
    sc.gravity.direction[:] = [0, 0, 0]
    o = oracle_mod.oracle_for_scene(sc)
    for st in (0, 1, 2, 3, 4, 5):
        o.stage(st)
    f = o.particles()[:, 8:11]
    assert np.isfinite(f).all()
    mag = np.linalg.norm(f, axis=1)
    assert (mag > 50.0).all()  # separation dominates (200 * 0.5 = 100 m/s^2 scale)
    d = np.array([math.sin(-1.0), math.cos(-2.0), math.sin(-3.0)])
    d /= np.linalg.norm(d)
    # particle in slot 0 gets a push along -dir(0-1) ... along +/- the index direction
    cosang = abs(np.dot(f[0], d)) / mag[0]
    assert cosang > 0.9


def test_mass_and_finiteness_over_steps(oracle_mod, scenes_mod):
    sc = scenes_mod.small_scene()
    o = oracle_mod.oracle_for_scene(sc)
    o.step(5)
    p = o.particles()
    assert np.isfinite(p).all()
    hw, hh, hd = sc.geom.half_width, sc.geom.half_height, sc.geom.half_depth
    assert (np.abs(p[:, 0]) <= hw + 1e-6).all() and (np.abs(p[:, 2]) <= hd + 1e-6).all()
    assert (p[:, 1] >= -1e-6).all() and (p[:, 1] <= 2 * hh + 1e-6).all()


def test_fp32_restatement_vs_fp64_twin(oracle_mod, scenes_mod):
    """Per-quantity FP32-vs-FP64 error of one step's density stage (by particle
    identity): within the 1e-5 density tolerance."""
    sc = scenes_mod.config0()
    o32 = oracle_mod.oracle_for_scene(sc, 32)
    o64 = oracle_mod.oracle_for_scene(sc, 64)
    for o in (o32, o64):
        for st in (0, 1, 2, 3):
            o.stage(st)
    s32 = o32.sorted_particles()[o32.index_maps()[0]]
    s64 = o64.particles_f64(sorted_=True)[o64.index_maps()[0]]
    dens = rel_err_stats(s32[:, 11], s64[:, 9])
    near = rel_err_stats(s32[:, 12], s64[:, 10])
    assert dens["max"] < 1e-5, dens
    assert near["max"] < 1e-5, near


def test_reorder_is_stable_and_deterministic(oracle_mod, scenes_mod):
    sc = scenes_mod.small_scene(seed=7)
    a = oracle_mod.oracle_for_scene(sc)
    b = oracle_mod.oracle_for_scene(sc)
    a.step(3)
    b.step(3)
    np.testing.assert_array_equal(a.particles(), b.particles())
    np.testing.assert_array_equal(a.index_maps()[1], b.index_maps()[1])


def test_empty_scene(oracle_mod, scenes_mod):
    sc = scenes_mod.make_scene("empty", np.zeros((0, 16), np.float32), (1, 1, 1))
    o = oracle_mod.oracle_for_scene(sc)
    o.step(2)
    counts, starts = o.cells()
    assert counts.sum() == 0 and starts[-1] == 0


def test_scene_generators_deterministic(scenes_mod):
    a = scenes_mod.config0(seed=0).particles
    b = scenes_mod.config0(seed=0).particles
    c = scenes_mod.config0(seed=1).particles
    assert a.shape == (49600, 16)
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, c)
    j = a[:, 0:3] - np.round((a[:, 0:3] + np.array([0.8, 0.0, 0.4], np.float32)) / 0.02) * 0.02 \
        + np.array([0.8, 0.0, 0.4], np.float32)
    assert np.abs(j).max() <= 0.002 + 1e-6
    # SplitMix64 reference values (seed 0)
    z = scenes_mod.splitmix64(0, 2)
    assert int(z[0]) == 0xE220A8397B1DCDAF and int(z[1]) == 0x6E789E6AA1B965F4


def test_fp32_sincos_accuracy(oracle_mod):
    """The fixed FP32 sin/cos of the close-pair direction against libm double
    on the integer arguments it receives (slot differences times 1..3): about
    one ulp up to 2^20, and under 3e-7 absolute up to 3 * 2^21."""
    rng = np.random.default_rng(0)
    near = np.concatenate([np.arange(-4096, 4097), rng.integers(-2**20, 2**20, 200000)])
    far = rng.integers(-3 * 2**21, 3 * 2**21, 200000)
    for x, tol in ((near, 8e-8), (far, 3e-7)):
        x = x.astype(np.float32)
        s, c = oracle_mod.sincos_f32(x)
        xd = x.astype(np.float64)
        assert np.abs(s - np.sin(xd)).max() < tol
        assert np.abs(c - np.cos(xd)).max() < tol
    s, c = oracle_mod.sincos_f32(np.zeros(1, np.float32))
    assert s[0] == 0.0 and c[0] == 1.0
