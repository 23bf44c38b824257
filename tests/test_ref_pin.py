"""The oracle restatement against the reference's own step shaders translated
to C++ (oracle/_ref), on fresh seeded scenes. Runs where the translation is
available (it is built from the reference sources); skipped elsewhere."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref_lib(oracle_mod):
    lib = oracle_mod.load_ref()
    if lib is None:
        pytest.skip("reference translation not available here")
    return lib


@pytest.mark.parametrize("seed,k", [(21, 1), (22, 2), (23, 5)])
def test_oracle_equals_reference_translation(oracle_mod, ref_lib, seed, k):
    from fluidsph import params as P
    from fluidsph import scenes
    sc = scenes.small_scene(nx=9 + seed % 3, ny=7, nz=6, seed=seed)
    sc.iterations = k
    sc.geom = P.container_geometry(0.6, 0.4, 0.0, 0.5, 0.05 * (seed % 4), -0.03, 250.0, 0.55)
    sc.rigid = P.rigid_body(position=(0.02, 0.1, -0.01), half_extent=0.07, active=True,
                            stiffness=250.0, shape=seed % 4, orientation=(0.0, 0.3, 0.0, 0.954))
    a = oracle_mod.oracle_for_scene(sc)
    b = oracle_mod.oracle_for_scene(sc, lib=ref_lib)
    for o in (a, b):
        o.clear_rigid_body_accum()
        o.step(3)
    for x, y in ((a.particles(), b.particles()), (a.sorted_particles(), b.sorted_particles())):
        assert ((x == y) | (np.isnan(x) & np.isnan(y))).all()
    np.testing.assert_array_equal(a.cells()[1], b.cells()[1])
    np.testing.assert_array_equal(a.index_maps()[1], b.index_maps()[1])
    assert a.read_rigid_body_accum() == b.read_rigid_body_accum()


def _splat_cases(sc, geom_clip):
    """MC grids over a scene's box: the reference's bounds (AABB + margin), a
    wider splat radius (2 SPH cells), clipping, and a grid reaching past the
    SPH grid's edge."""
    from fluidsph import params as P
    Lx, Ly, Lz = sc.box
    lo = (-Lx / 2 - 0.13, -0.13, -Lz / 2 - 0.13)
    hi = (Lx / 2 + 0.13, Ly + 0.13, Lz / 2 + 0.13)
    yield P.mc_grid_params(lo, hi, 24, 0.08), sc.geom
    yield P.mc_grid_params(lo, hi, 20, 0.08 * 1.6), geom_clip
    yield P.mc_grid_params((-2.3, -2.3, -2.3), (2.3, 2.3, 2.3), 16, 0.08), geom_clip


@pytest.mark.parametrize("seed", [31, 32])
def test_density_splat_equals_reference_translation(oracle_mod, ref_lib, seed):
    from fluidsph import params as P
    from fluidsph import scenes
    sc = scenes.small_scene(nx=9, ny=7, nz=6, seed=seed)
    sc.geom = P.container_geometry(0.6, 0.4, 0.0, 0.5, 0.04 * (seed % 3), -0.05, 250.0, 0.55)
    clip = P.container_geometry(0.6, 0.4, 0.0, 0.5, 0.04 * (seed % 3), -0.05, 250.0, 0.55,
                                clip_enabled=True, clip_margin=0.03)
    a = oracle_mod.oracle_for_scene(sc)
    b = oracle_mod.oracle_for_scene(sc, lib=ref_lib)
    for o in (a, b):
        o.step(2)
    for mc, geom in _splat_cases(sc, clip):
        fa = a.density_splat(mc, geom)
        fb = b.density_splat(mc, geom)
        np.testing.assert_array_equal(fa, fb)
        assert (fa > 0).any()
        if geom.clip_enabled:
            assert (fa == -1.0).any()


def test_mc_grid_params_matches_update_params():
    from fluidsph import params as P
    g = P.mc_grid_params((-1.0, -0.2, -0.5), (1.5, 1.0, 0.4), 100, 0.12, 300.0, 77)
    f32 = np.float32
    ext = max(f32(1.5) - f32(-1.0), f32(1.0) - f32(-0.2), f32(0.4) - f32(-0.5))
    assert g.cell_size == f32(ext) / f32(100)
    assert (g.grid_size, g.num_particles, g.max_vertices) == (100, 77, 4_000_000)
    assert g.kernel_radius == f32(0.12) and g.iso_value == 300.0


def test_spray_frames_equal_reference_translation(oracle_mod, ref_lib):
    """Whitewater frames (emit, ceiling update, simulate) of the restatement
    against the reference's own spray shaders, ring state carried over."""
    from fluidsph import scenes
    from fluidsph.abi import SPRAY_DTYPE
    from fluidsph.spray import spray_params
    sc = scenes.small_scene(nx=12, ny=10, nz=9, seed=61)
    a = oracle_mod.oracle_for_scene(sc)
    b = oracle_mod.oracle_for_scene(sc, lib=ref_lib)
    rings = [np.zeros(4096, SPRAY_DTYPE), np.zeros(4096, SPRAY_DTYPE)]
    state = [(0, (3.0, 1.0)), (0, (3.0, 1.0))]
    emitted = 0
    for frame in range(6):
        prm = spray_params(sc.n, sc.sph.dt * 3, frame_count=frame, max_particles=4096)
        out = []
        for k, o in enumerate((a, b)):
            o.step(3)
            head, lim = state[k]
            head, lim, live = o.spray_frame(prm, rings[k], head, lim)
            state[k] = (head, lim)
            out.append(live)
        np.testing.assert_array_equal(rings[0].view(np.uint32), rings[1].view(np.uint32))
        assert state[0] == state[1]
        np.testing.assert_array_equal(out[0], out[1])
        emitted = state[0][0]
    assert emitted > 0, "no spray emitted"
