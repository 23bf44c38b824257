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
