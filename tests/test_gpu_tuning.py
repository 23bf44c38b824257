"""The neighbour passes' load-depth autotuner (fs_kernel_forms and the
per-bucket table): the measurement runs on steps 8-17 whatever the fs_step
call sizes, each pass keeps its fastest depth, a later simulation of the same
particle-count bucket takes the table's depths without measuring, and every
depth gives the same bits (so simulations with any fixed depths, or measured
across calls, match each other exactly)."""
import numpy as np
import pytest

from helpers import assert_same_floats, gpu_sim_for_scene

pytestmark = pytest.mark.gpu

DEPTHS = (0, 4, 8, 16)                # density
SOLVE_DEPTHS = (0, 4, 8, 16)
XSPH_DEPTHS = (1, 4, 8, 16, 32)       # 32: the staged form


def _scene():
    from fluidsph import scenes
    sc = scenes.config0()
    sc.iterations = 7  # a bucket no other test uses: this test's simulation measures
    return sc


def _state(sim):
    p = sim.particles()
    return p[:, 0:3].copy(), p[:, 4:7].copy(), sim.sorted_particles()[:, 11:13].copy()


def test_forms_tuned_per_bucket_and_results_unchanged():
    from fluidsph.sim import kernel_forms_table
    sc = _scene()
    a = gpu_sim_for_scene(sc)
    a.step(7)
    assert a.kernel_forms()["decided"] == "pending"  # not measured before step 8
    assert a.load_batching() == (False, False)
    a.step(12)                                         # steps 8-17 measured inside
    f = a.kernel_forms()
    assert f["decided"] == "measured"
    assert f["density_loads"] in DEPTHS and f["solve_loads"] in SOLVE_DEPTHS
    assert f["xsph_loads"] in XSPH_DEPTHS
    assert all(t > 0 for row in f["ms"] for t in row)  # every depth of every pass timed
    # the kept depth is each pass's fastest (density and solve over their four)
    for k, key, lst in ((0, "density_loads", DEPTHS), (1, "xsph_loads", XSPH_DEPTHS),
                        (2, "solve_loads", SOLVE_DEPTHS)):
        assert lst[int(np.argmin(f["ms"][k][:len(lst)]))] == f[key]
    entry = [e for e in kernel_forms_table()
             if e["bucket"] == f["bucket"] and e["iterations"] == 7 and not e["many_scenes"]]
    assert len(entry) == 1 and entry[0]["density_loads"] == f["density_loads"]
    # a second simulation of the bucket takes the table's depths at once
    b = gpu_sim_for_scene(sc)
    b.step(1)
    g = b.kernel_forms()
    assert g["decided"] == "table"
    assert (g["density_loads"], g["solve_loads"], g["xsph_loads"]) == \
        (f["density_loads"], f["solve_loads"], f["xsph_loads"])
    b.close()
    ref = _state(a)
    # every depth, fixed for the whole run, and one mixed choice: the same bits
    for dens, solve, xsph in [(d, d, x) for d, x in zip(DEPTHS, XSPH_DEPTHS)] + \
            [(0, 16, 8), (16, 16, 32), (0, 0, 32)]:
        c = gpu_sim_for_scene(sc)
        c.set_kernel_forms(dens, solve, xsph)
        for _ in range(19):
            c.step(1)
        assert c.kernel_forms()["decided"] == "set"
        for x, y, what in zip(_state(c), ref, ("position", "velocity", "density")):
            assert_same_floats(x, y, f"{what} with depths {dens}/{solve}/{xsph}")
        c.close()
    a.close()


def test_set_kernel_forms_rejects_unknown_depths(fslib):
    sc = _scene()
    sim = gpu_sim_for_scene(sc)
    with pytest.raises(Exception):
        sim.set_kernel_forms(3, 4, 4)
    with pytest.raises(Exception):
        sim.set_kernel_forms(4, 4, 0)   # XSPH depths are 1, 4, 8, 16, 32
    with pytest.raises(Exception):
        sim.set_kernel_forms(32, 4, 4)  # the density pass has no staged form
    with pytest.raises(Exception):
        sim.set_kernel_forms(4, 32, 4)  # nor has the solve
    sim.set_kernel_forms(16, 0, 1)
    sim.set_kernel_forms()              # back to tuning
    assert sim.kernel_forms()["decided"] in ("pending", "table")
    sim.close()
