"""The per-simulation choice between the two forms of the density and solve
kernels (batched candidate loads or the plain loop, fs_load_batching): the
measurement runs on steps 8-11 whatever the fs_step call sizes, the choice is
then fixed, and the results are the same bits either way (so a simulation
stepped one step per call, which measures across calls, matches one stepped
in a single call)."""
import numpy as np
import pytest

from helpers import assert_same_floats, gpu_sim_for_scene

pytestmark = pytest.mark.gpu


def test_choice_is_measured_once_and_keeps_results():
    from fluidsph import scenes
    sc = scenes.config0()
    a = gpu_sim_for_scene(sc)
    b = gpu_sim_for_scene(sc)
    a.step(7)
    assert a.load_batching() == (False, False)  # not measured before step 8
    a.step(9)                                     # steps 8-11 measured inside
    batched, decided = a.load_batching()
    assert decided
    for _ in range(16):                           # one step per call
        b.step(1)
    assert b.load_batching()[1]
    pa, pb = a.particles(), b.particles()
    assert_same_floats(pa[:, 0:3], pb[:, 0:3], "position")
    assert_same_floats(pa[:, 4:7], pb[:, 4:7], "velocity")
    # the choice stays fixed afterwards
    a.step(5)
    assert a.load_batching() == (batched, True)
    a.close()
    b.close()
