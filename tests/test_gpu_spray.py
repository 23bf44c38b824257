"""GPU whitewater (fs_spray_*) against the FP32 oracle restatement, which
equals the reference's own spray shaders (tests/test_ref_pin.py): ring
records, write head, potential ceilings and live counts bit for bit over
several frames, including a ring that wraps, and a batch scene against its
plain simulation."""
import numpy as np
import pytest

from helpers import gpu_sim_for_scene

pytestmark = pytest.mark.gpu


def _run(sc, oracle_mod, frames, max_particles, substeps=3):
    from fluidsph.abi import SPRAY_DTYPE
    from fluidsph.spray import SpraySystem, spray_params
    sim = gpu_sim_for_scene(sc)
    orc = oracle_mod.oracle_for_scene(sc)
    spray = SpraySystem(sim, max_particles)
    ring = np.zeros(max_particles, SPRAY_DTYPE)
    head, lim = 0, (3.0, 1.0)
    for f in range(frames):
        prm = spray_params(sc.n, sc.sph.dt * substeps, frame_count=f, max_particles=max_particles)
        sim.step(substeps)
        orc.step(substeps)
        spray.step(prm)
        head, lim, live = orc.spray_frame(prm, ring, head, lim)
        g = spray.particles()
        np.testing.assert_array_equal(g.view(np.uint32), ring.view(np.uint32),
                                      err_msg=f"ring after frame {f}")
        (glim, ghead) = spray.auto_limits()
        assert ghead == head and np.float32(glim[0]) == np.float32(lim[0]) and \
            np.float32(glim[1]) == np.float32(lim[1]), (f, ghead, head, glim, lim)
        np.testing.assert_array_equal(spray.read_stats(), live)
    return head


def test_spray_matches_oracle(oracle_mod):
    from fluidsph import scenes
    sc = scenes.small_scene(nx=12, ny=10, nz=9, seed=61)
    assert _run(sc, oracle_mod, 6, 4096) > 1000


def test_spray_ring_wraps(oracle_mod):
    from fluidsph import scenes
    sc = scenes.small_scene(nx=12, ny=10, nz=9, seed=62)
    assert _run(sc, oracle_mod, 5, 700) > 700  # frames spawn more than the ring holds


def test_spray_dam_break_49600(oracle_mod):
    from fluidsph import scenes
    sc = scenes.config0()
    assert _run(sc, oracle_mod, 3, 100_000) > 0
