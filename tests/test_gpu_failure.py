"""Failure detection on the GPU without a GPU fault: the prefix scan's bounded
look-back wait is made to run out (fs_selftest_scan_wait polls a descriptor
that nothing publishes), the kernel finishes normally, and the expiry reaches
the host through the simulation's device error word as FS_E_DEVICE_TIMEOUT on
the next synchronising call, cleared on the call after. The simulation stays
usable: the next step is still bit-exact against the oracle."""
import ctypes as C

import numpy as np
import pytest

from helpers import assert_same_floats, gpu_sim_for_scene

pytestmark = pytest.mark.gpu

FS_OK, FS_E_DEVICE_TIMEOUT = 0, -5


def test_scan_wait_expiry_is_reported_once(fslib, oracle_mod):
    from fluidsph import scenes
    scene = scenes.config0()
    sim = gpu_sim_for_scene(scene)
    orc = oracle_mod.oracle_for_scene(scene)
    sim.step(1)
    orc.step(1)
    counts, starts = sim.cells()
    g = len(starts)
    assert g > 4096 * 2  # several scan tiles, so tiles after the first wait
    lib, h = fslib, sim._h
    out = np.zeros(g, np.uint32)

    # the unmodified wait: equals the step's scan, nothing reported
    assert lib.fs_selftest_scan_wait(h, 0, out.ctypes.data) == FS_OK
    np.testing.assert_array_equal(out, starts)
    assert lib.fs_sync(h) == FS_OK

    # every wait runs out: the kernel still finishes, with a wrong prefix
    out[:] = 0
    assert lib.fs_selftest_scan_wait(h, 1, out.ctypes.data) == FS_OK
    assert not np.array_equal(out, starts)
    np.testing.assert_array_equal(out[:4096], starts[:4096])  # the first tile waits for no one
    rc = lib.fs_sync(h)
    assert rc == FS_E_DEVICE_TIMEOUT
    assert b"scan look-back" in lib.fs_last_error()
    assert lib.fs_sync(h) == FS_OK  # reported once, then clear

    # the context and the simulation stay usable
    sim.step(1)
    orc.step(1)
    assert_same_floats(sim.particles(), orc.particles(), "step after the injected expiry")
    assert lib.fs_sync(h) == FS_OK
    sim.close()
