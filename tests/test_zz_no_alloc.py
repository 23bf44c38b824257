"""The allocation-free prefix scan (fs_prefix_scan_noalloc) against the scan
the simulation step itself runs.

For callers that cannot allocate device memory (stream capture without
allocation nodes, real-time loops, foreign memory pools), the library offers
one entry point whose scratch is a fixed device array. This test calls it
through the C ABI on the cell counts of a real step and checks its output
against the step's own cell_starts, on two calls in a row; it is collected
last so that a failure here cannot hide any other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_scan_matches_step_scan(fslib):
    import torch
    from fluidsph import abi, scenes
    from helpers import gpu_sim_for_scene

    scene = scenes.config0()
    sim = gpu_sim_for_scene(scene)
    sim.step(1)
    counts_ref, starts_ref = sim.cells()          # the step's scan (existing path)
    ptrs = sim.device_pointers()
    g = len(counts_ref)
    out = torch.full((g,), -1, dtype=torch.int32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):
        out.fill_(-1)
        torch.cuda.synchronize()
        rc = fslib.fs_prefix_scan_noalloc(C.c_void_p(ptrs.cell_counts), C.c_void_p(out.data_ptr()),
                                          g, C.c_void_p(status.data_ptr()), C.c_void_p(ptrs.stream))
        assert rc == 0, fslib.fs_last_error()
        sim.sync()
        got = out.cpu().numpy().view(np.uint32)
        np.testing.assert_array_equal(got, starts_ref, err_msg=f"call {call + 1}")
        assert int(status.item()) == 0
    sim.close()


def test_noalloc_scan_rejects_oversize_and_handles_ragged_sizes(fslib):
    import torch
    from fluidsph import abi

    rc = fslib.fs_prefix_scan_noalloc(C.c_void_p(1), C.c_void_p(1),
                                      abi.FS_NOALLOC_SCAN_MAX_CELLS + 1, None, None)
    assert rc == -3 and b"FS_NOALLOC_SCAN_MAX_CELLS" in fslib.fs_last_error()
    rng = np.random.default_rng(5)
    for g in (1, 4095, 4096, 4097, 1 << 17):
        counts = rng.integers(0, 50, g).astype(np.uint32)
        dev_in = torch.from_numpy(counts.view(np.int32)).cuda()
        dev_out = torch.empty(g, dtype=torch.int32, device="cuda")
        for _ in range(2):
            torch.cuda.synchronize()
            rc = fslib.fs_prefix_scan_noalloc(C.c_void_p(dev_in.data_ptr()),
                                              C.c_void_p(dev_out.data_ptr()), g, None, None)
            assert rc == 0, fslib.fs_last_error()
            torch.cuda.synchronize()
            got = dev_out.cpu().numpy().view(np.uint32)
            np.testing.assert_array_equal(got, np.cumsum(counts, dtype=np.uint32))
