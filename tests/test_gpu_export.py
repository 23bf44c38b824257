"""The device-side AoS export (fs_export_particles_aos): the 64-byte
SphParticle3D records a renderer instances from, written into device memory.
They must be byte for byte the records the host read-outs build
(fs_download_particles / fs_download_sorted and the per-scene batch
versions), for the canonical and the sorted view."""
import numpy as np
import pytest

from helpers import gpu_sim_for_scene

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _export(sim, count, sorted_view, scene=0):
    buf = torch.empty((count, 16), dtype=torch.float32, device="cuda")
    sim.export_particles_aos(buf.data_ptr(), count, sorted=sorted_view, scene=scene)
    sim.sync()
    return buf.cpu().numpy()


def _same_bytes(a, b):
    np.testing.assert_array_equal(np.ascontiguousarray(a).view(np.uint32),
                                  np.ascontiguousarray(b).view(np.uint32))


def test_export_matches_host_views():
    from fluidsph import scenes
    sc = scenes.config0()
    sim = gpu_sim_for_scene(sc)
    sim.step(3)
    n = sim.num_particles()
    _same_bytes(_export(sim, n, False), sim.particles())
    _same_bytes(_export(sim, n, True), sim.sorted_particles())
    # a prefix
    _same_bytes(_export(sim, 1000, False), sim.particles(1000))
    sim.close()


def test_export_batch_scene():
    from fluidsph import scenes
    from fluidsph.sim import SphBatch3DGrid
    scs = [scenes.batch_scene(k, 7, 2048, 6000, 10) for k in range(3)]
    b = SphBatch3DGrid([s.particles for s in scs], [s.sph for s in scs], [s.geom for s in scs])
    for k, s in enumerate(scs):
        b.update_scene(k, gravity=s.gravity)
    b.set_pcisph_iterations(scs[0].iterations)
    b.step(2)
    for k in (0, 2):
        n = scs[k].n
        _same_bytes(_export(b, n, False, scene=k), b.scene_particles(k))
        _same_bytes(_export(b, n, True, scene=k), b.scene_sorted_particles(k))
    b.close()


def test_export_rejects_bad_targets():
    from fluidsph import abi, scenes
    sc = scenes.config0()
    sim = gpu_sim_for_scene(sc)
    sim.step(1)
    n = sim.num_particles()
    host = np.zeros((16, 16), np.float32)
    with pytest.raises(abi.FluidSphError) as e:
        sim.export_particles_aos(host.ctypes.data, 16)
    assert e.value.code == -1  # host memory: FS_E_INVALID_ARGUMENT
    buf = torch.empty((17, 16), dtype=torch.float32, device="cuda")
    with pytest.raises(abi.FluidSphError) as e:
        sim.export_particles_aos(buf.data_ptr() + 4, 16)
    assert e.value.code == -1  # misaligned
    with pytest.raises(abi.FluidSphError) as e:
        sim.export_particles_aos(buf.data_ptr(), n + 1)
    assert e.value.code == -3  # FS_E_CAPACITY
    sim.export_particles_aos(buf.data_ptr(), 0)  # nothing to do
    sim.close()
