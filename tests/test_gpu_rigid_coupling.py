"""The device-resident rigid-body coupling (fs_frames) against the
reference's frame loop run from the host (app.rs:1205-1290): clear the
accumulator, step the substeps, read the accumulator back, integrate the
body on the CPU (fs_integrate_rigid_body) and upload its GpuRigidBody.
Particles, accumulators and the body's state must agree bit for bit after
every frame: a floating sphere, a sinking cube, a held torus, and a batch
scene against its plain simulation."""
import numpy as np
import pytest

from helpers import assert_same_floats, gpu_sim_for_scene

pytestmark = pytest.mark.gpu

SUBSTEPS = 3


def _scene(sc_mod, seed):
    return sc_mod.small_scene(nx=12, ny=9, nz=10, box=(0.6, 0.6, 0.5), seed=seed)


def _host_frames(sim, sc, state, frames):
    from fluidsph import params as P
    grav = list(sc.gravity.direction)
    for _ in range(frames):
        sim.update_rigid_body(P.rigid_body_to_gpu(state))
        sim.clear_rigid_body_accum()
        sim.step(SUBSTEPS)
        acc = sim.read_rigid_body_accum()
        if state.enabled and not state.held:
            P.integrate_rigid_body(state, sc.geom, sc.sph.dt, SUBSTEPS, grav, acc)
        elif state.enabled:
            import ctypes as C
            from fluidsph import abi
            abi.load().fs_clamp_rigid_body(C.byref(state), C.byref(sc.geom), 0)
    return state


def _fields(st):
    return np.array(list(st.position) + list(st.velocity) + list(st.orientation) +
                    list(st.angular_velocity), np.float32)


@pytest.mark.parametrize("shape,density,held", [(1, 300.0, False), (0, 3000.0, False),
                                                (3, 500.0, True)])
def test_device_frames_match_host_loop(shape, density, held):
    from fluidsph import params as P
    from fluidsph import scenes
    sc = _scene(scenes, 40 + shape)
    st0 = P.rigid_body_state(position=(0.02, 0.3, -0.01), half_extent=0.1, shape=shape,
                             density=density, orientation=(0.0, 0.2, 0.0, 0.98),
                             angular_velocity=(0.5, 0.0, -0.3), held=held, wall_stiffness=250.0)
    host = gpu_sim_for_scene(sc)
    dev = gpu_sim_for_scene(sc)
    st_host = type(st0).from_buffer_copy(st0)
    dev.rigid_coupling_set_state(st0)
    for frame in range(6):
        _host_frames(host, sc, st_host, 1)
        dev.frames(SUBSTEPS, 1)
        assert_same_floats(_fields(dev.rigid_coupling_get_state()), _fields(st_host),
                           f"rigid state after frame {frame}")
        assert dev.read_rigid_body_accum().as_tuple() == host.read_rigid_body_accum().as_tuple()
    assert_same_floats(dev.particles(), host.particles(), "particles")
    if not held:
        assert host.read_rigid_body_accum().contact_count > 0
    # graph replay of several frames at once
    dev.frames(SUBSTEPS, 4)
    _host_frames(host, sc, st_host, 4)
    assert_same_floats(_fields(dev.rigid_coupling_get_state()), _fields(st_host), "after 4 more")
    assert_same_floats(dev.particles(), host.particles(), "particles after 4 more")


def test_batch_scene_coupling_matches_plain():
    from fluidsph import params as P
    from fluidsph import scenes
    from fluidsph.sim import SphBatch3DGrid
    scs = [_scene(scenes, 50 + k) for k in range(3)]
    b = SphBatch3DGrid([s.particles for s in scs], [s.sph for s in scs], [s.geom for s in scs])
    for k, s in enumerate(scs):
        b.update_scene(k, gravity=s.gravity)
    b.set_pcisph_iterations(scs[0].iterations)
    st = P.rigid_body_state(position=(0.0, 0.25, 0.0), half_extent=0.09, shape=1, density=400.0)
    b.rigid_coupling_set_state(st, scene=1)
    plain = gpu_sim_for_scene(scs[1])
    plain.rigid_coupling_set_state(st)
    b.frames(SUBSTEPS, 5)
    plain.frames(SUBSTEPS, 5)
    assert_same_floats(_fields(b.rigid_coupling_get_state(1)), _fields(plain.rigid_coupling_get_state()),
                       "batch scene body")
    assert_same_floats(b.scene_particles(1), plain.particles(), "batch scene particles")
    # uncoupled scenes keep the default (inactive) body
    assert b.read_rigid_body_accums()[0].contact_count == 0
