"""The reverse pass on a batch: each scene's gradients (initial velocities,
viscosity, surface tension, near stiffness, PCISPH delta) against the same scene's plain reverse pass, and
each scene's loss against its plain loss. The reverse gathers may pick a
different lanes-per-particle variant for the batch's particle count (a
different fixed summation order), so gradients agree to a stated relative
tolerance rather than bit for bit; the losses are bit-identical (the forward
is)."""
import numpy as np
import pytest

from helpers import gpu_sim_for_scene

pytestmark = pytest.mark.gpu

RTOL = 1e-4


def test_batch_gradients_match_plain(oracle_mod):
    from fluidsph import scenes
    from fluidsph.adjoint import DifferentiableRollout
    from fluidsph.sim import SphBatch3DGrid
    scs, hidden = scenes.reference_physics_batch(num_scenes=3, steps=8, seed=3)
    grids = [scenes.loss_grid(s, 32) for s in scs]
    # targets: each scene's hidden-viscosity run
    targets = []
    for s, hdn, mc in zip(scs, hidden, grids):
        p = type(s.sph).from_buffer_copy(s.sph)
        p.viscosity = hdn["viscosity"]
        sim = gpu_sim_for_scene(s)
        sim.update_sph_params(p)
        r = DifferentiableRollout(sim, 4)
        r.forward(s.steps)
        targets.append(r.final_splat(mc, s.geom))
    b = SphBatch3DGrid([s.particles for s in scs], [s.sph for s in scs], [s.geom for s in scs])
    for k, s in enumerate(scs):
        b.update_scene(k, gravity=s.gravity)
    b.set_pcisph_iterations(scs[0].iterations)
    rb = DifferentiableRollout(b, 4)
    rb.forward(scs[0].steps)
    losses = [rb.splat_mse_loss(grids[k], scs[k].geom, targets[k], scene=k) for k in range(3)]
    dpos_b, dvel_b, _ = rb.backward(scenes=3)
    dpar_b = rb.param_gradients(scenes=3)
    off = 0
    for k, s in enumerate(scs):
        sim = gpu_sim_for_scene(s)
        r = DifferentiableRollout(sim, 4)
        r.forward(s.steps)
        loss = r.splat_mse_loss(grids[k], s.geom, targets[k])
        _, dvel, _ = r.backward()
        dpar = r.param_gradients()
        assert loss == losses[k]
        n = s.n
        g_b = dvel_b[off:off + n].astype(np.float64)
        scale = np.abs(dvel).max()
        assert np.abs(g_b - dvel).max() <= RTOL * scale, k
        for idx in (0, 2, 3, 4):  # viscosity, surface tension, near stiffness, delta
            assert abs(dpar_b[k, idx] - dpar[0, idx]) <= RTOL * abs(dpar[0, idx]), (k, idx)
        assert dpar_b[k, 1] == 0.0
        off += n


def test_batched_losses_match_single_scene_calls():
    """fs_adj_splat_mse_losses (one grid build, one read-back; host targets
    and device targets) gives each scene's single-call loss bit for bit and
    the same gradients, bit for bit."""
    import torch
    from fluidsph import scenes
    from fluidsph.adjoint import DifferentiableRollout
    from fluidsph.sim import SphBatch3DGrid
    scs, _ = scenes.reference_physics_batch(num_scenes=3, steps=6, seed=5)
    grids = [scenes.loss_grid(s, 32) for s in scs]
    rng = np.random.default_rng(7)
    targets = [rng.uniform(0.0, 50.0, (32, 32, 32)).astype(np.float32) for _ in scs]

    def run(mode):
        b = SphBatch3DGrid([s.particles for s in scs], [s.sph for s in scs],
                           [s.geom for s in scs])
        for k, s in enumerate(scs):
            b.update_scene(k, gravity=s.gravity)
        b.set_pcisph_iterations(scs[0].iterations)
        r = DifferentiableRollout(b, 3)
        r.forward(scs[0].steps)
        geoms = [s.geom for s in scs]
        if mode == "single":
            losses = np.array([r.splat_mse_loss(grids[k], geoms[k], targets[k], scene=k)
                               for k in range(3)])
        elif mode == "host":
            losses = r.splat_mse_losses(grids, geoms, targets)
        else:
            losses = r.splat_mse_losses(grids, geoms, [torch.from_numpy(t).cuda() for t in targets])
        dpos, dvel, _ = r.backward(scenes=3)
        dpar = r.param_gradients(scenes=3)
        r.close()
        b.close()
        return losses, dpos, dvel, dpar

    ref = run("single")
    for mode in ("host", "device"):
        got = run(mode)
        assert got[0].tobytes() == ref[0].tobytes(), mode
        for a, b in zip(got[1:], ref[1:]):
            assert a.tobytes() == b.tobytes(), mode
