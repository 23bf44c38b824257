"""The reverse pass (fs_adj_*) against forward-mode derivatives and finite
differences of the same discretisation.

Loss: the mean squared difference between the density splat of the final
positions (over the scene's box) and a hidden run's (different viscosity).
Checked quantities: dL/dviscosity, dL/dsurface_tension, dL/dstiffness (0: no
stage reads it), dL/dnear_stiffness and dL/dpcisph_delta (the live pressure
parameters: near pressure in the force pass, the PCISPH pressure update) and
the initial-velocity and initial-position gradients along random
directions.

* The rollout with the reference application's default physics (2,048
  particles, 20 steps, checkpoint every 6): the loss is smooth, so the GPU
  gradient must match the FP32 tangent (the oracle on dual numbers,
  following the GPU's own FP32 trajectory bit for bit) within EXACT_RTOL, the
  FP64 tangent (the exact derivative of the FP64 twin) within GRAD_RTOL and
  central FD of the FP64 loss within FD_RTOL (FD also sees the loss's kinks:
  viscosity switches, pressure clamps, the max(0, rho - rho0) of PCISPH).
* The 2,048-particle copy of the rollout workload (h 0.08, spacing 0.02,
  surface tension 6.5): its dynamics blow up within a few steps (hundreds of
  m/s, thousands of r < 0.1h pairs whose fallback direction jumps with the
  slot order), so the loss is discontinuous at float resolution and FD slopes
  do not converge. The reverse pass must still be the exact derivative of
  the piecewise-smooth map: it is compared with the FP32 tangent along the
  same trajectory over 1 and 2 steps.
* Determinism and independence of the checkpoint interval (bitwise).
"""
import numpy as np
import pytest

from helpers import gpu_sim_for_scene

pytestmark = pytest.mark.gpu

EXACT_RTOL = 2e-4   # vs the FP32 tangent on the identical trajectory
GRAD_RTOL = 1e-3    # vs the FP64 tangent (the FP64 trajectory differs slightly)
FD_RTOL = 1e-2      # vs central FD of the FP64 loss (eps 1e-4 relative)


def _with(p, **kw):
    q = type(p).from_buffer_copy(p)
    for k, v in kw.items():
        setattr(q, k, v)
    return q


def _target(oracle_mod, sc, mc, steps, **hidden):
    o = oracle_mod.OracleSim(sc.particles, _with(sc.sph, **hidden), sc.geom)
    o.update_gravity(sc.gravity)
    o.set_pcisph_iterations(sc.iterations)
    o.step(steps)
    for st in (0, 1, 2):  # grid build of the final positions
        o.stage(st)
    return o.density_splat(mc, sc.geom).astype(np.float32)


def _oracle_loss(oracle_mod, sc, mc, target, steps, visc=None, st=None, vel=None, near=None,
                 delta=None):
    p = _with(sc.sph, viscosity=sc.sph.viscosity if visc is None else visc,
              surface_tension=sc.sph.surface_tension if st is None else st,
              near_stiffness=sc.sph.near_stiffness if near is None else near,
              pcisph_delta=sc.sph.pcisph_delta if delta is None else delta)
    parts = sc.particles.copy()
    if vel is not None:
        parts[:, 4:7] = vel
    o = oracle_mod.OracleSim(parts, p, sc.geom, precision=64)
    o.update_gravity(sc.gravity)
    o.set_pcisph_iterations(sc.iterations)
    o.step(steps)
    for stage in (0, 1, 2):
        o.stage(stage)
    f = o.density_splat(mc, sc.geom)
    return float(np.mean((f - target.astype(np.float64)) ** 2))


def _gpu_grad(sc, mc, target, steps, every=6, tape_budget=0, info=None):
    from fluidsph.adjoint import DifferentiableRollout
    sim = gpu_sim_for_scene(sc)
    r = DifferentiableRollout(sim, every, tape_budget_bytes=tape_budget)
    r.forward(steps)
    loss = r.splat_mse_loss(mc, sc.geom, target)
    dpos, dvel, dpar = r.backward()
    full = r.param_gradients()
    # the five-parameter read-out repeats the backward's three
    assert np.array_equal(full[:, :3], dpar)
    if info is not None:
        info.append(r.tape_info())
    return loss, dpos.astype(np.float64), dvel.astype(np.float64), full


def _tangent(oracle_mod, sc, mc, target, steps, precision, **seed):
    return oracle_mod.tangent_rollout_loss(sc.particles, sc.sph, sc.geom, sc.gravity,
                                           sc.iterations, steps, mc, target,
                                           precision=precision, **seed)[1]


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.fixture(scope="module", params=[20, 5])
def smooth(request, oracle_mod):
    from fluidsph import scenes
    sc = scenes.reference_physics_rollout(steps=request.param)
    mc = scenes.loss_grid(sc, 48)
    target = _target(oracle_mod, sc, mc, sc.steps, viscosity=0.5)
    grads = _gpu_grad(sc, mc, target, sc.steps)
    return sc, mc, target, grads


def test_smooth_loss_matches_oracle(smooth, oracle_mod):
    sc, mc, target, (loss, *_ ) = smooth
    ref = _oracle_loss(oracle_mod, sc, mc, target, sc.steps)
    assert loss > 0 and _rel(loss, ref) < 1e-4, (loss, ref)


def _fd(oracle_mod, sc, mc, target, kw, base, rel_eps=1e-4):
    eps = rel_eps * abs(base)
    return (_oracle_loss(oracle_mod, sc, mc, target, sc.steps, **{kw: base + eps}) -
            _oracle_loss(oracle_mod, sc, mc, target, sc.steps, **{kw: base - eps})) / (2 * eps)


def test_smooth_parameter_gradients(smooth, oracle_mod):
    """Every gradient equals the FP32 tangent of the same trajectory; against
    the FP64 tangent and FD64 (eps 1e-4): viscosity over 20 steps, both
    parameters over 5. Over 20 steps the surface-tension gradient is a small
    remainder of cancelling contributions (about 3e9 per step at step 5 down
    to 7e6), which FP32 and FP64 trajectories resolve only to about 0.5%."""
    sc, mc, target, (_, _, _, dpar) = smooth
    assert dpar[0, 1] == 0.0  # stiffness: read by no stage
    for idx, name, kw in ((0, "viscosity", "visc"), (2, "surface_tension", "st")):
        seed = {"dvisc": 1.0} if idx == 0 else {"dst": 1.0}
        t32 = _tangent(oracle_mod, sc, mc, target, sc.steps, 32, **seed)
        t64 = _tangent(oracle_mod, sc, mc, target, sc.steps, 64, **seed)
        fd = _fd(oracle_mod, sc, mc, target, kw, getattr(sc.sph, name))
        g = dpar[0, idx]
        print(f"{sc.steps} steps dL/d{name}: reverse {g:.8e} tangent32 {t32:.8e} "
              f"tangent64 {t64:.8e} FD64 {fd:.8e}")
        assert _rel(g, t32) < EXACT_RTOL
        if idx == 0 or sc.steps <= 5:
            assert _rel(g, t64) < GRAD_RTOL
            assert _rel(g, fd) < FD_RTOL


def test_smooth_pressure_parameter_gradients(smooth, oracle_mod):
    """dL/dnear_stiffness and dL/dpcisph_delta (the pressure strength the
    step actually reads) equal the FP32 tangent of the same trajectory; over
    5 steps they also match the FP64 tangent and FD64 (eps 1e-4)."""
    sc, mc, target, (_, _, _, dpar) = smooth
    for idx, name, kw, seed in ((3, "near_stiffness", "near", "dnear"),
                                (4, "pcisph_delta", "delta", "ddelta")):
        t32 = _tangent(oracle_mod, sc, mc, target, sc.steps, 32, **{seed: 1.0})
        t64 = _tangent(oracle_mod, sc, mc, target, sc.steps, 64, **{seed: 1.0})
        fd = _fd(oracle_mod, sc, mc, target, kw, getattr(sc.sph, name))
        g = dpar[0, idx]
        print(f"{sc.steps} steps dL/d{name}: reverse {g:.8e} tangent32 {t32:.8e} "
              f"tangent64 {t64:.8e} FD64 {fd:.8e}")
        assert g != 0.0
        assert _rel(g, t32) < EXACT_RTOL
        if sc.steps <= 5:
            assert _rel(g, t64) < GRAD_RTOL
            assert _rel(g, fd) < FD_RTOL


def test_smooth_state_gradients(smooth, oracle_mod):
    sc, mc, target, (_, dpos, dvel, _) = smooth
    rng = np.random.default_rng(11)
    v0 = sc.particles[:, 4:7].astype(np.float64)
    for trial in range(2):
        d = rng.standard_normal(v0.shape)
        d /= np.linalg.norm(d)
        eps = 1e-4
        fd = (_oracle_loss(oracle_mod, sc, mc, target, sc.steps, vel=v0 + eps * d) -
              _oracle_loss(oracle_mod, sc, mc, target, sc.steps, vel=v0 - eps * d)) / (2 * eps)
        t32 = _tangent(oracle_mod, sc, mc, target, sc.steps, 32, dvel=d)
        t64 = _tangent(oracle_mod, sc, mc, target, sc.steps, 64, dvel=d)
        g = float(np.sum(dvel * d))
        print(f"{sc.steps} steps velocity direction {trial}: reverse {g:.8e} tangent32 {t32:.8e} "
              f"tangent64 {t64:.8e} FD64 {fd:.8e}")
        assert _rel(g, t32) < EXACT_RTOL
        if sc.steps <= 5:
            assert _rel(g, t64) < GRAD_RTOL
            assert _rel(g, fd) < FD_RTOL
        dp = rng.standard_normal(v0.shape)
        dp /= np.linalg.norm(dp)
        tp = _tangent(oracle_mod, sc, mc, target, sc.steps, 32, dpos=dp)
        gp = float(np.sum(dpos * dp))
        print(f"{sc.steps} steps position direction {trial}: reverse {gp:.8e} tangent32 {tp:.8e}")
        assert _rel(gp, tp) < EXACT_RTOL


@pytest.mark.parametrize("steps", [1, 2])
def test_workload_copy_exact_derivative(oracle_mod, steps):
    from fluidsph import scenes
    sc = scenes.config3_small()
    mc = scenes.loss_grid(sc)
    target = _target(oracle_mod, sc, mc, steps, viscosity=12.0, stiffness=30.0)
    _, dpos, dvel, dpar = _gpu_grad(sc, mc, target, steps, every=1)
    assert dpar[0, 1] == 0.0
    assert _rel(dpar[0, 0], _tangent(oracle_mod, sc, mc, target, steps, 32, dvisc=1.0)) < EXACT_RTOL
    assert _rel(dpar[0, 2], _tangent(oracle_mod, sc, mc, target, steps, 32, dst=1.0)) < EXACT_RTOL
    assert _rel(dpar[0, 3], _tangent(oracle_mod, sc, mc, target, steps, 32, dnear=1.0)) < EXACT_RTOL
    assert _rel(dpar[0, 4], _tangent(oracle_mod, sc, mc, target, steps, 32, ddelta=1.0)) < EXACT_RTOL
    d = np.random.default_rng(3).standard_normal(dvel.shape)
    d /= np.linalg.norm(d)
    t = _tangent(oracle_mod, sc, mc, target, steps, 32, dvel=d)
    assert _rel(float(np.sum(dvel * d)), t) < EXACT_RTOL


def test_backward_deterministic_and_checkpoint_independent(smooth):
    sc, mc, target, (_, dpos, dvel, dpar) = smooth
    _, dpos2, dvel2, dpar2 = _gpu_grad(sc, mc, target, sc.steps, every=6)
    assert np.array_equal(dpos, dpos2) and np.array_equal(dvel, dvel2)
    assert np.array_equal(dpar, dpar2)
    _, dpos3, dvel3, dpar3 = _gpu_grad(sc, mc, target, sc.steps, every=20)
    assert np.array_equal(dvel, dvel3) and np.array_equal(dpar, dpar3)


def test_tape_budget_keeps_gradients(smooth):
    """With a tape budget the forward records several segments and the
    backward reverses them without re-running them: same bits."""
    sc, mc, target, (loss, dpos, dvel, dpar) = smooth
    info = []
    loss2, dpos2, dvel2, dpar2 = _gpu_grad(sc, mc, target, sc.steps, every=6, info=info)
    assert info[-1][0] == 1 and info[-1][1] > 0  # default: one segment
    segs = -(-sc.steps // 6)
    loss3, dpos3, dvel3, dpar3 = _gpu_grad(sc, mc, target, sc.steps, every=6,
                                           tape_budget=info[-1][1] * segs, info=info)
    assert info[-1][0] == segs
    assert loss3 == loss and np.array_equal(dpos, dpos3) and np.array_equal(dvel, dvel3)
    assert np.array_equal(dpar, dpar3)
    # a budget of two segments: the last two recorded, the others re-run
    loss4, dpos4, dvel4, dpar4 = _gpu_grad(sc, mc, target, sc.steps, every=6,
                                           tape_budget=info[-1][1] * 2, info=info)
    assert info[-1][0] == min(2, segs)
    assert np.array_equal(dpos, dpos4) and np.array_equal(dpar, dpar4)
