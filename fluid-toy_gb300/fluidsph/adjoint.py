"""Reverse-mode differentiation of a rollout (fs_adj_*): the counterpart of a
``torch.autograd.Function`` over ``SphSimulation3DGrid.step``.

``DifferentiableRollout.forward(nsteps)`` records (checkpointing the state
every ``checkpoint_every`` steps); ``backward()`` consumes cotangents of the
final canonical state, set directly or through ``splat_mse_loss`` (the mean
squared difference of the marching-cubes density splat against a target
field), and returns dL/dpos0, dL/dvel0 as (N, 3) arrays and dL/d(viscosity,
stiffness, surface_tension) per scene. ``rollout_function`` wraps the same
calls as a torch.autograd.Function over the initial velocities and the
viscosity / surface tension.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .abi import check


class DifferentiableRollout:
    def __init__(self, sim, checkpoint_every: int = 20, tape_budget_bytes: int = 0):
        self._lib = abi.load()
        self.sim = sim
        h = C.c_void_p()
        check(self._lib.fs_adj_create(sim._h, int(checkpoint_every), C.byref(h)))
        self._h = h
        sim._register(self)
        if tape_budget_bytes:
            self.set_tape_budget(tape_budget_bytes)

    def set_tape_budget(self, nbytes: int) -> None:
        """Device memory the tape may take (fs_adj_set_tape_budget): segments
        that fit are recorded during forward() and not re-run by backward()."""
        check(self._lib.fs_adj_set_tape_budget(self._h, int(nbytes)))

    def tape_info(self) -> tuple[int, int]:
        """(tape segments of the last forward, bytes per segment)."""
        n = C.c_uint32()
        b = C.c_uint64()
        check(self._lib.fs_adj_tape_info(self._h, C.byref(n), C.byref(b)))
        return n.value, b.value

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.fs_adj_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, nsteps: int) -> None:
        check(self._lib.fs_adj_forward(self._h, int(nsteps)))

    @staticmethod
    def _rows(x):
        """(pointer, on_device, keepalive) of an (N, 3) float32 array or CUDA tensor."""
        if x is None:
            return None, 0, None
        if hasattr(x, "data_ptr") and getattr(x, "is_cuda", False):
            t = x.detach().to(dtype=__import__("torch").float32).contiguous()
            return t.data_ptr(), 1, t
        a = np.ascontiguousarray(x, np.float32).reshape(-1, 3)
        return a.ctypes.data, 0, a

    def set_cotangents(self, dl_dpos=None, dl_dvel=None) -> None:
        p, dev_p, kp = self._rows(dl_dpos)
        v, dev_v, kv = self._rows(dl_dvel)
        if p is not None and v is not None and dev_p != dev_v:
            raise ValueError("both cotangents on the host or both on the device")
        check(self._lib.fs_adj_set_cotangents(self._h, p, v, dev_p or dev_v))

    def splat_mse_loss(self, mc_params, container_geom, target, scene: int = 0) -> float:
        loss = C.c_double()
        if hasattr(target, "data_ptr") and getattr(target, "is_cuda", False):
            t = target.detach().float().contiguous()
            check(self._lib.fs_adj_splat_mse_loss(self._h, int(scene), C.byref(mc_params),
                                                  C.byref(container_geom), t.data_ptr(), 1,
                                                  C.byref(loss)))
        else:
            t = np.ascontiguousarray(target, np.float32)
            check(self._lib.fs_adj_splat_mse_loss(self._h, int(scene), C.byref(mc_params),
                                                  C.byref(container_geom), t.ctypes.data, 0,
                                                  C.byref(loss)))
        return loss.value

    def splat_mse_losses(self, mc_params, container_geoms, targets, scenes=None) -> np.ndarray:
        """splat_mse_loss for several scenes at once (fs_adj_splat_mse_losses:
        one grid build, one read-back): per scene k its grid mc_params[k],
        geometry container_geoms[k] and target targets[k] (all numpy arrays or
        all CUDA tensors); returns the losses."""
        n = len(targets)
        sc = list(range(n)) if scenes is None else [int(k) for k in scenes]
        if n == 0:
            return np.zeros(0, np.float64)
        if not (len(mc_params) == len(container_geoms) == len(sc) == n):
            raise ValueError("splat_mse_losses: one grid, geometry, target and scene per loss")
        grids = (type(mc_params[0]) * n)(*mc_params)
        geoms = (type(container_geoms[0]) * n)(*container_geoms)
        on_device = all(hasattr(t, "data_ptr") and getattr(t, "is_cuda", False) for t in targets)
        if on_device:
            keep = [t.detach().float().contiguous() for t in targets]
            ptrs = (C.c_void_p * n)(*[t.data_ptr() for t in keep])
        else:
            keep = [np.ascontiguousarray(t, np.float32) for t in targets]
            ptrs = (C.c_void_p * n)(*[t.ctypes.data for t in keep])
        out = np.zeros(n, np.float64)
        check(self._lib.fs_adj_splat_mse_losses(
            self._h, n, (C.c_uint32 * n)(*sc), grids, geoms, ptrs, 1 if on_device else 0,
            out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def final_splat(self, mc_params, container_geom, scene: int = 0) -> np.ndarray:
        """Density splat of the recorded rollout's final positions, (gs, gs, gs)."""
        gs = int(mc_params.grid_size)
        out = np.empty((gs, gs, gs), np.float32)
        check(self._lib.fs_adj_final_splat(self._h, int(scene), C.byref(mc_params),
                                           C.byref(container_geom), out.ctypes.data, 0))
        return out

    def backward(self, scenes: int = 1):
        n = self.sim.num_particles()
        dpos = np.empty((n, 3), np.float32)
        dvel = np.empty((n, 3), np.float32)
        dpar = np.zeros((scenes, 3), np.float64)
        check(self._lib.fs_adj_backward(self._h, dpos.ctypes.data, dvel.ctypes.data, 0,
                                        dpar.ctypes.data))
        return dpos, dvel, dpar

    PARAM_NAMES = ("viscosity", "stiffness", "surface_tension", "near_stiffness", "pcisph_delta")

    def param_gradients(self, scenes: int = 1) -> np.ndarray:
        """(scenes, 5) float64 gradients of the last backward() with respect
        to PARAM_NAMES (fs_adj_param_gradients)."""
        out = np.zeros((scenes, len(self.PARAM_NAMES)), np.float64)
        check(self._lib.fs_adj_param_gradients(self._h, out.ctypes.data, int(scenes)))
        return out


def rollout_function():
    """torch.autograd.Function: (vel0 (N,3), viscosity, surface_tension) ->
    final positions (N,3) of a plain simulation, with the backward through
    fs_adj_backward. Call as ``Fn.apply(vel0, visc, st, sim, base_particles,
    sph_params, nsteps, checkpoint_every)``."""
    import copy

    import torch

    from .abi import COL_VEL

    class Fn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, vel0, visc, st, sim, base_particles, sph_params, nsteps, every):
            parts = np.array(base_particles, np.float32, copy=True)
            parts[:, COL_VEL] = vel0.detach().cpu().numpy()
            p = copy.copy(sph_params)
            p.viscosity = float(visc)
            p.surface_tension = float(st)
            sim.update_sph_params(p)
            sim.upload_particles(parts)
            rollout = DifferentiableRollout(sim, int(every))
            rollout.forward(int(nsteps))
            ctx.rollout = rollout
            out = sim.particles()[:, 0:3]
            return torch.from_numpy(out.copy()).to(vel0.device)

        @staticmethod
        def backward(ctx, grad_pos):
            r = ctx.rollout
            r.set_cotangents(grad_pos.detach().cpu().numpy(), None)
            _, dvel, dpar = r.backward()
            r.close()
            dev = grad_pos.device
            return (torch.from_numpy(dvel).to(dev), torch.tensor(dpar[0, 0], device=dev),
                    torch.tensor(dpar[0, 2], device=dev), None, None, None, None, None)

    return Fn
