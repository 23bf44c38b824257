"""Python mirror of the reference's ``SphSimulation3DGrid``
(src/simulation/sph_3d_grid.rs:33-1569) over the C ABI of libfluidsph.so.

Method names and argument meaning follow the Rust type: ``new`` becomes the
constructor, ``step`` runs one substep (or ``nsteps``), the ``update_*``
methods upload parameter structs, ``set_pcisph_iterations`` clamps to >= 1,
``read_rigid_body_accum`` synchronises, ``spawn_particles`` clips at capacity.
Read-outs return numpy arrays. Errors raise ``FluidSphError`` (the reference
panics on wgpu validation errors; this library reports a status instead).
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import abi
from .abi import (FS_ABI_VERSION, FS_STAGE_COUNT, FS_STAT_COUNT, FsSceneInfo,
                  GpuContainerGeometry, GpuGravity, GpuGridParams, GpuMouseForce, GpuRigidBody,
                  GpuRigidBodyAccum, GpuSphParams3D, check)


class SphSimulation3DGrid:
    def __init__(self, particles: np.ndarray, sph_params: GpuSphParams3D,
                 container_geom: GpuContainerGeometry, max_particles: int = 0,
                 sdf: np.ndarray | None = None, device: int = 0):
        self._lib = abi.load()
        parts = abi.as_particles(particles) if len(particles) else np.zeros((0, 16), np.float32)
        self._parts_keep = parts
        sdf_ptr, sdf_res = None, 0
        if sdf is not None:
            sdf = np.ascontiguousarray(sdf, dtype=np.float32)
            sdf_res = int(round(sdf.size ** (1.0 / 3.0)))
            if sdf_res ** 3 != sdf.size:
                raise ValueError("sdf must hold res^3 values")
            sdf_ptr = sdf.ctypes.data
        h = C.c_void_p()
        check(self._lib.fs_create(parts.ctypes.data if len(parts) else None, len(parts),
                                  C.byref(sph_params), C.byref(container_geom),
                                  int(max_particles), sdf_ptr, sdf_res, int(device),
                                  FS_ABI_VERSION, C.byref(h)))
        self._h = h
        self._grid = GpuGridParams()
        check(self._lib.fs_grid_params(self._h, C.byref(self._grid)))

    # -- lifetime ---------------------------------------------------------------
    def _register(self, dependent) -> None:
        """Objects built on this simulation (rollouts, spray systems) are
        closed before it: their C handles point into it."""
        if not hasattr(self, "_dependents"):
            self._dependents = []
        self._dependents.append(weakref.ref(dependent))

    def close(self) -> None:
        for ref in getattr(self, "_dependents", []):
            dep = ref()
            if dep is not None:
                dep.close()
        self._dependents = []
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.fs_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- step and parameter uploads (sph_3d_grid.rs:1261-1477) --------------------
    def step(self, nsteps: int = 1) -> None:
        check(self._lib.fs_step(self._h, int(nsteps)))

    def prepare_steps(self, nsteps: int) -> None:
        """Capture the step graphs ``step(nsteps)`` will replay."""
        check(self._lib.fs_prepare_steps(self._h, int(nsteps)))

    def update_sph_params(self, params: GpuSphParams3D) -> None:
        check(self._lib.fs_update_sph_params(self._h, C.byref(params)))

    def update_container_geometry(self, geom: GpuContainerGeometry) -> None:
        check(self._lib.fs_update_container_geometry(self._h, C.byref(geom)))

    def update_mouse_force(self, mouse: GpuMouseForce) -> None:
        check(self._lib.fs_update_mouse_force(self._h, C.byref(mouse)))

    def update_gravity(self, gravity: GpuGravity) -> None:
        check(self._lib.fs_update_gravity(self._h, C.byref(gravity)))

    def update_rigid_body(self, body: GpuRigidBody) -> None:
        check(self._lib.fs_update_rigid_body(self._h, C.byref(body)))

    def set_pcisph_iterations(self, iterations: int) -> None:
        check(self._lib.fs_set_pcisph_iterations(self._h, int(iterations)))

    def clear_rigid_body_accum(self) -> None:
        check(self._lib.fs_clear_rigid_body_accum(self._h))

    def read_rigid_body_accum(self) -> GpuRigidBodyAccum:
        out = GpuRigidBodyAccum()
        check(self._lib.fs_read_rigid_body_accum(self._h, C.byref(out)))
        self._last_accum = out
        return out

    def rigid_body_accum(self) -> GpuRigidBodyAccum:
        return getattr(self, "_last_accum", GpuRigidBodyAccum())

    def num_particles(self) -> int:
        v = C.c_uint32()
        check(self._lib.fs_num_particles(self._h, C.byref(v)))
        return v.value

    def grid_params(self) -> GpuGridParams:
        g = GpuGridParams()
        check(self._lib.fs_grid_params(self._h, C.byref(g)))
        return g

    def spawn_particles(self, position, count: int, spread: float) -> int:
        pos = (C.c_float * 3)(*[float(v) for v in position])
        out = C.c_uint32()
        check(self._lib.fs_spawn_particles(self._h, pos, int(count), float(spread), C.byref(out)))
        return out.value

    def sync(self) -> None:
        check(self._lib.fs_sync(self._h))

    def set_stream(self, stream_ptr: int | None) -> None:
        check(self._lib.fs_set_stream(self._h, stream_ptr))

    # -- read-outs ------------------------------------------------------------------
    def particles(self, count: int | None = None) -> np.ndarray:
        n = self.num_particles() if count is None else int(count)
        out = np.empty((n, 16), np.float32)
        check(self._lib.fs_download_particles(self._h, out.ctypes.data, n))
        return out

    def load_batching(self) -> tuple[bool, bool]:
        """(batched candidate loads in use, choice measured yet): the density
        and solve kernel form the simulation picked (fs_load_batching)."""
        b, d = C.c_int(), C.c_int()
        check(self._lib.fs_load_batching(self._h, C.byref(b), C.byref(d)))
        return bool(b.value), bool(d.value)

    def kernel_forms(self) -> dict:
        """The neighbour passes' load depths and how they were chosen
        (fs_kernel_forms; waits for a pending measurement)."""
        f = abi.FsKernelForms()
        check(self._lib.fs_kernel_forms(self._h, C.byref(f)))
        return {"density_loads": f.density_loads, "solve_loads": f.solve_loads,
                "xsph_loads": f.xsph_loads,
                "decided": ("pending", "measured", "table", "set")[f.decided],
                "bucket": f.bucket, "ms": [list(row) for row in f.ms]}

    def set_kernel_forms(self, density_loads: int = -1, solve_loads: int = -1,
                         xsph_loads: int = -1) -> None:
        """Fix the load depths (no measurement, no host wait); all -1 to tune."""
        check(self._lib.fs_set_kernel_forms(self._h, int(density_loads), int(solve_loads),
                                            int(xsph_loads)))

    def export_particles_aos(self, device_ptr: int, count: int, sorted: bool = False,
                             scene: int = 0) -> None:
        """Write `count` 64-byte SphParticle3D records (canonical, or sorted
        slots) into device memory at `device_ptr`, asynchronously on the
        simulation's stream (fs_export_particles_aos)."""
        check(self._lib.fs_export_particles_aos(self._h, int(scene), 1 if sorted else 0,
                                                C.c_void_p(int(device_ptr)), int(count)))

    def upload_particles(self, particles: np.ndarray) -> None:
        p = abi.as_particles(particles)
        check(self._lib.fs_upload_particles(self._h, p.ctypes.data, len(p)))

    def sorted_particles(self, count: int | None = None) -> np.ndarray:
        n = self.num_particles() if count is None else int(count)
        out = np.empty((n, 16), np.float32)
        check(self._lib.fs_download_sorted(self._h, out.ctypes.data, n))
        return out

    def cells(self) -> tuple[np.ndarray, np.ndarray]:
        g = self._grid.total_cells
        counts = np.empty(g, np.uint32)
        starts = np.empty(g, np.uint32)
        check(self._lib.fs_download_cells(self._h, counts.ctypes.data, starts.ctypes.data, g))
        return counts, starts

    def index_maps(self) -> tuple[np.ndarray, np.ndarray]:
        n = self.num_particles()
        ci = np.empty(n, np.uint32)
        so = np.empty(n, np.uint32)
        check(self._lib.fs_download_index_maps(self._h, ci.ctypes.data, so.ctypes.data, n))
        return ci, so

    def density_splat(self, mc_params, container_geom, scene: int = 0,
                      out_device_ptr: int | None = None):
        """The MC density pass (mc_density.wgsl) over the last step's sorted
        positions: a (gs, gs, gs) float32 array indexed [z, y, x], or, with
        ``out_device_ptr``, written to that device memory asynchronously."""
        gs = int(mc_params.grid_size)
        if out_device_ptr is not None:
            check(self._lib.fs_density_splat(self._h, int(scene), C.byref(mc_params),
                                             C.byref(container_geom), int(out_device_ptr), 1))
            return None
        out = np.empty((gs, gs, gs), np.float32)
        check(self._lib.fs_density_splat(self._h, int(scene), C.byref(mc_params),
                                         C.byref(container_geom), out.ctypes.data, 0))
        return out

    # -- device-resident rigid-body coupling (app.rs:1205-1290 on the GPU) ---------
    def rigid_coupling_set_state(self, state, scene: int = 0) -> None:
        check(self._lib.fs_rigid_coupling_set_state(self._h, int(scene),
                                                    None if state is None else C.byref(state)))

    def rigid_coupling_get_state(self, scene: int = 0):
        out = abi.FsRigidBodyState()
        check(self._lib.fs_rigid_coupling_get_state(self._h, int(scene), C.byref(out)))
        return out

    def frames(self, substeps: int, frames: int = 1) -> None:
        check(self._lib.fs_frames(self._h, int(substeps), int(frames)))

    def device_pointers(self) -> abi.FsDevicePointers:
        p = abi.FsDevicePointers()
        check(self._lib.fs_device_pointers(self._h, C.byref(p)))
        return p

    # -- measurement ------------------------------------------------------------------
    def enable_stage_timing(self, enable: bool = True) -> None:
        check(self._lib.fs_enable_stage_timing(self._h, 1 if enable else 0))

    def stage_times(self, reset: bool = True) -> tuple[dict, int]:
        ms = (C.c_double * FS_STAGE_COUNT)()
        steps = C.c_uint32()
        check(self._lib.fs_stage_times(self._h, ms, C.byref(steps), 1 if reset else 0))
        return {name: ms[i] for i, name in enumerate(abi.STAGE_NAMES)}, steps.value

    def neighbor_stats(self, reset: bool = True) -> dict:
        out = (C.c_uint64 * FS_STAT_COUNT)()
        check(self._lib.fs_neighbor_stats(self._h, out, 1 if reset else 0))
        keys = ("cand_density", "hits_density", "hits_nonself", "cand_solve", "hits_solve",
                "coop_force")
        return {k: int(out[i]) for i, k in enumerate(keys)}


class SphBatch3DGrid(SphSimulation3DGrid):
    """Independent scenes stepped together (fs_batch_*): every stage is one
    launch over all scenes, and scene k evolves bit for bit like a
    ``SphSimulation3DGrid`` built from the same inputs. The simulation-wide
    methods (``step``, ``set_pcisph_iterations``, timing, statistics) are
    inherited; per-scene state goes through the ``*_scene`` methods."""

    def __init__(self, scenes_particles, sph_params, container_geoms, sdf=None, device: int = 0):
        self._lib = abi.load()
        counts = [len(p) for p in scenes_particles]
        if not counts:
            raise ValueError("a batch needs at least one scene")
        if not (len(sph_params) == len(container_geoms) == len(counts)):
            raise ValueError("one particle array, SphParams and geometry per scene")
        parts = np.concatenate([abi.as_particles(p) if len(p) else np.zeros((0, 16), np.float32)
                                for p in scenes_particles])
        self._parts_keep = parts
        c_counts = (C.c_uint32 * len(counts))(*counts)
        c_params = (GpuSphParams3D * len(counts))(*sph_params)
        c_geoms = (GpuContainerGeometry * len(counts))(*container_geoms)
        sdf_ptr, sdf_res = None, 0
        if sdf is not None:
            sdf = np.ascontiguousarray(sdf, dtype=np.float32)
            sdf_res = int(round(sdf.size ** (1.0 / 3.0)))
            if sdf_res ** 3 != sdf.size:
                raise ValueError("sdf must hold res^3 values")
            sdf_ptr = sdf.ctypes.data
        h = C.c_void_p()
        check(self._lib.fs_batch_create(parts.ctypes.data if len(parts) else None, c_counts,
                                        len(counts), C.cast(c_params, C.c_void_p),
                                        C.cast(c_geoms, C.c_void_p), sdf_ptr, sdf_res,
                                        int(device), FS_ABI_VERSION, C.byref(h)))
        self._h = h
        self.counts = counts

    def num_scenes(self) -> int:
        v = C.c_uint32()
        check(self._lib.fs_batch_num_scenes(self._h, C.byref(v)))
        return v.value

    def scene_info(self, scene: int) -> FsSceneInfo:
        out = FsSceneInfo()
        check(self._lib.fs_batch_scene_info(self._h, int(scene), C.byref(out)))
        return out

    def update_scene(self, scene: int, sph_params=None, container_geom=None, gravity=None,
                     mouse=None, rigid_body=None) -> None:
        ref = lambda x: C.byref(x) if x is not None else None
        check(self._lib.fs_batch_update_scene(self._h, int(scene), ref(sph_params),
                                              ref(container_geom), ref(gravity), ref(mouse),
                                              ref(rigid_body)))

    def read_rigid_body_accums(self) -> list:
        n = self.num_scenes()
        out = (GpuRigidBodyAccum * n)()
        check(self._lib.fs_batch_read_rigid_body_accum(self._h, C.cast(out, C.c_void_p), n))
        return list(out)

    def scene_particles(self, scene: int, count: int | None = None) -> np.ndarray:
        n = self.scene_info(scene).num_particles if count is None else int(count)
        out = np.empty((n, 16), np.float32)
        check(self._lib.fs_batch_download_scene(self._h, int(scene), out.ctypes.data, n))
        return out

    def scene_sorted_particles(self, scene: int, count: int | None = None) -> np.ndarray:
        n = self.scene_info(scene).active_particles if count is None else int(count)
        out = np.empty((n, 16), np.float32)
        check(self._lib.fs_batch_download_scene_sorted(self._h, int(scene), out.ctypes.data, n))
        return out

    def scene_cells(self, scene: int) -> tuple[np.ndarray, np.ndarray]:
        g = self.scene_info(scene).total_cells
        counts = np.empty(g, np.uint32)
        starts = np.empty(g, np.uint32)
        check(self._lib.fs_batch_download_scene_cells(self._h, int(scene), counts.ctypes.data,
                                                      starts.ctypes.data, g))
        return counts, starts

    def scene_index_maps(self, scene: int) -> tuple[np.ndarray, np.ndarray]:
        n = self.scene_info(scene).active_particles
        ci = np.empty(n, np.uint32)
        so = np.empty(n, np.uint32)
        check(self._lib.fs_batch_download_scene_index_maps(self._h, int(scene), ci.ctypes.data,
                                                           so.ctypes.data, n))
        return ci, so

    def upload_scene_particles(self, scene: int, particles: np.ndarray) -> None:
        p = abi.as_particles(particles)
        check(self._lib.fs_batch_upload_scene(self._h, int(scene), p.ctypes.data, len(p)))


def kernel_forms_table() -> list[dict]:
    """The process-wide per-bucket table of load depths (fs_kernel_forms_table)."""
    lib = abi.load()
    n = C.c_uint32()
    check(lib.fs_kernel_forms_table(None, 0, C.byref(n)))
    arr = (abi.FsKernelFormsEntry * max(n.value, 1))()
    check(lib.fs_kernel_forms_table(arr, n.value, C.byref(n)))
    return [{"bucket": e.bucket, "many_scenes": bool(e.many_scenes), "iterations": e.iterations,
             "density_loads": e.density_loads, "solve_loads": e.solve_loads,
             "xsph_loads": e.xsph_loads,
             "ms": {"density": [round(x, 3) for x in e.ms[0]], "xsph": [round(x, 3) for x in e.ms[1]],
                    "solve": [round(x, 3) for x in e.ms[2]]}}
            for e in arr[:n.value]]
