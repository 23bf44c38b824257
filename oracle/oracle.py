"""ctypes wrapper of the CPU oracle (oracle/sph_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check in
__graft_entry__.py and by bench.py's CPU-baseline and reference arms, as the
checker or the timed CPU baseline — never by the product path.

``build()`` compiles the FP32 restatement and its FP64 twin (one source,
template on the arithmetic type) into ``oracle/liboracle.so`` with
``-ffp-contract=off`` so results are identical on x86-64 and aarch64.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "sph_oracle.cpp"
LIB = HERE / "liboracle.so"

CXXFLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
            "-shared"]


def build(force: bool = False) -> Path:
    deps = [SRC, HERE / "dual.hpp"]
    if not force and LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    cxx = shutil.which("g++") or "c++"
    tmp = LIB.with_suffix(".so.tmp")
    r = subprocess.run([cxx, *CXXFLAGS, "-o", str(tmp), str(SRC)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


_lib = None
_ref_lib = None
REF_LIB = HERE / "_ref" / "libref.so"


def load_ref():
    """The reference's own step shaders translated to C++ (oracle/_ref), or
    None when they are not built (the reference sources are needed once)."""
    global _ref_lib
    if _ref_lib is None:
        try:
            import importlib.util
            spec = importlib.util.spec_from_file_location("build_ref", HERE / "build_ref.py")
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build(quiet=True)
        except Exception:
            pass
        if not REF_LIB.exists():
            return None
        _ref_lib = _bind(C.CDLL(str(REF_LIB)))
    return _ref_lib


_ref_host = None
REF_HOST_LIB = HERE / "_ref" / "libref_host.so"


def load_ref_host():
    """The reference's host functions (parameter builders, rigid-body
    integration, spawning) translated from its Rust sources (oracle/_ref), or
    None when they are not built (the reference sources are needed once)."""
    global _ref_host
    if _ref_host is None:
        try:
            import importlib.util
            spec = importlib.util.spec_from_file_location("build_ref", HERE / "build_ref.py")
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build_host(quiet=True)
        except Exception:
            pass
        if not REF_HOST_LIB.exists():
            return None
        lib = C.CDLL(str(REF_HOST_LIB))
        f, u32, vp, i = C.c_float, C.c_uint32, C.c_void_p, C.c_int
        fp = C.POINTER(C.c_float)
        lib.rh_compute_rest_density.restype = f
        lib.rh_compute_rest_density.argtypes = [f, f]
        lib.rh_compute_pcisph_delta.restype = f
        lib.rh_compute_pcisph_delta.argtypes = [f, f, f, f]
        lib.rh_to_gpu_params_3d.argtypes = [f, f, f, f, f, f, f, u32, f, vp]
        lib.rh_to_gpu_geometry.argtypes = [fp, f, f, i, f, vp]
        lib.rh_quat_to_rotation_rows.argtypes = [fp, fp]
        lib.rh_to_gpu_rigid_body.argtypes = [vp, f, vp]
        lib.rh_integrate_rigid_body.argtypes = [vp, fp, f, u32, fp, vp]
        lib.rh_clamp_rigid_body.argtypes = [vp, fp, i]
        lib.rh_spawn_particles.restype = u32
        lib.rh_spawn_particles.argtypes = [u32, u32, fp, u32, f, vp, C.POINTER(u32)]
        _ref_host = lib
    return _ref_host


def load():
    global _lib
    if _lib is None:
        build()
        _lib = _bind(C.CDLL(str(LIB)))
    return _lib


def _bind(lib):
    if True:
        vp, u32 = C.c_void_p, C.c_uint32
        lib.or_create.restype = vp
        lib.or_create.argtypes = [vp, u32, vp, vp, u32, vp, u32, C.c_int]
        lib.or_destroy.argtypes = [vp]
        lib.or_step.argtypes = [vp, u32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        lib.or_stage.argtypes = [vp, C.c_int, u32]
        for name in ("or_set_params", "or_set_geometry", "or_set_mouse", "or_set_rigid",
                     "or_get_accum", "or_get_grid"):
            getattr(lib, name).argtypes = [vp, vp]
        lib.or_set_gravity.argtypes = [vp, C.POINTER(C.c_float)]
        lib.or_set_iterations.argtypes = [vp, u32]
        if hasattr(lib, "or_set_cells_f32"):  # the restatement only
            lib.or_set_cells_f32.argtypes = [vp, C.c_int]
            lib.or_track_terms.argtypes = [vp, C.c_int]
            lib.or_get_term_magnitudes.argtypes = [vp, vp, u32]
        lib.or_clear_accum.argtypes = [vp]
        lib.or_get_particles.argtypes = [vp, vp, u32]
        lib.or_get_sorted.argtypes = [vp, vp, u32]
        lib.or_get_particles_f64.argtypes = [vp, vp, u32, C.c_int]
        lib.or_get_cells.argtypes = [vp, vp, vp]
        lib.or_get_index_maps.argtypes = [vp, vp, vp, u32]
        lib.or_get_predicted.argtypes = [vp, C.c_int, vp, u32]
        lib.or_sincos_f32.argtypes = [vp, vp, vp, u32]
        lib.or_set_threads.argtypes = [C.c_int]
        lib.or_density_splat.argtypes = [vp, vp, vp, vp]
        if hasattr(lib, "or_spray_frame"):
            lib.or_spray_frame.argtypes = [vp, vp, vp, vp, vp, vp]
        if hasattr(lib, "or_tangent_rollout_loss"):
            lib.or_tangent_rollout_loss.argtypes = [vp, u32, vp, vp, vp, u32, u32, vp, vp,
                                                    C.c_double, C.c_double, C.c_double,
                                                    C.c_double, vp, vp, C.c_int,
                                                    C.POINTER(C.c_double),
                                                    C.POINTER(C.c_double)]
        lib.or_max_threads.restype = C.c_int
    return lib


def sincos_f32(x: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """The FP32 sin/cos the restatement (and the GPU) use for the close-pair
    direction."""
    x = np.ascontiguousarray(x, np.float32)
    s = np.empty_like(x)
    c = np.empty_like(x)
    load().or_sincos_f32(x.ctypes.data, s.ctypes.data, c.ctypes.data, x.size)
    return s, c


def tangent_rollout_loss(particles, sph_params, container_geom, gravity, iterations: int,
                         steps: int, mc_params, target, dpos=None, dvel=None,
                         dvisc: float = 0.0, dst: float = 0.0, dnear: float = 0.0,
                         ddelta: float = 0.0, precision: int = 32):
    """(L, dL) of L = mean((splat(x_T) - target)^2) after `steps` steps, with
    dL its forward-mode derivative along (dpos, dvel, dvisc, dst, dnear,
    ddelta) (viscosity, surface tension, near stiffness, PCISPH delta): the
    oracle on dual numbers (precision 32: the FP32 restatement's own
    trajectory)."""
    lib = load()
    parts = np.ascontiguousarray(particles, np.float32)
    g = (C.c_float * 3)(*gravity.direction)
    t = np.ascontiguousarray(target, np.float32)
    dp = None if dpos is None else np.ascontiguousarray(dpos, np.float64)
    dv = None if dvel is None else np.ascontiguousarray(dvel, np.float64)
    loss, dloss = C.c_double(), C.c_double()
    lib.or_tangent_rollout_loss(parts.ctypes.data, len(parts), C.addressof(sph_params),
                                C.addressof(container_geom), g, int(iterations), int(steps),
                                None if dp is None else dp.ctypes.data,
                                None if dv is None else dv.ctypes.data, float(dvisc),
                                float(dst), float(dnear), float(ddelta), C.addressof(mc_params),
                                t.ctypes.data,
                                int(precision), C.byref(loss), C.byref(dloss))
    return loss.value, dloss.value


def set_threads(n: int) -> int:
    lib = load()
    lib.or_set_threads(int(n))
    return int(lib.or_max_threads())


class OracleSim:
    """The reference step on the CPU, precision 32 (FP32 restatement) or 64
    (FP64 twin). Same method names as fluidsph.sim.SphSimulation3DGrid."""

    def __init__(self, particles: np.ndarray, sph_params, container_geom, max_particles: int = 0,
                 sdf: np.ndarray | None = None, precision: int = 32, lib=None):
        self._lib = lib if lib is not None else load()
        parts = np.ascontiguousarray(particles, np.float32)
        self._n = len(parts)
        sdf_ptr, res = None, 0
        if sdf is not None:
            sdf = np.ascontiguousarray(sdf, np.float32)
            res = int(round(sdf.size ** (1 / 3)))
            sdf_ptr = sdf.ctypes.data
        self._h = self._lib.or_create(parts.ctypes.data if self._n else None, self._n,
                                      C.addressof(sph_params), C.addressof(container_geom),
                                      int(max_particles), sdf_ptr, res, int(precision))
        self.precision = precision
        self.last_candidates = 0
        self.last_hits = 0

    def close(self):
        if getattr(self, "_h", None):
            self._lib.or_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, nsteps: int = 1):
        cand, hits = C.c_uint64(), C.c_uint64()
        self._lib.or_step(self._h, int(nsteps), C.byref(cand), C.byref(hits))
        self.last_candidates, self.last_hits = cand.value, hits.value

    def stage(self, stage: int, arg: int = 0):
        self._lib.or_stage(self._h, int(stage), int(arg))

    def update_sph_params(self, p):
        self._lib.or_set_params(self._h, C.addressof(p))

    def update_container_geometry(self, g):
        self._lib.or_set_geometry(self._h, C.addressof(g))

    def update_gravity(self, g):
        arr = (C.c_float * 3)(*g.direction)
        self._lib.or_set_gravity(self._h, arr)

    def update_mouse_force(self, m):
        self._lib.or_set_mouse(self._h, C.addressof(m))

    def update_rigid_body(self, b):
        self._lib.or_set_rigid(self._h, C.addressof(b))

    def set_pcisph_iterations(self, k: int):
        self._lib.or_set_iterations(self._h, int(k))

    def track_terms(self, on: bool = True):
        """Keep, per particle, the sums of the magnitudes of the terms that
        the force pass, the last PCISPH iteration and the Akinci normal add
        (see term_magnitudes)."""
        self._lib.or_track_terms(self._h, 1 if on else 0)

    def term_magnitudes(self) -> np.ndarray:
        """(N, 3) float64, canonical order: sum over the force pass's pair
        terms of their magnitudes (plus |gravity|), the same for the last
        PCISPH iteration's pressure acceleration, and for the Akinci normal
        (scaled like the normal). Comparing them with the magnitude of the
        result gives the conditioning of each computed sum."""
        out = np.zeros((self._n, 3), np.float64)
        self._lib.or_get_term_magnitudes(self._h, out.ctypes.data, self._n)
        return out

    def set_cells_f32(self, on: bool = True):
        """Hash cells in FP32 arithmetic (for the FP64 twin): the integer
        stages then follow the FP32 pipeline's decisions."""
        self._lib.or_set_cells_f32(self._h, 1 if on else 0)

    def clear_rigid_body_accum(self):
        self._lib.or_clear_accum(self._h)

    def read_rigid_body_accum(self) -> tuple:
        out = (C.c_int32 * 8)()
        self._lib.or_get_accum(self._h, out)
        return tuple(out[:7])

    def particles(self) -> np.ndarray:
        out = np.empty((self._n, 16), np.float32)
        self._lib.or_get_particles(self._h, out.ctypes.data, self._n)
        return out

    def sorted_particles(self) -> np.ndarray:
        out = np.empty((self._n, 16), np.float32)
        self._lib.or_get_sorted(self._h, out.ctypes.data, self._n)
        return out

    def particles_f64(self, sorted_: bool = False) -> np.ndarray:
        out = np.empty((self._n, 14), np.float64)
        self._lib.or_get_particles_f64(self._h, out.ctypes.data, self._n, 1 if sorted_ else 0)
        return out

    def grid(self):
        from_buf = (C.c_uint32 * 12)()
        self._lib.or_get_grid(self._h, from_buf)
        return list(from_buf)

    def cells(self) -> tuple[np.ndarray, np.ndarray]:
        g = self.grid()[3]
        counts = np.empty(g, np.uint32)
        starts = np.empty(g, np.uint32)
        self._lib.or_get_cells(self._h, counts.ctypes.data, starts.ctypes.data)
        return counts, starts

    def index_maps(self) -> tuple[np.ndarray, np.ndarray]:
        ci = np.empty(self._n, np.uint32)
        so = np.empty(self._n, np.uint32)
        self._lib.or_get_index_maps(self._h, ci.ctypes.data, so.ctypes.data, self._n)
        return ci, so

    def density_splat(self, mc_params, container_geom) -> np.ndarray:
        """The MC density field (mc_density.wgsl) of the last step's sorted
        positions, shape (gs, gs, gs) indexed [z, y, x]; float64 (the FP32
        path's values are exact in it)."""
        gs = int(mc_params.grid_size)
        out = np.empty((gs, gs, gs), np.float64)
        self._lib.or_density_splat(self._h, C.addressof(mc_params), C.addressof(container_geom),
                                   out.ctypes.data)
        return out

    def spray_frame(self, params, ring: np.ndarray, head: int, limits) -> tuple:
        """One whitewater frame on `ring` (structured GpuSprayParticle array,
        modified in place); returns (head, limits, live counts)."""
        h = C.c_uint32(head)
        lim = (C.c_float * 2)(*limits)
        live = (C.c_uint32 * 4)()
        self._lib.or_spray_frame(self._h, C.addressof(params), ring.ctypes.data, C.byref(h), lim,
                                 live)
        return h.value, (lim[0], lim[1]), np.array(live, np.uint32)

    def predicted(self, which: int) -> np.ndarray:
        out = np.empty((self._n, 8), np.float32)
        self._lib.or_get_predicted(self._h, int(which), out.ctypes.data, self._n)
        return out


def oracle_for_scene(scene, precision: int = 32, lib=None, sdf=None) -> OracleSim:
    """An oracle simulation configured like a fluidsph.scenes.Scene (pass
    lib=load_ref() for the translated reference shaders)."""
    o = OracleSim(scene.particles, scene.sph, scene.geom, precision=precision, lib=lib, sdf=sdf)
    o.update_gravity(scene.gravity)
    o.set_pcisph_iterations(scene.iterations)
    if scene.rigid is not None:
        o.update_rigid_body(scene.rigid)
    return o
