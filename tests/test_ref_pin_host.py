"""The library's host-side restatements against the reference's own Rust
functions, translated mechanically to C++ (oracle/rs2cpp.py -> oracle/_ref),
bit for bit, on seeded random inputs. No GPU.

Pinned here (reference file:line -> library entry point):
  compute_rest_density   simulation.rs:402-427      fs_compute_rest_density
  compute_pcisph_delta   simulation.rs:429-480      fs_compute_pcisph_delta
  to_gpu_params_3d       simulation.rs:315-337      fs_sph_params_3d
  to_gpu_geometry        simulation.rs:137-184      fs_container_geometry
  quat_to_rotation_rows  rigid_body.rs:188-205      fs_quat_to_rotation_rows
  to_gpu_rigid_body      rigid_body.rs:131-146      fs_rigid_body_to_gpu
  integrate_rigid_body   rigid_body.rs:277-365      fs_integrate_rigid_body
  clamp_rigid_body_to_container  rigid_body.rs:400-479  fs_clamp_rigid_body
  spawn_particles        sph_3d_grid.rs:1534-1569   fs_spawn_positions
The oracle's own float32 restatement of the builders (oracle/host_params.py,
used by the bench's reference arm) is pinned the same way. Skipped where the
translation is not available (it is built from the reference sources)."""
import ctypes as C

import numpy as np
import pytest

f32 = np.float32


@pytest.fixture(scope="module")
def ref(oracle_mod):
    lib = oracle_mod.load_ref_host()
    if lib is None:
        pytest.skip("reference host translation not available here")
    return lib


def _bytes(s) -> bytes:
    return C.string_at(C.addressof(s), C.sizeof(s))


def _f(*v):
    return (C.c_float * len(v))(*v)


def _params_cases(rng, n):
    for _ in range(n):
        yield (f32(rng.uniform(0.01, 0.2)), f32(rng.uniform(0.1, 3.0)),
               f32(rng.uniform(100.0, 10000.0)), f32(rng.uniform(1e-4, 0.02)))
    yield f32(0.08), f32(1.0), f32(8000.0), f32(0.008)    # the configured workloads
    yield f32(0.035), f32(1.0), f32(1000.0), f32(1 / 360)  # the reference app's defaults
    yield f32(0.08), f32(1.0), f32(8000.0), f32(0.0)      # |denominator| <= 1e-10


def test_rest_density_and_pcisph_delta(fslib, ref):
    from oracle import host_params as H
    for h, m, rho, dt in _params_cases(np.random.default_rng(1), 40):
        a = f32(fslib.fs_compute_rest_density(h, m))
        b = f32(ref.rh_compute_rest_density(h, m))
        assert a.tobytes() == b.tobytes() == H.compute_rest_density(h, m).tobytes(), (h, m)
        a = f32(fslib.fs_compute_pcisph_delta(h, m, rho, dt))
        b = f32(ref.rh_compute_pcisph_delta(h, m, rho, dt))
        c = H.compute_pcisph_delta(h, m, rho, dt)
        assert a.tobytes() == b.tobytes() == c.tobytes(), (h, m, rho, dt)


def test_sph_params(fslib, ref):
    """to_gpu_params_3d derives the rest density; the library takes it as an
    argument (the configured workloads set 8000): with the derived value the
    64 bytes are the reference's."""
    from fluidsph import params as P
    from fluidsph.abi import GpuSphParams3D
    from oracle import host_params as H
    rng = np.random.default_rng(2)
    for h, m, _, dt in _params_cases(rng, 30):
        st, nk, vi, sig, xe = (float(f32(x)) for x in rng.uniform(0, 40, 5))
        n = int(rng.integers(0, 2 ** 31))
        out = GpuSphParams3D()
        ref.rh_to_gpu_params_3d(h, st, nk, vi, m, sig, xe, n, dt, C.addressof(out))
        mine = P.sph_params_3d(float(h), float(m), None, st, nk, vi, sig, xe, float(dt), n)
        theirs = H.sph_params_3d(float(h), float(m), None, st, nk, vi, sig, xe, float(dt), n)
        assert _bytes(mine) == _bytes(out) == _bytes(theirs)


def test_container_geometry(fslib, ref):
    from fluidsph import params as P
    from fluidsph.abi import GpuContainerGeometry
    from oracle import host_params as H
    rng = np.random.default_rng(3)
    cases = [(2.22, 1.8, -0.9, 1.8, 0.0, 0.0)]  # ContainerConfig::default
    cases += [tuple(float(f32(x)) for x in (rng.uniform(0.2, 5), rng.uniform(0.2, 5),
                                            rng.uniform(-2, 2), rng.uniform(0.2, 5),
                                            rng.uniform(-1.6, 1.6), rng.uniform(-1.6, 1.6)))
              for _ in range(60)]
    for k, c in enumerate(cases):
        wk, damp, clip, margin = float(f32(rng.uniform(0, 500))), float(f32(rng.random())), \
            bool(k % 2), float(f32(rng.uniform(0, 0.1)))
        out = GpuContainerGeometry()
        ref.rh_to_gpu_geometry(_f(*c), wk, damp, int(clip), margin, C.addressof(out))
        mine = P.container_geometry(c[0], c[1], c[2], c[3], c[4], c[5], wk, damp, clip, margin)
        theirs = H.container_geometry(c[0], c[1], c[2], c[3], c[4], c[5], wk, damp, clip, margin)
        assert _bytes(mine) == _bytes(out) == _bytes(theirs), c


def _random_state(rng, shape):
    from fluidsph import params as P
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    return P.rigid_body_state(position=tuple(rng.uniform(-1.2, 1.2, 3)),
                              half_extent=float(rng.uniform(0.02, 0.5)), shape=shape,
                              density=float(rng.uniform(-50, 3000)),
                              velocity=tuple(rng.uniform(-3, 3, 3)), orientation=tuple(q),
                              angular_velocity=tuple(rng.uniform(-5, 5, 3)),
                              enabled=bool(rng.random() < 0.8), held=bool(rng.random() < 0.3),
                              wall_stiffness=float(rng.uniform(50, 400)))


def _copy(state):
    return type(state).from_buffer_copy(state)


def test_quat_rows_and_gpu_rigid_body(fslib, ref):
    from fluidsph import params as P
    from fluidsph.abi import GpuRigidBody
    from oracle import host_params as H
    rng = np.random.default_rng(4)
    for k in range(200):
        q = rng.standard_normal(4) * (1.0 if k % 3 else rng.uniform(0.1, 3.0))
        rows_a, rows_b = (C.c_float * 12)(), (C.c_float * 12)()
        fslib.fs_quat_to_rotation_rows(_f(*q), rows_a)
        ref.rh_quat_to_rotation_rows(_f(*q), rows_b)
        assert bytes(rows_a) == bytes(rows_b)
        assert bytes(rows_a) == np.array(H.quat_to_rotation_rows(q), f32).tobytes()
        s = _random_state(rng, k % 5)
        out = GpuRigidBody()
        ref.rh_to_gpu_rigid_body(C.addressof(s), s.wall_stiffness, C.addressof(out))
        assert _bytes(P.rigid_body_to_gpu(s)) == _bytes(out)


def test_integrate_and_clamp_rigid_body(fslib, ref):
    """Random bodies of every shape, accumulators from zero to beyond the
    velocity clamps, tilted containers: the whole FsRigidBodyState after
    fs_integrate_rigid_body / fs_clamp_rigid_body is the reference's."""
    from fluidsph import params as P
    from fluidsph.abi import GpuRigidBodyAccum
    rng = np.random.default_rng(5)
    for k in range(400):
        c = tuple(float(f32(x)) for x in (rng.uniform(0.5, 3), rng.uniform(0.5, 3),
                                          rng.uniform(-1, 0.5), rng.uniform(0.5, 3),
                                          rng.uniform(-0.4, 0.4), rng.uniform(-0.4, 0.4)))
        geom = P.container_geometry(*c)
        s = _random_state(rng, k % 5)
        acc = GpuRigidBodyAccum()
        scale = [0, 10, 10 ** 4, 10 ** 7][k % 4]
        for name in ("force_x", "force_y", "force_z", "torque_x", "torque_y", "torque_z"):
            setattr(acc, name, int(rng.integers(-scale - 1, scale + 1)))
        dt = float(f32(rng.uniform(1e-4, 0.02)))
        subs = int(rng.integers(1, 9))
        g = _f(*rng.uniform(-12, 12, 3))
        a, b = _copy(s), _copy(s)
        assert fslib.fs_integrate_rigid_body(C.byref(a), C.byref(geom), dt, subs, g,
                                             C.byref(acc)) == 0
        ref.rh_integrate_rigid_body(C.addressof(b), _f(*c), dt, subs, g, C.addressof(acc))
        assert _bytes(a) == _bytes(b), k
        a, b = _copy(s), _copy(s)
        bounce = k % 2
        assert fslib.fs_clamp_rigid_body(C.byref(a), C.byref(geom), bounce) == 0
        ref.rh_clamp_rigid_body(C.addressof(b), _f(*c), bounce)
        assert _bytes(a) == _bytes(b), k


def test_spawn_positions(fslib, ref):
    """fs_spawn_positions (the records fs_spawn_particles writes) against
    spawn_particles: same count after the capacity clip, same 64-byte records
    bit for bit (cos/sin are the C library's on both sides), and the grid
    parameters' particle count."""
    rng = np.random.default_rng(6)
    for k in range(40):
        maxn = int(rng.integers(1, 5000))
        num = int(rng.integers(0, maxn + 1))
        count = int(rng.integers(0, 3000))
        spread = float(f32(rng.uniform(0.001, 0.5)))
        pos = _f(*rng.uniform(-1, 1, 3))
        n_exp = min(count, maxn - num)
        mine = np.zeros((max(n_exp, 1), 16), np.float32)
        theirs = np.zeros((max(n_exp, 1), 16), np.float32)
        got = C.c_uint32()
        assert fslib.fs_spawn_positions(pos, count, spread, num, maxn, mine.ctypes.data,
                                        C.byref(got)) == 0
        grid = C.c_uint32()
        n_ref = ref.rh_spawn_particles(maxn, num, pos, count, spread, theirs.ctypes.data,
                                       C.byref(grid))
        assert got.value == n_ref == n_exp
        assert mine.tobytes() == theirs.tobytes()
        if n_ref:
            assert grid.value == num + n_ref
