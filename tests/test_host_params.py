"""Host-side constants (no GPU): the library's restatements of
src/state/simulation.rs and src/state/rigid_body.rs, checked against an
independent numpy-f32 evaluation of the same formulas."""
import math

import numpy as np
import pytest

f32 = np.float32


def _powi(h, n):
    # f32::powi by binary exponentiation (LLVM powi lowering)
    r, a = None, f32(h)
    while n:
        if n & 1:
            r = a if r is None else f32(r * a)
        n >>= 1
        if n:
            a = f32(a * a)
    return r


def np_rest_density(h, mass):
    h = f32(h)
    spacing = f32(h * f32(0.6))
    cells = int(math.ceil(f32(h / spacing))) + 1
    h2 = f32(h * h)
    scale = f32(f32(315.0) / f32(f32(f32(64.0) * f32(math.pi)) * _powi(h, 9)))
    dens = f32(0)
    for dz in range(-cells, cells + 1):
        for dy in range(-cells, cells + 1):
            for dx in range(-cells, cells + 1):
                ax, ay, az = f32(f32(dx) * spacing), f32(f32(dy) * spacing), f32(f32(dz) * spacing)
                r2 = f32(f32(f32(ax * ax) + f32(ay * ay)) + f32(az * az))
                if r2 < h2:
                    d = f32(h2 - r2)
                    dens = f32(dens + f32(f32(f32(f32(f32(mass) * scale) * d) * d) * d))
    return dens


def test_rest_density_matches_restatement(fslib):
    for h, m in [(0.08, 1.0), (0.035, 1.0), (0.05, 2.0)]:
        got = fslib.fs_compute_rest_density(h, m)
        assert got == pytest.approx(float(np_rest_density(h, m)), rel=0, abs=0)


def test_rest_density_value_at_h008(fslib):
    # the derived rest density at h = 0.08 (spacing 0.6 h lattice) is about 8,679
    assert fslib.fs_compute_rest_density(0.08, 1.0) == pytest.approx(8678.83, abs=0.01)


def test_pcisph_delta_values(fslib):
    rho_ref = fslib.fs_compute_rest_density(0.08, 1.0)
    assert fslib.fs_compute_pcisph_delta(0.08, 1.0, rho_ref, 0.008) == pytest.approx(12.0357, rel=1e-4)
    d8000 = fslib.fs_compute_pcisph_delta(0.08, 1.0, 8000.0, 0.008)
    # delta scales with rho0^2 (beta = dt^2 m^2 / rho0^2)
    assert d8000 == pytest.approx(12.0357 * (8000.0 / rho_ref) ** 2, rel=1e-5)
    assert fslib.fs_compute_pcisph_delta(0.08, 1.0, 8000.0, 0.0) == 0.0  # |denom| <= 1e-10


def test_sph_params_powers(fslib):
    from fluidsph import params as P
    p = P.sph_params_3d(0.08, 1.0, 8000.0, 35.0, 0.45, 15.0, 6.5, 0.305, 0.008, 123)
    assert p.kernel_radius_sq == f32(f32(0.08) * f32(0.08))
    assert p.kernel_radius_pow5 == _powi(0.08, 5)
    assert p.kernel_radius_pow6 == _powi(0.08, 6)
    assert p.kernel_radius_pow9 == _powi(0.08, 9)
    assert p.num_particles == 123 and p.stiffness == f32(35.0)
    assert p.pcisph_delta == fslib.fs_compute_pcisph_delta(0.08, 1.0, 8000.0, 0.008)


def test_container_geometry_rotation(fslib):
    from fluidsph import params as P
    g = P.container_geometry(2.22, 1.8, -0.9, 1.8, 0.2, -0.3, 200.0, 0.55)
    assert g.half_width == f32(1.11) and g.half_depth == f32(0.9) and g.center_y == f32(0.0)
    F = np.array([g.forward_row0[:3], g.forward_row1[:3], g.forward_row2[:3]])
    I = np.array([g.inverse_row0[:3], g.inverse_row1[:3], g.inverse_row2[:3]])
    np.testing.assert_allclose(F @ I, np.eye(3), atol=1e-6)
    cx, sx, cz, sz = math.cos(0.2), math.sin(0.2), math.cos(-0.3), math.sin(-0.3)
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    np.testing.assert_allclose(F, Rz @ Rx, atol=1e-6)


def test_quat_rows_identity_and_rotation(fslib):
    from fluidsph import params as P
    b = P.rigid_body(orientation=(0, 0, 0, 1))
    assert list(b.rot_row0) == [1, 0, 0, 0] and list(b.rot_row2) == [0, 0, 1, 0]
    s = math.sin(math.pi / 4)
    b = P.rigid_body(orientation=(0, 0, s, s))  # 90 degrees about z
    rows = np.array([b.rot_row0[:3], b.rot_row1[:3], b.rot_row2[:3]])
    # rows are world->local (R^T): world +x maps to local -y
    np.testing.assert_allclose(rows @ np.array([1, 0, 0]), [0, -1, 0], atol=1e-6)


def test_grid_sizing(fslib):
    from fluidsph import params as P
    g = P.grid_params_for(0.08, 7)
    assert (g.grid_size_x, g.total_cells) == (52, 52 ** 3)
    assert g.grid_origin_x == f32(-2.08) and g.inv_cell_size == f32(12.5)
    g = P.grid_params_for(0.035, 7)
    assert g.grid_size_x == math.ceil(f32(4.0) / f32(0.035)) + 2
    import ctypes as C
    out = __import__("fluidsph.abi", fromlist=["GpuGridParams"]).GpuGridParams()
    assert fslib.fs_grid_params_for(0.0, 1, C.byref(out)) == -1      # invalid h
    assert fslib.fs_grid_params_for(0.001, 1, C.byref(out)) == -3    # grid too large


def _struct_bytes(s) -> bytes:
    import ctypes as C
    return C.string_at(C.addressof(s), C.sizeof(s))


def test_oracle_builders_equal_library_builders(fslib):
    """The oracle's float32 restatement of the host builders (used by the
    bench's reference arm) and the library's give byte-identical structs."""
    from fluidsph import params as P
    from oracle import host_params as H
    rng = np.random.default_rng(11)
    for _ in range(20):
        h = float(rng.uniform(0.02, 0.12))
        m = float(rng.uniform(0.5, 2.0))
        rho = None if rng.random() < 0.3 else float(rng.uniform(500, 9000))
        dt = float(rng.uniform(0.001, 0.01))
        args = (h, m, rho, 35.0, 0.45, 15.0, 6.5, 0.305, dt, int(rng.integers(1, 10**6)))
        assert _struct_bytes(P.sph_params_3d(*args)) == _struct_bytes(H.sph_params_3d(*args))
        g = (float(rng.uniform(0.5, 3)), float(rng.uniform(0.5, 3)), float(rng.uniform(-1, 1)),
             float(rng.uniform(0.5, 3)), float(rng.uniform(-0.3, 0.3)),
             float(rng.uniform(-0.3, 0.3)), 250.0, 0.55, bool(rng.random() < 0.5), 0.03)
        assert _struct_bytes(P.container_geometry(*g)) == _struct_bytes(H.container_geometry(*g))
        q = rng.standard_normal(4)
        q /= np.linalg.norm(q)
        kw = dict(position=tuple(rng.uniform(-1, 1, 3)), half_extent=0.2, active=True,
                  stiffness=250.0, shape=int(rng.integers(0, 5)), orientation=tuple(q))
        assert _struct_bytes(P.rigid_body(**kw)) == _struct_bytes(H.rigid_body(**kw))


def test_scenes_from_oracle_builders_are_identical(fslib):
    from fluidsph import scenes
    from oracle import host_params as H
    for cfg in (scenes.config0, scenes.config1):
        a, b = cfg(), cfg(builders=H)
        assert np.array_equal(a.particles, b.particles)
        for x, y in ((a.sph, b.sph), (a.geom, b.geom), (a.gravity, b.gravity)):
            assert _struct_bytes(x) == _struct_bytes(y)
        if a.rigid is not None:
            assert _struct_bytes(a.rigid) == _struct_bytes(b.rigid)


def test_batched_losses_check_their_lists():
    """DifferentiableRollout.splat_mse_losses refuses lists of different
    lengths before any library call (and returns no losses for none)."""
    import pytest
    from fluidsph.adjoint import DifferentiableRollout
    fake = object.__new__(DifferentiableRollout)
    assert DifferentiableRollout.splat_mse_losses(fake, [], [], []).shape == (0,)
    with pytest.raises(ValueError):
        DifferentiableRollout.splat_mse_losses(fake, [1, 2], [1], [np.zeros(1), np.zeros(1)])
