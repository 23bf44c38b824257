"""Host restatement of the reference's CPU rigid-body integration
(src/state/rigid_body.rs:277-479), fs_integrate_rigid_body, against an
independent numpy float32 restatement: bit-exact on random states and
accumulators for every shape, held clamps included."""
import numpy as np
import pytest

f32 = np.float32
PI = f32(np.pi)


def _volume(shape, he):
    if shape == 0:
        side = f32(2) * he
        return side * side * side
    if shape == 2:
        return PI * he * he * (f32(2) * he)
    if shape == 3:
        small = he * f32(0.3)
        return f32(2) * PI * PI * he * small * small
    return (f32(4) / f32(3)) * PI * he * he * he


def _inertia(shape, mass, he):
    if shape == 0:
        side = f32(2) * he
        return (f32(1) / f32(6)) * mass * side * side
    if shape == 2:
        r, h = he, f32(2) * he
        return (f32(1) / f32(12)) * mass * (f32(3) * r * r + h * h)
    if shape == 3:
        big, small = he, he * f32(0.3)
        return mass * (big * big + f32(0.75) * small * small)
    return (f32(2) / f32(5)) * mass * he * he


def _rows(q):
    x, y, z, w = q
    xx, yy, zz, xy, xz, yz = x * x, y * y, z * z, x * y, x * z, y * z
    wx, wy, wz = w * x, w * y, w * z
    one, two = f32(1), f32(2)
    return [[one - two * (yy + zz), two * (xy + wz), two * (xz - wy)],
            [two * (xy - wz), one - two * (xx + zz), two * (yz + wx)],
            [two * (xz + wy), two * (yz - wx), one - two * (xx + yy)]]


def _clamp(st, g, bounce):
    inv = [list(map(f32, g.inverse_row0[:3])), list(map(f32, g.inverse_row1[:3])),
           list(map(f32, g.inverse_row2[:3]))]
    fwd = [list(map(f32, g.forward_row0[:3])), list(map(f32, g.forward_row1[:3])),
           list(map(f32, g.forward_row2[:3]))]
    he = st["he"]
    if st["shape"] == 1:
        aabb = [he, he, he]
    else:
        lh = [he + f32(0.3) * he, f32(0.3) * he, he + f32(0.3) * he] if st["shape"] == 3 else [he] * 3
        br = _rows(st["q"])
        aabb = []
        for i in range(3):
            s = f32(0)
            for j in range(3):
                m = inv[i][0] * br[j][0] + inv[i][1] * br[j][1] + inv[i][2] * br[j][2]
                s = s + abs(m) * lh[j]
            aabb.append(s)
    cy_ = f32(g.center_y)
    p, v = st["p"], st["v"]
    cy = [p[0], p[1] - cy_, p[2]]
    lp = [inv[i][0] * cy[0] + inv[i][1] * cy[1] + inv[i][2] * cy[2] for i in range(3)]
    lv = [inv[i][0] * v[0] + inv[i][1] * v[1] + inv[i][2] * v[2] for i in range(3)]
    H = [f32(g.half_width), f32(g.half_height), f32(g.half_depth)]
    for i in range(3):
        if lp[i] - aabb[i] < -H[i]:
            lp[i] = -H[i] + aabb[i]
            if bounce:
                lv[i] = abs(lv[i]) * f32(0.3)
        if lp[i] + aabb[i] > H[i]:
            lp[i] = H[i] - aabb[i]
            if bounce:
                lv[i] = -abs(lv[i]) * f32(0.3)
    st["p"] = [fwd[0][0] * lp[0] + fwd[0][1] * lp[1] + fwd[0][2] * lp[2],
               fwd[1][0] * lp[0] + fwd[1][1] * lp[1] + fwd[1][2] * lp[2] + cy_,
               fwd[2][0] * lp[0] + fwd[2][1] * lp[1] + fwd[2][2] * lp[2]]
    if bounce:
        st["v"] = [fwd[i][0] * lv[0] + fwd[i][1] * lv[1] + fwd[i][2] * lv[2] for i in range(3)]


def _integrate(st, g, dt, n, grav, acc):
    reaction = [f32(a) / f32(1000) for a in acc[0:3]]
    he = st["he"]
    mass = st["density"] * _volume(st["shape"], he)
    total = f32(n) * dt
    if mass <= 0:
        return
    dv = [dt * reaction[i] / mass for i in range(3)]
    max_dv = total * f32(200)
    mag = np.sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2], dtype=f32)
    if mag > max_dv:
        sc = max_dv / mag
        dv = [d * sc for d in dv]
    v = st["v"]
    for i in range(3):
        v[i] = v[i] + (dv[i] + total * grav[i])
        v[i] = v[i] * f32(0.995)
    st["p"] = [st["p"][i] + total * v[i] for i in range(3)]
    torque = [f32(a) / f32(1000) for a in acc[4:7]]
    inertia = _inertia(st["shape"], mass, he)
    if inertia > 0:
        dw = [dt * torque[i] / inertia for i in range(3)]
        max_dw = total * f32(50)
        mag = np.sqrt(dw[0] * dw[0] + dw[1] * dw[1] + dw[2] * dw[2], dtype=f32)
        if mag > max_dw:
            sc = max_dw / mag
            dw = [d * sc for d in dw]
        w = st["w"]
        for i in range(3):
            w[i] = w[i] + dw[i]
            w[i] = w[i] * f32(0.98)
        ax, ay, az, aw = w[0], w[1], w[2], f32(0)
        bx, by, bz, bw = st["q"]
        qd = [aw * bx + ax * bw + ay * bz - az * by, aw * by - ax * bz + ay * bw + az * bx,
              aw * bz + ax * by - ay * bx + az * bw, aw * bw - ax * bx - ay * by - az * bz]
        qn = [st["q"][i] + f32(0.5) * total * qd[i] for i in range(4)]
        ln = np.sqrt(qn[0] * qn[0] + qn[1] * qn[1] + qn[2] * qn[2] + qn[3] * qn[3], dtype=f32)
        st["q"] = [f32(0), f32(0), f32(0), f32(1)] if ln < f32(1e-10) else [c / ln for c in qn]
    _clamp(st, g, True)


def test_integrate_rigid_body_matches_independent_restatement(fslib):
    from fluidsph import abi
    from fluidsph import params as P
    rng = np.random.default_rng(5)
    with np.errstate(all="ignore"):
        for trial in range(300):
            shape = trial % 5
            geom = P.container_geometry(float(rng.uniform(0.6, 2)), float(rng.uniform(0.6, 2)),
                                        0.0, float(rng.uniform(0.6, 2)),
                                        float(rng.uniform(-0.3, 0.3)), float(rng.uniform(-0.3, 0.3)))
            q = rng.standard_normal(4)
            q /= np.linalg.norm(q)
            st = P.rigid_body_state(position=rng.uniform(-1, 1, 3), half_extent=float(rng.uniform(0.05, 0.3)),
                                    shape=shape, density=float(rng.uniform(50, 2000)),
                                    velocity=rng.uniform(-2, 2, 3), orientation=q,
                                    angular_velocity=rng.uniform(-3, 3, 3))
            acc = abi.GpuRigidBodyAccum()
            vals = rng.integers(-2_000_000, 2_000_000, 7)
            acc.force_x, acc.force_y, acc.force_z = (int(v) for v in vals[:3])
            acc.torque_x, acc.torque_y, acc.torque_z = (int(v) for v in vals[4:7])
            acc.contact_count = int(abs(vals[3]) % 5000)
            py = {"p": [f32(x) for x in st.position], "v": [f32(x) for x in st.velocity],
                  "w": [f32(x) for x in st.angular_velocity], "q": [f32(x) for x in st.orientation],
                  "he": f32(st.half_extent), "density": f32(st.density), "shape": shape}
            dt, n, grav = f32(1 / 60 / 6), 6, [f32(0), f32(-9.81), f32(0)]
            P.integrate_rigid_body(st, geom, float(dt), n, [float(g) for g in grav], acc)
            _integrate(py, geom, dt, n, grav, acc.as_tuple())
            np.testing.assert_array_equal(np.array(st.position, f32), np.array(py["p"], f32))
            np.testing.assert_array_equal(np.array(st.velocity, f32), np.array(py["v"], f32))
            np.testing.assert_array_equal(np.array(st.orientation, f32), np.array(py["q"], f32))
            np.testing.assert_array_equal(np.array(st.angular_velocity, f32), np.array(py["w"], f32))


def test_rigid_body_to_gpu_matches_rows(fslib):
    import ctypes as C
    from fluidsph import abi
    from fluidsph import params as P
    st = P.rigid_body_state(position=(0.1, 0.2, 0.3), half_extent=0.12, shape=3,
                            orientation=(0.1, 0.2, 0.3, 0.927), enabled=True, wall_stiffness=250.0)
    g = P.rigid_body_to_gpu(st)
    rows = (C.c_float * 12)()
    q = (C.c_float * 4)(*st.orientation)
    abi.load().fs_quat_to_rotation_rows(q, rows)
    assert list(g.rot_row0) + list(g.rot_row1) + list(g.rot_row2) == list(rows)
    assert (g.is_active, g.shape, g.stiffness, g.half_extent) == (1, 3, np.float32(250.0), np.float32(0.12))
