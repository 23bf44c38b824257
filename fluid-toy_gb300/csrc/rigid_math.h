// rigid_math.h — the reference's CPU rigid-body integration
// (src/state/rigid_body.rs), restated once for the host entry points
// (host_params.cpp) and the device-resident coupling loop (rigid_kernels.cu).
//
// Every expression keeps the Rust source's operation order; host code is
// built with -ffp-contract=off and device code with -fmad=false, and sqrt and
// division are IEEE on both, so host and device produce the same bits as each
// other and as the reference's f32 arithmetic.
#pragma once

#include <math.h>
#include <stdint.h>

#include "../../include/fluidsph.h"

#ifdef __CUDACC__
#define FS_HD __host__ __device__ __forceinline__
#else
#define FS_HD inline
#endif

namespace fs {
namespace rb {

constexpr float PI_F32 = 3.14159265358979323846f;  // std::f32::consts::PI

// RigidBodyShape::volume, rigid_body.rs:28-52
FS_HD float shape_volume(uint32_t shape, float he) {
  switch (shape) {
    case 0: {
      const float side = 2.0f * he;
      return side * side * side;
    }
    case 2: return PI_F32 * he * he * (2.0f * he);
    case 3: {
      const float small_r = he * 0.3f;
      return 2.0f * PI_F32 * PI_F32 * he * small_r * small_r;
    }
    default: return (4.0f / 3.0f) * PI_F32 * he * he * he;  // sphere, custom
  }
}

// RigidBodyShape::moment_of_inertia, rigid_body.rs:54-83
FS_HD float moment_of_inertia(uint32_t shape, float mass, float he) {
  switch (shape) {
    case 0: {
      const float side = 2.0f * he;
      return (1.0f / 6.0f) * mass * side * side;
    }
    case 2: {
      const float r = he, h = 2.0f * he;
      return (1.0f / 12.0f) * mass * (3.0f * r * r + h * h);
    }
    case 3: {
      const float big_r = he, small_r = he * 0.3f;
      return mass * (big_r * big_r + 0.75f * small_r * small_r);
    }
    default: return (2.0f / 5.0f) * mass * he * he;  // sphere, custom
  }
}

// quat_normalize / quat_mul / quat_to_rotation_rows, rigid_body.rs:166-205
FS_HD void quat_normalize(const float q[4], float out[4]) {
  const float len = sqrtf(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  if (len < 1e-10f) {
    out[0] = 0.0f; out[1] = 0.0f; out[2] = 0.0f; out[3] = 1.0f;
    return;
  }
  out[0] = q[0] / len; out[1] = q[1] / len; out[2] = q[2] / len; out[3] = q[3] / len;
}
FS_HD void quat_mul(const float a[4], const float b[4], float out[4]) {
  const float ax = a[0], ay = a[1], az = a[2], aw = a[3];
  const float bx = b[0], by = b[1], bz = b[2], bw = b[3];
  out[0] = aw * bx + ax * bw + ay * bz - az * by;
  out[1] = aw * by - ax * bz + ay * bw + az * bx;
  out[2] = aw * bz + ax * by - ay * bx + az * bw;
  out[3] = aw * bw - ax * bx - ay * by - az * bz;
}
FS_HD void quat_rows(const float q[4], float r[3][4]) {
  const float x = q[0], y = q[1], z = q[2], w = q[3];
  const float xx = x * x, yy = y * y, zz = z * z;
  const float xy = x * y, xz = x * z, yz = y * z;
  const float wx = w * x, wy = w * y, wz = w * z;
  r[0][0] = 1.0f - 2.0f * (yy + zz); r[0][1] = 2.0f * (xy + wz); r[0][2] = 2.0f * (xz - wy); r[0][3] = 0.0f;
  r[1][0] = 2.0f * (xy - wz); r[1][1] = 1.0f - 2.0f * (xx + zz); r[1][2] = 2.0f * (yz + wx); r[1][3] = 0.0f;
  r[2][0] = 2.0f * (xz + wy); r[2][1] = 2.0f * (yz - wx); r[2][2] = 1.0f - 2.0f * (xx + yy); r[2][3] = 0.0f;
}

// RigidBodyConfig::to_gpu_rigid_body, rigid_body.rs:131-146
FS_HD void to_gpu(const FsRigidBodyState &s, GpuRigidBody &g) {
  float rows[3][4];
  quat_rows(s.orientation, rows);
  g.position[0] = s.position[0]; g.position[1] = s.position[1]; g.position[2] = s.position[2];
  g.half_extent = s.half_extent;
  g.velocity[0] = s.velocity[0]; g.velocity[1] = s.velocity[1]; g.velocity[2] = s.velocity[2];
  g.is_active = s.enabled ? 1u : 0u;
  g.stiffness = s.wall_stiffness;
  g.shape = s.shape;
  g._pad1 = 0.0f;
  g._pad2 = 0.0f;
  for (int k = 0; k < 4; k++) {
    g.rot_row0[k] = rows[0][k];
    g.rot_row1[k] = rows[1][k];
    g.rot_row2[k] = rows[2][k];
  }
}

// rotated_aabb_half_extents, rigid_body.rs:371-412 (inv = the container's
// inverse rows, world -> container local)
FS_HD void rotated_aabb(uint32_t shape, float he, const float q[4], const float inv[3][3],
                        float aabb[3]) {
  if (shape == 1u) {
    aabb[0] = he; aabb[1] = he; aabb[2] = he;
    return;
  }
  float local_he[3];
  if (shape == 3u) {
    const float r_minor = 0.3f * he;
    local_he[0] = he + r_minor; local_he[1] = r_minor; local_he[2] = he + r_minor;
  } else {
    local_he[0] = he; local_he[1] = he; local_he[2] = he;
  }
  float br[3][4];
  quat_rows(q, br);
  for (int i = 0; i < 3; i++) {
    float sum = 0.0f;
    for (int j = 0; j < 3; j++) {
      const float m_ij = inv[i][0] * br[j][0] + inv[i][1] * br[j][1] + inv[i][2] * br[j][2];
      sum += fabsf(m_ij) * local_he[j];
    }
    aabb[i] = sum;
  }
}

// clamp_rigid_body_to_container, rigid_body.rs:415-479
FS_HD void clamp_to_container(FsRigidBodyState &s, const GpuContainerGeometry &c, bool bounce) {
  const float inv[3][3] = {{c.inverse_row0[0], c.inverse_row0[1], c.inverse_row0[2]},
                           {c.inverse_row1[0], c.inverse_row1[1], c.inverse_row1[2]},
                           {c.inverse_row2[0], c.inverse_row2[1], c.inverse_row2[2]}};
  const float fwd[3][3] = {{c.forward_row0[0], c.forward_row0[1], c.forward_row0[2]},
                           {c.forward_row1[0], c.forward_row1[1], c.forward_row1[2]},
                           {c.forward_row2[0], c.forward_row2[1], c.forward_row2[2]}};
  float aabb[3];
  rotated_aabb(s.shape, s.half_extent, s.orientation, inv, aabb);
  const float center_y = c.center_y;
  const float cy[3] = {s.position[0], s.position[1] - center_y, s.position[2]};
  float lp[3], lv[3];
  for (int i = 0; i < 3; i++) {
    lp[i] = inv[i][0] * cy[0] + inv[i][1] * cy[1] + inv[i][2] * cy[2];
    lv[i] = inv[i][0] * s.velocity[0] + inv[i][1] * s.velocity[1] + inv[i][2] * s.velocity[2];
  }
  const float H[3] = {c.half_width, c.half_height, c.half_depth};
  for (int i = 0; i < 3; i++) {
    if (lp[i] - aabb[i] < -H[i]) {
      lp[i] = -H[i] + aabb[i];
      if (bounce) lv[i] = fabsf(lv[i]) * 0.3f;
    }
    if (lp[i] + aabb[i] > H[i]) {
      lp[i] = H[i] - aabb[i];
      if (bounce) lv[i] = -fabsf(lv[i]) * 0.3f;
    }
  }
  s.position[0] = fwd[0][0] * lp[0] + fwd[0][1] * lp[1] + fwd[0][2] * lp[2];
  s.position[1] = fwd[1][0] * lp[0] + fwd[1][1] * lp[1] + fwd[1][2] * lp[2] + center_y;
  s.position[2] = fwd[2][0] * lp[0] + fwd[2][1] * lp[1] + fwd[2][2] * lp[2];
  if (bounce)
    for (int i = 0; i < 3; i++)
      s.velocity[i] = fwd[i][0] * lv[0] + fwd[i][1] * lv[1] + fwd[i][2] * lv[2];
}

// integrate_rigid_body, rigid_body.rs:277-365: reaction forces -> velocity ->
// position, torque -> angular velocity -> orientation, then the container
// clamp with bounce.
FS_HD void integrate(FsRigidBodyState &s, const GpuContainerGeometry &c, float delta_time,
                     uint32_t num_substeps, const float gravity[3], const GpuRigidBodyAccum &a) {
  const float reaction[3] = {float(a.force_x) / 1000.0f, float(a.force_y) / 1000.0f,
                             float(a.force_z) / 1000.0f};
  const float he = s.half_extent;
  const float volume = shape_volume(s.shape, he);
  const float body_mass = s.density * volume;
  const float total_dt = float(num_substeps) * delta_time;
  if (body_mass <= 0.0f) return;
  float dv[3];
  for (int i = 0; i < 3; i++) dv[i] = delta_time * reaction[i] / body_mass;
  const float max_dv = total_dt * 200.0f;
  const float dv_mag = sqrtf(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
  if (dv_mag > max_dv) {
    const float scale = max_dv / dv_mag;
    for (int i = 0; i < 3; i++) dv[i] *= scale;
  }
  for (int i = 0; i < 3; i++) {
    s.velocity[i] += dv[i] + total_dt * gravity[i];
    s.velocity[i] *= 0.995f;
  }
  for (int i = 0; i < 3; i++) s.position[i] += total_dt * s.velocity[i];
  const float torque[3] = {float(a.torque_x) / 1000.0f, float(a.torque_y) / 1000.0f,
                           float(a.torque_z) / 1000.0f};
  const float inertia = moment_of_inertia(s.shape, body_mass, he);
  if (inertia > 0.0f) {
    float dw[3];
    for (int i = 0; i < 3; i++) dw[i] = delta_time * torque[i] / inertia;
    const float max_dw = total_dt * 50.0f;
    const float dw_mag = sqrtf(dw[0] * dw[0] + dw[1] * dw[1] + dw[2] * dw[2]);
    if (dw_mag > max_dw) {
      const float scale = max_dw / dw_mag;
      for (int i = 0; i < 3; i++) dw[i] *= scale;
    }
    for (int i = 0; i < 3; i++) {
      s.angular_velocity[i] += dw[i];
      s.angular_velocity[i] *= 0.98f;
    }
    const float omega[4] = {s.angular_velocity[0], s.angular_velocity[1],
                            s.angular_velocity[2], 0.0f};
    float q_dot[4];
    quat_mul(omega, s.orientation, q_dot);
    const float qn[4] = {s.orientation[0] + 0.5f * total_dt * q_dot[0],
                         s.orientation[1] + 0.5f * total_dt * q_dot[1],
                         s.orientation[2] + 0.5f * total_dt * q_dot[2],
                         s.orientation[3] + 0.5f * total_dt * q_dot[3]};
    quat_normalize(qn, s.orientation);
  }
  clamp_to_container(s, c, true);
}

}  // namespace rb
}  // namespace fs
