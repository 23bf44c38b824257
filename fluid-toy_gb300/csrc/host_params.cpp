// host_params.cpp — host-side constants of the SPH step, restating the
// reference's parameter builders in f32 with the same operation order
// (compiled with -ffp-contract=off, so no multiply-add is fused):
//   compute_rest_density      src/state/simulation.rs:402-425
//   compute_pcisph_delta      src/state/simulation.rs:429-480
//   to_gpu_params_3d          src/state/simulation.rs:315-337
//   rotation_matrices + to_gpu_geometry  src/state/simulation.rs:139-184
//   quat_to_rotation_rows     src/state/rigid_body.rs:188-205
//   grid sizing               src/simulation/sph_3d_grid.rs:121-143
#include <algorithm>
#include <cmath>
#include <cstring>

#include "../../include/fluidsph.h"
#include "rigid_math.h"

namespace {

const float PI_F32 = 3.14159265358979323846f;  // std::f32::consts::PI

// f32::powi for the exponents the reference uses (binary exponentiation, the
// product order of LLVM's powi lowering).
inline float powi5(float h) {
  const float h2 = h * h, h4 = h2 * h2;
  return h * h4;
}
inline float powi6(float h) {
  const float h2 = h * h, h4 = h2 * h2;
  return h2 * h4;
}
inline float powi9(float h) {
  const float h2 = h * h, h4 = h2 * h2, h8 = h4 * h4;
  return h * h8;
}

}  // namespace

extern "C" {

float fs_compute_rest_density(float h, float mass) {
  const float spacing = h * 0.6f;
  const int cells = int(std::ceil(h / spacing)) + 1;
  const float h2 = h * h;
  const float h9 = powi9(h);
  const float scale = 315.0f / (64.0f * PI_F32 * h9);
  float density = 0.0f;
  for (int dz = -cells; dz <= cells; dz++)
    for (int dy = -cells; dy <= cells; dy++)
      for (int dx = -cells; dx <= cells; dx++) {
        const float ax = float(dx) * spacing, ay = float(dy) * spacing, az = float(dz) * spacing;
        const float r_sq = ax * ax + ay * ay + az * az;
        if (r_sq < h2) {
          const float diff = h2 - r_sq;
          density += mass * scale * diff * diff * diff;
        }
      }
  return density;
}

float fs_compute_pcisph_delta(float h, float mass, float rest_density, float dt) {
  const float spacing = h * 0.6f;
  const int cells = int(std::ceil(h / spacing)) + 1;
  float sum_grad[3] = {0.0f, 0.0f, 0.0f};
  float sum_grad_sq = 0.0f;
  const float h6 = powi6(h);
  for (int dz = -cells; dz <= cells; dz++)
    for (int dy = -cells; dy <= cells; dy++)
      for (int dx = -cells; dx <= cells; dx++) {
        if (dx == 0 && dy == 0 && dz == 0) continue;
        const float rv[3] = {float(dx) * spacing, float(dy) * spacing, float(dz) * spacing};
        const float r_sq = rv[0] * rv[0] + rv[1] * rv[1] + rv[2] * rv[2];
        if (r_sq < h * h && r_sq > 1e-12f) {
          const float r = std::sqrt(r_sq);
          const float grad_mag = 45.0f / (PI_F32 * h6) * (h - r) * (h - r);
          const float g[3] = {grad_mag * rv[0] / r, grad_mag * rv[1] / r, grad_mag * rv[2] / r};
          sum_grad[0] += g[0];
          sum_grad[1] += g[1];
          sum_grad[2] += g[2];
          sum_grad_sq += g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
        }
      }
  const float sum_grad_dot = sum_grad[0] * sum_grad[0] + sum_grad[1] * sum_grad[1] +
                             sum_grad[2] * sum_grad[2];
  const float beta = dt * dt * mass * mass / (rest_density * rest_density);
  const float denom = beta * (sum_grad_dot + sum_grad_sq);
  const float omega = 0.2f;
  return std::fabs(denom) > 1e-10f ? omega / denom : 0.0f;
}

int fs_sph_params_3d(float kernel_radius, float mass, float rest_density, float stiffness,
                     float near_stiffness, float viscosity, float surface_tension,
                     float xsph_epsilon, float dt, uint32_t num_particles,
                     GpuSphParams3D *out) {
  if (!out) return FS_E_INVALID_ARGUMENT;
  const float h = kernel_radius;
  GpuSphParams3D p;
  std::memset(&p, 0, sizeof(p));
  p.kernel_radius = h;
  p.kernel_radius_sq = h * h;
  p.kernel_radius_pow5 = powi5(h);
  p.kernel_radius_pow6 = powi6(h);
  p.kernel_radius_pow9 = powi9(h);
  p.mass = mass;
  p.rest_density = rest_density;
  p.stiffness = stiffness;
  p.near_stiffness = near_stiffness;
  p.viscosity = viscosity;
  p.dt = dt;
  p.num_particles = num_particles;
  p.surface_tension = surface_tension;
  p.pcisph_delta = fs_compute_pcisph_delta(h, mass, rest_density, dt);
  p.xsph_epsilon = xsph_epsilon;
  p._padding_st = 0.0f;
  *out = p;
  return FS_OK;
}

int fs_container_geometry(float width, float depth, float floor_y, float height, float tilt_x,
                          float tilt_z, float wall_stiffness, float damping,
                          uint32_t clip_enabled, float clip_margin,
                          GpuContainerGeometry *out) {
  if (!out) return FS_E_INVALID_ARGUMENT;
  const float sx = std::sin(tilt_x), cx = std::cos(tilt_x);
  const float sz = std::sin(tilt_z), cz = std::cos(tilt_z);
  GpuContainerGeometry g;
  std::memset(&g, 0, sizeof(g));
  const float fwd[3][4] = {{cz, -sz * cx, sz * sx, 0.0f},
                           {sz, cz * cx, -cz * sx, 0.0f},
                           {0.0f, sx, cx, 0.0f}};
  const float inv[3][4] = {{cz, sz, 0.0f, 0.0f},
                           {-sz * cx, cz * cx, sx, 0.0f},
                           {sz * sx, -cz * sx, cx, 0.0f}};
  g.half_width = width / 2.0f;
  g.half_height = height / 2.0f;
  g.half_depth = depth / 2.0f;
  g.center_y = floor_y + height / 2.0f;
  std::memcpy(g.forward_row0, fwd[0], 16);
  std::memcpy(g.forward_row1, fwd[1], 16);
  std::memcpy(g.forward_row2, fwd[2], 16);
  std::memcpy(g.inverse_row0, inv[0], 16);
  std::memcpy(g.inverse_row1, inv[1], 16);
  std::memcpy(g.inverse_row2, inv[2], 16);
  g.wall_stiffness = wall_stiffness;
  g.damping = damping;
  g.clip_enabled = clip_enabled ? 1u : 0u;
  g.clip_margin = clip_margin;
  *out = g;
  return FS_OK;
}

int fs_quat_to_rotation_rows(const float q[4], float rows[12]) {
  if (!q || !rows) return FS_E_INVALID_ARGUMENT;
  const float x = q[0], y = q[1], z = q[2], w = q[3];
  const float xx = x * x, yy = y * y, zz = z * z;
  const float xy = x * y, xz = x * z, yz = y * z;
  const float wx = w * x, wy = w * y, wz = w * z;
  const float r[12] = {1.0f - 2.0f * (yy + zz), 2.0f * (xy + wz), 2.0f * (xz - wy), 0.0f,
                       2.0f * (xy - wz), 1.0f - 2.0f * (xx + zz), 2.0f * (yz + wx), 0.0f,
                       2.0f * (xz + wy), 2.0f * (yz - wx), 1.0f - 2.0f * (xx + yy), 0.0f};
  std::memcpy(rows, r, sizeof(r));
  return FS_OK;
}

int fs_grid_params_for(float kernel_radius, uint32_t num_particles, GpuGridParams *out) {
  if (!out) return FS_E_INVALID_ARGUMENT;
  if (!(kernel_radius > 0.0f) || !std::isfinite(kernel_radius)) return FS_E_INVALID_ARGUMENT;
  const float cell_size = kernel_radius;
  const float bounds_extent = 2.0f;
  const float cells_f = std::ceil((2.0f * bounds_extent) / cell_size);
  // total_cells must fit the u32 buffers (the reference's u32 product)
  if (!(cells_f < 1288.0f)) return FS_E_CAPACITY;
  const uint32_t gs = uint32_t(cells_f) + 2u;
  GpuGridParams g;
  std::memset(&g, 0, sizeof(g));
  g.grid_size_x = g.grid_size_y = g.grid_size_z = gs;
  g.total_cells = gs * gs * gs;
  g.cell_size = cell_size;
  g.inv_cell_size = 1.0f / cell_size;
  g.grid_origin_x = -bounds_extent - cell_size;
  g.grid_origin_y = -bounds_extent - cell_size;
  g.grid_origin_z = -bounds_extent - cell_size;
  g.num_particles = num_particles;
  *out = g;
  return FS_OK;
}

int fs_mc_grid_params(const float grid_min[3], const float grid_max[3], uint32_t grid_size,
                      float kernel_radius, float iso_value, uint32_t num_particles,
                      GpuMcGridParams *out) {
  if (!out || !grid_min || !grid_max || grid_size == 0) return FS_E_INVALID_ARGUMENT;
  const float ex = grid_max[0] - grid_min[0];
  const float ey = grid_max[1] - grid_min[1];
  const float ez = grid_max[2] - grid_min[2];
  GpuMcGridParams p;
  std::memset(&p, 0, sizeof(p));
  std::memcpy(p.grid_min, grid_min, 12);
  std::memcpy(p.grid_max, grid_max, 12);
  p.grid_size = grid_size;
  p.cell_size = std::max(std::max(ex, ey), ez) / float(grid_size);
  p.kernel_radius = kernel_radius;
  p.iso_value = iso_value;
  p.num_particles = num_particles;
  p.max_vertices = 4000000u;
  *out = p;
  return FS_OK;
}

int fs_spawn_positions(const float position[3], uint32_t count, float spread,
                       uint32_t num_particles, uint32_t max_particles, SphParticle3D *out,
                       uint32_t *spawned) {
  if (!position || !spawned) return FS_E_INVALID_ARGUMENT;
  *spawned = 0;
  if (num_particles > max_particles) return FS_E_INVALID_ARGUMENT;
  const uint32_t available = max_particles - num_particles;
  const uint32_t spawn = std::min(count, available);
  if (spawn == 0) return FS_OK;
  if (!out) return FS_E_INVALID_ARGUMENT;
  // golden-angle spiral in layers of 20, sph_3d_grid.rs:1546-1557; the
  // records are SphParticle3D::new (particle.rs:19-31): zero but the position
  for (uint32_t i = 0; i < spawn; i++) {
    const float angle = float(i) * 2.39996f;
    const float r = spread * std::sqrt(float(i) / float(spawn));
    const uint32_t layer = i / 20u;
    std::memset(&out[i], 0, sizeof(SphParticle3D));
    out[i].position[0] = position[0] + r * std::cos(angle);
    out[i].position[1] = position[1] + float(layer) * spread * 0.3f;
    out[i].position[2] = position[2] + r * std::sin(angle);
  }
  *spawned = spawn;
  return FS_OK;
}

int fs_rigid_body_to_gpu(const FsRigidBodyState *state, GpuRigidBody *out) {
  if (!state || !out) return FS_E_INVALID_ARGUMENT;
  fs::rb::to_gpu(*state, *out);
  return FS_OK;
}

int fs_integrate_rigid_body(FsRigidBodyState *state, const GpuContainerGeometry *container,
                            float substep_dt, uint32_t num_substeps, const float gravity[3],
                            const GpuRigidBodyAccum *accum) {
  if (!state || !container || !gravity || !accum) return FS_E_INVALID_ARGUMENT;
  fs::rb::integrate(*state, *container, substep_dt, num_substeps, gravity, *accum);
  return FS_OK;
}

int fs_clamp_rigid_body(FsRigidBodyState *state, const GpuContainerGeometry *container,
                        int bounce_velocity) {
  if (!state || !container) return FS_E_INVALID_ARGUMENT;
  fs::rb::clamp_to_container(*state, *container, bounce_velocity != 0);
  return FS_OK;
}

}  // extern "C"

namespace fs {
float pow_int_f32(float x, unsigned n);
}

float fs::pow_int_f32(float x, unsigned n) {
  double r = 1.0, b = double(x);
  for (; n; n >>= 1) {
    if (n & 1u) r *= b;
    b *= b;
  }
  return float(r);
}
