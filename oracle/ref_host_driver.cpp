// ref_host_driver.cpp — C ABI over the reference's host functions, translated
// from its Rust sources by oracle/rs2cpp.py (oracle/_ref/ref_host.hpp).
//
// TEST INFRASTRUCTURE ONLY: built into oracle/_ref/libref_host.so by
// oracle/build_ref.py where the reference sources are present, and used by
// tests/test_ref_pin_host.py to pin the library's restatements
// (fs_compute_rest_density, fs_compute_pcisph_delta, fs_sph_params_3d,
// fs_container_geometry, fs_quat_to_rotation_rows, fs_rigid_body_to_gpu,
// fs_integrate_rigid_body, fs_clamp_rigid_body, fs_spawn_positions) bit for
// bit. Each entry builds the Rust value the function takes from plain
// arguments and copies its result out; the arithmetic is the translation's.
#include <cstdint>
#include <cstring>

#include "ref_host.hpp"

using namespace refhost;

namespace {

static_assert(sizeof(GpuSphParams3D) == 64, "GpuSphParams3D layout");
static_assert(sizeof(GpuContainerGeometry) == 128, "GpuContainerGeometry layout");
static_assert(sizeof(GpuRigidBody) == 96, "GpuRigidBody layout");
static_assert(sizeof(GpuRigidBodyAccum) == 32, "GpuRigidBodyAccum layout");
static_assert(sizeof(SphParticle3D) == 64, "SphParticle3D layout");
static_assert(sizeof(GpuGridParams) == 48, "GpuGridParams layout");

// The simulated part of RigidBodyConfig (src/state/rigid_body.rs:86-107) as
// plain data, in the field order of the library's FsRigidBodyState.
struct RigidState {
  float position[3];
  float half_extent;
  float velocity[3];
  float density;
  float orientation[4];
  float angular_velocity[3];
  uint32_t shape;
  uint32_t enabled;
  uint32_t held;
  float wall_stiffness;
  uint32_t pad;
};

RigidBodyConfig to_config(const RigidState &s) {
  RigidBodyConfig c{};
  c.enabled = s.enabled != 0;
  c.held = s.held != 0;
  c.shape = RigidBodyShape(int32_t(s.shape));
  for (int k = 0; k < 3; k++) {
    c.position[k] = s.position[k];
    c.velocity[k] = s.velocity[k];
    c.angular_velocity[k] = s.angular_velocity[k];
  }
  for (int k = 0; k < 4; k++) c.orientation[k] = s.orientation[k];
  c.half_extent = s.half_extent;
  c.density = s.density;
  return c;
}

void from_config(const RigidBodyConfig &c, RigidState &s) {
  for (int k = 0; k < 3; k++) {
    s.position[k] = c.position[k];
    s.velocity[k] = c.velocity[k];
    s.angular_velocity[k] = c.angular_velocity[k];
  }
  for (int k = 0; k < 4; k++) s.orientation[k] = c.orientation[k];
}

ContainerConfig container(const float c[6]) {  // width, depth, floor_y, height, tilt_x, tilt_z
  ContainerConfig k{};
  k.width = c[0];
  k.depth = c[1];
  k.floor_y = c[2];
  k.height = c[3];
  k.tilt_x = c[4];
  k.tilt_z = c[5];
  return k;
}

}  // namespace

extern "C" {

float rh_compute_rest_density(float h, float mass) { return rs_compute_rest_density(h, mass); }

float rh_compute_pcisph_delta(float h, float mass, float rest_density, float dt) {
  return rs_compute_pcisph_delta(h, mass, rest_density, dt);
}

// SphConfig::to_gpu_params_3d (rest density derived from h and mass)
void rh_to_gpu_params_3d(float kernel_radius, float stiffness, float near_stiffness,
                         float viscosity, float mass, float surface_tension,
                         float xsph_epsilon, uint32_t num_particles, float dt, void *out) {
  SphConfig c{};
  c.kernel_radius = kernel_radius;
  c.stiffness = stiffness;
  c.near_stiffness = near_stiffness;
  c.viscosity = viscosity;
  c.mass = mass;
  c.surface_tension = surface_tension;
  c.xsph_epsilon = xsph_epsilon;
  const GpuSphParams3D p = m_to_gpu_params_3d(c, num_particles, dt);
  std::memcpy(out, &p, sizeof(p));
}

// ContainerConfig::to_gpu_geometry; c = width, depth, floor_y, height, tilt_x, tilt_z
void rh_to_gpu_geometry(const float c[6], float wall_stiffness, float damping, int clip_enabled,
                        float clip_margin, void *out) {
  const GpuContainerGeometry g =
      m_to_gpu_geometry(container(c), wall_stiffness, damping, clip_enabled != 0, clip_margin);
  std::memcpy(out, &g, sizeof(g));
}

void rh_quat_to_rotation_rows(const float q[4], float rows[12]) {
  const auto r = rs_quat_to_rotation_rows({q[0], q[1], q[2], q[3]});
  std::memcpy(rows, r.data(), sizeof(float) * 12);
}

void rh_to_gpu_rigid_body(const void *state, float wall_stiffness, void *out) {
  const GpuRigidBody b =
      m_to_gpu_rigid_body(to_config(*static_cast<const RigidState *>(state)), wall_stiffness);
  std::memcpy(out, &b, sizeof(b));
}

// integrate_rigid_body (the state's position, velocity, orientation and
// angular velocity are updated in place)
void rh_integrate_rigid_body(void *state, const float c[6], float delta_time,
                             uint32_t num_substeps, const float gravity[3], const void *accum) {
  auto &s = *static_cast<RigidState *>(state);
  RigidBodyConfig cfg = to_config(s);
  GpuRigidBodyAccum a{};
  std::memcpy(&a, accum, sizeof(a));
  rs_integrate_rigid_body(cfg, container(c), delta_time, num_substeps,
                          {gravity[0], gravity[1], gravity[2]}, a);
  from_config(cfg, s);
}

void rh_clamp_rigid_body(void *state, const float c[6], int bounce_velocity) {
  auto &s = *static_cast<RigidState *>(state);
  RigidBodyConfig cfg = to_config(s);
  rs_clamp_rigid_body_to_container(cfg, container(c), bounce_velocity != 0);
  from_config(cfg, s);
}

// SphSimulation3DGrid::spawn_particles on a simulation holding num_particles
// of max_particles: returns the spawned count; the records it wrote at the
// end of the particle buffer go to out (64 bytes each) and the grid
// parameters' particle count to *grid_count.
uint32_t rh_spawn_particles(uint32_t max_particles, uint32_t num_particles, const float position[3],
                            uint32_t count, float spread, void *out, uint32_t *grid_count) {
  SphSimulation3DGrid sim;
  sim.max_particles = max_particles;
  sim.num_particles = num_particles;
  const rs::wgpu_Queue queue;
  const uint32_t n = m_spawn_particles(sim, queue, {position[0], position[1], position[2]},
                                       count, spread);
  const size_t off = size_t(num_particles) * sizeof(SphParticle3D);
  if (n) std::memcpy(out, sim.particle_buffer.bytes.data() + off, size_t(n) * sizeof(SphParticle3D));
  if (grid_count) {
    GpuGridParams g{};
    if (sim.grid_params_buffer.bytes.size() >= sizeof(g))
      std::memcpy(&g, sim.grid_params_buffer.bytes.data(), sizeof(g));
    *grid_count = g.num_particles;
  }
  return n;
}

}  // extern "C"
