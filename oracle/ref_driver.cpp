// ref_driver.cpp — runs the reference's own step shaders (translated
// mechanically to C++ by oracle/wgsl2cpp.py into _ref/ref_shaders.hpp) with
// the buffers, bind groups and dispatch sequence of
// SphSimulation3DGrid::step() (src/simulation/sph_3d_grid.rs:1261-1444).
//
// TEST INFRASTRUCTURE ONLY: it pins the oracle restatement and generates the
// committed golden fixtures. It exports the same C entry points as
// sph_oracle.cpp so the same Python wrapper drives either.
#include <algorithm>
#include <cstring>
#include <vector>

#include "ref_shaders.hpp"

namespace {

using namespace wgsl;

struct ParticleF {  // SphParticle3D as the 64-byte host record
  float position[3], pad0, velocity[3], pad1, force[3], density, near_density, normal[3];
};
static_assert(sizeof(ParticleF) == 64, "particle record");

// the translated structs whose host layout equals the reference's POD layout
static_assert(sizeof(sph_density::SphParams) == 64, "SphParams");
static_assert(sizeof(grid_build::GridParams) == 48, "GridParams");
static_assert(sizeof(sph_density::ContainerGeometry) == 128, "ContainerGeometry");
static_assert(sizeof(sph_force::Gravity) == 16, "Gravity");
static_assert(sizeof(sph_integrate::MouseForce) == 48, "MouseForce");
static_assert(sizeof(sph_integrate::RigidBody) == 96, "RigidBody");
static_assert(sizeof(sph_integrate::RigidBodyAccum) == 32, "RigidBodyAccum");
static_assert(offsetof(sph_integrate::MouseForce, direction) == 32, "MouseForce layout");
static_assert(offsetof(sph_integrate::RigidBody, rot_row0) == 48, "RigidBody layout");

using Particle = grid_build::SphParticle3D;  // every shader declares the same struct

using Pred = pcisph_predict::PredictedState;

template <class To, class From>
To *as(From *p) {
  static_assert(sizeof(To) == sizeof(From), "layout-compatible buffers only");
  return reinterpret_cast<To *>(p);
}

struct RefSim {
  uint32_t num_particles = 0, max_particles = 0, iterations = 5;
  uint8_t sph[64], grid[48], geom[128], gravity[16], mouse[48], rigid[96];
  sph_integrate::RigidBodyAccum accum{};
  std::vector<Particle> P, S;
  std::vector<u32> counts, starts, offsets, cell_idx, s2o, block_sums;
  std::vector<Pred> A, B;
  std::vector<f32> pressure;
  std::vector<float> sdf;
  int sdf_res = 1;

  u32 params_n() const {
    u32 n;
    std::memcpy(&n, sph + 44, 4);
    return n;
  }
  u32 total_cells() const {
    u32 t;
    std::memcpy(&t, grid + 12, 4);
    return t;
  }

  template <class S_>
  void set_params(S_ &dst) const { std::memcpy(&dst, sph, 64); }
  template <class G_>
  void set_grid(G_ &dst) const { std::memcpy(&dst, grid, 48); }

  // step(), sph_3d_grid.rs:1261-1444
  void step() {
    const u32 particle_workgroups = (num_particles + 63u) / 64u;
    const u32 cell_workgroups = (total_cells() + 255u) / 256u;
    // 1. grid clear
    grid_clear::cell_counts = counts.data();
    set_grid(grid_clear::grid);
    grid_clear::dispatch_main(cell_workgroups);
    std::fill(offsets.begin(), offsets.end(), 0u);  // clear_buffer(cell_offsets)
    // 2. grid build
    grid_build::particles = P.data();
    grid_build::cell_counts = counts.data();
    grid_build::particle_cell_indices = cell_idx.data();
    set_grid(grid_build::grid);
    grid_build::dispatch_main(particle_workgroups);
    // copy counts -> starts, then the three scan dispatches
    starts = counts;
    prefix_scan::data = starts.data();
    prefix_scan::block_sums = block_sums.data();
    set_grid(prefix_scan::grid);
    prefix_scan::dispatch_scan_blocks(cell_workgroups);
    prefix_scan::dispatch_scan_block_sums(1);
    prefix_scan::dispatch_add_block_offsets(cell_workgroups);
    // 4. reorder
    grid_reorder::particles_in = as<grid_reorder::SphParticle3D>(P.data());
    grid_reorder::particles_out = as<grid_reorder::SphParticle3D>(S.data());
    grid_reorder::particle_cell_indices = cell_idx.data();
    grid_reorder::cell_offsets = offsets.data();
    grid_reorder::cell_starts = starts.data();
    grid_reorder::cell_counts = counts.data();
    grid_reorder::sorted_to_orig = s2o.data();
    set_grid(grid_reorder::grid);
    grid_reorder::dispatch_main(particle_workgroups);
    // 5. density (container_common prepended)
    set_params(sph_density::params);
    sph_density::sorted_particles = as<sph_density::SphParticle3D>(S.data());
    sph_density::cell_starts = starts.data();
    sph_density::cell_counts = counts.data();
    set_grid(sph_density::grid);
    std::memcpy(&sph_density::container, geom, 128);
    sph_density::dispatch_main(particle_workgroups);
    // 6. XSPH
    set_params(xsph::params);
    xsph::particles = as<xsph::SphParticle3D>(P.data());
    xsph::sorted_particles = as<xsph::SphParticle3D>(S.data());
    xsph::cell_starts = starts.data();
    xsph::cell_counts = counts.data();
    set_grid(xsph::grid);
    xsph::sorted_to_orig = s2o.data();
    xsph::dispatch_main(particle_workgroups);
    // 7. force
    set_params(sph_force::params);
    sph_force::particles = as<sph_force::SphParticle3D>(P.data());
    sph_force::sorted_particles = as<sph_force::SphParticle3D>(S.data());
    sph_force::cell_starts = starts.data();
    sph_force::cell_counts = counts.data();
    set_grid(sph_force::grid);
    std::memcpy(&sph_force::gravity, gravity, 16);
    sph_force::sorted_to_orig = s2o.data();
    sph_force::dispatch_main(particle_workgroups);
    // 8. PCISPH predict -> A
    set_params(pcisph_predict::params);
    pcisph_predict::particles = as<pcisph_predict::SphParticle3D>(P.data());
    pcisph_predict::sorted_predicted = A.data();
    pcisph_predict::sorted_index = cell_idx.data();
    pcisph_predict::prev_pressure = pressure.data();
    pcisph_predict::dispatch_main(particle_workgroups);
    // 9. solve iterations, ping-pong A -> B -> A ...
    set_params(pcisph_solve::params);
    pcisph_solve::particles = as<pcisph_solve::SphParticle3D>(P.data());
    pcisph_solve::cell_starts = starts.data();
    pcisph_solve::cell_counts = counts.data();
    set_grid(pcisph_solve::grid);
    pcisph_solve::sorted_to_orig = s2o.data();
    for (u32 it = 0; it < iterations; it++) {
      auto *in = it % 2 == 0 ? A.data() : B.data();
      auto *out = it % 2 == 0 ? B.data() : A.data();
      pcisph_solve::sorted_predicted_in = as<pcisph_solve::PredictedState>(in);
      pcisph_solve::sorted_predicted_out = as<pcisph_solve::PredictedState>(out);
      pcisph_solve::dispatch_main(particle_workgroups);
    }
    // 10. finalize from A if the iteration count is even, else B (:1409-1413)
    set_params(pcisph_finalize::params);
    pcisph_finalize::particles = as<pcisph_finalize::SphParticle3D>(P.data());
    pcisph_finalize::sorted_predicted =
        as<pcisph_finalize::PredictedState>(iterations % 2 == 0 ? A.data() : B.data());
    pcisph_finalize::sorted_index = cell_idx.data();
    pcisph_finalize::pressure_out = pressure.data();
    pcisph_finalize::dispatch_main(particle_workgroups);
    // 11. integrate
    set_params(sph_integrate::params);
    sph_integrate::particles = as<sph_integrate::SphParticle3D>(P.data());
    std::memcpy(&sph_integrate::container, geom, 128);
    std::memcpy(&sph_integrate::mouse_force, mouse, 48);
    std::memcpy(&sph_integrate::rigid_body, rigid, 96);
    sph_integrate::body_accum = accum;
    sph_integrate::sdf_texture.data = sdf.data();
    sph_integrate::sdf_texture.res = sdf_res;
    sph_integrate::dispatch_main(particle_workgroups);
    accum = sph_integrate::body_accum;
  }
};

Particle from_f(const ParticleF &q) {
  Particle p{};
  p.position = vec3<f32>(q.position[0], q.position[1], q.position[2]);
  p.velocity = vec3<f32>(q.velocity[0], q.velocity[1], q.velocity[2]);
  p.force = vec3<f32>(q.force[0], q.force[1], q.force[2]);
  p.density = q.density;
  p.near_density = q.near_density;
  p.normal_x = q.normal[0];
  p.normal_y = q.normal[1];
  p.normal_z = q.normal[2];
  return p;
}
ParticleF to_f(const Particle &p) {
  ParticleF q{};
  q.position[0] = p.position.x; q.position[1] = p.position.y; q.position[2] = p.position.z;
  q.velocity[0] = p.velocity.x; q.velocity[1] = p.velocity.y; q.velocity[2] = p.velocity.z;
  q.force[0] = p.force.x; q.force[1] = p.force.y; q.force[2] = p.force.z;
  q.density = p.density;
  q.near_density = p.near_density;
  q.normal[0] = p.normal_x; q.normal[1] = p.normal_y; q.normal[2] = p.normal_z;
  return q;
}

// Grid sizing of SphSimulation3DGrid::new (sph_3d_grid.rs:121-143).
void make_grid(float cell_size, uint32_t n, uint8_t out[48]) {
  const float bounds_extent = 2.0f;
  const u32 gs = u32(std::ceil((2.0f * bounds_extent) / cell_size)) + 2u;
  grid_build::GridParams g{};
  g.grid_size_x = g.grid_size_y = g.grid_size_z = gs;
  g.total_cells = gs * gs * gs;
  g.cell_size = cell_size;
  g.inv_cell_size = 1.0f / cell_size;
  g.grid_origin_x = g.grid_origin_y = g.grid_origin_z = -bounds_extent - cell_size;
  g.num_particles = n;
  std::memcpy(out, &g, 48);
}

}  // namespace

extern "C" {

void *or_create(const void *particles, uint32_t n, const void *params, const void *geom,
                uint32_t max_particles, const float *sdf, uint32_t sdf_res, int /*precision*/) {
  auto *s = new RefSim();
  s->num_particles = n;
  s->max_particles = std::max(max_particles, n);
  std::memcpy(s->sph, params, 64);
  std::memcpy(s->geom, geom, 128);
  float h;
  std::memcpy(&h, s->sph, 4);
  // the same effective-count rule as the oracle and the library:
  // min(params.num_particles, n) for every stage
  const u32 eff = std::min(s->params_n(), n);
  std::memcpy(s->sph + 44, &eff, 4);
  make_grid(h, eff, s->grid);
  const float g[4] = {0.0f, -9.8f, 0.0f, 0.0f};
  std::memcpy(s->gravity, g, 16);
  sph_integrate::MouseForce m{};
  m.radius = 0.5f;
  m.strength = 30.0f;
  m.direction = vec3<f32>(0.0f, 0.0f, -1.0f);
  std::memcpy(s->mouse, &m, 48);
  sph_integrate::RigidBody rb{};
  rb.half_extent = 0.15f;
  rb.stiffness = 200.0f;
  rb.rot_row0 = vec4<f32>(1, 0, 0, 0);
  rb.rot_row1 = vec4<f32>(0, 1, 0, 0);
  rb.rot_row2 = vec4<f32>(0, 0, 1, 0);
  std::memcpy(s->rigid, &rb, 96);
  const u32 M = s->max_particles;
  s->P.assign(M, Particle{});
  s->S.assign(M, Particle{});
  for (u32 i = 0; i < n; i++) s->P[i] = from_f(((const ParticleF *)particles)[i]);
  const u32 G = s->total_cells();
  s->counts.assign(G, 0u);
  s->starts.assign(G, 0u);
  s->offsets.assign(G, 0u);
  s->block_sums.assign((G + 255u) / 256u, 0u);
  s->cell_idx.assign(M, 0u);
  s->s2o.assign(M, 0u);
  s->A.assign(M, Pred{});
  s->B.assign(M, Pred{});
  s->pressure.assign(M, 0.0f);
  if (sdf && sdf_res) {
    s->sdf.assign(sdf, sdf + size_t(sdf_res) * sdf_res * sdf_res);
    s->sdf_res = int(sdf_res);
  } else {
    s->sdf.assign(1, 1.0f);
  }
  return s;
}

void or_destroy(void *h) { delete (RefSim *)h; }
void or_set_threads(int) {}
int or_max_threads(void) { return 1; }

void or_step(void *h, uint32_t nsteps, uint64_t *cand, uint64_t *hits) {
  auto *s = (RefSim *)h;
  for (uint32_t k = 0; k < nsteps; k++) s->step();
  if (cand) *cand = 0;
  if (hits) *hits = 0;
}
void or_stage(void *, int, uint32_t) {}

void or_set_params(void *h, const void *q) {
  auto *s = (RefSim *)h;
  std::memcpy(s->sph, q, 64);
  const u32 eff = std::min(s->params_n(), s->num_particles);
  std::memcpy(s->sph + 44, &eff, 4);
  std::memcpy(s->grid + 36, &eff, 4);  // update_sph_params syncs the grid count
}
void or_set_geometry(void *h, const void *q) { std::memcpy(((RefSim *)h)->geom, q, 128); }
void or_set_gravity(void *h, const float *g) {
  const float v[4] = {g[0], g[1], g[2], 0.0f};
  std::memcpy(((RefSim *)h)->gravity, v, 16);
}
void or_set_mouse(void *h, const void *q) { std::memcpy(((RefSim *)h)->mouse, q, 48); }
void or_set_rigid(void *h, const void *q) { std::memcpy(((RefSim *)h)->rigid, q, 96); }
void or_set_iterations(void *h, uint32_t it) { ((RefSim *)h)->iterations = std::max(it, 1u); }
void or_clear_accum(void *h) { ((RefSim *)h)->accum = sph_integrate::RigidBodyAccum{}; }
void or_get_accum(void *h, void *out) { std::memcpy(out, &((RefSim *)h)->accum, 32); }
void or_get_particles(void *h, void *out, uint32_t n) {
  auto *s = (RefSim *)h;
  for (uint32_t i = 0; i < n; i++) ((ParticleF *)out)[i] = to_f(s->P[i]);
}
void or_get_sorted(void *h, void *out, uint32_t n) {
  auto *s = (RefSim *)h;
  for (uint32_t i = 0; i < n; i++) ((ParticleF *)out)[i] = to_f(s->S[i]);
}
void or_get_particles_f64(void *, double *, uint32_t, int) {}
void or_get_cells(void *h, uint32_t *counts, uint32_t *starts) {
  auto *s = (RefSim *)h;
  if (counts) std::copy(s->counts.begin(), s->counts.end(), counts);
  if (starts) std::copy(s->starts.begin(), s->starts.end(), starts);
}
void or_get_index_maps(void *h, uint32_t *cell_idx, uint32_t *s2o, uint32_t n) {
  auto *s = (RefSim *)h;
  if (cell_idx) std::copy(s->cell_idx.begin(), s->cell_idx.begin() + n, cell_idx);
  if (s2o) std::copy(s->s2o.begin(), s->s2o.begin() + n, s2o);
}
void or_get_predicted(void *, int, float *, uint32_t) {}
void or_get_grid(void *h, void *out) { std::memcpy(out, ((RefSim *)h)->grid, 48); }
void or_sincos_f32(const float *, float *, float *, uint32_t) {}

// spray.rs:40-50 (f32)
static float update_auto_limit(float current, float frame_max, float floor_v) {
  if (frame_max <= 1e-6f) return current;
  const float alpha = frame_max > current ? 0.05f : 0.01f;
  return std::max(current + alpha * (frame_max - current), floor_v);
}

// One whitewater frame with the reference's own shaders (spray.rs:348-385):
// the emit pass over the sorted particles of the last step (invocations in
// index order, so the atomic write head hands out slots in that order), the
// ceiling update from this frame's maxima, then the simulate pass over the
// ring. params: GpuSprayParams (its ceilings replaced by `limits`); ring:
// max_particles records of 48 bytes.
void or_spray_frame(void *hv, const void *params, void *ring, uint32_t *head, float *limits,
                    uint32_t *live_stats) {
  auto *h = (RefSim *)hv;
  static_assert(sizeof(spray_emit::SprayParams) == 80, "SprayParams");
  static_assert(sizeof(spray_emit::SprayParticle) == 48, "SprayParticle");
  static_assert(sizeof(spray_emit::SphParticle) == 64, "SphParticle");
  std::memcpy(&spray_emit::params, params, 80);
  spray_emit::params.ta_limit = limits[0];
  spray_emit::params.wc_limit = limits[1];
  spray_emit::sorted_particles = as<spray_emit::SphParticle>(h->S.data());
  spray_emit::spray_particles = (spray_emit::SprayParticle *)ring;
  spray_emit::write_head = *head;
  std::memcpy(&spray_emit::sph_params, h->sph, 64);
  spray_emit::cell_starts = h->starts.data();
  spray_emit::cell_counts = h->counts.data();
  std::memcpy(&spray_emit::grid, h->grid, 48);
  spray_emit::emit_stats = {};
  const u32 n = spray_emit::params.num_sph_particles;
  spray_emit::dispatch_main((n + 63u) / 64u);
  *head = spray_emit::write_head;
  float ta_max, wc_max;
  std::memcpy(&ta_max, &spray_emit::emit_stats[0], 4);
  std::memcpy(&wc_max, &spray_emit::emit_stats[1], 4);
  limits[0] = update_auto_limit(limits[0], ta_max, 0.2f);
  limits[1] = update_auto_limit(limits[1], wc_max, 0.05f);
  std::memcpy(&spray_simulate::params, params, 80);
  std::memcpy(&spray_simulate::container, h->geom, 128);
  spray_simulate::spray_particles = (spray_simulate::SprayParticle *)ring;
  spray_simulate::sorted_particles = as<spray_simulate::SphParticle>(h->S.data());
  spray_simulate::cell_starts = h->starts.data();
  spray_simulate::cell_counts = h->counts.data();
  std::memcpy(&spray_simulate::grid, h->grid, 48);
  std::memcpy(&spray_simulate::sph_params, h->sph, 64);
  spray_simulate::live_stats = {};
  const u32 m = spray_simulate::params.max_particles;
  spray_simulate::dispatch_main((m + 63u) / 64u);
  for (int k = 0; k < 4; k++) live_stats[k] = spray_simulate::live_stats[k];
}

// The MC density pass exactly as mc_density.wgsl runs it, on the sorted
// buffer and cell tables of the last step (bindings of marching_cubes.rs).
void or_density_splat(void *hv, const void *mc, const void *geom, double *out) {
  auto *h = (RefSim *)hv;
  static_assert(sizeof(mc_density::GridParams) == 48, "MC GridParams");
  std::memcpy(&mc_density::params, mc, 48);
  std::memcpy(&mc_density::container, geom, 128);
  std::memcpy(&mc_density::sph_grid, h->grid, 48);
  mc_density::sorted_particles = as<mc_density::SphParticle3D>(h->S.data());
  mc_density::cell_starts = h->starts.data();
  mc_density::cell_counts = h->counts.data();
  mc_density::aniso_params = mc_density::AnisoParams{};  // enabled = 0
  const u32 gs = mc_density::params.grid_size;
  std::vector<float> field(size_t(gs) * gs * gs);
  mc_density::density_field.data = field.data();
  mc_density::density_field.dim = gs;
  const u32 groups = (gs + 3u) / 4u;
  mc_density::dispatch_main(groups, groups, groups);
  for (size_t i = 0; i < field.size(); i++) out[i] = field[i];
}

}  // extern "C"
