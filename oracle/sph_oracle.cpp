// sph_oracle.cpp — CPU oracle for the SPH step (TEST INFRASTRUCTURE ONLY).
//
// This file is the checker, never the product: only tests/, the smoke check of
// __graft_entry__ and bench.py's CPU-baseline / reference arm load it. It is a
// plain C++17 restatement of fluid-toy's per-substep compute pipeline,
// `SphSimulation3DGrid::step()` (src/simulation/sph_3d_grid.rs:1261-1444),
// stage by stage, in the operation order of the WGSL shaders it cites, with
// the reference's buffer dataflow kept literally (64-byte AoS canonical and
// sorted particle buffers, inclusive cell-end scan, orig->slot and slot->orig
// maps, A/B predicted-state ping-pong).
//
// Template parameter R selects the arithmetic: `float` is the FP32
// restatement (compiled with -ffp-contract=off so no multiply-add is fused and
// results are identical on x86-64 and aarch64), `double` is the FP64 twin of
// the same discretisation.
//
// Parity pin: the reference has no tests, golden vectors or fixtures for this
// path, and its WGSL cannot run here (no wgpu/naga, no graphics stack). This
// restatement is pinned against a mechanical C++ translation of the
// reference's own WGSL files (oracle/wgsl2cpp.py, built into oracle/_ref/ when
// the reference sources are present) through the committed fixtures under
// tests/golden/.
//
// Within-cell order: the reference takes a reorder slot with atomicAdd
// (src/shaders/grid_reorder.wgsl:51), so its order inside a cell is
// unspecified. The oracle fixes it to ascending original index (a stable
// counting sort — exactly what the reference's shader produces when its
// invocations run in index order), and the GPU library uses the same order.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <type_traits>
#include <vector>

#include "dual.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---- boundary structs (same layouts as include/fluidsph.h) ----------------
struct ParticleF {  // SphParticle3D, src/simulation/particle.rs:8-17
  float position[3], pad0, velocity[3], pad1, force[3], density, near_density,
      normal[3];
};
struct SphParamsF {  // GpuSphParams3D, src/state/simulation.rs:344-361
  float kernel_radius, kernel_radius_sq, kernel_radius_pow5, kernel_radius_pow6,
      kernel_radius_pow9, mass, rest_density, stiffness, near_stiffness,
      viscosity, dt;
  uint32_t num_particles;
  float surface_tension, pcisph_delta, xsph_epsilon, pad;
};
struct GeomF {  // GpuContainerGeometry, src/state/simulation.rs:367-386
  float half_width, half_height, half_depth, center_y;
  float f0[4], f1[4], f2[4], i0[4], i1[4], i2[4];
  float wall_stiffness, damping;
  uint32_t clip_enabled;
  float clip_margin;
};
struct GravityF {
  float direction[3], pad;
};
struct MouseF {  // GpuMouseForce, src/state/interaction.rs:102-111
  float position[3], radius, strength;
  uint32_t is_active, mode;
  float pad, direction[3], pad2;
};
struct RigidF {  // GpuRigidBody, src/state/rigid_body.rs:212-224
  float position[3], half_extent, velocity[3];
  uint32_t is_active;
  float stiffness;
  uint32_t shape;
  float pad1, pad2, r0[4], r1[4], r2[4];
};
struct AccumI {  // GpuRigidBodyAccum, src/state/rigid_body.rs:247-256
  int32_t force_x, force_y, force_z;
  uint32_t contact_count;
  int32_t torque_x, torque_y, torque_z;
  uint32_t pad;
};
struct GridF {  // GpuGridParams, src/simulation/sph_3d_grid.rs:15-30
  uint32_t gx, gy, gz, total_cells;
  float cell_size, inv_cell_size, ox, oy, oz;
  uint32_t num_particles, pad[2];
};
static_assert(sizeof(ParticleF) == 64, "particle");
static_assert(sizeof(SphParamsF) == 64, "params");
static_assert(sizeof(GeomF) == 128, "geom");
static_assert(sizeof(MouseF) == 48, "mouse");
static_assert(sizeof(RigidF) == 96, "rigid");
static_assert(sizeof(AccumI) == 32, "accum");
static_assert(sizeof(GridF) == 48, "grid");
struct McGridF {  // GpuGridParams of the MC renderer, src/render/marching_cubes.rs:56-66
  float grid_min[3];
  uint32_t grid_size;
  float grid_max[3];
  float cell_size, kernel_radius, iso_value;
  uint32_t num_particles, max_vertices;
};
static_assert(sizeof(McGridF) == 48, "mc grid");

struct SprayParamsF {  // GpuSprayParams, src/state/interaction.rs:129-153
  float min_speed, emission_rate, lifetime, lifetime_variation, drag, speed_multiplier,
      velocity_jitter, dt;
  uint32_t max_particles, num_sph_particles, frame_count;
  float gravity_y, k_trapped_air, k_wave_crest, ta_limit, bubble_buoyancy, bubble_drag, wc_limit,
      pad0, pad1;
};
static_assert(sizeof(SprayParamsF) == 80, "spray params");
struct SprayPartF {  // GpuSprayParticle, src/state/interaction.rs:155-174
  float pos[3], lifetime, vel[3], max_lifetime;
  uint32_t kind;
  float age, pad1, pad2;
};
static_assert(sizeof(SprayPartF) == 48, "spray particle");

// spray_emit.wgsl:140-152
inline uint32_t spray_hash(uint32_t x) {
  x = x ^ (x >> 16u);
  x = x * 0x45d9f3bu;
  x = x ^ (x >> 16u);
  x = x * 0x45d9f3bu;
  x = x ^ (x >> 16u);
  return x;
}
inline float spray_hash_float(uint32_t seed) { return float(spray_hash(seed) & 0xFFFFu) / 65535.0f; }
inline float remap_clamp(float x, float lo, float hi) {
  return std::min(std::max((x - lo) / (hi - lo), 0.0f), 1.0f);
}

// WGSL pow(x, n.0) for an integral n >= 1: binary exponentiation in double,
// rounded once (the library's definition; WGSL leaves pow's precision open).
inline double pow_int_d(double x, unsigned n) {
  double r = 1.0, b = x;
  for (; n; n >>= 1) {
    if (n & 1u) r *= b;
    b *= b;
  }
  return r;
}

// ---- small vector type: every operator is one IEEE op per component --------
template <class R>
struct V3 {
  R x, y, z;
};
template <class R> inline V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
// dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z, left to right, no fusion.
template <class R> inline R dot3(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// math on R: the std functions for float/double, dual.hpp's for Dual
template <class R, class = std::enable_if_t<std::is_arithmetic_v<R>>>
inline R sqrt_(R x) { return std::sqrt(x); }
template <class R, class = std::enable_if_t<std::is_arithmetic_v<R>>>
inline R floor_(R x) { return std::floor(x); }
template <class R, class = std::enable_if_t<std::is_arithmetic_v<R>>>
inline R fabs_(R x) { return std::fabs(x); }
template <class R> inline R len3(V3<R> a) { return sqrt_(dot3(a, a)); }
template <class R> inline V3<R> normalize3(V3<R> a) { return a / len3(a); }
template <class R> inline double norm_d(V3<R> a) {
  const double x = double(a.x), y = double(a.y), z = double(a.z);
  return std::sqrt(x * x + y * y + z * z);
}
template <class R> inline V3<R> cross3(V3<R> a, V3<R> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> inline V3<R> from4(const float *r) { return {R(r[0]), R(r[1]), R(r[2])}; }
template <class R, class = std::enable_if_t<std::is_arithmetic_v<R>>>
inline R fmax_(R a, R b) { return std::fmax(a, b); }
template <class R, class = std::enable_if_t<std::is_arithmetic_v<R>>>
inline R fmin_(R a, R b) { return std::fmin(a, b); }
template <class R> inline R clamp_(R e, R lo, R hi) { return fmin_(fmax_(e, lo), hi); }
template <class R> inline R sign_(R x) { return x > R(0) ? R(1) : (x < R(0) ? R(-1) : R(0)); }
// sin/cos of the close-pair fallback direction (sph_force_3d_grid.wgsl:
// 167-172). WGSL leaves their accuracy to the implementation; the FP32
// restatement fixes one deterministic evaluation so that CPU and GPU agree
// bit for bit: Cody-Waite reduction by pi/2 (three-part constant, each step
// one correctly rounded fma), then the Taylor polynomials of sin and cos on
// [-pi/4, pi/4] in Horner form. The arguments are integer-valued
// (slot differences times 1, 2, 3). The FP64 twin uses libm.
inline float reduce_half_pi(float x, int *quadrant) {
  const float k = std::rint(x * 0.636619747f);
  float r = std::fma(-k, 1.57079637f, x);
  r = std::fma(-k, -4.37113883e-08f, r);
  r = std::fma(-k, -1.71512451e-15f, r);
  *quadrant = int(k) & 3;
  return r;
}
inline float sin_poly(float r) {
  const float r2 = r * r;
  float p = std::fma(r2, 2.75573188e-06f, -1.98412701e-04f);
  p = std::fma(r2, p, 8.33333377e-03f);
  p = std::fma(r2, p, -0.166666672f);
  return std::fma(r * r2, p, r);
}
inline float cos_poly(float r) {
  const float r2 = r * r;
  float p = std::fma(r2, -2.755732e-07f, 2.48015876e-05f);
  p = std::fma(r2, p, -1.38888892e-03f);
  p = std::fma(r2, p, 4.16666679e-02f);
  p = std::fma(r2, p, -0.5f);
  return std::fma(r2, p, 1.0f);
}
inline float sin_f32(float x) {
  int q;
  const float r = reduce_half_pi(x, &q);
  const float s = sin_poly(r), c = cos_poly(r);
  return q == 0 ? s : (q == 1 ? c : (q == 2 ? -s : -c));
}
inline float cos_f32(float x) {
  int q;
  const float r = reduce_half_pi(x, &q);
  const float s = sin_poly(r), c = cos_poly(r);
  return q == 0 ? c : (q == 1 ? -s : (q == 2 ? -c : s));
}
inline float sin_(float x) { return sin_f32(x); }
inline float cos_(float x) { return cos_f32(x); }
inline double sin_(double x) { return std::sin(x); }
inline double cos_(double x) { return std::cos(x); }
template <class V> inline Dual<V> sin_(Dual<V> x) {
  return Dual<V>(sin_(x.v), std::cos(double(x.v)) * x.d);
}
template <class V> inline Dual<V> cos_(Dual<V> x) {
  return Dual<V>(cos_(x.v), -std::sin(double(x.v)) * x.d);
}

// WGSL f32 -> i32 conversion: truncate toward zero, saturate, NaN -> 0.
inline int32_t f2i_sat(double x) {
  if (std::isnan(x)) return 0;
  if (x >= 2147483647.0) return INT32_MAX;
  if (x <= -2147483648.0) return INT32_MIN;
  return int32_t(x);
}

const float PI_F = 3.14159265359f;  // `const PI: f32` in every step shader

template <class R> struct value_is_f32 : std::is_same<R, float> {};
template <> struct value_is_f32<Dual<float>> : std::true_type {};

// ---- per-particle records at precision R ---------------------------------
template <class R>
struct Part {  // SphParticle3D at precision R (field order as the reference)
  V3<R> pos;
  R pad0;
  V3<R> vel;
  R pad1;
  V3<R> force;
  R density, near_density;
  V3<R> normal;
};
template <class R>
struct Pred {  // PredictedState, src/shaders/pcisph_predict.wgsl:33-42
  V3<R> x;
  R pressure;
  V3<R> v;
  R density;
};

template <class R>
struct Params {  // GpuSphParams3D widened to R
  R h, h2, h5, h6, h9, mass, rho0, stiffness, near_k, visc, dt;
  uint32_t n;
  R st, delta, xsph_eps;
};
template <class R>
struct Geom {
  R hw, hh, hd, cy;
  V3<R> f0, f1, f2, i0, i1, i2;
  R wall_k, damping;
};

// container_common.wgsl:28-64
template <class R> inline V3<R> world_to_local(const Geom<R> &c, V3<R> p) {
  V3<R> q{p.x, p.y - c.cy, p.z};
  return {dot3(c.i0, q), dot3(c.i1, q), dot3(c.i2, q)};
}
template <class R> inline V3<R> local_to_world(const Geom<R> &c, V3<R> l) {
  V3<R> r{dot3(c.f0, l), dot3(c.f1, l), dot3(c.f2, l)};
  return {r.x, r.y + c.cy, r.z};
}
template <class R> inline V3<R> world_dir_to_local(const Geom<R> &c, V3<R> d) {
  return {dot3(c.i0, d), dot3(c.i1, d), dot3(c.i2, d)};
}
template <class R> inline V3<R> local_dir_to_world(const Geom<R> &c, V3<R> d) {
  return {dot3(c.f0, d), dot3(c.f1, d), dot3(c.f2, d)};
}

template <class R>
struct Oracle {
  GridF grid{};
  Params<R> p{};
  R gravity[3]{R(0), R(-9.8f), R(0)};  // default, sph_3d_grid.rs:271-274
  Geom<R> geom{};
  MouseF mouse{};
  RigidF rigid{};
  AccumI accum{};
  uint32_t iterations = 5;  // struct default, sph_3d_grid.rs:1253
  uint32_t num_particles = 0, max_particles = 0;
  std::vector<Part<R>> P, S;              // canonical, sorted (AoS)
  std::vector<uint32_t> counts, starts;   // cell_counts, cell_starts (inclusive)
  std::vector<uint32_t> cell_idx, s2o;    // particle_cell_indices, sorted_to_orig
  std::vector<Pred<R>> A, B;              // sorted_predicted_{a,b}
  std::vector<float> sdf;                 // SDF texture texels (x fastest)
  uint32_t sdf_res = 1;

  // Cell coordinates in FP32 arithmetic whatever R is (set on the FP64 twin
  // for per-particle error reports: the integer stages then take the FP32
  // pipeline's decisions, so only the continuous arithmetic differs).
  bool cells_in_f32 = false;
  // Per-particle sums of the magnitudes of the terms each sum adds (canonical
  // order), kept when track_terms is set: the conditioning of the computed
  // sums, for error reports (|sum| << sum of |terms| means cancellation).
  bool track_terms = false;
  std::vector<double> tmag_force, tmag_solve, tmag_normal;
  // grid_build.wgsl:33-44 / sph_density_3d_grid.wgsl:68-81
  inline void position_to_cell(V3<R> pos, int32_t c[3]) const {
    if (cells_in_f32) {
      const float lx = float(pos.x) - grid.ox, ly = float(pos.y) - grid.oy,
                  lz = float(pos.z) - grid.oz;
      c[0] = f2i_sat(double(std::floor(lx * grid.inv_cell_size)));
      c[1] = f2i_sat(double(std::floor(ly * grid.inv_cell_size)));
      c[2] = f2i_sat(double(std::floor(lz * grid.inv_cell_size)));
      return;
    }
    V3<R> l{pos.x - R(grid.ox), pos.y - R(grid.oy), pos.z - R(grid.oz)};
    c[0] = f2i_sat(double(floor_(l.x * R(grid.inv_cell_size))));
    c[1] = f2i_sat(double(floor_(l.y * R(grid.inv_cell_size))));
    c[2] = f2i_sat(double(floor_(l.z * R(grid.inv_cell_size))));
  }
  inline uint32_t cell_to_index_clamped(const int32_t c[3]) const {
    int32_t cx = std::min(std::max(c[0], 0), int32_t(grid.gx) - 1);
    int32_t cy = std::min(std::max(c[1], 0), int32_t(grid.gy) - 1);
    int32_t cz = std::min(std::max(c[2], 0), int32_t(grid.gz) - 1);
    return uint32_t(cx) + uint32_t(cy) * grid.gx + uint32_t(cz) * grid.gx * grid.gy;
  }
  inline bool valid(int32_t x, int32_t y, int32_t z) const {
    return x >= 0 && x < int32_t(grid.gx) && y >= 0 && y < int32_t(grid.gy) && z >= 0 &&
           z < int32_t(grid.gz);
  }
  // Visit neighbour slots j of the 3x3x3 block around the UNCLAMPED cell of
  // `pos`, in the shaders' order: dz, dy, dx outer loops, slot order inside a
  // cell (e.g. sph_density_3d_grid.wgsl:129-167).
  template <class F>
  inline void for_neighbors(V3<R> pos, F &&f) const {
    int32_t c[3];
    position_to_cell(pos, c);
    for (int dz = -1; dz <= 1; dz++)
      for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++) {
          int32_t nx = c[0] + dx, ny = c[1] + dy, nz = c[2] + dz;
          if (!valid(nx, ny, nz)) continue;
          uint32_t idx = uint32_t(nx) + uint32_t(ny) * grid.gx + uint32_t(nz) * grid.gx * grid.gy;
          uint32_t count = counts[idx];
          uint32_t end = starts[idx];
          uint32_t start = end - count;
          for (uint32_t k = 0; k < count; k++) f(start + k);
        }
  }

  // ---- stages -------------------------------------------------------------
  // 1. grid_clear.wgsl:23-29 and the encoder clear of cell_offsets.
  // 2. grid_build.wgsl:46-62: cell index (clamped) + atomic count.
  void stage_hash() {
    std::fill(counts.begin(), counts.end(), 0u);
    const uint32_t n = grid.num_particles;
    for (uint32_t i = 0; i < n; i++) {
      int32_t c[3];
      position_to_cell(P[i].pos, c);
      uint32_t ci = cell_to_index_clamped(c);
      cell_idx[i] = ci;
      counts[ci] += 1u;
    }
  }
  // 3. copy counts -> starts (sph_3d_grid.rs:1295-1301) and the three scan
  //    dispatches of prefix_scan.wgsl:50-122: an inclusive prefix sum.
  void stage_scan() {
    uint32_t acc = 0;
    for (uint32_t c = 0; c < grid.total_cells; c++) {
      acc += counts[c];
      starts[c] = acc;
    }
  }
  // 4. grid_reorder.wgsl:37-63, invocations in index order (stable).
  void stage_reorder() {
    const uint32_t n = grid.num_particles;
    std::vector<uint32_t> offs(grid.total_cells, 0u);
    for (uint32_t i = 0; i < n; i++) {
      uint32_t ci = cell_idx[i];
      uint32_t start = starts[ci] - counts[ci];
      uint32_t slot = offs[ci]++;
      uint32_t dest = start + slot;
      S[dest] = P[i];
      cell_idx[i] = dest;
      s2o[dest] = i;
    }
  }
  // boundary_gamma, sph_density_3d_grid.wgsl:86-109
  R boundary_gamma(V3<R> pos) const {
    const R h = p.h;
    V3<R> l = world_to_local(geom, pos);
    R gamma = R(1);
    R d_nx = l.x - (-geom.hw);
    R d_px = geom.hw - l.x;
    R d_fl = l.y - (-geom.hh);
    R d_ce = geom.hh - l.y;
    R d_nz = l.z - (-geom.hd);
    R d_pz = geom.hd - l.z;
    if (d_nx < h) gamma *= R(0.5f) + R(0.5f) * clamp_(d_nx / h, R(0), R(1));
    if (d_px < h) gamma *= R(0.5f) + R(0.5f) * clamp_(d_px / h, R(0), R(1));
    if (d_fl < h) gamma *= R(0.5f) + R(0.5f) * clamp_(d_fl / h, R(0), R(1));
    if (d_ce < h) gamma *= R(0.5f) + R(0.5f) * clamp_(d_ce / h, R(0), R(1));
    if (d_nz < h) gamma *= R(0.5f) + R(0.5f) * clamp_(d_nz / h, R(0), R(1));
    if (d_pz < h) gamma *= R(0.5f) + R(0.5f) * clamp_(d_pz / h, R(0), R(1));
    return fmax_(gamma, R(0.1f));
  }
  // 5. sph_density_3d_grid.wgsl:111-194 (writes the sorted copy only).
  void stage_density(uint64_t *cand_out, uint64_t *hit_out) {
    const uint32_t n = p.n;
    const R scale_d = R(315.0f) / (R(64.0f) * R(PI_F) * p.h9);
    const R scale_n = R(15.0f) / (R(PI_F) * p.h6);
    const R m_over_rho0 = p.mass / p.rho0;
    const R h8 = p.h6 * p.h * p.h;
    const R normal_scale = R(945.0f) / (R(32.0f) * R(PI_F) * h8);
    uint64_t cand = 0, hits = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : cand, hits)
    for (int64_t si = 0; si < int64_t(n); si++) {
      const uint32_t s = uint32_t(si);
      V3<R> pos_i = S[s].pos;
      R density = R(0), near_density = R(0);
      V3<R> normal{R(0), R(0), R(0)};
      double tnorm = 0.0;
      for_neighbors(pos_i, [&](uint32_t j) {
        V3<R> r_vec = pos_i - S[j].pos;
        R r_sq = dot3(r_vec, r_vec);
        cand++;
        if (r_sq < p.h2) {
          hits++;
          R r = sqrt_(r_sq);
          R diff = p.h2 - r_sq;
          density += p.mass * (scale_d * diff * diff * diff);
          R dn = p.h - r;
          near_density += p.mass * (scale_n * dn * dn * dn);
          if (r_sq > R(1e-12f)) {
            R diff2 = p.h2 - r_sq;
            normal = normal + m_over_rho0 * r_vec * diff2 * diff2;
            if (track_terms) tnorm += norm_d(m_over_rho0 * r_vec * diff2 * diff2);
          }
        }
      });
      if (track_terms) tmag_normal[s2o[s]] = tnorm * double(normal_scale);
      R gamma = boundary_gamma(pos_i);
      density = density / gamma;
      normal = normal * normal_scale;
      S[s].density = density;
      S[s].near_density = near_density;
      S[s].normal = normal;
    }
    if (cand_out) *cand_out = cand;
    if (hit_out) *hit_out = hits;
  }
  // 6. xsph.wgsl:81-138 (scatters to the canonical velocity).
  void stage_xsph() {
    const uint32_t n = p.n;
    const R eps = p.xsph_eps;
    if (eps <= R(0)) return;  // xsph.wgsl:94-97
    const R scale_d = R(315.0f) / (R(64.0f) * R(PI_F) * p.h9);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t si = 0; si < int64_t(n); si++) {
      const uint32_t s = uint32_t(si);
      V3<R> pos_i = S[s].pos, vel_i = S[s].vel;
      V3<R> corr{R(0), R(0), R(0)};
      for_neighbors(pos_i, [&](uint32_t j) {
        V3<R> r_vec = pos_i - S[j].pos;
        R r_sq = dot3(r_vec, r_vec);
        if (r_sq < p.h2 && r_sq > R(1e-12f)) {
          R density_j = fmax_(S[j].density, R(1));
          V3<R> vel_j = S[j].vel;
          R diff = p.h2 - r_sq;
          R w = scale_d * diff * diff * diff;
          corr = corr + (p.mass / density_j) * (vel_j - vel_i) * w;
        }
      });
      P[s2o[s]].vel = vel_i + eps * corr;
    }
  }
  // 7. sph_force_3d_grid.wgsl:105-227 (writes canonical `force` = a_np).
  void stage_force() {
    const uint32_t n = p.n;
    const R h = p.h;
    const R scale_g = R(45.0f) / (R(PI_F) * p.h6);  // both spiky gradients
    const R scale_c = R(32.0f) / (R(PI_F) * p.h9);  // Akinci cohesion
    const R g0 = gravity[0], g1 = gravity[1], g2 = gravity[2];
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t si = 0; si < int64_t(n); si++) {
      const uint32_t s = uint32_t(si);
      const uint32_t orig = s2o[s];
      V3<R> pos_i = S[s].pos;
      V3<R> vel_i = P[orig].vel;
      R density_i = fmax_(S[s].density, R(1));
      R near_density_i = fmax_(S[s].near_density, R(1));
      V3<R> n_i = S[s].normal;
      R near_pressure_i = p.near_k * near_density_i;
      V3<R> a_p{R(0), R(0), R(0)}, a_v{R(0), R(0), R(0)}, a_c{R(0), R(0), R(0)};
      double tf = 0.0, tc = 0.0;
      for_neighbors(pos_i, [&](uint32_t j) {
        V3<R> pos_j = S[j].pos;
        V3<R> r_vec = pos_i - pos_j;
        R r_sq = dot3(r_vec, r_vec);
        if (r_sq < p.h2 && r_sq > R(1e-12f)) {
          R r = sqrt_(r_sq);
          V3<R> dir;
          R min_dist = h * R(0.1f);
          if (r < min_dist) {
            R idx_diff = R(float(s)) - R(float(j));
            dir = normalize3(v3(sin_(idx_diff * R(1)), cos_(idx_diff * R(2)),
                                sin_(idx_diff * R(3))));
          } else {
            dir = normalize3(pos_j - pos_i);
          }
          R density_j = fmax_(S[j].density, R(1));
          R near_density_j = fmax_(S[j].near_density, R(1));
          R near_pressure_j = p.near_k * near_density_j;
          R dg = h - r;
          R grad = scale_g * dg * dg;
          a_p = a_p + (-p.mass * (near_pressure_i + near_pressure_j) /
                       (R(2) * density_i * near_density_j)) * dir * grad;
          if (track_terms)
            tf += norm_d((-p.mass * (near_pressure_i + near_pressure_j) /
                          (R(2) * density_i * near_density_j)) * dir * grad);
          if (r < min_dist) {
            R sep = R(200.0f) * (R(1) - r / min_dist);
            a_p = a_p + (-sep) * dir;
            if (track_terms) tf += std::fabs(double(sep));
          }
          V3<R> vel_j = S[j].vel;
          V3<R> v_ij = vel_i - vel_j;
          V3<R> x_ij = pos_i - pos_j;
          R v_dot_x = dot3(v_ij, x_ij);
          if (v_dot_x < R(0)) {
            R mu = h * v_dot_x / (r_sq + R(0.01f) * p.h2);
            R avg_density = (density_i + density_j) * R(0.5f);
            R pi_visc = -p.visc * mu / avg_density;
            a_v = a_v + (-p.mass * pi_visc * grad) * dir;
            if (track_terms) tf += norm_d((-p.mass * pi_visc * grad) * dir);
          }
          R K_ij = R(2) * p.rho0 / (density_i + density_j);
          // akinci_cohesion_kernel, sph_force_3d_grid.wgsl:77-88
          R r3 = r * r * r;
          R coh;
          if (r >= h * R(0.5f)) {
            coh = scale_c * dg * dg * dg * r3;
          } else {
            coh = scale_c * (R(2) * dg * dg * dg * r3 - p.h6 / R(64.0f));
          }
          a_c = a_c + (p.mass * K_ij * coh) * dir;
          V3<R> n_j = S[j].normal;
          a_c = a_c - (p.mass * K_ij) * (n_i - n_j);
          if (track_terms)
            tc += norm_d((p.mass * K_ij * coh) * dir) + norm_d((p.mass * K_ij) * (n_i - n_j));
        }
      });
      if (track_terms)
        tmag_force[orig] = tf + tc * std::fabs(double(p.st)) +
                           std::sqrt(double(g0) * double(g0) + double(g1) * double(g1) +
                                     double(g2) * double(g2));
      a_c = a_c * p.st;
      V3<R> a_g{g0, g1, g2};
      P[orig].force = a_p + a_v + a_c + a_g;
    }
  }
  // 8. pcisph_predict.wgsl:50-73 (canonical order, writes A[slot]).
  void stage_predict() {
    const uint32_t n = p.n;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < int64_t(n); ii++) {
      const uint32_t i = uint32_t(ii);
      V3<R> v_star = P[i].vel + p.dt * P[i].force;
      V3<R> x_star = P[i].pos + p.dt * v_star;
      Pred<R> &o = A[cell_idx[i]];
      o.x = x_star;
      o.pressure = R(0);
      o.v = v_star;
      o.density = R(0);
    }
  }
  // 9. pcisph_solve.wgsl:99-208, one iteration (in -> out).
  void stage_solve(const std::vector<Pred<R>> &in, std::vector<Pred<R>> &out) {
    const uint32_t n = p.n;
    const R h = p.h;
    const R scale_d = R(315.0f) / (R(64.0f) * R(PI_F) * p.h9);
    const R scale_g = R(45.0f) / (R(PI_F) * p.h6);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t si = 0; si < int64_t(n); si++) {
      const uint32_t s = uint32_t(si);
      const uint32_t orig = s2o[s];
      const Pred<R> self = in[s];
      V3<R> pred_pos = self.x;
      R old_p = self.pressure;
      V3<R> pos_i = P[orig].pos;
      R pred_density = R(0);
      V3<R> a_p{R(0), R(0), R(0)};
      double ts = 0.0;
      for_neighbors(pos_i, [&](uint32_t j) {
        const Pred<R> &nb = in[j];
        V3<R> r_vec = pred_pos - nb.x;
        R r_sq = dot3(r_vec, r_vec);
        if (r_sq < p.h2) {
          R diff = p.h2 - r_sq;
          pred_density += p.mass * (scale_d * diff * diff * diff);
          if (r_sq > R(1e-12f)) {
            R r = sqrt_(r_sq);
            R nd = fmax_(nb.density, R(1));
            R np = nb.pressure;
            R sd = fmax_(self.density, R(1));
            V3<R> dir = (-r_vec) / r;
            R dg = h - r;
            R grad = scale_g * dg * dg;
            a_p = a_p + (-p.mass * (old_p / (sd * sd) + np / (nd * nd)) * grad) * dir;
            if (track_terms)
              ts += norm_d((-p.mass * (old_p / (sd * sd) + np / (nd * nd)) * grad) * dir);
          }
        }
      });
      if (track_terms) tmag_solve[orig] = ts;
      R density_error = fmax_(R(0), pred_density - p.rho0);
      R new_p = old_p + p.delta * density_error;
      R max_accel = R(0.25f) * h / (p.dt * p.dt);
      R mag_sq = dot3(a_p, a_p);
      R max_sq = max_accel * max_accel;
      if (mag_sq > max_sq) a_p = a_p * (max_accel / sqrt_(mag_sq));
      V3<R> a_total = P[orig].force + a_p;
      V3<R> v_star = P[orig].vel + p.dt * a_total;
      V3<R> x_star = P[orig].pos + p.dt * v_star;
      Pred<R> &o = out[s];
      o.x = x_star;
      o.pressure = new_p;
      o.v = v_star;
      o.density = pred_density;
    }
  }
  // 10. pcisph_finalize.wgsl:50-74
  void stage_finalize(const std::vector<Pred<R>> &fin) {
    const uint32_t n = p.n;
#pragma omp parallel for schedule(static)
    for (int64_t ii = 0; ii < int64_t(n); ii++) {
      const uint32_t i = uint32_t(ii);
      V3<R> corrected = fin[cell_idx[i]].v;
      V3<R> original = P[i].vel;
      P[i].force = corrected - original;
      P[i].vel = corrected;
    }
  }
  // SDF texture sample with clamp-to-edge trilinear filtering
  // (sph_3d_grid.rs:336-344; exact FP32 weights).
  R sample_sdf(V3<R> uvw) const {
    const int res = int(sdf_res);
    auto texel = [&](int x, int y, int z) -> R {
      x = std::min(std::max(x, 0), res - 1);
      y = std::min(std::max(y, 0), res - 1);
      z = std::min(std::max(z, 0), res - 1);
      return R(sdf[size_t(x) + size_t(y) * res + size_t(z) * res * res]);
    };
    R tx = uvw.x * R(float(res)) - R(0.5f);
    R ty = uvw.y * R(float(res)) - R(0.5f);
    R tz = uvw.z * R(float(res)) - R(0.5f);
    R fx0 = floor_(tx), fy0 = floor_(ty), fz0 = floor_(tz);
    R ax = tx - fx0, ay = ty - fy0, az = tz - fz0;
    int x0 = std::min(std::max(f2i_sat(double(fx0)), -1), res);
    int y0 = std::min(std::max(f2i_sat(double(fy0)), -1), res);
    int z0 = std::min(std::max(f2i_sat(double(fz0)), -1), res);
    auto mix = [](R a, R b, R t) { return a * (R(1) - t) + b * t; };
    R c00 = mix(texel(x0, y0, z0), texel(x0 + 1, y0, z0), ax);
    R c10 = mix(texel(x0, y0 + 1, z0), texel(x0 + 1, y0 + 1, z0), ax);
    R c01 = mix(texel(x0, y0, z0 + 1), texel(x0 + 1, y0, z0 + 1), ax);
    R c11 = mix(texel(x0, y0 + 1, z0 + 1), texel(x0 + 1, y0 + 1, z0 + 1), ax);
    R c0 = mix(c00, c10, ay);
    R c1 = mix(c01, c11, ay);
    return mix(c0, c1, az);
  }
  // 11. sph_integrate_3d.wgsl:91-388
  void stage_integrate() {
    const uint32_t n = p.n;
    const R h = p.h;
    const Geom<R> &c = geom;
    // fixed-point accumulators: 32-bit wrapping sums (order-independent)
    uint32_t fx = 0, fy = 0, fz = 0, cnt = 0, tx = 0, ty = 0, tz = 0;
#pragma omp parallel for schedule(static) reduction(+ : fx, fy, fz, cnt, tx, ty, tz)
    for (int64_t ii = 0; ii < int64_t(n); ii++) {
      const uint32_t i = uint32_t(ii);
      V3<R> pos = P[i].pos, vel = P[i].vel;
      V3<R> accel{R(0), R(0), R(0)};
      V3<R> lp = world_to_local(c, pos);
      V3<R> lv = world_dir_to_local(c, vel);
      const R bl = h * R(0.4f);
      const R wd = R(8.0f);
      V3<R> wa{R(0), R(0), R(0)};
      R d = lp.x - (-c.hw);
      if (d < bl) { R t = R(1) - d / bl; wa.x += c.wall_k * t * t; if (lv.x < R(0)) wa.x -= lv.x * wd * t; }
      d = c.hw - lp.x;
      if (d < bl) { R t = R(1) - d / bl; wa.x -= c.wall_k * t * t; if (lv.x > R(0)) wa.x -= lv.x * wd * t; }
      d = lp.y - (-c.hh);
      if (d < bl) { R t = R(1) - d / bl; wa.y += c.wall_k * t * t; if (lv.y < R(0)) wa.y -= lv.y * wd * t; }
      d = c.hh - lp.y;
      if (d < bl) { R t = R(1) - d / bl; wa.y -= c.wall_k * t * t; if (lv.y > R(0)) wa.y -= lv.y * wd * t; }
      d = lp.z - (-c.hd);
      if (d < bl) { R t = R(1) - d / bl; wa.z += c.wall_k * t * t; if (lv.z < R(0)) wa.z -= lv.z * wd * t; }
      d = c.hd - lp.z;
      if (d < bl) { R t = R(1) - d / bl; wa.z -= c.wall_k * t * t; if (lv.z > R(0)) wa.z -= lv.z * wd * t; }
      accel = accel + local_dir_to_world(c, wa);

      // mouse force, sph_integrate_3d.wgsl:162-200
      if (mouse.is_active == 1u) {
        V3<R> to_mouse = from4<R>(mouse.position) - pos;
        R dist = len3(to_mouse);
        if (dist < R(mouse.radius) && dist > R(0.001f)) {
          R falloff = R(1) - dist / R(mouse.radius);
          V3<R> fd = normalize3(to_mouse);
          R sm = R(mouse.strength) * falloff;
          switch (mouse.mode) {
            case 1: accel = accel + fd * sm; break;  // pull
            case 2: {                                // vortex
              V3<R> axis = normalize3(from4<R>(mouse.direction));
              V3<R> tangent = cross3(fd, axis);
              R tlen = len3(tangent);
              if (tlen > R(0.001f)) accel = accel + (tangent / tlen) * sm;
              break;
            }
            case 3: accel = accel - fd * sm * R(3); break;  // explode
            case 4: {                                        // drain
              V3<R> dd = normalize3(fd + v3(R(0), R(-1), R(0)));
              accel = accel + dd * sm;
              break;
            }
            default: accel = accel - fd * sm; break;  // push
          }
        }
      }

      // rigid-body penalty, sph_integrate_3d.wgsl:202-341
      if (rigid.is_active != 0u) {
        V3<R> world_rel = pos - from4<R>(rigid.position);
        V3<R> rr0 = from4<R>(rigid.r0), rr1 = from4<R>(rigid.r1), rr2 = from4<R>(rigid.r2);
        V3<R> rl{dot3(rr0, world_rel), dot3(rr1, world_rel), dot3(rr2, world_rel)};
        const R he = R(rigid.half_extent);
        R sdf_v;
        V3<R> ln{R(0), R(0), R(0)};
        switch (rigid.shape) {
          case 1: {  // sphere
            R dist = len3(rl);
            sdf_v = dist - he;
            if (dist > R(0.001f)) ln = rl / dist; else ln = v3(R(0), R(1), R(0));
            break;
          }
          case 2: {  // cylinder
            R radial = sqrt_(rl.x * rl.x + rl.z * rl.z);
            R d_radial = radial - he;
            R d_cap = fabs_(rl.y) - he;
            sdf_v = fmax_(d_radial, d_cap);
            if (d_radial > d_cap) {
              if (radial > R(0.001f)) ln = v3(rl.x / radial, R(0), rl.z / radial);
              else ln = v3(R(1), R(0), R(0));
            } else {
              ln = v3(R(0), sign_(rl.y), R(0));
            }
            break;
          }
          case 3: {  // torus
            R minor_r = he * R(0.3f);
            R xz_len = sqrt_(rl.x * rl.x + rl.z * rl.z);
            R qx = xz_len - he, qy = rl.y;
            R q_len = sqrt_(qx * qx + qy * qy);
            sdf_v = q_len - minor_r;
            if (q_len > R(0.001f) && xz_len > R(0.001f)) {
              R rdx = qx / q_len, rdy = qy / q_len;
              ln = v3(rdx * rl.x / xz_len, rdy, rdx * rl.z / xz_len);
            } else {
              ln = v3(R(0), R(1), R(0));
            }
            break;
          }
          case 4: {  // custom SDF
            V3<R> nrm = rl / he;
            V3<R> uvw = nrm * R(0.5f) + v3(R(0.5f), R(0.5f), R(0.5f));
            R raw = sample_sdf(uvw);
            sdf_v = raw * he;
            const R e = R(1.0f / 32.0f);
            R gx = sample_sdf(uvw + v3(e, R(0), R(0))) - sample_sdf(uvw - v3(e, R(0), R(0)));
            R gy = sample_sdf(uvw + v3(R(0), e, R(0))) - sample_sdf(uvw - v3(R(0), e, R(0)));
            R gz = sample_sdf(uvw + v3(R(0), R(0), e)) - sample_sdf(uvw - v3(R(0), R(0), e));
            V3<R> g{gx, gy, gz};
            R gl = len3(g);
            if (gl > R(1e-6f)) ln = g / gl;
            else ln = normalize3(rl + v3(R(0), R(1e-6f), R(0)));
            break;
          }
          default: {  // cube
            V3<R> dd{fabs_(rl.x) - he, fabs_(rl.y) - he, fabs_(rl.z) - he};
            sdf_v = fmax_(dd.x, fmax_(dd.y, dd.z));
            if (dd.x >= dd.y && dd.x >= dd.z) ln = v3(sign_(rl.x), R(0), R(0));
            else if (dd.y >= dd.x && dd.y >= dd.z) ln = v3(R(0), sign_(rl.y), R(0));
            else ln = v3(R(0), R(0), sign_(rl.z));
            break;
          }
        }
        const R range = h * R(0.7f);
        if (sdf_v < range) {
          V3<R> nw{rr0.x * ln.x + rr1.x * ln.y + rr2.x * ln.z,
                   rr0.y * ln.x + rr1.y * ln.y + rr2.y * ln.z,
                   rr0.z * ln.x + rr1.z * ln.y + rr2.z * ln.z};
          R pen = range - sdf_v;
          R t = pen / range;
          V3<R> penalty = nw * R(rigid.stiffness) * t * t;
          accel = accel + penalty;
          V3<R> damp{R(0), R(0), R(0)};
          V3<R> rel_vel = vel - from4<R>(rigid.velocity);
          R vn = dot3(rel_vel, nw);
          if (vn < R(0)) {
            damp = (-nw) * vn * R(5.0f);
            accel = accel + damp;
          }
          V3<R> reaction = (-(penalty + damp)) * p.mass;
          fx += uint32_t(f2i_sat(double(reaction.x * R(1000.0f))));
          fy += uint32_t(f2i_sat(double(reaction.y * R(1000.0f))));
          fz += uint32_t(f2i_sat(double(reaction.z * R(1000.0f))));
          cnt += 1u;
          V3<R> torque = cross3(world_rel, reaction);
          tx += uint32_t(f2i_sat(double(torque.x * R(1000.0f))));
          ty += uint32_t(f2i_sat(double(torque.y * R(1000.0f))));
          tz += uint32_t(f2i_sat(double(torque.z * R(1000.0f))));
        }
      }

      vel = vel + p.dt * accel;
      pos = pos + p.dt * vel;

      // hard backstop, sph_integrate_3d.wgsl:347-384
      V3<R> lpn = world_to_local(c, pos);
      V3<R> lvn = world_dir_to_local(c, vel);
      const R rest = c.damping;
      if (lpn.x < -c.hw) { lpn.x = -c.hw; lvn.x = fabs_(lvn.x) * rest; }
      else if (lpn.x > c.hw) { lpn.x = c.hw; lvn.x = -fabs_(lvn.x) * rest; }
      if (lpn.y < -c.hh) { lpn.y = -c.hh; lvn.y = fabs_(lvn.y) * rest; }
      else if (lpn.y > c.hh) { lpn.y = c.hh; lvn.y = -fabs_(lvn.y) * rest; }
      if (lpn.z < -c.hd) { lpn.z = -c.hd; lvn.z = fabs_(lvn.z) * rest; }
      else if (lpn.z > c.hd) { lpn.z = c.hd; lvn.z = -fabs_(lvn.z) * rest; }
      P[i].pos = local_to_world(c, lpn);
      P[i].vel = local_dir_to_world(c, lvn);
    }
    accum.force_x = int32_t(uint32_t(accum.force_x) + fx);
    accum.force_y = int32_t(uint32_t(accum.force_y) + fy);
    accum.force_z = int32_t(uint32_t(accum.force_z) + fz);
    accum.contact_count += cnt;
    accum.torque_x = int32_t(uint32_t(accum.torque_x) + tx);
    accum.torque_y = int32_t(uint32_t(accum.torque_y) + ty);
    accum.torque_z = int32_t(uint32_t(accum.torque_z) + tz);
  }

  // step(), sph_3d_grid.rs:1261-1444
  void step(uint64_t *cand, uint64_t *hits) {
    stage_hash();
    stage_scan();
    stage_reorder();
    stage_density(cand, hits);
    stage_xsph();
    stage_force();
    stage_predict();
    for (uint32_t it = 0; it < iterations; it++) {
      if (it % 2 == 0) stage_solve(A, B); else stage_solve(B, A);
    }
    stage_finalize(iterations % 2 == 0 ? A : B);
    stage_integrate();
  }

  // ---- marshalling ----------------------------------------------------------
  static Part<R> from_f(const ParticleF &q) {
    Part<R> r;
    r.pos = v3(R(q.position[0]), R(q.position[1]), R(q.position[2]));
    r.pad0 = R(q.pad0);
    r.vel = v3(R(q.velocity[0]), R(q.velocity[1]), R(q.velocity[2]));
    r.pad1 = R(q.pad1);
    r.force = v3(R(q.force[0]), R(q.force[1]), R(q.force[2]));
    r.density = R(q.density);
    r.near_density = R(q.near_density);
    r.normal = v3(R(q.normal[0]), R(q.normal[1]), R(q.normal[2]));
    return r;
  }
  static ParticleF to_f(const Part<R> &r) {
    ParticleF q;
    q.position[0] = float(r.pos.x); q.position[1] = float(r.pos.y); q.position[2] = float(r.pos.z);
    q.pad0 = float(r.pad0);
    q.velocity[0] = float(r.vel.x); q.velocity[1] = float(r.vel.y); q.velocity[2] = float(r.vel.z);
    q.pad1 = float(r.pad1);
    q.force[0] = float(r.force.x); q.force[1] = float(r.force.y); q.force[2] = float(r.force.z);
    q.density = float(r.density);
    q.near_density = float(r.near_density);
    q.normal[0] = float(r.normal.x); q.normal[1] = float(r.normal.y); q.normal[2] = float(r.normal.z);
    return q;
  }
  void set_params(const SphParamsF &q) {
    p.h = R(q.kernel_radius); p.h2 = R(q.kernel_radius_sq); p.h5 = R(q.kernel_radius_pow5);
    p.h6 = R(q.kernel_radius_pow6); p.h9 = R(q.kernel_radius_pow9); p.mass = R(q.mass);
    p.rho0 = R(q.rest_density); p.stiffness = R(q.stiffness); p.near_k = R(q.near_stiffness);
    p.visc = R(q.viscosity); p.dt = R(q.dt);
    p.n = std::min(q.num_particles, num_particles);
    p.st = R(q.surface_tension); p.delta = R(q.pcisph_delta); p.xsph_eps = R(q.xsph_epsilon);
    grid.num_particles = p.n;  // update_sph_params keeps both counts in sync
  }
  // mc_density.wgsl:130-231, isotropic path (anisotropy off): the poly6
  // density of the sorted positions S at the centres of gs^3 voxels (x
  // fastest), over the SPH cells within ceil(h / cell) of the voxel's
  // unclamped cell in dz, dy, dx, slot order; -1 outside the box when
  // clipping; else divided by the five-wall gamma (mc_density.wgsl:110-128).
  // The cell radius is an index quantity and is taken in f32 at any R.
  template <class T>
  void splat_into(const McGridF &mc, const GeomF &cgf, T *out) const {
    Geom<R> cg;
    cg.hw = R(cgf.half_width); cg.hh = R(cgf.half_height); cg.hd = R(cgf.half_depth);
    cg.cy = R(cgf.center_y);
    cg.i0 = from4<R>(cgf.i0); cg.i1 = from4<R>(cgf.i1); cg.i2 = from4<R>(cgf.i2);
    const uint32_t gs = mc.grid_size;
    const R h = R(mc.kernel_radius);
    const R h_sq = h * h;
    const R pow9 = value_is_f32<R>::value ? R(float(pow_int_d(double(mc.kernel_radius), 9)))
                                          : R(pow_int_d(double(mc.kernel_radius), 9));
    const R coeff = R(315) / (R(64) * R(PI_F) * pow9);
    const int32_t cr = f2i_sat(double(std::ceil(mc.kernel_radius * grid.inv_cell_size)));
    const R cs = R(mc.cell_size);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t zi = 0; zi < int64_t(gs); zi++) {
      const uint32_t z = uint32_t(zi);
      for (uint32_t y = 0; y < gs; y++)
        for (uint32_t x = 0; x < gs; x++) {
          const V3<R> wp{R(mc.grid_min[0]) + (R(float(x)) + R(0.5f)) * cs,
                         R(mc.grid_min[1]) + (R(float(y)) + R(0.5f)) * cs,
                         R(mc.grid_min[2]) + (R(float(z)) + R(0.5f)) * cs};
          int32_t c[3];
          position_to_cell(wp, c);
          R density = R(0);
          for (int32_t dz = -cr; dz <= cr; dz++)
            for (int32_t dy = -cr; dy <= cr; dy++)
              for (int32_t dx = -cr; dx <= cr; dx++) {
                const int64_t nx = int64_t(c[0]) + dx, ny = int64_t(c[1]) + dy,
                              nz = int64_t(c[2]) + dz;
                if (nx < 0 || nx >= int64_t(grid.gx) || ny < 0 || ny >= int64_t(grid.gy) ||
                    nz < 0 || nz >= int64_t(grid.gz))
                  continue;
                const uint32_t idx = uint32_t(nx) + uint32_t(ny) * grid.gx +
                                     uint32_t(nz) * grid.gx * grid.gy;
                const uint32_t count = counts[idx];
                const uint32_t start = starts[idx] - count;
                for (uint32_t k = 0; k < count; k++) {
                  const V3<R> d = wp - S[start + k].pos;
                  const R r_sq = dot3(d, d);
                  if (r_sq < h_sq) {
                    const R diff = h_sq - r_sq;
                    density += coeff * diff * diff * diff;
                  }
                }
              }
          const V3<R> q{wp.x, wp.y - cg.cy, wp.z};
          const V3<R> l{dot3(cg.i0, q), dot3(cg.i1, q), dot3(cg.i2, q)};
          T &o = out[size_t(x) + size_t(gs) * (size_t(y) + size_t(gs) * z)];
          if (cgf.clip_enabled != 0u &&
              !(l.x >= -cg.hw && l.x <= cg.hw && l.y >= -cg.hh && l.y <= cg.hh &&
                l.z >= -cg.hd && l.z <= cg.hd)) {
            o = T(-1.0);
            continue;
          }
          R gamma = R(1);
          const R dnx = l.x + cg.hw, dpx = cg.hw - l.x, dfl = l.y + cg.hh;
          const R dnz = l.z + cg.hd, dpz = cg.hd - l.z;
          auto fac = [&](R dd) {
            R t = dd / h;
            t = std::min(std::max(t, R(0)), R(1));
            return R(0.5f) + R(0.5f) * t;
          };
          if (dnx < h) gamma *= fac(dnx);
          if (dpx < h) gamma *= fac(dpx);
          if (dfl < h) gamma *= fac(dfl);
          if (dnz < h) gamma *= fac(dnz);
          if (dpz < h) gamma *= fac(dpz);
          gamma = std::max(gamma, R(0.15f));
          o = T(density / gamma);
        }
    }
  }

  // spray_emit.wgsl:180-372 over the sorted particles in index order: the
  // write head hands out ring slots sequentially. stats: per-frame maxima
  // bits (trapped air, wave crest). ta/wc: this frame's ceilings.
  void spray_emit(const SprayParamsF &prm, float ta, float wc, SprayPartF *ring, uint32_t *head,
                  uint32_t stats[2]) const {
    const float PI_S = 3.14159265359f, TWO_PI_S = 6.28318530718f;
    const uint32_t n = std::min(prm.num_sph_particles, p.n);
    const float h = float(p.h), h_sq = float(p.h2);
    const float mass = float(p.mass);
    const float poly6_norm = 315.0f / (64.0f * PI_S * float(p.h9));
    for (uint32_t i = 0; i < n; i++) {
      const Part<R> &pi = S[i];
      const V3<float> pos{float(pi.pos.x), float(pi.pos.y), float(pi.pos.z)};
      const V3<float> vel{float(pi.vel.x), float(pi.vel.y), float(pi.vel.z)};
      const float speed = len3(vel);
      if (speed < prm.min_speed) continue;
      const V3<float> normal_i{float(pi.normal.x), float(pi.normal.y), float(pi.normal.z)};
      const float n_len_i = len3(normal_i);
      const bool crest_eligible = n_len_i > 1e-4f && float(pi.density) < float(p.rho0) * 0.9f;
      V3<float> n_hat_i{0.0f, 1.0f, 0.0f};
      if (crest_eligible) n_hat_i = normal_i / n_len_i;
      float trapped_air = 0.0f, crest = 0.0f, divergence = 0.0f;
      uint32_t n_neighbors = 0u;
      for_neighbors(pi.pos, [&](uint32_t j) {
        const Part<R> &pj = S[j];
        const V3<float> pjp{float(pj.pos.x), float(pj.pos.y), float(pj.pos.z)};
        const V3<float> r_vec = pos - pjp;
        const float r_sq = dot3(r_vec, r_vec);
        if (r_sq >= h_sq || r_sq < 1e-12f) return;
        const float r = std::sqrt(r_sq);
        const float w = 1.0f - r / h;
        const V3<float> x_hat = r_vec / r;
        n_neighbors += 1u;
        const float d2 = h_sq - r_sq;
        const float w_vol = (mass / std::max(float(pj.density), 1e-6f)) * poly6_norm * d2 * d2 * d2;
        const V3<float> v_ij = vel - V3<float>{float(pj.vel.x), float(pj.vel.y), float(pj.vel.z)};
        const float v_ij_len = len3(v_ij);
        if (v_ij_len > 1e-6f) trapped_air += v_ij_len * (1.0f - dot3(v_ij / v_ij_len, x_hat)) * w_vol;
        divergence += dot3(v_ij, x_hat) * w;
        if (crest_eligible && dot3(-x_hat, n_hat_i) < 0.0f) {
          const V3<float> normal_j{float(pj.normal.x), float(pj.normal.y), float(pj.normal.z)};
          const float n_len_j = len3(normal_j);
          if (n_len_j > 1e-4f) crest += (1.0f - dot3(n_hat_i, normal_j / n_len_j)) * w_vol;
        }
      });
      if (n_neighbors < 10u) continue;
      if (dot3(vel / speed, n_hat_i) < 0.6f) crest = 0.0f;
      uint32_t bits;
      if (trapped_air > 0.0f) {
        std::memcpy(&bits, &trapped_air, 4);
        stats[0] = std::max(stats[0], bits);
      }
      if (crest > 0.0f) {
        std::memcpy(&bits, &crest, 4);
        stats[1] = std::max(stats[1], bits);
      }
      const float phi_div = remap_clamp(divergence, 0.0f, 0.5f);
      const float ta_hi = std::max(ta, 1e-4f), wc_hi = std::max(wc, 1e-4f);
      const float phi_ta = remap_clamp(trapped_air, 0.1f * ta_hi, ta_hi);
      const float phi_wc = remap_clamp(crest, 0.1f * wc_hi, wc_hi) * phi_div;
      const float phi_k = remap_clamp(speed, prm.min_speed, 2.5f);
      const float rate = phi_k * (prm.k_trapped_air * phi_ta + prm.k_wave_crest * phi_wc) * prm.emission_rate;
      const float expected = rate * prm.dt;
      const uint32_t base_seed = i + prm.frame_count * 7919u;
      uint32_t n_emit = uint32_t(std::floor(expected));
      if (spray_hash_float(base_seed * 13u + 5u) < expected - std::floor(expected)) n_emit = n_emit + 1u;
      n_emit = std::min(n_emit, 16u);
      if (n_emit == 0u) continue;
      const V3<float> v_dir = vel / speed;
      V3<float> ref_axis{0.0f, 1.0f, 0.0f};
      if (std::fabs(v_dir.y) > 0.99f) ref_axis = V3<float>{1.0f, 0.0f, 0.0f};
      const V3<float> e1 = normalize3(cross3(v_dir, ref_axis));
      const V3<float> e2 = cross3(v_dir, e1);
      for (uint32_t e = 0u; e < n_emit; e = e + 1u) {
        const uint32_t slot = ((*head)++) % prm.max_particles;
        const uint32_t seed = base_seed + e * 3571u;
        const float r0 = spray_hash_float(seed), r1 = spray_hash_float(seed + 1u);
        const float r2 = spray_hash_float(seed + 2u), r3 = spray_hash_float(seed + 3u);
        const float r4 = spray_hash_float(seed + 4u) * 2.0f - 1.0f;
        const float r5 = spray_hash_float(seed + 5u) * 2.0f - 1.0f;
        const float r6 = spray_hash_float(seed + 6u) * 2.0f - 1.0f;
        const float disc_r = h * 0.5f * std::sqrt(r0);
        const float theta = TWO_PI_S * r1;
        const float along = r2 * prm.dt * speed;
        const V3<float> sp = pos + e1 * (disc_r * cos_f32(theta)) +
                             e2 * (disc_r * sin_f32(theta)) + v_dir * along;
        const V3<float> jitter = V3<float>{r4, r5, r6} * prm.velocity_jitter;
        const V3<float> spawn_vel = vel * prm.speed_multiplier + jitter;
        const float lt_min = prm.lifetime * (1.0f - prm.lifetime_variation);
        const float lt_span = 2.0f * prm.lifetime * prm.lifetime_variation;
        const float lt = lt_min + phi_k * r3 * lt_span;
        SprayPartF q{{sp.x, sp.y, sp.z}, lt, {spawn_vel.x, spawn_vel.y, spawn_vel.z}, lt, 0u, 0.0f,
                     0.0f, 0.0f};
        ring[slot] = q;
      }
    }
  }

  // spray_simulate.wgsl:158-280 over every ring slot.
  void spray_simulate(const SprayParamsF &prm, SprayPartF *ring, uint32_t live[4]) const {
    const float h = float(p.h), h_sq = float(p.h2), dt = prm.dt;
    auto cap = [](float t) {
      const float tc = std::min(std::max(t, 0.0f), 1.0f);
      return tc * tc * (3.0f - tc) * 0.25f;
    };
    for (uint32_t idx = 0; idx < prm.max_particles; idx++) {
      SprayPartF q = ring[idx];
      if (q.lifetime <= 0.0f) continue;
      const V3<float> pos{q.pos[0], q.pos[1], q.pos[2]};
      V3<float> vel{q.vel[0], q.vel[1], q.vel[2]};
      uint32_t neighbor_count = 0u;
      float w_sum = 0.0f;
      V3<float> v_avg{0.0f, 0.0f, 0.0f};
      for_neighbors(V3<R>{R(pos.x), R(pos.y), R(pos.z)}, [&](uint32_t j) {
        const Part<R> &pj = S[j];
        const V3<float> r_vec = pos - V3<float>{float(pj.pos.x), float(pj.pos.y), float(pj.pos.z)};
        const float r_sq = dot3(r_vec, r_vec);
        if (r_sq < h_sq) {
          const float w = 1.0f - std::sqrt(r_sq) / h;
          neighbor_count = neighbor_count + 1u;
          w_sum = w_sum + w;
          v_avg = v_avg + V3<float>{float(pj.vel.x), float(pj.vel.y), float(pj.vel.z)} * w;
        }
      });
      if (w_sum > 1e-6f) v_avg = v_avg / w_sum;
      uint32_t kind = 1u;
      if (neighbor_count <= 6u) kind = 0u;
      else if (neighbor_count >= 20u) kind = 2u;
      const float hw = float(geom.hw), hh = float(geom.hh), hd = float(geom.hd);
      auto to_local = [&](V3<float> w) {
        const V3<float> c{w.x, w.y - float(geom.cy), w.z};
        const V3<float> i0{float(geom.i0.x), float(geom.i0.y), float(geom.i0.z)};
        const V3<float> i1{float(geom.i1.x), float(geom.i1.y), float(geom.i1.z)};
        const V3<float> i2{float(geom.i2.x), float(geom.i2.y), float(geom.i2.z)};
        return V3<float>{dot3(i0, c), dot3(i1, c), dot3(i2, c)};
      };
      if (kind == 1u) {
        const V3<float> lp = to_local(pos);
        const float he[3] = {hw, hh, hd}, la[3] = {lp.x, lp.y, lp.z};
        float missing = 0.0f;
        for (int a = 0; a < 3; a++) {
          const float dlo = he[a] + la[a], dhi = he[a] - la[a];
          if (dlo < h) missing += cap(1.0f - dlo / h);
          if (dhi < h) missing += cap(1.0f - dhi / h);
        }
        const float visible = std::max(1.0f - missing, 0.25f);
        if (uint32_t(std::nearbyint(float(neighbor_count) / visible)) >= 20u) kind = 2u;
      }
      if (kind == 1u && q.age < 0.15f) kind = 0u;
      const V3<float> gravity{0.0f, prm.gravity_y, 0.0f};
      float decay = 0.0f;
      if (kind == 0u) {
        vel = vel + dt * (gravity - prm.drag * vel);
      } else if (kind == 1u) {
        vel = v_avg;
        decay = 1.0f;
      } else {
        vel = vel + dt * (-prm.bubble_buoyancy * gravity);
        const float t = std::min(std::max(prm.bubble_drag, 0.0f), 1.0f);
        vel = vel * (1.0f - t) + v_avg * t;
      }
      const V3<float> np = pos + dt * vel;
      q.pos[0] = np.x; q.pos[1] = np.y; q.pos[2] = np.z;
      q.vel[0] = vel.x; q.vel[1] = vel.y; q.vel[2] = vel.z;
      q.kind = kind;
      q.age = q.age + dt;
      q.lifetime = q.lifetime - dt * decay;
      const V3<float> l = to_local(np);
      if (!(l.x >= -hw && l.x <= hw && l.y >= -hh && l.y <= hh && l.z >= -hd && l.z <= hd))
        q.lifetime = 0.0f;
      if (q.lifetime > 0.0f) {
        live[0] += 1u;
        live[1 + kind] += 1u;
      }
      ring[idx] = q;
    }
  }

  void density_splat(const McGridF &mc, const GeomF &cgf, double *out) const {
    splat_into<double>(mc, cgf, out);
  }

  void set_geom(const GeomF &q) {
    geom.hw = R(q.half_width); geom.hh = R(q.half_height); geom.hd = R(q.half_depth);
    geom.cy = R(q.center_y);
    geom.f0 = from4<R>(q.f0); geom.f1 = from4<R>(q.f1); geom.f2 = from4<R>(q.f2);
    geom.i0 = from4<R>(q.i0); geom.i1 = from4<R>(q.i1); geom.i2 = from4<R>(q.i2);
    geom.wall_k = R(q.wall_stiffness); geom.damping = R(q.damping);
  }
};

// Grid sizing, sph_3d_grid.rs:121-143 (f32 arithmetic as the reference).
GridF make_grid(float cell_size, uint32_t n) {
  const float bounds_extent = 2.0f;
  uint32_t gs = uint32_t(std::ceil((2.0f * bounds_extent) / cell_size)) + 2u;
  GridF g{};
  g.gx = g.gy = g.gz = gs;
  g.total_cells = gs * gs * gs;
  g.cell_size = cell_size;
  g.inv_cell_size = 1.0f / cell_size;
  g.ox = g.oy = g.oz = -bounds_extent - cell_size;
  g.num_particles = n;
  return g;
}

struct Handle {
  int precision;  // 32 or 64
  Oracle<float> *f = nullptr;
  Oracle<double> *d = nullptr;
};

template <class R>
Oracle<R> *create_impl(const ParticleF *parts, uint32_t n, const SphParamsF *params,
                       const GeomF *geom, uint32_t max_particles, const float *sdf,
                       uint32_t sdf_res) {
  auto *o = new Oracle<R>();
  o->num_particles = n;
  o->max_particles = std::max(max_particles, n);
  o->grid = make_grid(params->kernel_radius, n);
  o->P.resize(o->max_particles);
  o->S.resize(o->max_particles);
  for (uint32_t i = 0; i < n; i++) o->P[i] = Oracle<R>::from_f(parts[i]);
  o->counts.assign(o->grid.total_cells, 0u);
  o->starts.assign(o->grid.total_cells, 0u);
  o->cell_idx.assign(o->max_particles, 0u);
  o->s2o.assign(o->max_particles, 0u);
  o->A.resize(o->max_particles);
  o->B.resize(o->max_particles);
  // Effective count: min(params.num_particles, n) for every stage (the GPU
  // library applies the same rule; see set_params).
  o->set_params(*params);
  o->set_geom(*geom);
  // GpuMouseForce::default(), interaction.rs:113-128; GpuRigidBody::default(),
  // rigid_body.rs:226-242
  o->mouse = MouseF{{0, 0, 0}, 0.5f, 30.0f, 0u, 0u, 0.0f, {0, 0, -1}, 0.0f};
  o->rigid = RigidF{{0, 0, 0}, 0.15f, {0, 0, 0}, 0u, 200.0f, 0u, 0, 0,
                    {1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}};
  if (sdf && sdf_res > 0) {
    o->sdf.assign(sdf, sdf + size_t(sdf_res) * sdf_res * sdf_res);
    o->sdf_res = sdf_res;
  } else {
    o->sdf.assign(1, 1.0f);
    o->sdf_res = 1;
  }
  return o;
}

}  // namespace

// Forward-mode derivative of the rollout loss L = mean((splat(x_T) - target)^2)
// along one direction of (initial positions, initial velocities, viscosity,
// surface tension): the oracle run on Dual<V> numbers (V = float follows the
// FP32 restatement's trajectory bit for bit, V = double the FP64 twin's).
template <class V>
void tangent_loss_impl(const ParticleF *parts, uint32_t n, const SphParamsF *params,
                       const GeomF *geom, const float *gravity, uint32_t iterations,
                       uint32_t steps, const double *dpos, const double *dvel, double dvisc,
                       double dst, double dnear, double ddelta, const McGridF *mc,
                       const float *target, double *loss, double *dloss) {
  using R = Dual<V>;
  std::unique_ptr<Oracle<R>> o(create_impl<R>(parts, n, params, geom, 0, nullptr, 0));
  for (int a = 0; a < 3; a++) o->gravity[a] = R(gravity[a]);
  o->iterations = std::max(iterations, 1u);
  for (uint32_t i = 0; i < n; i++) {
    if (dpos) {
      o->P[i].pos.x.d = dpos[3 * size_t(i)];
      o->P[i].pos.y.d = dpos[3 * size_t(i) + 1];
      o->P[i].pos.z.d = dpos[3 * size_t(i) + 2];
    }
    if (dvel) {
      o->P[i].vel.x.d = dvel[3 * size_t(i)];
      o->P[i].vel.y.d = dvel[3 * size_t(i) + 1];
      o->P[i].vel.z.d = dvel[3 * size_t(i) + 2];
    }
  }
  o->p.visc.d = dvisc;
  o->p.st.d = dst;
  o->p.near_k.d = dnear;
  o->p.delta.d = ddelta;
  for (uint32_t k = 0; k < steps; k++) o->step(nullptr, nullptr);
  o->stage_hash();
  o->stage_scan();
  o->stage_reorder();
  const size_t nvox = size_t(mc->grid_size) * mc->grid_size * mc->grid_size;
  std::vector<R> f(nvox);
  o->template splat_into<R>(*mc, *geom, f.data());
  double L = 0.0, dL = 0.0;
  for (size_t v = 0; v < nvox; v++) {
    const double diff = double(f[v].v) - double(target[v]);
    L += diff * diff;
    dL += 2.0 * diff * f[v].d;
  }
  *loss = L / double(nvox);
  *dloss = dL / double(nvox);
}

// ---- C ABI for the test harness (ctypes) ------------------------------------
extern "C" {

void *or_create(const void *particles, uint32_t n, const void *params, const void *geom,
                uint32_t max_particles, const float *sdf, uint32_t sdf_res, int precision) {
  auto *h = new Handle();
  h->precision = precision;
  if (precision == 64)
    h->d = create_impl<double>((const ParticleF *)particles, n, (const SphParamsF *)params,
                               (const GeomF *)geom, max_particles, sdf, sdf_res);
  else
    h->f = create_impl<float>((const ParticleF *)particles, n, (const SphParamsF *)params,
                              (const GeomF *)geom, max_particles, sdf, sdf_res);
  return h;
}

void or_destroy(void *hv) {
  auto *h = (Handle *)hv;
  delete h->f;
  delete h->d;
  delete h;
}

#define DISPATCH(h, expr)          \
  do {                             \
    if ((h)->f) {                  \
      auto *o = (h)->f;            \
      expr;                        \
    } else {                       \
      auto *o = (h)->d;            \
      expr;                        \
    }                              \
  } while (0)

void or_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : omp_get_num_procs());
#else
  (void)n;
#endif
}

int or_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void or_step(void *hv, uint32_t nsteps, uint64_t *cand, uint64_t *hits) {
  auto *h = (Handle *)hv;
  for (uint32_t k = 0; k < nsteps; k++) DISPATCH(h, o->step(cand, hits));
}

// Stage-by-stage driving, for stage-level parity checks. stage ids: 0 hash,
// 1 scan, 2 reorder, 3 density, 4 xsph, 5 force, 6 predict, 7 one solve
// iteration (arg = iteration index), 8 finalize (arg = iterations), 9 integrate.
void or_stage(void *hv, int stage, uint32_t arg) {
  auto *h = (Handle *)hv;
  DISPATCH(h, {
    switch (stage) {
      case 0: o->stage_hash(); break;
      case 1: o->stage_scan(); break;
      case 2: o->stage_reorder(); break;
      case 3: o->stage_density(nullptr, nullptr); break;
      case 4: o->stage_xsph(); break;
      case 5: o->stage_force(); break;
      case 6: o->stage_predict(); break;
      case 7: if (arg % 2 == 0) o->stage_solve(o->A, o->B); else o->stage_solve(o->B, o->A); break;
      case 8: o->stage_finalize(arg % 2 == 0 ? o->A : o->B); break;
      case 9: o->stage_integrate(); break;
      default: break;
    }
  });
}

void or_set_params(void *hv, const void *q) {
  auto *h = (Handle *)hv;
  DISPATCH(h, o->set_params(*(const SphParamsF *)q));
}
void or_set_geometry(void *hv, const void *q) {
  auto *h = (Handle *)hv;
  DISPATCH(h, o->set_geom(*(const GeomF *)q));
}
void or_set_gravity(void *hv, const float *g) {
  auto *h = (Handle *)hv;
  DISPATCH(h, { o->gravity[0] = g[0]; o->gravity[1] = g[1]; o->gravity[2] = g[2]; });
}
void or_set_mouse(void *hv, const void *q) {
  auto *h = (Handle *)hv;
  DISPATCH(h, o->mouse = *(const MouseF *)q);
}
void or_set_rigid(void *hv, const void *q) {
  auto *h = (Handle *)hv;
  DISPATCH(h, o->rigid = *(const RigidF *)q);
}
void or_track_terms(void *hv, int on) {
  auto *h = (Handle *)hv;
  DISPATCH(h, {
    o->track_terms = on != 0;
    const size_t n = o->P.size();
    o->tmag_force.assign(n, 0.0);
    o->tmag_solve.assign(n, 0.0);
    o->tmag_normal.assign(n, 0.0);
  });
}
// Term-magnitude sums of the last step, canonical order: force pass, last
// PCISPH iteration's pressure acceleration, Akinci normal (3 doubles each).
void or_get_term_magnitudes(void *hv, double *out, uint32_t n) {
  auto *h = (Handle *)hv;
  DISPATCH(h, {
    for (uint32_t i = 0; i < n && i < o->tmag_force.size(); i++) {
      out[3 * size_t(i)] = o->tmag_force[i];
      out[3 * size_t(i) + 1] = o->tmag_solve[i];
      out[3 * size_t(i) + 2] = o->tmag_normal[i];
    }
  });
}
void or_set_cells_f32(void *hv, int on) {
  auto *h = (Handle *)hv;
  DISPATCH(h, o->cells_in_f32 = on != 0);
}
void or_set_iterations(void *hv, uint32_t it) {
  auto *h = (Handle *)hv;
  DISPATCH(h, o->iterations = std::max(it, 1u));
}
void or_clear_accum(void *hv) {
  auto *h = (Handle *)hv;
  DISPATCH(h, o->accum = AccumI{});
}
void or_get_accum(void *hv, void *out) {
  auto *h = (Handle *)hv;
  DISPATCH(h, std::memcpy(out, &o->accum, sizeof(AccumI)));
}
void or_get_particles(void *hv, void *out, uint32_t n) {
  auto *h = (Handle *)hv;
  DISPATCH(h, { for (uint32_t i = 0; i < n; i++) ((ParticleF *)out)[i] = o->to_f(o->P[i]); });
}
void or_get_sorted(void *hv, void *out, uint32_t n) {
  auto *h = (Handle *)hv;
  DISPATCH(h, { for (uint32_t i = 0; i < n; i++) ((ParticleF *)out)[i] = o->to_f(o->S[i]); });
}
// FP64 twin: read the canonical/sorted state without rounding to float.
// Layout per particle (14 doubles): pos[3], vel[3], force[3], density,
// near_density, normal[3].
void or_get_particles_f64(void *hv, double *out, uint32_t n, int sorted) {
  auto *h = (Handle *)hv;
  DISPATCH(h, {
    const auto &src = sorted ? o->S : o->P;
    for (uint32_t i = 0; i < n; i++) {
      const auto &r = src[i];
      double *d = out + size_t(i) * 14;
      d[0] = r.pos.x; d[1] = r.pos.y; d[2] = r.pos.z;
      d[3] = r.vel.x; d[4] = r.vel.y; d[5] = r.vel.z;
      d[6] = r.force.x; d[7] = r.force.y; d[8] = r.force.z;
      d[9] = r.density; d[10] = r.near_density;
      d[11] = r.normal.x; d[12] = r.normal.y; d[13] = r.normal.z;
    }
  });
}
void or_get_cells(void *hv, uint32_t *counts, uint32_t *starts) {
  auto *h = (Handle *)hv;
  DISPATCH(h, {
    if (counts) std::copy(o->counts.begin(), o->counts.end(), counts);
    if (starts) std::copy(o->starts.begin(), o->starts.end(), starts);
  });
}
void or_get_index_maps(void *hv, uint32_t *cell_idx, uint32_t *s2o, uint32_t n) {
  auto *h = (Handle *)hv;
  DISPATCH(h, {
    if (cell_idx) std::copy(o->cell_idx.begin(), o->cell_idx.begin() + n, cell_idx);
    if (s2o) std::copy(o->s2o.begin(), o->s2o.begin() + n, s2o);
  });
}
// Predicted-state buffer (which = 0 for A, 1 for B), 8 floats per slot.
void or_get_predicted(void *hv, int which, float *out, uint32_t n) {
  auto *h = (Handle *)hv;
  DISPATCH(h, {
    const auto &src = which ? o->B : o->A;
    for (uint32_t i = 0; i < n; i++) {
      float *d = out + size_t(i) * 8;
      d[0] = float(src[i].x.x); d[1] = float(src[i].x.y); d[2] = float(src[i].x.z);
      d[3] = float(src[i].pressure);
      d[4] = float(src[i].v.x); d[5] = float(src[i].v.y); d[6] = float(src[i].v.z);
      d[7] = float(src[i].density);
    }
  });
}
// The FP32 sin/cos of the close-pair direction, for accuracy tests.
void or_sincos_f32(const float *x, float *s, float *c, uint32_t n) {
  for (uint32_t i = 0; i < n; i++) {
    s[i] = sin_f32(x[i]);
    c[i] = cos_f32(x[i]);
  }
}

void or_get_grid(void *hv, void *out) {
  auto *h = (Handle *)hv;
  DISPATCH(h, std::memcpy(out, &o->grid, sizeof(GridF)));
}

// Tangent of the rollout loss (see tangent_loss_impl); precision 32 or 64.
void or_tangent_rollout_loss(const void *particles, uint32_t n, const void *params,
                             const void *geom, const float *gravity, uint32_t iterations,
                             uint32_t steps, const double *dpos, const double *dvel, double dvisc,
                             double dst, double dnear, double ddelta, const void *mc,
                             const float *target, int precision, double *loss, double *dloss) {
  if (precision == 64)
    tangent_loss_impl<double>((const ParticleF *)particles, n, (const SphParamsF *)params,
                              (const GeomF *)geom, gravity, iterations, steps, dpos, dvel, dvisc,
                              dst, dnear, ddelta, (const McGridF *)mc, target, loss, dloss);
  else
    tangent_loss_impl<float>((const ParticleF *)particles, n, (const SphParamsF *)params,
                             (const GeomF *)geom, gravity, iterations, steps, dpos, dvel, dvisc,
                             dst, dnear, ddelta, (const McGridF *)mc, target, loss, dloss);
}

// One whitewater frame (FP32 restatement): emit, ceiling update, simulate.
void or_spray_frame(void *hv, const void *params, void *ring, uint32_t *head, float *limits,
                    uint32_t *live_stats) {
  auto *h = (Handle *)hv;
  if (!h->f) return;  // FP32 only
  const SprayParamsF &prm = *(const SprayParamsF *)params;
  uint32_t stats[2] = {0u, 0u};
  h->f->spray_emit(prm, limits[0], limits[1], (SprayPartF *)ring, head, stats);
  auto update = [](float current, uint32_t bits, float floor_v) {
    float frame_max;
    std::memcpy(&frame_max, &bits, 4);
    if (frame_max <= 1e-6f) return current;
    const float alpha = frame_max > current ? 0.05f : 0.01f;
    return std::max(current + alpha * (frame_max - current), floor_v);
  };
  limits[0] = update(limits[0], stats[0], 0.2f);
  limits[1] = update(limits[1], stats[1], 0.05f);
  for (int k = 0; k < 4; k++) live_stats[k] = 0u;
  h->f->spray_simulate(prm, (SprayPartF *)ring, live_stats);
}

// The MC density field of the last step's sorted positions (gs^3 doubles).
void or_density_splat(void *hv, const void *mc, const void *geom, double *out) {
  auto *h = (Handle *)hv;
  DISPATCH(h, o->density_splat(*(const McGridF *)mc, *(const GeomF *)geom, out));
}

}  // extern "C"
