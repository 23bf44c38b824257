// spray_kernels.cu — whitewater emission and simulation on sm_103a
// (spray_emit.wgsl, spray_simulate.wgsl; src/simulation/spray.rs).
//
// Emission runs in three launches instead of the shader's one: every sorted
// fluid particle computes its two potentials and its spawn count
// (k_spray_count), an exclusive scan turns the counts into ring slots
// (the library's prefix scan), and k_spray_spawn writes the records. A
// frame's spawns therefore take consecutive slots in sorted particle order —
// the shader's atomic write head, executed in invocation order. Compiled with
// -fmad=false: every expression keeps the shaders' evaluation order, so the
// records are bit-identical to the FP32 restatement; sin/cos use the
// library's fixed FP32 evaluation (sph_device.cuh).
#include "spray_internal.h"
#include "sph_device.cuh"

namespace fs {
namespace {

constexpr float SPRAY_PI = 3.14159265359f;
constexpr float SPRAY_TWO_PI = 6.28318530718f;
constexpr float AUTO_LIMIT_MIN_FRAC = 0.1f;
constexpr uint32_t EMIT_MIN_NEIGHBORS = 10u;
constexpr float KINETIC_MAX_SPEED = 2.5f;
constexpr float CREST_DENSITY_FRAC = 0.9f;
constexpr float CREST_VEL_NORMAL_MIN = 0.6f;
constexpr float CREST_DIVERGENCE_MIN = 0.0f;
constexpr float CREST_DIVERGENCE_MAX = 0.5f;
constexpr uint32_t MAX_EMIT_PER_FRAME = 16u;

// spray_emit.wgsl:140-152
__device__ __forceinline__ uint32_t spray_hash(uint32_t x) {
  x = x ^ (x >> 16u);
  x = x * 0x45d9f3bu;
  x = x ^ (x >> 16u);
  x = x * 0x45d9f3bu;
  x = x ^ (x >> 16u);
  return x;
}
__device__ __forceinline__ float hash_float(uint32_t seed) {
  return float(spray_hash(seed) & 0xFFFFu) / 65535.0f;
}
__device__ __forceinline__ float remap_clamp(float x, float lo, float hi) {
  return clampf((x - lo) / (hi - lo), 0.0f, 1.0f);
}

// What k_spray_spawn needs to redo an emitter's spawn geometry.
struct Emitter {
  float3 pos, vel;
  float speed, phi_k;
  uint32_t n_emit;
};

// spray_emit.wgsl:180-316 up to the spawn count, for the scene-local sorted
// index i (global slot s).
__device__ __forceinline__ Emitter emitter(const SprayView &sv, uint32_t i, uint32_t s,
                                           const SprayFrame &f) {
  Emitter em;
  em.n_emit = 0u;
  const DevUniforms &U = *sv.u;
  const GpuSphParams3D &sp = U.sph;
  const GpuSprayParams &prm = f.params;
  const float4 pos4 = sv.s_pos[s];
  const float4 vel4 = sv.s_vel[s];
  em.pos = xyz(pos4);
  em.vel = xyz(vel4);
  em.speed = len3(em.vel);
  if (em.speed < prm.min_speed) return em;
  const float h = sp.kernel_radius, h_sq = sp.kernel_radius_sq;
  const float2 dens_i = sv.s_dens[s];
  const float3 normal_i = xyz(sv.s_nrm[s]);
  const float n_len_i = len3(normal_i);
  const bool crest_eligible = n_len_i > 1e-4f && dens_i.x < sp.rest_density * CREST_DENSITY_FRAC;
  float3 n_hat_i = f3(0.0f, 1.0f, 0.0f);
  if (crest_eligible) n_hat_i = normal_i / n_len_i;
  float trapped_air = 0.0f, crest = 0.0f, divergence = 0.0f;
  uint32_t n_neighbors = 0u;
  const float poly6_norm = 315.0f / (64.0f * SPRAY_PI * sp.kernel_radius_pow9);
  Runs R;
  neighbor_runs(em.pos, U.grid, sv.begin, R);
  for (int r = 0; r < R.count; r++) {
    for (uint32_t j = R.lo[r]; j < R.hi[r]; j++) {
      const float3 pj = xyz(__ldg(sv.s_pos + j));
      const float3 r_vec = em.pos - pj;
      const float r_sq = dot3(r_vec, r_vec);
      if (r_sq >= h_sq || r_sq < 1e-12f) continue;
      const float rr = sqrtf(r_sq);
      const float w = 1.0f - rr / h;
      const float3 x_hat = r_vec / rr;
      n_neighbors += 1u;
      const float d2 = h_sq - r_sq;
      const float w_vol = (sp.mass / fmaxf(__ldg(&sv.s_dens[j].x), 1e-6f)) * poly6_norm * d2 * d2 * d2;
      const float3 v_ij = em.vel - xyz(__ldg(sv.s_vel + j));
      const float v_ij_len = len3(v_ij);
      if (v_ij_len > 1e-6f)
        trapped_air += v_ij_len * (1.0f - dot3(v_ij / v_ij_len, x_hat)) * w_vol;
      divergence += dot3(v_ij, x_hat) * w;
      if (crest_eligible && dot3(-x_hat, n_hat_i) < 0.0f) {
        const float3 normal_j = xyz(__ldg(sv.s_nrm + j));
        const float n_len_j = len3(normal_j);
        if (n_len_j > 1e-4f) crest += (1.0f - dot3(n_hat_i, normal_j / n_len_j)) * w_vol;
      }
    }
  }
  if (n_neighbors < EMIT_MIN_NEIGHBORS) return em;
  if (dot3(em.vel / em.speed, n_hat_i) < CREST_VEL_NORMAL_MIN) crest = 0.0f;
  if (trapped_air > 0.0f) atomicMax(sv.emit_stats + 0, __float_as_uint(trapped_air));
  if (crest > 0.0f) atomicMax(sv.emit_stats + 1, __float_as_uint(crest));
  const float phi_div = remap_clamp(divergence, CREST_DIVERGENCE_MIN, CREST_DIVERGENCE_MAX);
  const float ta_hi = fmaxf(sv.limits[0], 1e-4f);  // this frame's ceilings
  const float wc_hi = fmaxf(sv.limits[1], 1e-4f);
  const float phi_ta = remap_clamp(trapped_air, AUTO_LIMIT_MIN_FRAC * ta_hi, ta_hi);
  const float phi_wc = remap_clamp(crest, AUTO_LIMIT_MIN_FRAC * wc_hi, wc_hi) * phi_div;
  em.phi_k = remap_clamp(em.speed, prm.min_speed, KINETIC_MAX_SPEED);
  const float rate = em.phi_k * (prm.k_trapped_air * phi_ta + prm.k_wave_crest * phi_wc) *
                     prm.emission_rate;
  const float expected = rate * prm.dt;
  const uint32_t base_seed = i + prm.frame_count * 7919u;
  const float fl = floorf(expected);
  uint32_t n_emit = uint32_t(fl);  // expected >= 0
  if (hash_float(base_seed * 13u + 5u) < expected - fl) n_emit = n_emit + 1u;
  em.n_emit = min(n_emit, MAX_EMIT_PER_FRAME);
  return em;
}

__global__ void __launch_bounds__(128)
    k_spray_count(SprayView sv, SprayFrame f, uint32_t n, uint32_t *__restrict__ counts) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  counts[i] = emitter(sv, i, sv.s_offset + i, f).n_emit;
}

// spray_emit.wgsl:318-372 for the emitters with spawns; their first slot is
// head + (inclusive end - count).
__global__ void __launch_bounds__(128)
    k_spray_spawn(SprayView sv, SprayFrame f, uint32_t n, const uint32_t *__restrict__ counts,
                  const uint32_t *__restrict__ ends, GpuSprayParticle *__restrict__ ring) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t cnt = counts[i];
  if (cnt == 0u) return;
  // recompute the emitter (its spawn count is deterministic; the maxima
  // atomics repeat the same values)
  const Emitter em = emitter(sv, i, sv.s_offset + i, f);
  const GpuSprayParams &prm = f.params;
  const float h = sv.u->sph.kernel_radius;
  const float3 v_dir = em.vel / em.speed;
  float3 ref_axis = f3(0.0f, 1.0f, 0.0f);
  if (fabsf(v_dir.y) > 0.99f) ref_axis = f3(1.0f, 0.0f, 0.0f);
  const float3 e1 = normalize3(cross3(v_dir, ref_axis));
  const float3 e2 = cross3(v_dir, e1);
  const uint32_t base_seed = i + prm.frame_count * 7919u;
  const uint32_t start = ends[i] - cnt;  // this frame's spawn index of the first record
  const uint32_t total = ends[n - 1];
  for (uint32_t e = 0u; e < cnt; e = e + 1u) {
    // a frame that spawns more than the ring holds keeps the last records,
    // as the sequential write head does
    if (uint64_t(start + e) + prm.max_particles < uint64_t(total)) continue;
    const uint32_t slot = (*sv.write_head + start + e) % prm.max_particles;
    const uint32_t seed = base_seed + e * 3571u;
    const float r0 = hash_float(seed);
    const float r1 = hash_float(seed + 1u);
    const float r2 = hash_float(seed + 2u);
    const float r3 = hash_float(seed + 3u);
    const float r4 = hash_float(seed + 4u) * 2.0f - 1.0f;
    const float r5 = hash_float(seed + 5u) * 2.0f - 1.0f;
    const float r6 = hash_float(seed + 6u) * 2.0f - 1.0f;
    const float disc_r = h * 0.5f * sqrtf(r0);
    const float theta = SPRAY_TWO_PI * r1;
    const float along = r2 * prm.dt * em.speed;
    const float3 pos = em.pos + e1 * (disc_r * cos_d(theta)) + e2 * (disc_r * sin_d(theta)) +
                       v_dir * along;
    const float3 jitter = f3(r4, r5, r6) * prm.velocity_jitter;
    const float3 spawn_vel = em.vel * prm.speed_multiplier + jitter;
    const float lt_min = prm.lifetime * (1.0f - prm.lifetime_variation);
    const float lt_span = 2.0f * prm.lifetime * prm.lifetime_variation;
    const float lt = lt_min + em.phi_k * r3 * lt_span;
    GpuSprayParticle q;
    q.pos[0] = pos.x; q.pos[1] = pos.y; q.pos[2] = pos.z;
    q.lifetime = lt;
    q.vel[0] = spawn_vel.x; q.vel[1] = spawn_vel.y; q.vel[2] = spawn_vel.z;
    q.max_lifetime = lt;
    q.kind = 0u;
    q.age = 0.0f;
    q._pad[0] = 0.0f;
    q._pad[1] = 0.0f;
    ring[slot] = q;
  }
}

// spray.rs:40-50, on the device: the ceilings follow this frame's maxima.
__device__ __forceinline__ float update_auto_limit(float current, float frame_max, float floor_v) {
  if (frame_max <= 1e-6f) return current;
  const float alpha = frame_max > current ? 0.05f : 0.01f;
  return fmaxf(current + alpha * (frame_max - current), floor_v);
}

__global__ void k_spray_advance(SprayView sv, uint32_t n, const uint32_t *__restrict__ ends) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (n) *sv.write_head += ends[n - 1];
  sv.limits[0] = update_auto_limit(sv.limits[0], __uint_as_float(sv.emit_stats[0]), 0.2f);
  sv.limits[1] = update_auto_limit(sv.limits[1], __uint_as_float(sv.emit_stats[1]), 0.05f);
}

// spray_simulate.wgsl:132-156
__device__ __forceinline__ float cap_volume_fraction(float t) {
  const float tc = clampf(t, 0.0f, 1.0f);
  return tc * tc * (3.0f - tc) * 0.25f;
}

// spray_simulate.wgsl:158-280, one ring slot
__global__ void __launch_bounds__(128)
    k_spray_simulate(SprayView sv, SprayFrame f, GpuSprayParticle *__restrict__ ring) {
  const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
  const GpuSprayParams &prm = f.params;
  if (idx >= prm.max_particles) return;
  GpuSprayParticle p = ring[idx];
  if (p.lifetime <= 0.0f) return;
  const DevUniforms &U = *sv.u;
  const float dt = prm.dt;
  const float3 pos = f3(p.pos[0], p.pos[1], p.pos[2]);
  float3 vel = f3(p.vel[0], p.vel[1], p.vel[2]);
  const float h = U.sph.kernel_radius, h_sq = U.sph.kernel_radius_sq;
  uint32_t neighbor_count = 0u;
  float w_sum = 0.0f;
  float3 v_avg = f3(0.0f, 0.0f, 0.0f);
  Runs R;
  neighbor_runs(pos, U.grid, sv.begin, R);
  for (int r = 0; r < R.count; r++) {
    for (uint32_t j = R.lo[r]; j < R.hi[r]; j++) {
      const float3 r_vec = pos - xyz(__ldg(sv.s_pos + j));
      const float r_sq = dot3(r_vec, r_vec);
      if (r_sq < h_sq) {
        const float w = 1.0f - sqrtf(r_sq) / h;
        neighbor_count = neighbor_count + 1u;
        w_sum = w_sum + w;
        v_avg = v_avg + xyz(__ldg(sv.s_vel + j)) * w;
      }
    }
  }
  if (w_sum > 1e-6f) v_avg = v_avg / w_sum;
  uint32_t kind = 1u;  // foam
  if (neighbor_count <= 6u) kind = 0u;
  else if (neighbor_count >= 20u) kind = 2u;
  const GpuContainerGeometry &c = U.geom;
  if (kind == 1u) {
    const float3 lp = world_to_local(c, pos);
    const float he[3] = {c.half_width, c.half_height, c.half_depth};
    const float lpa[3] = {lp.x, lp.y, lp.z};
    float missing = 0.0f;
    for (int a = 0; a < 3; a++) {
      const float dist_lo = he[a] + lpa[a];
      const float dist_hi = he[a] - lpa[a];
      if (dist_lo < h) missing += cap_volume_fraction(1.0f - dist_lo / h);
      if (dist_hi < h) missing += cap_volume_fraction(1.0f - dist_hi / h);
    }
    const float visible = fmaxf(1.0f - missing, 0.25f);
    if (uint32_t(rintf(float(neighbor_count) / visible)) >= 20u) kind = 2u;
  }
  if (kind == 1u && p.age < 0.15f) kind = 0u;
  const float3 gravity = f3(0.0f, prm.gravity_y, 0.0f);
  float lifetime_decay = 0.0f;
  if (kind == 0u) {
    vel = vel + dt * (gravity - prm.drag * vel);
  } else if (kind == 1u) {
    vel = v_avg;
    lifetime_decay = 1.0f;
  } else {
    vel = vel + dt * (-prm.bubble_buoyancy * gravity);
    const float t = clampf(prm.bubble_drag, 0.0f, 1.0f);
    vel = vel * (1.0f - t) + v_avg * t;
  }
  const float3 new_pos = pos + dt * vel;
  p.pos[0] = new_pos.x; p.pos[1] = new_pos.y; p.pos[2] = new_pos.z;
  p.vel[0] = vel.x; p.vel[1] = vel.y; p.vel[2] = vel.z;
  p.kind = kind;
  p.age = p.age + dt;
  p.lifetime = p.lifetime - dt * lifetime_decay;
  const float3 lp = world_to_local(c, new_pos);
  if (!(lp.x >= -c.half_width && lp.x <= c.half_width && lp.y >= -c.half_height &&
        lp.y <= c.half_height && lp.z >= -c.half_depth && lp.z <= c.half_depth))
    p.lifetime = 0.0f;
  if (p.lifetime > 0.0f) {
    atomicAdd(sv.live_stats + 0, 1u);
    atomicAdd(sv.live_stats + 1 + kind, 1u);
  }
  ring[idx] = p;
}

inline unsigned blocks_for(uint32_t n, unsigned threads) { return (n + threads - 1) / threads; }

}  // namespace

cudaError_t launch_spray_frame(const SprayView &sv, const SprayFrame &f, uint32_t n,
                               uint32_t *counts, uint32_t *ends, unsigned long long *scan_tiles,
                               uint32_t *err, GpuSprayParticle *ring, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(sv.emit_stats, 0, sizeof(uint32_t) * 8, st);  // + live stats
  if (e != cudaSuccess) return e;
  if (n) {
    k_spray_count<<<blocks_for(n, 128), 128, 0, st>>>(sv, f, n, counts);
    e = cudaMemsetAsync(scan_tiles, 0, sizeof(unsigned long long) * (scan_tiles_for(n) + 1), st);
    if (e != cudaSuccess) return e;
    e = launch_scan_with_scratch(counts, ends, n, scan_tiles, err, st);
    if (e != cudaSuccess) return e;
    k_spray_spawn<<<blocks_for(n, 128), 128, 0, st>>>(sv, f, n, counts, ends, ring);
  }
  k_spray_advance<<<1, 32, 0, st>>>(sv, n, ends);
  const uint32_t slots = f.params.max_particles;
  if (slots) k_spray_simulate<<<blocks_for(slots, 128), 128, 0, st>>>(sv, f, ring);
  return cudaGetLastError();
}

}  // namespace fs
