// sph_kernels.cu — per-particle SPH stages of the step on sm_103a.
//
// Reference stages (WGSL, src/shaders/):
//   density + near density + Akinci normal   sph_density_3d_grid.wgsl:56-194
//   XSPH velocity smoothing                  xsph.wgsl:60-138
//   near-pressure/viscosity/cohesion force   sph_force_3d_grid.wgsl:63-227
//   PCISPH predict (fused into force)        pcisph_predict.wgsl:50-73
//   PCISPH solve, one iteration              pcisph_solve.wgsl:71-208
//   PCISPH finalize + integrate (fused)      pcisph_finalize.wgsl:50-74,
//                                            sph_integrate_3d.wgsl:91-388
//
// Numerics. This translation unit is compiled with -fmad=false and IEEE
// division/sqrt, and every expression keeps the shaders' evaluation order, so
// results are bit-identical to the FP32 restatement of the shaders. sin/cos
// (the close-pair fallback direction) use one fixed FP32 evaluation shared
// with the restatement (see sin_d below).
//
// Neighbour walk. For a particle in unclamped cell (cx,cy,cz) the shaders
// visit the valid cells of the 3x3x3 block in dz, dy, dx order and each cell
// in slot order. Cells adjacent in x are adjacent in the sorted arrays, so the
// three dx cells of a (dy,dz) row form ONE contiguous slot range
// [begin[row+x0], begin[row+x1+1]): nine contiguous runs per particle, visited
// in exactly the shaders' order.
#include <type_traits>

#include "sph_device.cuh"

namespace fs {
namespace {

// Candidate records loaded ahead per lane (batched_loop; <= 1: plain loop).
// Each neighbour pass has one instantiation per load depth in
// kLoadDepths (density, solve) or kXsphDepths (XSPH, two records per
// candidate): deeper batches hide more load latency per lane but take more
// registers, so fewer warps fit an SM. Which depth is fastest depends on the
// workload (on the 1M-particle dam break, clumps of ~10,000, density at 16
// records takes 4.11 -> 3.22 ms and the four solve iterations 7.22 -> 4.92
// ms against the plain loop; on the 256-scene ensemble the plain loop was
// faster), so the simulation measures them (DevState::load_*, chosen per
// particle-count bucket by fs_step's tuner). Every depth gives the same bits.
// PCISPH iteration 0 runs on the pressure-free kernel at every depth (its
// pressures are all 0, the skipped sum is +0 exactly); its batched forms are
// bounded to four blocks per SM, without which the compiler serialised their
// loads (solve 4.78 -> 4.65 ms on the 1M-particle dam break against running
// iteration 0 on the pressure kernel with zero terms).
constexpr int kLoadDepths[kNumLoadDepths] = {0, 4, 8, 16, 32};
constexpr int kXsphDepths[kNumLoadDepths] = {1, 4, 8, 16, 32};
static_assert(kLoadDepths[3] == int(kDensityDepths[3]) && kXsphDepths[0] == int(kXsphDepthList[0]),
              "depth lists agree");
// The staged form (load depth kStagedLoads, XSPH): in a
// warp whose 32 lanes are all in one cell (the same neighbour runs: the dense
// clumps, where the time goes), candidate records go through shared memory in
// chunks of 32, each lane loading one record of the next chunk while the warp
// works on the current one: the latency hiding of 32 records in flight per
// lane at the registers of one. Every lane still visits its candidates in the
// shaders' order, so the bits are those of the other forms; other warps run
// the plain loop. (Streaming the union of the runs of lanes in x-adjacent
// cells, each lane taking only its own candidates, was measured slower: the
// lanes idle over the union's extra cell. A staged form of the PCISPH solve
// was measured slower than its batched loads on every workload and is not
// built: 6.1 against 4.8 ms per step on the 1M-particle dam break.)
constexpr int kStagedLoads = 32;

// Whether every lane of the warp is active with the same runs (one cell).
__device__ __forceinline__ bool warp_same_runs(bool active, const Runs &R) {
  if (!__all_sync(0xffffffffu, active)) return false;
  const int c0 = __shfl_sync(0xffffffffu, R.count, 0);
  const uint32_t rows0 = __shfl_sync(0xffffffffu, R.rows, 0);
  if (!__all_sync(0xffffffffu, R.count == c0 && R.rows == rows0)) return false;
  // every lane executes every shuffle (no short-circuit around them: a
  // full-mask shuffle that some lanes skip is undefined)
  bool same = true;
#pragma unroll
  for (int r = 0; r < 9; r++) {
    const bool in = r < c0;  // the same on every lane (counts are equal)
    const uint32_t lo = in ? R.lo[r] : 0u, hi = in ? R.hi[r] : 0u;
    const uint32_t lo0 = __shfl_sync(0xffffffffu, lo, 0);
    const uint32_t hi0 = __shfl_sync(0xffffffffu, hi, 0);
    same = same & (lo == lo0) & (hi == hi0);
  }
  return __all_sync(0xffffffffu, same);
}

// Position in the chunk sequence of a set of runs: for each run in order,
// chunks of up to 32 consecutive candidates from its start.
struct StagedChunks {
  int r;
  uint32_t base, cnt;
  bool valid;
  __device__ __forceinline__ explicit StagedChunks(const Runs &U) : r(0), base(0), cnt(0) {
    valid = false;
    for (; r < U.count; r++)
      if (U.hi[r] > U.lo[r]) {
        base = U.lo[r];
        cnt = min(32u, U.hi[r] - base);
        valid = true;
        break;
      }
  }
  __device__ __forceinline__ void advance(const Runs &U) {
    if (base + 32u < U.hi[r]) {
      base += 32u;
      cnt = min(32u, U.hi[r] - base);
      return;
    }
    valid = false;
    for (r++; r < U.count; r++)
      if (U.hi[r] > U.lo[r]) {
        base = U.lo[r];
        cnt = min(32u, U.hi[r] - base);
        valid = true;
        return;
      }
  }
};

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Visit the neighbours j with test(j) true in the shaders' order (rows in
// dz, dy order, slots ascending inside a row), calling body(j) right after
// its test. Used for cheap bodies and as the fallback of the mask walks.
template <class Test, class Body>
__device__ __forceinline__ void for_each_hit(const Runs &R, Test &&test, Body &&body) {
  for (int r = 0; r < R.count; r++) {
#pragma unroll 4
    for (uint32_t j = R.lo[r]; j < R.hi[r]; j++)
      if (test(j)) body(j);
  }
}

// ---- hit masks ----------------------------------------------------------------
// The heavy per-hit body (force) runs over a per-particle bitmask of
// in-range neighbours written by the density pass. Each run's candidates start
// a new word: bit k of the run's word w is candidate lo + 32w + k, so a run of
// length L owns ceil(L / 32) words and a particle R.words words in run order.
// Walking the mask gives every lane its own hits, one per loop iteration, in
// the shaders' order, so a warp runs as long as its busiest lane (not as long
// as the union of its lanes' candidate positions), and no candidate is tested
// twice.

// Word offset of each particle's mask, allocated per warp from a bump counter.
// Particles that do not fit the capacity get MASK_NONE and use the tested
// (unmasked) path.
__device__ __forceinline__ uint32_t alloc_mask(bool active, uint32_t nwords,
                                               unsigned long long *__restrict__ alloc,
                                               unsigned long long capacity) {
  const unsigned lane = threadIdx.x & 31u;
  uint32_t incl = active ? nwords : 0u;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (int(lane) >= o) incl += y;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  unsigned long long base = 0;
  if (lane == 31u && total) base = atomicAdd(alloc, (unsigned long long)total);
  base = __shfl_sync(0xffffffffu, base, 31);
  const unsigned long long off = base + incl - (active ? nwords : 0u);
  if (!active || off + nwords > capacity || off >= MASK_NONE) return MASK_NONE;
  return uint32_t(off);
}

template <class Body>
__device__ __forceinline__ void walk_mask(const Runs &R, const uint32_t *words, Body &&body) {
  MaskWalk m;
  m.init(R, words);
  uint32_t j;
  while (m.next(R, j)) body(j);
}

// Per-particle neighbour records, written by the density pass for the later
// gathers: pos = (position, max(density, 1)), vel = (pre-XSPH velocity,
// mass / max(density, 1)), nrm = (Akinci normal, max(near density, 1)). Each
// value is the exact expression the shaders evaluate per neighbour, computed
// once per particle instead of once per pair.
struct NbrRecords {
  float4 *pos, *vel, *nrm;
  uint32_t *hits;  // per slot: pairs with r^2 < h^2 (statistics of dedupe copies)
  unsigned long long *step_hits;  // the step's pairs with 1e-12 < r^2 < h^2
};

__global__ void __launch_bounds__(256) k_dir_table(float4 *__restrict__ tab, int dir_half) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t > 2 * dir_half) return;
  const float3 d = fallback_dir_eval(float(t - dir_half));
  tab[t] = make_float4(d.x, d.y, d.z, 0.0f);
}


// sph_density_3d_grid.wgsl:111-194 (writes the sorted copy only). Besides the
// density it records each particle's hit mask (1e-12 < r^2 < h^2, the XSPH and
// force criterion) and its neighbour records for the later passes. The body
// is evaluated for every candidate and the sums are updated with selects
// (x = hit ? x + t : x, the same bits as the shader's branch), so lanes never
// split inside the loop.
template <int B>
__device__ __forceinline__ void density_one(
    uint32_t s, SceneView v, const float4 *__restrict__ s_pos,
              const float4 *__restrict__ s_vel,
              const uint32_t *__restrict__ begin, float2 *__restrict__ s_dens,
              float4 *__restrict__ s_nrm, NbrRecords nb, unsigned long long *__restrict__ stats,
              uint32_t *__restrict__ mask_words, uint32_t *__restrict__ mask_off,
              uint32_t *__restrict__ mask_hits, unsigned long long *__restrict__ mask_alloc,
              unsigned long long mask_cap) {
  const bool active = s < v.b->n_sorted;
  const DevUniforms *U = v.u + (active ? v.scene_of_slot[s] : 0u);
  const GpuSphParams3D &P = U->sph;
  const float h = P.kernel_radius, h2 = P.kernel_radius_sq, mass = P.mass;
  const float scale_d = 315.0f / (64.0f * PI_F * P.kernel_radius_pow9);
  const float scale_n = 15.0f / (PI_F * P.kernel_radius_pow6);
  const float m_over_rho0 = mass / P.rest_density;
  uint32_t hits = 0u, nonself = 0u;
  float3 pos_i = f3(0.f, 0.f, 0.f);
  Runs R;
  R.count = 0;
  R.total = 0;
  R.words = 0;
  if (active) {
    pos_i = xyz(s_pos[s]);
    neighbor_runs(pos_i, U->grid, begin + U->c_offset, R);
  }
  const uint32_t off = alloc_mask(active, R.words, mask_alloc, mask_cap);
  if (active) {
    mask_off[s] = off;
    uint32_t *words = mask_words + (off == MASK_NONE ? 0u : off);
    float density = 0.0f, near_density = 0.0f;
    float3 normal = f3(0.f, 0.f, 0.f);
    uint32_t widx = 0u;
    for (int r = 0; r < R.count; r++) {
      for (uint32_t base = R.lo[r]; base < R.hi[r]; base += 32u) {
        const uint32_t cnt = min(32u, R.hi[r] - base);
        uint32_t word = 0u;
        batched_loop<B>(
            cnt, [&](uint32_t k) { return __ldg(s_pos + base + k); },
            [&](uint32_t k, const float4 pj) {
          const float rx = pos_i.x - pj.x, ry = pos_i.y - pj.y, rz = pos_i.z - pj.z;
          const float r_sq = rx * rx + ry * ry + rz * rz;
          const bool hit = r_sq < h2;
          const bool ns = hit && r_sq > 1e-12f;
          float rr;
          if constexpr (B > 1) {
            // correctly rounded fast square root (the batched form only: it
            // is what the clumped workloads that pick it gain from); r_sq = +0
            // (coincident particles) gives +0 as sqrtf does; anything else
            // outside the validated range takes sqrtf
            rr = r_sq == 0.0f ? 0.0f : sqrt_fast(r_sq);
            if (!(fast_ok(r_sq) || r_sq == 0.0f)) rr = sqrtf(r_sq);
          } else {
            rr = sqrtf(r_sq);
          }
          const float diff = h2 - r_sq;
          const float td = mass * (scale_d * diff * diff * diff);
          const float dn = h - rr;
          const float tn = mass * (scale_n * dn * dn * dn);
          density = hit ? density + td : density;
          near_density = hit ? near_density + tn : near_density;
          const float nx = normal.x + m_over_rho0 * rx * diff * diff;
          const float ny = normal.y + m_over_rho0 * ry * diff * diff;
          const float nz = normal.z + m_over_rho0 * rz * diff * diff;
          normal.x = ns ? nx : normal.x;
          normal.y = ns ? ny : normal.y;
          normal.z = ns ? nz : normal.z;
          hits += hit ? 1u : 0u;
          word |= ns ? (1u << k) : 0u;
        });
        if (off != MASK_NONE) words[widx] = word;
        widx++;
        nonself += uint32_t(__popc(word));
      }
    }
    mask_hits[s] = nonself;
    nb.hits[s] = hits;
    const float gamma = boundary_gamma(U->geom, h, pos_i);
    density = density / gamma;
    const float h8 = P.kernel_radius_pow6 * h * h;
    const float normal_scale = 945.0f / (32.0f * PI_F * h8);
    normal = normal * normal_scale;
    s_dens[s] = make_float2(density, near_density);
    s_nrm[s] = make_float4(normal.x, normal.y, normal.z, 0.0f);
    const float dmax = fmaxf(density, 1.0f);
    const float4 vs = s_vel[s];
    nb.pos[s] = make_float4(pos_i.x, pos_i.y, pos_i.z, dmax);
    nb.vel[s] = make_float4(vs.x, vs.y, vs.z, mass / dmax);
    nb.nrm[s] = make_float4(normal.x, normal.y, normal.z, fmaxf(near_density, 1.0f));
  }
  const unsigned long long cand = warp_sum_u64(R.total);
  const unsigned long long hsum = warp_sum_u64(hits);
  const unsigned long long nsum = warp_sum_u64(nonself);
  if ((threadIdx.x & 31) == 0 && cand) {
    atomicAdd(stats + STAT_CAND_DENSITY, cand);
    atomicAdd(stats + STAT_HIT_DENSITY, hsum);
    atomicAdd(stats + STAT_HIT_NONSELF, nsum);
    atomicAdd(nb.step_hits, nsum);
  }
}

// ---- XSPH -------------------------------------------------------------------
// xsph.wgsl:81-138; the result is the post-XSPH velocity in sorted order (the
// reference scatters it to the canonical array). mass / density_j comes from
// the neighbour record (the same quotient, evaluated once per particle). The
// per-neighbour body is short, so every candidate is tested in a branch-free
// loop (the term is added where 1e-12 < r^2 < h^2, in the shader's order):
// faster here than walking the hit mask, whose per-hit cost is the walk and
// two dependent gathers.
template <int B>
__device__ __forceinline__ void xsph_one(uint32_t s, SceneView v,
                                              const float4 *__restrict__ s_vel,
                                              const float4 *__restrict__ nb_pos,
                                              const float4 *__restrict__ nb_vel,
                                              const uint32_t *__restrict__ begin,
                                              float4 *__restrict__ vel_x) {
  // the pair term, shared by the forms (xsph.wgsl:106-135)
  auto term = [](float3 pos_i, float3 vel_i, float h2, float scale_d, float3 &corr, float4 pj,
                 float4 vj) {
    const float rx = pos_i.x - pj.x, ry = pos_i.y - pj.y, rz = pos_i.z - pj.z;
    const float r_sq = rx * rx + ry * ry + rz * rz;
    const bool hit = r_sq < h2 && r_sq > 1e-12f;
    const float diff = h2 - r_sq;
    const float w = scale_d * diff * diff * diff;
    const float3 c = corr + vj.w * (xyz(vj) - vel_i) * w;
    corr = hit ? c : corr;
  };
  if constexpr (B == kStagedLoads) {
    // staged (see kStagedLoads): warps whose lanes share one cell
    __shared__ float4 st_p[4][32], st_v[4][32];
    const bool act = s < v.b->n_sorted;
    const DevUniforms *U = v.u + (act ? v.scene_of_slot[s] : 0u);
    const GpuSphParams3D &P = U->sph;
    const bool work = act && P.xsph_epsilon > 0.0f;
    Runs R;
    R.count = 0;
    R.total = 0;
    R.words = 0;
    float3 pos_i = f3(0.f, 0.f, 0.f);
    if (work) {
      pos_i = xyz(nb_pos[s]);
      neighbor_runs(pos_i, U->grid, begin + U->c_offset, R);
    }
    if (warp_same_runs(work, R)) {
      const float4 vi4 = s_vel[s];
      const float3 vel_i = xyz(vi4);
      const float h2 = P.kernel_radius_sq;
      const float scale_d = 315.0f / (64.0f * PI_F * P.kernel_radius_pow9);
      const unsigned lane = threadIdx.x & 31u;
      float4 *sp = st_p[threadIdx.x >> 5], *sv = st_v[threadIdx.x >> 5];
      float3 corr = f3(0.f, 0.f, 0.f);
      StagedChunks ch(R);
      float4 pf_p = make_float4(0.f, 0.f, 0.f, 0.f), pf_v = pf_p;
      if (ch.valid && lane < ch.cnt) {
        pf_p = __ldg(nb_pos + ch.base + lane);
        pf_v = __ldg(nb_vel + ch.base + lane);
      }
      while (ch.valid) {
        const uint32_t cnt = ch.cnt;
        const float4 cur_p = pf_p, cur_v = pf_v;
        ch.advance(R);
        if (ch.valid && lane < ch.cnt) {
          pf_p = __ldg(nb_pos + ch.base + lane);
          pf_v = __ldg(nb_vel + ch.base + lane);
        }
        __syncwarp();  // the previous chunk's readers are done
        sp[lane] = cur_p;
        sv[lane] = cur_v;
        __syncwarp();
#pragma unroll 4
        for (uint32_t k = 0; k < cnt; k++) term(pos_i, vel_i, h2, scale_d, corr, sp[k], sv[k]);
      }
      const float3 vn = vel_i + P.xsph_epsilon * corr;
      vel_x[s] = make_float4(vn.x, vn.y, vn.z, vi4.w);
      return;
    }
  }
  if (s >= v.b->n_sorted) return;
  const DevUniforms *U = v.u + v.scene_of_slot[s];
  const GpuSphParams3D &P = U->sph;
  const float4 vi4 = s_vel[s];
  const float eps = P.xsph_epsilon;
  if (eps <= 0.0f) {  // xsph.wgsl:94-97: the velocity stays pre-XSPH
    vel_x[s] = vi4;
    return;
  }
  const float3 vel_i = xyz(vi4);
  const float h2 = P.kernel_radius_sq;
  const float scale_d = 315.0f / (64.0f * PI_F * P.kernel_radius_pow9);
  const float3 pos_i = xyz(nb_pos[s]);
  Runs R;
  neighbor_runs(pos_i, U->grid, begin + U->c_offset, R);
  float3 corr = f3(0.f, 0.f, 0.f);
  struct PV {
    float4 p, v;
  };
  for (int r = 0; r < R.count; r++) {
    const uint32_t lo = R.lo[r];
    batched_loop<(B == kStagedLoads ? 1 : B)>(
        R.hi[r] - lo, [&](uint32_t k) { return PV{__ldg(nb_pos + lo + k), __ldg(nb_vel + lo + k)}; },
        [&](uint32_t, const PV &q) { term(pos_i, vel_i, h2, scale_d, corr, q.p, q.v); });
  }
  const float3 vn = vel_i + eps * corr;
  vel_x[s] = make_float4(vn.x, vn.y, vn.z, vi4.w);
}

// ---- small coordinates --------------------------------------------------------
// A position coordinate c with 0 < |c| < 2^-34. When no particle has one,
// every nonzero coordinate difference of two particles is >= 2^-57 in
// magnitude (both coordinates are zero or multiples of 2^-57, or they have
// opposite signs), so the force pass, which divides those differences by r,
// skips their per-pair lower-bound checks. k_warp_work sets the step's flag.
__device__ __forceinline__ bool small_coord(float c) {
  const float a = fabsf(c);
  return a < 0x1p-34f && a != 0.0f;
}

// ---- force + PCISPH predict ---------------------------------------------------
// Three hits per walk iteration: their records are loaded together and their
// terms computed side by side, then added in order (6.15 -> 5.76 ms on the
// 1M-particle dam break against two, 123 registers; with the larger per-hit
// body before the range proofs three measured no faster than two; four
// spill).
constexpr bool kForceHitTriples = true;
// Threads per block of the force pass: four blocks of 128 per SM (its
// registers).
constexpr int kForceThreads = 128;
// Heavy particles of the force pass go cooperative (a warp each) when their
// hits exceed kCoopFactor times the step's pairs per resident lane, and at
// least kCoopMinHits: with few particles (the 32,768-particle rollout, the
// 49,600-particle dam break) the heaviest lanes' serial walks bound the pass.
// Measured factors (force ms, 49.6k / 32.8k particles): none 0.44 / 0.29;
// 2: 0.50 / 0.29; 4: 0.35 / 0.25; 8: 0.54 / 0.25; 16: 0.44 / 0.29. At 1M
// particles no lane reaches the threshold, and the two-kernel form cost 1%
// (its rest kernel compiles differently), so large simulations keep the
// single kernel over every slot.
constexpr unsigned long long kCoopFactor = 4;
constexpr uint32_t kCoopMinHits = 128;
// Simulations of at least this many sorted slots run the force pass without
// the cooperative path (one kernel over every slot).
constexpr uint32_t kCoopMaxParticles = 262144;
// sph_force_3d_grid.wgsl:105-227, then pcisph_predict.wgsl:61-72 for the same
// particle (sorted order).
template <bool COOP>
__device__ __forceinline__ void force_predict_one(
    uint32_t s, SceneView v, const float4 *__restrict__ s_pos,
                    const float4 *__restrict__ nb_pos, const float4 *__restrict__ nb_vel,
                    const float4 *__restrict__ nb_nrm, const float2 *__restrict__ s_dens,
                    const float4 *__restrict__ s_nrm, const float4 *__restrict__ vel_x,
                    const uint32_t *__restrict__ begin, const float4 *__restrict__ dir_tab,
                    int dir_half, const uint32_t *__restrict__ mask_words,
                    const uint32_t *__restrict__ mask_off,
                    const uint32_t *__restrict__ small_flag, float4 *__restrict__ anp,
                    float4 *__restrict__ pred_xp, float *__restrict__ pred_rho,
                    float *__restrict__ pterm0) {
  if (s >= v.b->n_sorted) return;
  const DevUniforms *U = v.u + v.scene_of_slot[s];
  const GpuSphParams3D &P = U->sph;
  const float h = P.kernel_radius, h2 = P.kernel_radius_sq, mass = P.mass;
  const float scale_g = 45.0f / (PI_F * P.kernel_radius_pow6);
  const float scale_c = 32.0f / (PI_F * P.kernel_radius_pow9);
  const float near_k = P.near_stiffness, visc = P.viscosity, rho0 = P.rest_density;
  const float min_dist = h * 0.1f;
  const float y_min_dist = __frcp_rn(min_dist);
  const float two_rho0 = 2.0f * rho0;
  // Operand ranges that hold for every pair the walk visits. The walked pairs
  // are the density pass's hits, 1e-12 < r^2 < h^2 (the same r^2 bit for bit:
  // the same positions and expression), so with h^2 < 2^59 the values r^2, r
  // and the viscosity denominator r^2 + 0.01 h^2 lie in [2^-60, 2^60).
  // Densities and near densities are clamped to >= 1, so the near-pressure
  // denominator and the density sum are >= 2 and need only an upper bound.
  // What is checked per pair: the numerators and those two upper bounds.
  const bool fast_particle = h2 < 0x1p59f && rcp_den_ok(min_dist) && fast_num_ok(two_rho0);
  const float3 pos_i = xyz(s_pos[s]);
  const float3 vel_i = xyz(vel_x[s]);
  const float2 di = s_dens[s];
  const float density_i = fmaxf(di.x, 1.0f);
  const float near_density_i = fmaxf(di.y, 1.0f);
  const float3 n_i = xyz(s_nrm[s]);
  const float near_pressure_i = near_k * near_density_i;
  float3 a_p = f3(0.f, 0.f, 0.f), a_v = f3(0.f, 0.f, 0.f), a_c = f3(0.f, 0.f, 0.f);
  Runs R;
  neighbor_runs(pos_i, U->grid, begin + U->c_offset, R);
  // Every arm of the shader's branches is evaluated and the accumulators are
  // updated with selects (x = c ? x + t : x), which leaves their bits exactly
  // as the branches would: lanes of a warp then never split inside the body.
  // Each hit's terms are computed first (they depend on the hit only) and
  // then added in the shader's order, so the terms of consecutive hits can
  // overlap while the sums keep their order.
  struct Rec {
    float4 p, v, n;
  };
  struct Terms {
    float3 p;    // near-pressure term
    float3 sep;  // close-pair separation term
    float3 v;    // viscosity term
    float3 c1;   // cohesion term
    float3 c2;   // normal-difference term
    bool close, ok;
  };
  auto load = [&](uint32_t j) {
    return Rec{__ldg(nb_pos + j), __ldg(nb_vel + j), __ldg(nb_nrm + j)};
  };
  // The pair's terms, with the correctly rounded fast reciprocal, square
  // root and quotients (FAST; t.ok reports whether every operand was in
  // their validated range) or with the IEEE operations.
  auto terms_impl = [&](uint32_t j, const Rec &q, auto fast, auto dv_check) {
    constexpr bool FAST = decltype(fast)::value;
    constexpr bool DV_CHECK = decltype(dv_check)::value;
    Terms t;
    bool ok = fast_particle;
    const float3 pos_j = xyz(q.p);
    const float3 vel_j = xyz(q.v);
    const float3 n_j = xyz(q.n);
    const float3 r_vec = pos_i - pos_j;
    const float r_sq = dot3(r_vec, r_vec);
    float rr, y_rr;
    if constexpr (FAST) {
      rr = sqrt_fast(r_sq);
      y_rr = rcp_fast(rr);
    } else {
      rr = sqrtf(r_sq);
      y_rr = __frcp_rn(rr);
    }
    t.close = rr < min_dist;
    // normalize(pos_j - pos_i): its length is sqrt(dot(-r, -r)) == rr bit for
    // bit, so dividing by rr is the same operation sequence
    // (pos_j - pos_i) / rr with one shared reciprocal, bit-identical; and
    // pos_j - pos_i is -r_vec exactly (IEEE subtraction is sign-symmetric).
    const float dvx = -r_vec.x, dvy = -r_vec.y, dvz = -r_vec.z;
    float3 dir;
    if constexpr (FAST) {
      // (markstein_nz: every quotient of the pair only scales terms of the
      // three sums a_p, a_v, a_c, which start at +0)
      dir = f3(markstein_nz(dvx, rr, y_rr), markstein_nz(dvy, rr, y_rr),
               markstein_nz(dvz, rr, y_rr));
      // the components' magnitudes are below r < 2^30; without DV_CHECK no
      // position has a coordinate 0 < |c| < 2^-34, so they are also 0 or
      // >= 2^-57
      if constexpr (DV_CHECK)
        ok = ok && fast_num_lo_ok(dvx) && fast_num_lo_ok(dvy) && fast_num_lo_ok(dvz);
    } else {
      dir = f3(dvx / rr, dvy / rr, dvz / rr);
    }
    // r < 0.1 h (rare: a few pairs per particle even in the clumps): the
    // slot-difference direction and the separation term
    // (sph_force_3d_grid.wgsl:160-176)
    t.sep = f3(0.f, 0.f, 0.f);
    if (t.close) {
      const int d = int(s) - int(j);
      if (d >= -dir_half && d <= dir_half)
        dir = xyz(__ldg(dir_tab + (d + dir_half)));
      else
        dir = fallback_dir_eval(float(s - U->s_offset) - float(j - U->s_offset));
      const float q_sep = FAST ? markstein_nz(rr, min_dist, y_min_dist) : rr / min_dist;
      const float sep = 200.0f * (1.0f - q_sep);
      t.sep = (-sep) * dir;
    }
    const float density_j = q.p.w;       // max(density_j, 1)
    const float near_density_j = q.n.w;  // max(near density_j, 1)
    const float near_pressure_j = near_k * near_density_j;
    const float dg = h - rr;
    const float grad = scale_g * dg * dg;
    const float np_num = -mass * (near_pressure_i + near_pressure_j);
    const float np_den = 2.0f * density_i * near_density_j;
    const float3 v_ij = vel_i - vel_j;
    const float v_dot_x = dot3(v_ij, r_vec);
    const float mu_num = h * v_dot_x;
    const float mu_den = r_sq + 0.01f * h2;
    const float dsum = density_i + density_j;
    const float avg_density = dsum * 0.5f;
    float np_q, mu, pi_visc, K_ij;
    if constexpr (FAST) {
      // 1 / avg_density is 2 / dsum: with y = RN(1 / dsum), 2 y = RN(1 / avg_density)
      // exactly (dsum in [2, 2^60): the halving and doubling are exact)
      const float y_sum = rcp_fast(dsum);
      np_q = markstein_nz(np_num, np_den, rcp_fast(np_den));
      mu = markstein_nz(mu_num, mu_den, rcp_fast(mu_den));
      const float pi_num = -visc * mu;
      pi_visc = markstein_nz(pi_num, avg_density, 2.0f * y_sum);
      K_ij = markstein_nz(two_rho0, dsum, y_sum);
      ok = ok && fast_num_ok(np_num) && np_den < 0x1p60f && fast_num_ok(mu_num) &&
           fast_num_ok(pi_num) && dsum < 0x1p60f;
    } else {
      np_q = np_num / np_den;
      mu = mu_num / mu_den;
      pi_visc = (-visc * mu) / avg_density;
      K_ij = two_rho0 / dsum;
    }
    t.p = np_q * dir * grad;
    // the viscosity term where v_ij . r_ij < 0, else (+0) * dir: adding a
    // zero leaves the sum's bits (the sums start at +0 and an RN sum is -0
    // only when both operands are), so the shader's branch is one select
    const float visc_c = v_dot_x < 0.0f ? -mass * pi_visc * grad : 0.0f;
    t.v = visc_c * dir;
    // akinci_cohesion_kernel: r >= h/2: s_c dg^3 r^3; else s_c (2 dg^3 r^3 -
    // h^6/64), each product chain in the shader's order from its first factor
    const float r3 = rr * rr * rr;
    const bool coh_far = rr >= h * 0.5f;
    const float coh_chain = (coh_far ? scale_c : 2.0f) * dg * dg * dg * r3;
    const float coh = coh_far ? coh_chain : scale_c * (coh_chain - P.kernel_radius_pow6 / 64.0f);
    t.c1 = (mass * K_ij * coh) * dir;
    t.c2 = (mass * K_ij) * (n_i - n_j);
    t.ok = ok;
    return t;
  };
  // the fast form, recomputed with IEEE operations when an operand is out of
  // range (never on ordinary inputs: one rarely taken branch per pair)
  auto terms = [&](uint32_t j, const Rec &q, auto dv_check) {
    Terms t = terms_impl(j, q, std::true_type{}, dv_check);
    if (!t.ok) t = terms_impl(j, q, std::false_type{}, dv_check);
    return t;
  };
  auto add = [&](const Terms &t) {
    a_p = a_p + t.p;
    if (t.close) a_p = a_p + t.sep;
    a_v = a_v + t.v;
    a_c = a_c + t.c1;
    a_c = a_c - t.c2;
  };
  const uint32_t off = mask_off[s];
  // the mask walk, with or without the direction numerators' checks (the
  // step-wide small-coordinate flag decides, the same for every particle)
  auto walk = [&](auto dv_check) {
    auto body = [&](uint32_t j) { add(terms(j, load(j), dv_check)); };
    MaskWalk m;
    m.init(R, mask_words + off);
    if (kForceHitTriples) {
      uint32_t j0, j1, j2;
      while (m.next(R, j0)) {
        if (!m.next(R, j1)) {
          body(j0);
          break;
        }
        if (!m.next(R, j2)) {
          const Terms t0 = terms(j0, load(j0), dv_check);
          const Terms t1 = terms(j1, load(j1), dv_check);
          add(t0);
          add(t1);
          break;
        }
        const Rec q0 = load(j0), q1 = load(j1), q2 = load(j2);
        const Terms t0 = terms(j0, q0, dv_check);
        const Terms t1 = terms(j1, q1, dv_check);
        const Terms t2 = terms(j2, q2, dv_check);
        add(t0);
        add(t1);
        add(t2);
      }
    } else {
      walk_mask(R, mask_words + off, body);
    }
  };
  // Cooperative (a heavy particle, the whole warp on it; every lane has the
  // same s and a mask): per mask word, lane L computes the terms of candidate
  // base + L if it is a hit and stores them at the hit's rank in the word;
  // then lanes 0-8 each carry one accumulator component (a_p, a_v, a_c: x, y,
  // z) through the word's hits in order, with the additions of the lane walk
  // (a_p + p, then + sep for close pairs; a_v + v; a_c + c1, then + (-c2),
  // which is a_c - c2 exactly). Same terms, same order: the same bits.
  __shared__ float co_terms[kForceThreads / 32][32][20];  // referenced by COOP only
  auto walk_coop = [&](auto dv_check) {
    const unsigned lane = threadIdx.x & 31u;
    float(*ct)[20] = co_terms[threadIdx.x >> 5];
    const uint32_t *words = mask_words + off;
    const int kind = int(lane) / 3, comp = int(lane) % 3;  // lanes 0-8
    float acc = 0.0f;
    StagedChunks ch(R);
    uint32_t widx = 0u;
    while (ch.valid) {
      const uint32_t base = ch.base;
      const uint32_t bits = words[widx++];
      ch.advance(R);
      if ((bits >> lane) & 1u) {
        const uint32_t r = uint32_t(__popc(bits & ((1u << lane) - 1u)));
        const uint32_t j = base + lane;
        const Terms t = terms(j, load(j), dv_check);
        float *e = ct[r];
        e[0] = t.p.x; e[1] = t.p.y; e[2] = t.p.z;
        e[3] = t.v.x; e[4] = t.v.y; e[5] = t.v.z;
        e[6] = t.c1.x; e[7] = t.c1.y; e[8] = t.c1.z;
        e[9] = t.sep.x; e[10] = t.sep.y; e[11] = t.sep.z;
        e[12] = 0.0f; e[13] = 0.0f; e[14] = 0.0f;
        e[15] = -t.c2.x; e[16] = -t.c2.y; e[17] = -t.c2.z;
        e[18] = t.close ? 1.0f : 0.0f;
      }
      __syncwarp();
      if (lane < 9u) {
        const uint32_t m = uint32_t(__popc(bits));
        for (uint32_t r = 0; r < m; r++) {
          const float *e = ct[r];
          acc = acc + e[lane];
          const bool second = kind == 2 || (kind == 0 && e[18] != 0.0f);
          if (second) acc = acc + e[9 + lane];
        }
      }
      __syncwarp();
    }
    (void)comp;
    a_p = f3(__shfl_sync(0xffffffffu, acc, 0), __shfl_sync(0xffffffffu, acc, 1),
             __shfl_sync(0xffffffffu, acc, 2));
    a_v = f3(__shfl_sync(0xffffffffu, acc, 3), __shfl_sync(0xffffffffu, acc, 4),
             __shfl_sync(0xffffffffu, acc, 5));
    a_c = f3(__shfl_sync(0xffffffffu, acc, 6), __shfl_sync(0xffffffffu, acc, 7),
             __shfl_sync(0xffffffffu, acc, 8));
  };
  if constexpr (COOP) {
    if (__ldg(small_flag) == 0u)
      walk_coop(std::false_type{});
    else
      walk_coop(std::true_type{});
    if ((threadIdx.x & 31u) != 0u) return;  // lane 0 writes the particle
  } else if (off != MASK_NONE) {
    if (__ldg(small_flag) == 0u)
      walk(std::false_type{});
    else
      walk(std::true_type{});
  } else {
    for_each_hit(
        R,
        [&](uint32_t j) {
          const float4 pj = __ldg(nb_pos + j);
          const float rx = pos_i.x - pj.x, ry = pos_i.y - pj.y, rz = pos_i.z - pj.z;
          const float r_sq = rx * rx + ry * ry + rz * rz;
          return r_sq < h2 && r_sq > 1e-12f;
        },
        [&](uint32_t j) { add(terms(j, load(j), std::true_type{})); });
  }
  a_c = a_c * P.surface_tension;
  const float3 a_g = xyz(U->gravity.direction);
  const float3 a = a_p + a_v + a_c + a_g;
  anp[s] = make_float4(a.x, a.y, a.z, 0.0f);
  const float dt = P.dt;
  const float3 v_star = vel_i + dt * a;
  const float3 x_star = pos_i + dt * v_star;
  pred_xp[s] = make_float4(x_star.x, x_star.y, x_star.z, 0.0f);
  pred_rho[s] = 0.0f;
  pterm0[s] = 0.0f;  // iteration 0's pressure terms (see launch_solve)
}

// ---- PCISPH solve -------------------------------------------------------------
// One iteration in -> out (pcisph_solve.wgsl:99-208). The predicted density is
// summed inline while the candidates are tested; with pressure, the hits with
// r^2 > 1e-12 are recorded in the particle's mask (the density pass's word
// range, same candidate list) and the pressure term is then summed by walking
// it. Iteration 0 reads the predict output, where every pressure is 0: the
// pressure sum is +0 exactly, so it is skipped (HAS_PRESSURE=false) with
// bit-identical results. The last iteration only produces the corrected
// velocity. Each other iteration also writes every particle's pressure term
// p / max(rho, 1)^2 (the shader's per-neighbour quotient, which depends on
// the neighbour only), so the next iteration reads it instead of dividing per
// pair. When recording (hit_out), the iteration also records each particle's
// in-range candidates (r^2 < h^2 at the predicted positions) in a hit mask in
// the density mask's layout and offsets (same runs), for the reverse pass:
// iteration 0 writes it, later iterations OR theirs in (one union mask).
template <bool HAS_PRESSURE, bool LAST, bool RECORD, int B>
__device__ __forceinline__ void solve_one(
    uint32_t s, SceneView v, const float4 *__restrict__ s_pos,
            const float4 *__restrict__ vel_x, const float4 *__restrict__ anp,
            const uint32_t *__restrict__ begin, const float4 *__restrict__ xp_in,
            const float *__restrict__ pterm_in, float4 *__restrict__ xp_out,
            float *__restrict__ rho_out, float *__restrict__ pterm_out,
            float4 *__restrict__ v_out, unsigned long long *__restrict__ stats,
            float4 *__restrict__ ap_out, const uint32_t *__restrict__ mask_off,
            uint32_t *__restrict__ hit_out, bool hit_or) {
  const bool active = s < v.b->n_sorted;
  const DevUniforms *U = v.u + (active ? v.scene_of_slot[s] : 0u);
  const GpuSphParams3D &P = U->sph;
  const float h = P.kernel_radius, h2 = P.kernel_radius_sq, mass = P.mass;
  const float scale_d = 315.0f / (64.0f * PI_F * P.kernel_radius_pow9);
  const float scale_g = 45.0f / (PI_F * P.kernel_radius_pow6);
  uint32_t hits = 0u;
  Runs R;
  R.count = 0;
  R.total = 0;
  R.words = 0;
  float3 pos_i = f3(0.f, 0.f, 0.f);
  if (active) {
    pos_i = xyz(s_pos[s]);  // current position decides the cells
    neighbor_runs(pos_i, U->grid, begin + U->c_offset, R);
    const float4 self_xp = xp_in[s];
    const float3 pred_pos = xyz(self_xp);
    const float old_p = self_xp.w;
    float pred_density = 0.0f;
    float3 a_p = f3(0.f, 0.f, 0.f);
    // old_p / (sd * sd) with sd = max(rho_in[s], 1), written by the previous
    // iteration (read only when there is pressure)
    const float self_term = HAS_PRESSURE ? pterm_in[s] : 0.0f;
    const bool fast_h2 = h2 < 0x1p59f;
    auto pressure = [&](uint32_t j, float3 r_vec, float r_sq) {
      const float pt = __ldg(pterm_in + j);  // np / (nd * nd)
      const float3 nr = -r_vec;
      // correctly rounded fast square root, reciprocal and quotients, one
      // range check for the pair (IEEE operations outside it). The pair is a
      // hit, 1e-12 < r^2 < h^2, so with h^2 < 2^59 r^2 and r are in the
      // validated range and |nr| < r: only the numerators' lower bound is
      // checked per pair.
      float rr = sqrt_fast(r_sq);
      const float y_rr = rcp_fast(rr);
      // (markstein_nz: the direction only scales terms of a_p, which starts
      // at +0)
      float3 dir = f3(markstein_nz(nr.x, rr, y_rr), markstein_nz(nr.y, rr, y_rr),
                      markstein_nz(nr.z, rr, y_rr));
      if (!(fast_h2 && fast_num_lo_ok(nr.x) && fast_num_lo_ok(nr.y) && fast_num_lo_ok(nr.z))) {
        rr = sqrtf(r_sq);
        dir = f3(nr.x / rr, nr.y / rr, nr.z / rr);
      }
      const float dg = h - rr;
      const float grad = scale_g * dg * dg;
      a_p = a_p + (-mass * (self_term + pt) * grad) * dir;
    };
    uint32_t *hit_words = nullptr;
    if (RECORD) {
      const uint32_t off = mask_off[s];
      hit_words = off == MASK_NONE ? nullptr : hit_out + off;
    }
    // candidates in chunks of up to 32: the predicted density is summed while
    // testing; the pressure hits of the chunk go to a per-lane bitmask that
    // each lane then walks (its own hits only, ascending)
    uint32_t widx = 0u;
    for (int r = 0; r < R.count; r++) {
      for (uint32_t base = R.lo[r]; base < R.hi[r]; base += 32u) {
        const uint32_t cnt = min(32u, R.hi[r] - base);
        uint32_t chunk = 0u, hitw = 0u;
        batched_loop<B>(
            cnt, [&](uint32_t k) { return __ldg(xp_in + base + k); },
            [&](uint32_t k, const float4 nb) {
              const float3 r_vec = pred_pos - xyz(nb);
              const float r_sq = dot3(r_vec, r_vec);
              if (r_sq < h2) {
                hits++;
                const float diff = h2 - r_sq;
                pred_density += mass * (scale_d * diff * diff * diff);
                if (HAS_PRESSURE && r_sq > 1e-12f) chunk |= 1u << k;
                if (RECORD) hitw |= 1u << k;
              }
            });
        if (RECORD) {
          if (hit_words) hit_words[widx] = hit_or ? (hit_words[widx] | hitw) : hitw;
          widx++;
        }
        if (HAS_PRESSURE) {
          while (chunk) {
            const uint32_t j = base + uint32_t(__ffs(chunk) - 1);
            chunk &= chunk - 1u;
            const float4 nb = __ldg(xp_in + j);
            const float3 r_vec = pred_pos - xyz(nb);
            pressure(j, r_vec, dot3(r_vec, r_vec));
          }
        }
      }
    }
    const float density_error = fmaxf(0.0f, pred_density - P.rest_density);
    const float new_p = old_p + P.pcisph_delta * density_error;
    const float dt = P.dt;
    const float max_accel = 0.25f * h / (dt * dt);
    const float mag_sq = dot3(a_p, a_p);
    const float max_sq = max_accel * max_accel;
    if (ap_out) ap_out[s] = make_float4(a_p.x, a_p.y, a_p.z, 0.0f);  // recording for the reverse pass
    if (mag_sq > max_sq) a_p = a_p * (max_accel / sqrtf(mag_sq));
    const float3 a_total = xyz(anp[s]) + a_p;
    const float3 v_star = xyz(vel_x[s]) + dt * a_total;
    if (LAST) {
      v_out[s] = make_float4(v_star.x, v_star.y, v_star.z, 0.0f);
    } else {
      const float3 x_star = pos_i + dt * v_star;
      xp_out[s] = make_float4(x_star.x, x_star.y, x_star.z, new_p);
      rho_out[s] = pred_density;
      const float nd = fmaxf(pred_density, 1.0f);
      pterm_out[s] = new_p / (nd * nd);
    }
  }
  const unsigned long long cand = warp_sum_u64(R.total);
  const unsigned long long hsum = warp_sum_u64(hits);
  if ((threadIdx.x & 31) == 0 && cand) {
    atomicAdd(stats + STAT_CAND_SOLVE, cand);
    atomicAdd(stats + STAT_HIT_SOLVE, hsum);
  }
}

// ---- work ordering -------------------------------------------------------------
// The neighbour passes' cost per particle ranges over two orders of
// magnitude (the clumps carry most of the pairs). Persistent warps take
// 32-slot tasks from a queue ordered heaviest first (longest-processing-time
// scheduling). Density, XSPH and solve, which test every candidate, take
// warps of 32 consecutive sorted slots (neighbouring particles share their
// neighbours' loads in L1); the force pass, which walks the hit mask (its
// lanes run as many iterations as they have hits), takes 32 slots of similar
// hit count from a permutation built by a counting sort on a log-linear work
// key, so its lanes finish together. Which lane computes a particle does not
// change its result.
__device__ __forceinline__ uint32_t work_key(uint32_t c) {
  return c < 4096u ? c : 4096u + min((c - 4096u) >> 4, 4095u);
}

// The hit-count keys are histogrammed and scattered per block of KEY_CHUNK
// slots in shared memory (a bucket receives one global atomic per block):
// most particles share a few hundred hit counts, and per-warp global atomics
// on those buckets serialised (4.35M slots of the 256-scene ensemble: 0.26 ms
// per kernel).
constexpr unsigned KEY_THREADS = 1024, KEY_ITEMS = 8, KEY_CHUNK = KEY_THREADS * KEY_ITEMS;

// Adds 1 to h[k] for every active lane, warp-aggregated; returns the lane's
// rank among all additions to h[k] (the old value plus its rank among the
// warp's lanes with the same key).
__device__ __forceinline__ uint32_t shared_rank(bool active, uint32_t k, uint32_t *h) {
  const unsigned act = __ballot_sync(0xffffffffu, active);
  if (!active) return 0u;
  const unsigned peers = __match_any_sync(act, k);
  const int leader = __ffs(peers) - 1;
  const unsigned lane = threadIdx.x & 31u;
  uint32_t old = 0u;
  if (int(lane) == leader) old = atomicAdd(&h[k], uint32_t(__popc(peers)));
  old = __shfl_sync(peers, old, leader);
  return old + uint32_t(__popc(peers & ((1u << lane) - 1u)));
}

// Adds a block's bucket counts (shared) to the global histogram, one atomic
// per non-empty bucket; all threads of the block call it.
template <int NB>
__device__ __forceinline__ void flush_buckets(const uint32_t (&h)[NB], uint32_t *hist) {
  __syncthreads();
  if (threadIdx.x < unsigned(NB) && h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], h[threadIdx.x]);
}

// Task order, heaviest first: k_warp_work puts every warp (32 sorted slots)
// in a bucket floor(log2(max candidates of its particles)) + 1 and counts the
// buckets; k_scatter_order writes the warps bucket by bucket, heaviest bucket
// first (the order inside a bucket is immaterial). k_warp_work also keeps
// each slot's candidate count (the density dedupe's tasks and statistics) and
// sets the positions' small-coordinate flag.
constexpr int ORDER_BUCKETS = 33;
static_assert(ORDER_HIST_WORDS == 2 * ORDER_BUCKETS + 4 && ORDER_HIST_STEP_HITS % 2 == 0,
              "order_hist layout");
__global__ void __launch_bounds__(256)
    k_warp_work(SceneView v, const float4 *__restrict__ s_pos,
                const uint32_t *__restrict__ begin, uint8_t *__restrict__ warp_bucket,
                uint32_t *__restrict__ hist, uint32_t *__restrict__ cand,
                uint32_t *__restrict__ small_flag) {
  __shared__ uint32_t h[ORDER_BUCKETS];
  if (threadIdx.x < unsigned(ORDER_BUCKETS)) h[threadIdx.x] = 0u;
  __syncthreads();
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t total = 0u;
  const bool active = s < v.b->n_sorted;
  bool small = false;
  if (active) {
    const DevUniforms *U = v.u + v.scene_of_slot[s];
    const float4 p = s_pos[s];
    small = small_coord(p.x) || small_coord(p.y) || small_coord(p.z);
    Runs R;
    neighbor_runs(xyz(p), U->grid, begin + U->c_offset, R);
    total = R.total;
    cand[s] = total;
  }
  if (__any_sync(0xffffffffu, small) && (threadIdx.x & 31u) == 0u) atomicOr(small_flag, 1u);
  const uint32_t m = __reduce_max_sync(0xffffffffu, total);
  if ((threadIdx.x & 31u) == 0u && active) {
    const uint32_t b = 32u - uint32_t(__clz(m));
    warp_bucket[s >> 5] = uint8_t(b);
    atomicAdd(&h[b], 1u);
  }
  flush_buckets(h, hist);
}

// Each block ranks its warps per bucket in shared memory and reserves one
// range per bucket with a global atomic.
__global__ void __launch_bounds__(256)
    k_scatter_order(SceneView v, const uint8_t *__restrict__ warp_bucket,
                    const uint32_t *__restrict__ hist, uint32_t *__restrict__ cursor,
                    uint32_t *__restrict__ order, const uint32_t *__restrict__ count) {
  __shared__ uint32_t base[ORDER_BUCKETS], local[ORDER_BUCKETS];
  if (threadIdx.x == 0) {
    uint32_t acc = 0u;
    for (int b = ORDER_BUCKETS - 1; b >= 0; b--) {
      base[b] = acc;
      acc += hist[b];
    }
  }
  if (threadIdx.x < unsigned(ORDER_BUCKETS)) local[threadIdx.x] = 0u;
  __syncthreads();
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = w < ((count ? *count : v.b->n_sorted) + 31u) / 32u;
  const uint32_t b = active ? uint32_t(warp_bucket[w]) : 0u;
  const uint32_t r = shared_rank(active, b, local);
  __syncthreads();
  if (threadIdx.x < unsigned(ORDER_BUCKETS) && local[threadIdx.x])
    local[threadIdx.x] = atomicAdd(&cursor[threadIdx.x], local[threadIdx.x]);
  __syncthreads();
  if (active) order[base[b] + local[b] + r] = w;
}

__global__ void __launch_bounds__(KEY_THREADS)
    k_hit_keys(SceneView v, const uint32_t *__restrict__ mask_hits,
               const uint32_t *__restrict__ mask_off,
               const unsigned long long *__restrict__ step_hits, uint32_t coop_lanes,
               uint16_t *__restrict__ key, uint32_t *__restrict__ hist,
               unsigned long long *__restrict__ stats) {
  __shared__ uint32_t h[KEY_BUCKETS];
  for (unsigned i = threadIdx.x; i < unsigned(KEY_BUCKETS); i += KEY_THREADS) h[i] = 0u;
  __syncthreads();
  const uint32_t n = v.b->n_sorted;
  const uint32_t first = blockIdx.x * KEY_CHUNK + threadIdx.x;
  uint32_t hits[KEY_ITEMS];
#pragma unroll
  for (unsigned k = 0; k < KEY_ITEMS; k++) {
    const uint32_t s = first + k * KEY_THREADS;
    hits[k] = s < n ? mask_hits[s] : 0u;
  }
  // the cooperative threshold: a slot whose hits exceed kCoopFactor times a
  // resident lane's share of the step's pairs is on the pass's critical path
  uint32_t coop_min = 0xffffffffu;
  if (coop_lanes) {
    const unsigned long long t = (__ldg(step_hits) * kCoopFactor) / coop_lanes;
    coop_min = uint32_t(max(min(t, 0xffffffffull), (unsigned long long)kCoopMinHits));
  }
#pragma unroll
  for (unsigned k = 0; k < KEY_ITEMS; k++) {
    const uint32_t s = first + k * KEY_THREADS;
    const bool coop = s < n && hits[k] >= coop_min && mask_off[s] != MASK_NONE;
    const uint32_t c = coop ? uint32_t(KEY_BUCKETS - 1) : min(work_key(hits[k]), uint32_t(KEY_BUCKETS - 2));
    if (s < n) key[s] = uint16_t(c);
    shared_rank(s < n, c, h);
  }
  __syncthreads();
  for (unsigned i = threadIdx.x; i < unsigned(KEY_BUCKETS); i += KEY_THREADS)
    if (h[i]) atomicAdd(&hist[i], h[i]);
  if (threadIdx.x == 0u && h[KEY_BUCKETS - 1])
    atomicAdd(stats + STAT_COOP_FORCE, (unsigned long long)h[KEY_BUCKETS - 1]);
}

// Exclusive bases of the key buckets, heaviest bucket first (one block).
__global__ void __launch_bounds__(1024) k_key_bases(const uint32_t *__restrict__ hist,
                                                    uint32_t *__restrict__ base) {
  constexpr int PER = KEY_BUCKETS / 1024;
  __shared__ uint32_t part[1024];
  const int t = threadIdx.x;
  uint32_t local[PER], sum = 0u;
#pragma unroll
  for (int i = 0; i < PER; i++) {
    local[i] = hist[KEY_BUCKETS - 1 - (t * PER + i)];
    sum += local[i];
  }
  part[t] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const uint32_t add = t >= off ? part[t - off] : 0u;
    __syncthreads();
    part[t] += add;
    __syncthreads();
  }
  uint32_t run = part[t] - sum;
#pragma unroll
  for (int i = 0; i < PER; i++) {
    base[KEY_BUCKETS - 1 - (t * PER + i)] = run;
    run += local[i];
  }
}

// Each block ranks its slots per key in shared memory, reserves one range
// per key with a global atomic, then writes its slots (the order inside a
// key is immaterial).
__global__ void __launch_bounds__(KEY_THREADS)
    k_key_scatter(SceneView v, const uint16_t *__restrict__ key, const uint32_t *__restrict__ base,
                  uint32_t *__restrict__ cursor, uint32_t *__restrict__ perm) {
  __shared__ uint32_t h[KEY_BUCKETS];
  for (unsigned i = threadIdx.x; i < unsigned(KEY_BUCKETS); i += KEY_THREADS) h[i] = 0u;
  __syncthreads();
  const uint32_t n = v.b->n_sorted;
  const uint32_t first = blockIdx.x * KEY_CHUNK + threadIdx.x;
  uint32_t kk[KEY_ITEMS], rank[KEY_ITEMS];
#pragma unroll
  for (unsigned k = 0; k < KEY_ITEMS; k++) {
    const uint32_t s = first + k * KEY_THREADS;
    kk[k] = s < n ? uint32_t(key[s]) : 0u;
  }
#pragma unroll
  for (unsigned k = 0; k < KEY_ITEMS; k++) rank[k] = shared_rank(first + k * KEY_THREADS < n, kk[k], h);
  __syncthreads();
  for (unsigned i = threadIdx.x; i < unsigned(KEY_BUCKETS); i += KEY_THREADS) {
    const uint32_t c = h[i];
    if (c) h[i] = base[i] + atomicAdd(&cursor[i], c);
  }
  __syncthreads();
#pragma unroll
  for (unsigned k = 0; k < KEY_ITEMS; k++) {
    const uint32_t s = first + k * KEY_THREADS;
    if (s < n) perm[h[kk[k]] + rank[k]] = s;
  }
}

// ---- density dedupe ------------------------------------------------------------
// Particles at bit-identical positions (and of the same scene) have the same
// candidate runs and the same r^2 to every candidate, so their density, near
// density, normal, hit mask and neighbour records are identical: the density
// pass computes one representative per group and copies the rest. Groups are
// found inside each 32-slot warp (__match_any_sync on the position bits) and
// the representatives of all warps are compacted in slot order into tasks of
// 32, heaviest first. Over-compressed starts clamp thousands of particles to
// the same wall corner coordinates (the 1M-particle dam break: ~57,000
// particles in such groups, 28% of the pass's candidate tests).
__global__ void __launch_bounds__(256)
    k_dedupe_mark(SceneView v, const float4 *__restrict__ s_pos, uint32_t *__restrict__ rep_of,
                  uint32_t *__restrict__ warp_reps) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t n = v.b->n_sorted;
  const bool active = s < n;
  const unsigned act = __ballot_sync(0xffffffffu, active);
  bool is_rep = false;
  if (active) {
    const float4 p = s_pos[s];
    const unsigned m = __match_any_sync(act, __float_as_uint(p.x)) &
                       __match_any_sync(act, __float_as_uint(p.y)) &
                       __match_any_sync(act, __float_as_uint(p.z)) &
                       __match_any_sync(act, uint32_t(v.scene_of_slot[s]));
    const int leader = __ffs(m) - 1;
    rep_of[s] = (s & ~31u) + uint32_t(leader);
    is_rep = int(lane) == leader;
  }
  const unsigned reps = __ballot_sync(0xffffffffu, is_rep);
  if (lane == 0u && (s >> 5) < (n + 31u) / 32u) warp_reps[s >> 5] = uint32_t(__popc(reps));
}

__global__ void __launch_bounds__(256)
    k_dedupe_list(SceneView v, const uint32_t *__restrict__ rep_of,
                  const uint32_t *__restrict__ warp_incl, uint32_t *__restrict__ list) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned lane = threadIdx.x & 31u;
  const bool is_rep = s < v.b->n_sorted && rep_of[s] == s;
  const unsigned reps = __ballot_sync(0xffffffffu, is_rep);
  if (is_rep)
    list[warp_incl[s >> 5] - uint32_t(__popc(reps)) + uint32_t(__popc(reps & ((1u << lane) - 1u)))] = s;
}

// Task buckets of the compacted list (as k_warp_work, over list entries,
// from the candidate counts k_warp_work kept).
__global__ void __launch_bounds__(256)
    k_list_work(const uint32_t *__restrict__ list, const uint32_t *__restrict__ count,
                const uint32_t *__restrict__ cand, uint8_t *__restrict__ task_bucket,
                uint32_t *__restrict__ hist) {
  __shared__ uint32_t h[ORDER_BUCKETS];
  if (threadIdx.x < unsigned(ORDER_BUCKETS)) h[threadIdx.x] = 0u;
  __syncthreads();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t entries = *count;
  uint32_t total = 0u;
  const bool active = i < entries;
  if (active) total = cand[list[i]];
  const uint32_t m = __reduce_max_sync(0xffffffffu, total);
  if ((threadIdx.x & 31u) == 0u && active) {
    const uint32_t b = 32u - uint32_t(__clz(m));
    task_bucket[i >> 5] = uint8_t(b);
    atomicAdd(&h[b], 1u);
  }
  flush_buckets(h, hist);
}

// The copies: each slot that is not a representative takes its
// representative's results (its own pre-XSPH velocity in its record) and adds
// the representative's pair counts to the statistics.
__global__ void __launch_bounds__(256)
    k_dedupe_copy(SceneView v, const uint32_t *__restrict__ rep_of, const float4 *__restrict__ s_vel,
                  float2 *__restrict__ s_dens, float4 *__restrict__ s_nrm, NbrRecords nb,
                  uint32_t *__restrict__ mask_off, uint32_t *__restrict__ mask_hits,
                  const uint32_t *__restrict__ cand, unsigned long long *__restrict__ stats) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t c = 0u, h = 0u, ns = 0u;
  if (s < v.b->n_sorted) {
    const uint32_t r = rep_of[s];
    if (r != s) {
      s_dens[s] = s_dens[r];
      s_nrm[s] = s_nrm[r];
      nb.pos[s] = nb.pos[r];
      nb.nrm[s] = nb.nrm[r];
      const float4 vs = s_vel[s];
      nb.vel[s] = make_float4(vs.x, vs.y, vs.z, nb.vel[r].w);
      mask_off[s] = mask_off[r];
      ns = mask_hits[r];
      mask_hits[s] = ns;
      h = nb.hits[r];
      nb.hits[s] = h;
      c = cand[r];
    }
  }
  const unsigned long long cs = warp_sum_u64(c), hs = warp_sum_u64(h), nss = warp_sum_u64(ns);
  if ((threadIdx.x & 31u) == 0u && cs) {
    atomicAdd(stats + STAT_CAND_DENSITY, cs);
    atomicAdd(stats + STAT_HIT_DENSITY, hs);
    atomicAdd(stats + STAT_HIT_NONSELF, nss);
    atomicAdd(nb.step_hits, nss);
  }
}

template <int B>
__global__ void __launch_bounds__(128)
    k_density(TaskQueue q, SceneView v, const float4 *__restrict__ s_pos,
              const float4 *__restrict__ s_vel, const uint32_t *__restrict__ begin,
              float2 *__restrict__ s_dens, float4 *__restrict__ s_nrm, NbrRecords nb,
              unsigned long long *__restrict__ stats, uint32_t *__restrict__ mask_words,
              uint32_t *__restrict__ mask_off, uint32_t *__restrict__ mask_hits,
              unsigned long long *__restrict__ mask_alloc, unsigned long long mask_cap) {
  for_warp_tasks(q, [&](uint32_t s) {
    density_one<B>(s, v, s_pos, s_vel, begin, s_dens, s_nrm, nb, stats, mask_words, mask_off,
                   mask_hits, mask_alloc, mask_cap);
  });
}

template <int B>
__global__ void __launch_bounds__(128)
    k_xsph(TaskQueue q, SceneView v, const float4 *__restrict__ s_vel,
           const float4 *__restrict__ nb_pos, const float4 *__restrict__ nb_vel,
           const uint32_t *__restrict__ begin, float4 *__restrict__ vel_x) {
  for_warp_tasks(q, [&](uint32_t s) { xsph_one<B>(s, v, s_vel, nb_pos, nb_vel, begin, vel_x); });
}


// The heavy particles, one warp each (cooperative): the first *coop_count
// slots of the hit permutation. Its own kernel, launched before
// k_force_predict, so that only it holds the shared memory of the
// cooperative walk (the other kernel keeps the whole L1).
__global__ void __launch_bounds__(kForceThreads, 512 / kForceThreads)
    k_force_coop(TaskQueue q, const uint32_t *__restrict__ coop_count, SceneView v,
                 const float4 *__restrict__ s_pos, const float4 *__restrict__ nb_pos,
                 const float4 *__restrict__ nb_vel, const float4 *__restrict__ nb_nrm,
                 const float2 *__restrict__ s_dens, const float4 *__restrict__ s_nrm,
                 const float4 *__restrict__ vel_x, const uint32_t *__restrict__ begin,
                 const float4 *__restrict__ dir_tab, int dir_half,
                 const uint32_t *__restrict__ mask_words, const uint32_t *__restrict__ mask_off,
                 const uint32_t *__restrict__ small_flag, float4 *__restrict__ anp,
                 float4 *__restrict__ pred_xp, float *__restrict__ pred_rho,
                 float *__restrict__ pterm0) {
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t nc = min(__ldg(coop_count), q.n);
  while (true) {
    uint32_t t = 0u;
    if (lane == 0u) t = atomicAdd(q.counter, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= nc) break;
    force_predict_one<true>(__ldg(q.perm + t), v, s_pos, nb_pos, nb_vel, nb_nrm, s_dens, s_nrm,
                            vel_x, begin, dir_tab, dir_half, mask_words, mask_off, small_flag, anp,
                            pred_xp, pred_rho, pterm0);
  }
}

// Every slot of the hit permutation in tasks of 32 (simulations of
// kCoopMaxParticles or more, where no lane reaches the cooperative threshold).
__global__ void __launch_bounds__(kForceThreads, 512 / kForceThreads)
    k_force_all(TaskQueue q, SceneView v, const float4 *__restrict__ s_pos,
                const float4 *__restrict__ nb_pos, const float4 *__restrict__ nb_vel,
                const float4 *__restrict__ nb_nrm, const float2 *__restrict__ s_dens,
                const float4 *__restrict__ s_nrm, const float4 *__restrict__ vel_x,
                const uint32_t *__restrict__ begin, const float4 *__restrict__ dir_tab,
                int dir_half, const uint32_t *__restrict__ mask_words,
                const uint32_t *__restrict__ mask_off, const uint32_t *__restrict__ small_flag,
                float4 *__restrict__ anp, float4 *__restrict__ pred_xp,
                float *__restrict__ pred_rho, float *__restrict__ pterm0) {
  for_warp_tasks(q, [&](uint32_t s) {
    force_predict_one<false>(s, v, s_pos, nb_pos, nb_vel, nb_nrm, s_dens, s_nrm, vel_x, begin,
                             dir_tab, dir_half, mask_words, mask_off, small_flag, anp, pred_xp,
                             pred_rho, pterm0);
  });
}

// The other slots of the hit permutation (after the *coop_count cooperative
// ones), in tasks of 32.
__global__ void __launch_bounds__(kForceThreads, 512 / kForceThreads)
    k_force_predict(TaskQueue q, const uint32_t *__restrict__ coop_count, SceneView v,
                    const float4 *__restrict__ s_pos, const float4 *__restrict__ nb_pos,
                    const float4 *__restrict__ nb_vel, const float4 *__restrict__ nb_nrm,
                    const float2 *__restrict__ s_dens, const float4 *__restrict__ s_nrm,
                    const float4 *__restrict__ vel_x, const uint32_t *__restrict__ begin,
                    const float4 *__restrict__ dir_tab, int dir_half,
                    const uint32_t *__restrict__ mask_words,
                    const uint32_t *__restrict__ mask_off,
                    const uint32_t *__restrict__ small_flag, float4 *__restrict__ anp,
                    float4 *__restrict__ pred_xp, float *__restrict__ pred_rho,
                    float *__restrict__ pterm0) {
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t nc = min(__ldg(coop_count), q.n);
  const uint32_t ntasks = (q.n - nc + 31u) / 32u;
  while (true) {
    uint32_t t = 0u;
    if (lane == 0u) t = atomicAdd(q.counter, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= ntasks) break;
    const uint32_t idx = nc + t * 32u + lane;
    const uint32_t s = idx < q.n ? __ldg(q.perm + idx) : 0xffffffffu;
    force_predict_one<false>(s, v, s_pos, nb_pos, nb_vel, nb_nrm, s_dens, s_nrm, vel_x, begin,
                             dir_tab, dir_half, mask_words, mask_off, small_flag, anp, pred_xp,
                             pred_rho, pterm0);
  }
}

template <bool HAS_PRESSURE, bool LAST, bool RECORD, int B>
__global__ void __launch_bounds__(128, (!HAS_PRESSURE && B > 1) ? 4 : 0)
    k_solve(TaskQueue q, SceneView v, const float4 *__restrict__ s_pos,
            const float4 *__restrict__ vel_x, const float4 *__restrict__ anp,
            const uint32_t *__restrict__ begin, const float4 *__restrict__ xp_in,
            const float *__restrict__ pterm_in, float4 *__restrict__ xp_out,
            float *__restrict__ rho_out, float *__restrict__ pterm_out,
            float4 *__restrict__ v_out, unsigned long long *__restrict__ stats,
            float4 *__restrict__ ap_out, const uint32_t *__restrict__ mask_off,
            uint32_t *__restrict__ hit_out, bool hit_or) {
  for_warp_tasks(q, [&](uint32_t s) {
    solve_one<HAS_PRESSURE, LAST, RECORD, B>(s, v, s_pos, vel_x, anp, begin, xp_in, pterm_in, xp_out,
                                          rho_out, pterm_out, v_out, stats, ap_out, mask_off,
                                          hit_out, hit_or);
  });
}

// ---- finalize + integrate ----------------------------------------------------
// SDF texture with clamp-to-edge trilinear filtering (exact FP32 weights).
__device__ __forceinline__ float sample_sdf(const float *__restrict__ sdf, int res, float3 uvw) {
  auto texel = [&](int x, int y, int z) -> float {
    x = min(max(x, 0), res - 1);
    y = min(max(y, 0), res - 1);
    z = min(max(z, 0), res - 1);
    return __ldg(sdf + size_t(x) + size_t(y) * res + size_t(z) * res * res);
  };
  const float tx = uvw.x * float(res) - 0.5f;
  const float ty = uvw.y * float(res) - 0.5f;
  const float tz = uvw.z * float(res) - 0.5f;
  const float fx0 = floorf(tx), fy0 = floorf(ty), fz0 = floorf(tz);
  const float ax = tx - fx0, ay = ty - fy0, az = tz - fz0;
  // clamp before the +1 neighbour so the index arithmetic cannot overflow
  const int x0 = min(max(__float2int_rz(fx0), -1), res);
  const int y0 = min(max(__float2int_rz(fy0), -1), res);
  const int z0 = min(max(__float2int_rz(fz0), -1), res);
  auto mix = [](float a, float b, float t) { return a * (1.0f - t) + b * t; };
  const float c00 = mix(texel(x0, y0, z0), texel(x0 + 1, y0, z0), ax);
  const float c10 = mix(texel(x0, y0 + 1, z0), texel(x0 + 1, y0 + 1, z0), ax);
  const float c01 = mix(texel(x0, y0, z0 + 1), texel(x0 + 1, y0, z0 + 1), ax);
  const float c11 = mix(texel(x0, y0 + 1, z0 + 1), texel(x0 + 1, y0 + 1, z0 + 1), ax);
  const float c0 = mix(c00, c10, ay);
  const float c1 = mix(c01, c11, ay);
  return mix(c0, c1, az);
}

__device__ __forceinline__ int f2i_rz(float x) { return __float2int_rz(x); }  // saturating, NaN -> 0

__global__ void __launch_bounds__(128)
    k_finalize_integrate(SceneView v, const float4 *__restrict__ s_pos,
                         const float4 *__restrict__ s_vel, const float4 *__restrict__ vel_x,
                         const float4 *__restrict__ v_fin, const uint32_t *__restrict__ s2o,
                         const float *__restrict__ sdf, float4 *__restrict__ p_pos,
                         float4 *__restrict__ p_vel, float4 *__restrict__ p_force,
                         GpuRigidBodyAccum *__restrict__ accum) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  int32_t rfx = 0, rfy = 0, rfz = 0, rtx = 0, rty = 0, rtz = 0;
  uint32_t contact = 0;
  const bool active = s < v.b->n_sorted;
  const uint32_t scene = active ? v.scene_of_slot[s] : 0u;
  if (active) {
    const DevUniforms *U = v.u + scene;
    const GpuSphParams3D &P = U->sph;
    const GpuContainerGeometry &c = U->geom;
    const uint32_t orig = s2o[s];
    // pcisph_finalize.wgsl:57-72
    const float3 corrected = xyz(v_fin[s]);
    const float3 original = xyz(vel_x[s]);
    const float3 dv = corrected - original;
    p_force[orig] = make_float4(dv.x, dv.y, dv.z, 0.0f);
    // sph_integrate_3d.wgsl:98-388
    const float4 pos4 = s_pos[s];
    float3 pos = xyz(pos4);
    float3 vel = corrected;
    const float h = P.kernel_radius;
    float3 accel = f3(0.f, 0.f, 0.f);
    const float3 lp = world_to_local(c, pos);
    const float3 lv = world_dir_to_local(c, vel);
    const float bl = h * 0.4f;
    const float wd = 8.0f;
    float3 wa = f3(0.f, 0.f, 0.f);
    float d;
    d = lp.x - (-c.half_width);
    if (d < bl) { const float t = 1.0f - d / bl; wa.x += c.wall_stiffness * t * t; if (lv.x < 0.0f) wa.x -= lv.x * wd * t; }
    d = c.half_width - lp.x;
    if (d < bl) { const float t = 1.0f - d / bl; wa.x -= c.wall_stiffness * t * t; if (lv.x > 0.0f) wa.x -= lv.x * wd * t; }
    d = lp.y - (-c.half_height);
    if (d < bl) { const float t = 1.0f - d / bl; wa.y += c.wall_stiffness * t * t; if (lv.y < 0.0f) wa.y -= lv.y * wd * t; }
    d = c.half_height - lp.y;
    if (d < bl) { const float t = 1.0f - d / bl; wa.y -= c.wall_stiffness * t * t; if (lv.y > 0.0f) wa.y -= lv.y * wd * t; }
    d = lp.z - (-c.half_depth);
    if (d < bl) { const float t = 1.0f - d / bl; wa.z += c.wall_stiffness * t * t; if (lv.z < 0.0f) wa.z -= lv.z * wd * t; }
    d = c.half_depth - lp.z;
    if (d < bl) { const float t = 1.0f - d / bl; wa.z -= c.wall_stiffness * t * t; if (lv.z > 0.0f) wa.z -= lv.z * wd * t; }
    accel = accel + local_dir_to_world(c, wa);

    const GpuMouseForce &M = U->mouse;
    if (M.is_active == 1u) {
      const float3 to_mouse = xyz(M.position) - pos;
      const float dist = len3(to_mouse);
      if (dist < M.radius && dist > 0.001f) {
        const float falloff = 1.0f - dist / M.radius;
        const float3 fd = normalize3(to_mouse);
        const float sm = M.strength * falloff;
        switch (M.mode) {
          case 1: accel = accel + fd * sm; break;
          case 2: {
            const float3 axis = normalize3(xyz(M.direction));
            const float3 tangent = cross3(fd, axis);
            const float tlen = len3(tangent);
            if (tlen > 0.001f) accel = accel + (tangent / tlen) * sm;
            break;
          }
          case 3: accel = accel - fd * sm * 3.0f; break;
          case 4: {
            const float3 dd = normalize3(fd + f3(0.0f, -1.0f, 0.0f));
            accel = accel + dd * sm;
            break;
          }
          default: accel = accel - fd * sm; break;
        }
      }
    }

    const GpuRigidBody &B = U->rigid;
    if (B.is_active != 0u) {
      const float3 world_rel = pos - xyz(B.position);
      const float3 rr0 = xyz(B.rot_row0), rr1 = xyz(B.rot_row1), rr2 = xyz(B.rot_row2);
      const float3 rl = f3(dot3(rr0, world_rel), dot3(rr1, world_rel), dot3(rr2, world_rel));
      const float he = B.half_extent;
      float sdf_v;
      float3 ln = f3(0.f, 0.f, 0.f);
      switch (B.shape) {
        case 1: {
          const float dist = len3(rl);
          sdf_v = dist - he;
          ln = dist > 0.001f ? rl / dist : f3(0.f, 1.f, 0.f);
          break;
        }
        case 2: {
          const float radial = sqrtf(rl.x * rl.x + rl.z * rl.z);
          const float d_radial = radial - he;
          const float d_cap = fabsf(rl.y) - he;
          sdf_v = fmaxf(d_radial, d_cap);
          if (d_radial > d_cap) {
            ln = radial > 0.001f ? f3(rl.x / radial, 0.f, rl.z / radial) : f3(1.f, 0.f, 0.f);
          } else {
            ln = f3(0.f, signf(rl.y), 0.f);
          }
          break;
        }
        case 3: {
          const float minor_r = he * 0.3f;
          const float xz_len = sqrtf(rl.x * rl.x + rl.z * rl.z);
          const float qx = xz_len - he, qy = rl.y;
          const float q_len = sqrtf(qx * qx + qy * qy);
          sdf_v = q_len - minor_r;
          if (q_len > 0.001f && xz_len > 0.001f) {
            const float rdx = qx / q_len, rdy = qy / q_len;
            ln = f3(rdx * rl.x / xz_len, rdy, rdx * rl.z / xz_len);
          } else {
            ln = f3(0.f, 1.f, 0.f);
          }
          break;
        }
        case 4: {
          const int res = int(U->sdf_res);
          const float3 nrm = rl / he;
          const float3 uvw = nrm * 0.5f + f3(0.5f, 0.5f, 0.5f);
          const float raw = sample_sdf(sdf, res, uvw);
          sdf_v = raw * he;
          const float e = 1.0f / 32.0f;
          const float gx = sample_sdf(sdf, res, uvw + f3(e, 0.f, 0.f)) - sample_sdf(sdf, res, uvw - f3(e, 0.f, 0.f));
          const float gy = sample_sdf(sdf, res, uvw + f3(0.f, e, 0.f)) - sample_sdf(sdf, res, uvw - f3(0.f, e, 0.f));
          const float gz = sample_sdf(sdf, res, uvw + f3(0.f, 0.f, e)) - sample_sdf(sdf, res, uvw - f3(0.f, 0.f, e));
          const float3 g = f3(gx, gy, gz);
          const float gl = len3(g);
          ln = gl > 1e-6f ? g / gl : normalize3(rl + f3(0.f, 1e-6f, 0.f));
          break;
        }
        default: {
          const float3 dd = f3(fabsf(rl.x) - he, fabsf(rl.y) - he, fabsf(rl.z) - he);
          sdf_v = fmaxf(dd.x, fmaxf(dd.y, dd.z));
          if (dd.x >= dd.y && dd.x >= dd.z) ln = f3(signf(rl.x), 0.f, 0.f);
          else if (dd.y >= dd.x && dd.y >= dd.z) ln = f3(0.f, signf(rl.y), 0.f);
          else ln = f3(0.f, 0.f, signf(rl.z));
          break;
        }
      }
      const float range = h * 0.7f;
      if (sdf_v < range) {
        const float3 nw = f3(rr0.x * ln.x + rr1.x * ln.y + rr2.x * ln.z,
                             rr0.y * ln.x + rr1.y * ln.y + rr2.y * ln.z,
                             rr0.z * ln.x + rr1.z * ln.y + rr2.z * ln.z);
        const float pen = range - sdf_v;
        const float t = pen / range;
        const float3 penalty = nw * B.stiffness * t * t;
        accel = accel + penalty;
        float3 damp = f3(0.f, 0.f, 0.f);
        const float3 rel_vel = vel - xyz(B.velocity);
        const float vn = dot3(rel_vel, nw);
        if (vn < 0.0f) {
          damp = (-nw) * vn * 5.0f;
          accel = accel + damp;
        }
        const float3 reaction = (-(penalty + damp)) * P.mass;
        rfx = f2i_rz(reaction.x * 1000.0f);
        rfy = f2i_rz(reaction.y * 1000.0f);
        rfz = f2i_rz(reaction.z * 1000.0f);
        contact = 1u;
        const float3 torque = cross3(world_rel, reaction);
        rtx = f2i_rz(torque.x * 1000.0f);
        rty = f2i_rz(torque.y * 1000.0f);
        rtz = f2i_rz(torque.z * 1000.0f);
      }
    }

    const float dt = P.dt;
    vel = vel + dt * accel;
    pos = pos + dt * vel;
    float3 lpn = world_to_local(c, pos);
    float3 lvn = world_dir_to_local(c, vel);
    const float rest = c.damping;
    if (lpn.x < -c.half_width) { lpn.x = -c.half_width; lvn.x = fabsf(lvn.x) * rest; }
    else if (lpn.x > c.half_width) { lpn.x = c.half_width; lvn.x = -fabsf(lvn.x) * rest; }
    if (lpn.y < -c.half_height) { lpn.y = -c.half_height; lvn.y = fabsf(lvn.y) * rest; }
    else if (lpn.y > c.half_height) { lpn.y = c.half_height; lvn.y = -fabsf(lvn.y) * rest; }
    if (lpn.z < -c.half_depth) { lpn.z = -c.half_depth; lvn.z = fabsf(lvn.z) * rest; }
    else if (lpn.z > c.half_depth) { lpn.z = c.half_depth; lvn.z = -fabsf(lvn.z) * rest; }
    const float3 pw = local_to_world(c, lpn);
    const float3 vw = local_dir_to_world(c, lvn);
    p_pos[orig] = make_float4(pw.x, pw.y, pw.z, pos4.w);
    p_vel[orig] = make_float4(vw.x, vw.y, vw.z, s_vel[s].w);
  }
  // rigid-body reaction: integer sums are order independent, so reduce in
  // the warp and add once per warp (sph_integrate_3d.wgsl:328-339). A warp
  // whose contacts span two scenes (a scene boundary inside the warp) adds
  // lane by lane into each scene's accumulator instead.
  const unsigned any = __ballot_sync(0xffffffffu, contact != 0u);
  if (any) {
    const uint32_t s0 = __shfl_sync(0xffffffffu, scene, __ffs(any) - 1);
    if (__all_sync(0xffffffffu, contact == 0u || scene == s0)) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        rfx += __shfl_xor_sync(0xffffffffu, rfx, o);
        rfy += __shfl_xor_sync(0xffffffffu, rfy, o);
        rfz += __shfl_xor_sync(0xffffffffu, rfz, o);
        rtx += __shfl_xor_sync(0xffffffffu, rtx, o);
        rty += __shfl_xor_sync(0xffffffffu, rty, o);
        rtz += __shfl_xor_sync(0xffffffffu, rtz, o);
      }
      if ((threadIdx.x & 31) == 0) {
        GpuRigidBodyAccum *a = accum + s0;
        atomicAdd(&a->force_x, rfx);
        atomicAdd(&a->force_y, rfy);
        atomicAdd(&a->force_z, rfz);
        atomicAdd(&a->contact_count, uint32_t(__popc(any)));
        atomicAdd(&a->torque_x, rtx);
        atomicAdd(&a->torque_y, rty);
        atomicAdd(&a->torque_z, rtz);
      }
    } else if (contact) {
      GpuRigidBodyAccum *a = accum + scene;
      atomicAdd(&a->force_x, rfx);
      atomicAdd(&a->force_y, rfy);
      atomicAdd(&a->force_z, rfz);
      atomicAdd(&a->contact_count, 1u);
      atomicAdd(&a->torque_x, rtx);
      atomicAdd(&a->torque_y, rty);
      atomicAdd(&a->torque_z, rtz);
    }
  }
}

inline unsigned blocks_for(uint32_t n, unsigned threads) {
  return unsigned((n + threads - 1) / threads);
}

}  // namespace

cudaError_t launch_dir_table(const DevState &d, cudaStream_t st) {
  const int count = 2 * d.dir_half + 1;
  k_dir_table<<<(count + 255) / 256, 256, 0, st>>>(d.dir_tab, d.dir_half);
  return cudaGetLastError();
}

namespace {
// Persistent grid: as many resident blocks as the kernel's occupancy allows.
// the positions' small-coordinate flag in order_hist (see small_coord)
uint32_t *position_small_flag(const DevState &d) { return d.order_hist + 2 * ORDER_BUCKETS; }
// the step's in-range pair count in order_hist (summed by the density pass)
unsigned long long *step_hits(const DevState &d) {
  return reinterpret_cast<unsigned long long *>(d.order_hist + ORDER_HIST_STEP_HITS);
}

template <class K>
unsigned persistent_blocks(K kernel, int sm_count, int threads = 128) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  return unsigned(per_sm * sm_count);
}

unsigned force_blocks(const DevState &d) {
  static unsigned blocks = 0;
  if (!blocks) blocks = persistent_blocks(k_force_predict, d.sm_count, kForceThreads);
  return blocks;
}

cudaError_t prepare_queue(const DevState &d, const uint32_t *order, bool slots, uint32_t n,
                          int slot, cudaStream_t st, TaskQueue *q) {
  q->perm = order;
  q->slots = slots;
  q->counter = d.task_counters + slot;
  q->n = n;
  q->nwarps = (n + 31u) / 32u;
  return cudaMemsetAsync(q->counter, 0, sizeof(uint32_t), st);
}

cudaError_t order_by_keys(const DevState &d, uint32_t n, uint32_t *perm, cudaStream_t st) {
  k_key_bases<<<1, 1024, 0, st>>>(d.key_hist, d.key_hist + KEY_BUCKETS);
  k_key_scatter<<<blocks_for(n, KEY_CHUNK), KEY_THREADS, 0, st>>>(
      d.view(), d.work_key, d.key_hist + KEY_BUCKETS, d.key_hist + 2 * KEY_BUCKETS, perm);
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_order_warps(const DevState &d, uint32_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(d.order_hist, 0, sizeof(uint32_t) * ORDER_HIST_WORDS, st);
  if (e != cudaSuccess) return e;
  k_warp_work<<<blocks_for(n, 256), 256, 0, st>>>(d.view(), d.s_pos, d.cell_begin, d.warp_bucket,
                                                  d.order_hist, d.dens_cand,
                                                  position_small_flag(d));
  const uint32_t nwarps = (n + 31u) / 32u;
  k_scatter_order<<<blocks_for(nwarps, 256), 256, 0, st>>>(d.view(), d.warp_bucket, d.order_hist,
                                                           d.order_hist + ORDER_BUCKETS,
                                                           d.warp_order, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_order_hits(const DevState &d, uint32_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(d.key_hist, 0, sizeof(uint32_t) * 3 * KEY_BUCKETS, st);
  if (e != cudaSuccess) return e;
  k_hit_keys<<<blocks_for(n, KEY_CHUNK), KEY_THREADS, 0, st>>>(
      d.view(), d.mask_hits, d.mask_off, step_hits(d),
      n < kCoopMaxParticles ? force_blocks(d) * kForceThreads : 0u, d.work_key, d.key_hist,
      d.stats);
  return order_by_keys(d, n, d.perm_hit, st);
}

cudaError_t launch_density(const DevState &d, uint32_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(d.mask_alloc, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  // dedupe, except while recording for the reverse pass (the recorded PCISPH
  // levels write per-particle masks at the density mask's offsets, which
  // copies would share)
  const bool dedupe = d.rec_hits == nullptr;
  const uint32_t nwarps = (n + 31u) / 32u;
  TaskQueue q;
  if (dedupe) {
    // representatives per warp, their inclusive scan (decoupled look-back),
    // the compacted list; its size is the scan's last entry
    const uint32_t *dd_count = d.dd_incl + (nwarps - 1u);
    k_dedupe_mark<<<blocks_for(n, 256), 256, 0, st>>>(d.view(), d.s_pos, d.rep_of, d.dd_warp);
    e = cudaMemsetAsync(d.dd_tiles, 0, sizeof(unsigned long long) * (scan_tiles(nwarps) + 1), st);
    if (e != cudaSuccess) return e;
    e = launch_scan_with_scratch(d.dd_warp, d.dd_incl, nwarps, d.dd_tiles, d.err, st);
    if (e != cudaSuccess) return e;
    k_dedupe_list<<<blocks_for(n, 256), 256, 0, st>>>(d.view(), d.rep_of, d.dd_incl, d.dd_list);
    e = cudaMemsetAsync(d.dd_hist, 0, sizeof(uint32_t) * 2 * ORDER_BUCKETS, st);
    if (e != cudaSuccess) return e;
    k_list_work<<<blocks_for(n, 256), 256, 0, st>>>(d.dd_list, dd_count, d.dens_cand, d.dd_bucket,
                                                    d.dd_hist);
    k_scatter_order<<<blocks_for(nwarps, 256), 256, 0, st>>>(
        d.view(), d.dd_bucket, d.dd_hist, d.dd_hist + ORDER_BUCKETS, d.dd_order, dd_count);
    e = prepare_queue(d, d.dd_order, false, n, TASK_COUNTERS - 1, st, &q);
    q.list = d.dd_list;
    q.count = dd_count;
  } else {
    e = prepare_queue(d, d.warp_order, false, n, TASK_COUNTERS - 1, st, &q);
  }
  if (e != cudaSuccess) return e;
  const NbrRecords nb{d.nb_pos, d.nb_vel, d.nb_nrm, d.dens_hits, step_hits(d)};
#define FS_DENSITY(I_)                                                                      \
  do {                                                                                      \
    static unsigned blocks = 0;                                                             \
    if (!blocks) blocks = persistent_blocks(k_density<kLoadDepths[I_]>, d.sm_count);        \
    k_density<kLoadDepths[I_]><<<blocks, 128, 0, st>>>(                                     \
        q, d.view(), d.s_pos, d.s_vel, d.cell_begin, d.s_dens, d.s_nrm, nb, d.stats,        \
        d.mask_words, d.mask_off, d.mask_hits, d.mask_alloc, d.mask_cap);                   \
  } while (0)
  switch (d.load_density) {
    case 1: FS_DENSITY(1); break;
    case 2: FS_DENSITY(2); break;
    case 3:
    case 4: FS_DENSITY(3); break;  // no staged density form
    default: FS_DENSITY(0); break;
  }
#undef FS_DENSITY
  if (dedupe)
    k_dedupe_copy<<<blocks_for(n, 256), 256, 0, st>>>(d.view(), d.rep_of, d.s_vel, d.s_dens,
                                                      d.s_nrm, nb, d.mask_off, d.mask_hits,
                                                      d.dens_cand, d.stats);
  return cudaGetLastError();
}

cudaError_t launch_xsph(const DevState &d, uint32_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  TaskQueue q;
  cudaError_t e = prepare_queue(d, d.warp_order, false, n, 0, st, &q);
  if (e != cudaSuccess) return e;
#define FS_XSPH(I_)                                                                          \
  do {                                                                                       \
    static unsigned blocks = 0;                                                              \
    if (!blocks) blocks = persistent_blocks(k_xsph<kXsphDepths[I_]>, d.sm_count);            \
    k_xsph<kXsphDepths[I_]><<<blocks, 128, 0, st>>>(q, d.view(), d.s_vel, d.nb_pos, d.nb_vel, \
                                                    d.cell_begin, d.vel_x);                  \
  } while (0)
  switch (d.load_xsph) {
    case 0: FS_XSPH(0); break;
    case 2: FS_XSPH(2); break;
    case 3: FS_XSPH(3); break;
    case 4: FS_XSPH(4); break;
    default: FS_XSPH(1); break;
  }
#undef FS_XSPH
  return cudaGetLastError();
}

cudaError_t launch_force_predict(const DevState &d, uint32_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  TaskQueue q, qc;
  cudaError_t e = prepare_queue(d, d.perm_hit, true, n, 1, st, &q);
  if (e != cudaSuccess) return e;
  e = prepare_queue(d, d.perm_hit, true, n, TASK_COUNTERS - 2, st, &qc);
  if (e != cudaSuccess) return e;
  float4 *xp_out = d.rec_xp ? d.rec_xp[0] : d.pred_xp[0];
  float *rho_out = d.rec_rho ? d.rec_rho[0] : d.pred_rho[0];
  // the cooperative slots: the count of the top hit-count key
  const uint32_t *coop_count = d.key_hist + (KEY_BUCKETS - 1);
  if (n >= kCoopMaxParticles) {
    static unsigned all_blocks = 0;
    if (!all_blocks) all_blocks = persistent_blocks(k_force_all, d.sm_count, kForceThreads);
    k_force_all<<<all_blocks, kForceThreads, 0, st>>>(
        q, d.view(), d.s_pos, d.nb_pos, d.nb_vel, d.nb_nrm, d.s_dens, d.s_nrm, d.vel_x,
        d.cell_begin, d.dir_tab, d.dir_half, d.mask_words, d.mask_off, position_small_flag(d),
        d.anp, xp_out, rho_out, d.pterm[0]);
    return cudaGetLastError();
  }
  static unsigned coop_blocks = 0;
  if (!coop_blocks) coop_blocks = persistent_blocks(k_force_coop, d.sm_count, kForceThreads);
  k_force_coop<<<coop_blocks, kForceThreads, 0, st>>>(
      qc, coop_count, d.view(), d.s_pos, d.nb_pos, d.nb_vel, d.nb_nrm, d.s_dens, d.s_nrm,
      d.vel_x, d.cell_begin, d.dir_tab, d.dir_half, d.mask_words, d.mask_off,
      position_small_flag(d), d.anp, xp_out, rho_out, d.pterm[0]);
  k_force_predict<<<force_blocks(d), kForceThreads, 0, st>>>(
      q, coop_count, d.view(), d.s_pos, d.nb_pos, d.nb_vel, d.nb_nrm, d.s_dens, d.s_nrm,
      d.vel_x, d.cell_begin, d.dir_tab, d.dir_half, d.mask_words, d.mask_off,
      position_small_flag(d), d.anp, xp_out, rho_out, d.pterm[0]);
  return cudaGetLastError();
}

cudaError_t launch_solve(const DevState &d, uint32_t n, int iter, int last, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const int in = iter & 1, out = in ^ 1;
  // ping-pong, or the recorded levels iter -> iter + 1 when recording
  const float4 *xp_in = d.rec_xp ? d.rec_xp[iter] : d.pred_xp[in];
  float4 *xp_out = d.rec_xp ? d.rec_xp[iter + 1] : d.pred_xp[out];
  float *rho_out = d.rec_rho ? d.rec_rho[iter + 1] : d.pred_rho[out];
  float4 *ap_out = d.rec_ap ? d.rec_ap[iter] : nullptr;
  uint32_t *hit_out = d.rec_hits;
  const bool hit_or = iter > 0;
  TaskQueue q;
  cudaError_t e = prepare_queue(d, d.warp_order, false, n, 2 + (iter % (TASK_COUNTERS - 3)), st, &q);
  if (e != cudaSuccess) return e;
#define FS_SOLVE_B(P_, L_, R_, B_, Q_)                                                        \
  do {                                                                                        \
    static unsigned blocks = 0;                                                               \
    if (!blocks) blocks = persistent_blocks(k_solve<P_, L_, R_, B_>, d.sm_count);            \
    k_solve<P_, L_, R_, B_><<<blocks, 128, 0, st>>>(Q_, d.view(), d.s_pos, d.vel_x, d.anp,     \
                                                    d.cell_begin, xp_in, d.pterm[in], xp_out, \
                                                    rho_out, d.pterm[out], d.pred_v, d.stats, \
                                                    ap_out, d.mask_off, hit_out, hit_or);     \
  } while (0)
#define FS_SOLVE(P_, L_, R_)                                       \
  do {                                                             \
    switch (d.load_solve) {                                        \
      case 1: FS_SOLVE_B(P_, L_, R_, kLoadDepths[1], q); break;    \
      case 2: FS_SOLVE_B(P_, L_, R_, kLoadDepths[2], q); break;    \
      case 3: FS_SOLVE_B(P_, L_, R_, kLoadDepths[3], q); break;    \
      default: FS_SOLVE_B(P_, L_, R_, kLoadDepths[0], q); break;   \
    }                                                              \
  } while (0)
#define FS_SOLVE_R(P_, L_)            \
  do {                                \
    if (hit_out) FS_SOLVE(P_, L_, true); \
    else FS_SOLVE(P_, L_, false);     \
  } while (0)
  // iteration 0 reads the predict output, where every pressure is 0: the
  // pressure-free kernel
  if (iter == 0 && last) FS_SOLVE_R(false, true);
  else if (iter == 0) FS_SOLVE_R(false, false);
  else if (last) FS_SOLVE_R(true, true);
  else FS_SOLVE_R(true, false);
#undef FS_SOLVE_R
#undef FS_SOLVE
#undef FS_SOLVE_B
  return cudaGetLastError();
}

cudaError_t launch_finalize_integrate(const DevState &d, uint32_t n, int /*final_buf*/,
                                      cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_finalize_integrate<<<blocks_for(n, 128), 128, 0, st>>>(d.view(), d.s_pos, d.s_vel, d.vel_x,
                                                           d.pred_v, d.s2o, d.sdf, d.p_pos,
                                                           d.p_vel, d.p_force, d.accum);
  return cudaGetLastError();
}

}  // namespace fs
