// adj_kernels.cu — reverse-mode (adjoint) kernels of one SPH step on sm_103a.
//
// The step maps the canonical state (x, v) to (x', v') through the stages of
// sph_3d_grid.rs:1261-1444. Cell assignment and every neighbour set are
// piecewise constant: they are taken from the recorded forward step and not
// differentiated. Each kernel below is the vector-Jacobian product of one
// stage, derived by hand from the forward arithmetic in sph_kernels.cu:
//
//   k_adj_integrate   sph_integrate_3d.wgsl:98-388 (walls, backstop) and
//                     pcisph_finalize.wgsl:57-72, then the first half of the
//                     last PCISPH iteration's reverse (clamp, velocity)
//   k_adj_solve       one PCISPH iteration, pcisph_solve.wgsl:99-208 (the
//                     predicted density and pressure-force pair sums), fused
//                     with the elementwise half of the previous iteration's
//                     reverse, or with pcisph_predict.wgsl:61-72 for level 0
//   k_adj_force       sph_force_3d_grid.wgsl:105-227
//   k_adj_xsph        xsph.wgsl:81-138
//   k_adj_density     sph_density_3d_grid.wgsl:111-194 with boundary_gamma
//   k_adj_to_canonical  the reorder permutation (grid_reorder.wgsl:54-62)
//
// Every pair sum is reversed as a GATHER: the adjoint of particle q collects
// the i-side derivative of each pair (q, j) and the j-side derivative of
// each pair (j, q), evaluating both orientations with the neighbour's own
// recorded inputs and cotangents. No atomics, deterministic. This needs the
// neighbour relation to be symmetric, which holds while every particle's
// cell is inside the grid (clamping breaks it); the kernels check it and set
// ERR_ADJ_OUTSIDE_GRID otherwise.
//
// Per-particle adjoints are FP32; the scalar-parameter gradients (viscosity,
// surface tension, near stiffness, the PCISPH pressure factor delta) are
// summed per particle and reduced per scene in FP64.
#include "adj_internal.h"
#include "sph_device.cuh"

namespace fs {
namespace {

constexpr float MIN_R2 = 1e-12f;  // the shaders' non-self test (r^2 > 1e-12)

__device__ __forceinline__ float3 f3of(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float4 f4(float3 a, float w) { return make_float4(a.x, a.y, a.z, w); }
__device__ __forceinline__ float3 add3(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 mad3(float3 a, float s, float3 b) {  // a + s b
  return f3(a.x + s * b.x, a.y + s * b.y, a.z + s * b.z);
}

// Neighbour runs of the RECORDED step (its cell table) around `pos`; also
// reports whether pos's cell lies inside the grid (neighbour symmetry).
__device__ __forceinline__ bool runs_checked(float3 pos, const GpuGridParams &g,
                                             const uint32_t *begin, Runs &R) {
  const long long cx = __float2int_rd((pos.x - g.grid_origin_x) * g.inv_cell_size);
  const long long cy = __float2int_rd((pos.y - g.grid_origin_y) * g.inv_cell_size);
  const long long cz = __float2int_rd((pos.z - g.grid_origin_z) * g.inv_cell_size);
  neighbor_runs(pos, g, begin, R);
  return cx >= 0 && cy >= 0 && cz >= 0 && cx < (long long)g.grid_size_x &&
         cy < (long long)g.grid_size_y && cz < (long long)g.grid_size_z;
}

// L lanes share one particle's candidate list: lane `sub` of the group takes
// the flat candidate indices congruent to sub mod L. Small particle counts
// leave the GPU latency bound at one particle per lane; splitting each list
// multiplies the warps in flight. Partial sums then combine in a fixed
// butterfly, so the result depends on L but not on the run.
template <int L, class F>
__device__ __forceinline__ void for_candidates_sub(const Runs &R, uint32_t sub, F &&f) {
  uint32_t base = 0;
  for (int r = 0; r < R.count; r++) {
    const uint32_t lo = R.lo[r], hi = R.hi[r];
    const uint32_t first = L == 1 ? lo : lo + (sub + L - base % L) % L;
    for (uint32_t j = first; j < hi; j += L) f(j);
    base += hi - lo;
  }
}
template <int L>
__device__ __forceinline__ float group_sum(float x) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}
template <int L>
__device__ __forceinline__ float3 group_sum3(float3 x) {
  return make_float3(group_sum<L>(x.x), group_sum<L>(x.y), group_sum<L>(x.z));
}
// Tasks of 32 / L slots with L lanes per particle: each 32-slot warp of the
// recorded task order (heaviest first) split L ways, so a heavy warp's
// particles spread over L concurrently running warps and the critical path
// (the heaviest particle's candidate list) shrinks L-fold.
// With a slot permutation (q.slots) the 32 slots of task group t / L are
// perm[32 (t / L) .. 32 (t / L) + 31] (0xffffffff past the end).
template <int L, class F>
__device__ __forceinline__ void for_warp_tasks_sub(const TaskQueue &q, F &&f) {
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t ntasks = q.nwarps * uint32_t(L);
  while (true) {
    uint32_t t = 0u;
    if (lane == 0u) t = atomicAdd(q.counter, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= ntasks) break;
    const uint32_t within = (t % L) * (32u / L) + lane / L;
    uint32_t slot;
    if (q.slots) {
      const uint32_t idx = (t / L) * 32u + within;
      slot = idx < q.n ? __ldg(q.perm + idx) : 0xffffffffu;
    } else {
      slot = __ldg(q.perm + t / L) * 32u + within;
    }
    f(slot, lane % L);
  }
}

// q's in-range neighbours j (1e-12 < r^2 < h^2, the force / XSPH / normal
// criterion): walked from the recorded step's hit mask when q has one (the
// forward's own decisions, no candidate tests), else found by testing the
// candidates. Lane `sub` of q's L lanes takes every L-th mask word (every
// L-th candidate when testing).
template <int L, class InRange, class Body>
__device__ __forceinline__ void for_hits_sub(const Runs &R, const TapeView &t, uint32_t q,
                                             uint32_t sub, InRange &&in_range, Body &&body,
                                             const uint32_t *words = nullptr) {
  const uint32_t off = t.mask_off[q];
  if (off != MASK_NONE) {
    MaskWalk m;
    m.init(R, (words ? words : t.mask_words) + off, sub, uint32_t(L));
    uint32_t j = 0u;
    while (m.next(R, j)) body(j);
  } else {
    for_candidates_sub<L>(R, sub, [&](uint32_t j) {
      if (in_range(j)) body(j);
    });
  }
}

// Reverse of the acceleration clamp |a| <= A (pcisph_solve.wgsl:190-196):
// a = a~ * A / |a~| when |a~|^2 > A^2, whose Jacobian is (A/|a~|)(I - e e^T).
__device__ __forceinline__ float3 clamp_adjoint(float3 a_raw, float3 abar, float max_accel) {
  const float m2 = dot3(a_raw, a_raw);
  if (!(m2 > max_accel * max_accel)) return abar;
  const float m = sqrtf(m2);
  const float3 e = a_raw * (1.0f / m);
  return (abar - e * dot3(e, abar)) * (max_accel / m);
}

__device__ __forceinline__ void flag_outside(uint32_t *err, bool inside) {
  if (!inside) atomicOr(err, ERR_ADJ_OUTSIDE_GRID);
}

// Level k's record of particle s (see AdjView::lv): its predicted position,
// p / max(rho*, 1)^2 and the cotangents u, rhat.
__device__ __forceinline__ void put_level_record(float4 *lv, uint32_t s, const TapeView &t, int k,
                                                 float3 u, float rhat) {
  const float4 x = t.xp[k][s];
  const float rt = fmaxf(t.rho[k][s], 1.0f);
  lv[2 * size_t(s)] = make_float4(x.x, x.y, x.z, x.w / (rt * rt));
  lv[2 * size_t(s) + 1] = f4(u, rhat);
}

// ---- integrate + finalize --------------------------------------------------------
__global__ void __launch_bounds__(128)
    k_adj_integrate(SceneView v, TapeView t, AdjView a, const float4 *__restrict__ xbar_in,
                    const float4 *__restrict__ vbar_in, const float4 *__restrict__ ap_last,
                    int K) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.b->n_sorted) return;
  const DevUniforms *U = v.u + t.scene_of_slot[s];
  const GpuSphParams3D &P = U->sph;
  const GpuContainerGeometry &c = U->geom;
  const uint32_t orig = t.s2o[s];
  const float3 Xb = f3of(xbar_in[orig]);
  const float3 Vb = f3of(vbar_in[orig]);
  // forward recomputation (sph_integrate_3d.wgsl:98-150, 340-388)
  const float3 pos = f3of(t.pos[s]);
  const float3 vf = f3of(t.vfin[s]);
  const float h = P.kernel_radius, dt = P.dt;
  const float bl = h * 0.4f, wd = 8.0f, k_w = c.wall_stiffness;
  const float3 lp = world_to_local(c, pos);
  const float3 lv = world_dir_to_local(c, vf);
  const float lpa[3] = {lp.x, lp.y, lp.z}, lva[3] = {lv.x, lv.y, lv.z};
  const float H[3] = {c.half_width, c.half_height, c.half_depth};
  float wa[3] = {0.f, 0.f, 0.f};
  for (int ax = 0; ax < 3; ax++) {
    float d = lpa[ax] - (-H[ax]);
    if (d < bl) { const float tt = 1.0f - d / bl; wa[ax] += k_w * tt * tt; if (lva[ax] < 0.0f) wa[ax] -= lva[ax] * wd * tt; }
    d = H[ax] - lpa[ax];
    if (d < bl) { const float tt = 1.0f - d / bl; wa[ax] -= k_w * tt * tt; if (lva[ax] > 0.0f) wa[ax] -= lva[ax] * wd * tt; }
  }
  const float3 accel = local_dir_to_world(c, f3(wa[0], wa[1], wa[2]));
  const float3 vel = vf + dt * accel;
  const float3 pos2 = pos + dt * vel;
  const float3 lpn = world_to_local(c, pos2);
  const float3 lvn = world_dir_to_local(c, vel);
  // reverse: out = Rf * clamp(lpn), Rf * reflect(lvn)
  float3 lpn_b = world_dir_to_local(c, Xb);  // Rf^T = Ri (rotation)
  float3 lvn_b = world_dir_to_local(c, Vb);
  float lpb[3] = {lpn_b.x, lpn_b.y, lpn_b.z}, lvb[3] = {lvn_b.x, lvn_b.y, lvn_b.z};
  const float lpna[3] = {lpn.x, lpn.y, lpn.z}, lvna[3] = {lvn.x, lvn.y, lvn.z};
  const float rest = c.damping;
  for (int ax = 0; ax < 3; ax++) {
    const float sg = lvna[ax] > 0.f ? 1.f : (lvna[ax] < 0.f ? -1.f : 0.f);
    if (lpna[ax] < -H[ax]) { lpb[ax] = 0.f; lvb[ax] *= sg * rest; }
    else if (lpna[ax] > H[ax]) { lpb[ax] = 0.f; lvb[ax] *= -sg * rest; }
  }
  const float3 pos2_b = local_dir_to_world(c, f3(lpb[0], lpb[1], lpb[2]));  // Ri^T = Rf
  float3 vel_b = local_dir_to_world(c, f3(lvb[0], lvb[1], lvb[2]));
  float3 xb = pos2_b;
  vel_b = vel_b + dt * pos2_b;
  float3 vfb = vel_b;
  const float3 acc_b = dt * vel_b;
  const float3 wab3 = world_dir_to_local(c, acc_b);
  const float wab[3] = {wab3.x, wab3.y, wab3.z};
  float lpg[3] = {0.f, 0.f, 0.f}, lvg[3] = {0.f, 0.f, 0.f};
  for (int ax = 0; ax < 3; ax++) {
    float d = lpa[ax] - (-H[ax]);
    if (d < bl) {  // d t / d lp = -1/bl
      const float tt = 1.0f - d / bl;
      lpg[ax] += wab[ax] * (-2.0f * k_w * tt / bl);
      if (lva[ax] < 0.0f) { lpg[ax] += wab[ax] * (lva[ax] * wd / bl); lvg[ax] += wab[ax] * (-wd * tt); }
    }
    d = H[ax] - lpa[ax];
    if (d < bl) {  // d t / d lp = +1/bl
      const float tt = 1.0f - d / bl;
      lpg[ax] += wab[ax] * (-2.0f * k_w * tt / bl);
      if (lva[ax] > 0.0f) { lpg[ax] += wab[ax] * (-lva[ax] * wd / bl); lvg[ax] += wab[ax] * (-wd * tt); }
    }
  }
  xb = xb + local_dir_to_world(c, f3(lpg[0], lpg[1], lpg[2]));
  vfb = vfb + local_dir_to_world(c, f3(lvg[0], lvg[1], lvg[2]));
  // finalize: v_fin = v*^K. Elementwise half of the last iteration's reverse:
  // v*^K = vhat + dt (a + clamp(a~p)); its x*, p, rho* outputs are unused.
  const float max_accel = 0.25f * h / (dt * dt);
  const float3 apb = clamp_adjoint(f3of(ap_last[s]), dt * vfb, max_accel);
  a.gx[s] = f4(xb, 0.f);
  a.gvhat[s] = f4(vfb, 0.f);
  a.ga[s] = f4(dt * vfb, 0.f);
  put_level_record(a.lv[(K - 1) & 1], s, t, K - 1, apb, 0.f);
  a.gp[s] = 0.f;
  a.gv[s] = make_float4(0.f, 0.f, 0.f, 0.f);
  a.grho[s] = make_float2(0.f, 0.f);
  a.gn[s] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// ---- one PCISPH iteration (level k) ------------------------------------------------
// Level k's recorded arrays come as arguments (xpk = x*^k with p^k, rhok =
// rho*^k, ap_prev = iteration k-1's pressure acceleration before the clamp);
// lv_in holds level k's records (AdjView::lv), from which the neighbours'
// values are read, and lv_out receives level k-1's.
template <int L>
__device__ __forceinline__ void adj_solve_one(uint32_t q, uint32_t sub, const SceneView &v,
                                              const TapeView &t, const AdjView &a,
                                              const float4 *__restrict__ xpk,
                                              const float *__restrict__ rhok,
                                              const float4 *__restrict__ ap_prev,
                                              const float4 *__restrict__ lv_in,
                                              float4 *__restrict__ lv_out, int k, int K) {
  const bool active = q < v.b->n_sorted;
  const uint32_t qq = active ? q : 0u;
  const DevUniforms *U = v.u + t.scene_of_slot[qq];
  const GpuSphParams3D &P = U->sph;
  const float h = P.kernel_radius, h2 = P.kernel_radius_sq, mass = P.mass, dt = P.dt;
  const float4 xq4 = xpk[qq];
  const float pq = xq4.w;
  const float rho_q = rhok[qq];
  const float rt_q = fmaxf(rho_q, 1.0f);
  float3 xsb = f3(0.f, 0.f, 0.f);
  float phisum = 0.f;  // sum over pairs of m g e.du (pressure terms of p and rho*)
  if (active) {
    const float scale_d = 315.0f / (64.0f * PI_F * P.kernel_radius_pow9);
    const float scale_g = 45.0f / (PI_F * P.kernel_radius_pow6);
    const float3 xq = f3of(xq4);
    const float cq = pq / (rt_q * rt_q);
    const float4 uq4 = lv_in[2 * size_t(q) + 1];
    const float3 uq = f3of(uq4);
    const float rhat_q = uq4.w;
    const bool has_rho = k < K - 1;  // level K's density and pressure are unused
    const bool has_p = k >= 1;       // level 0 holds zero pressures
    Runs R;
    flag_outside(a.err, runs_checked(f3of(t.pos[q]), U->grid, t.cell_begin + U->c_offset, R));
    const float c_rho = -6.0f * mass * scale_d;
    // the level's in-range pairs (r^2 < h^2 at the predicted positions):
    // walked from the union of the levels' recorded masks, each pair kept
    // where it is in range at this level (selects keep the lanes together)
    for_hits_sub<L>(
        R, t, q, sub,
        [&](uint32_t j) {
          const float3 r = xq - f3of(__ldg(lv_in + 2 * size_t(j)));
          return dot3(r, r) < h2;
        },
        [&](uint32_t j) {
          const float4 xj4 = __ldg(lv_in + 2 * size_t(j));  // x*_j, c_j
          const float3 r = xq - f3of(xj4);
          const float r2 = dot3(r, r);
          const bool in = r2 < h2;
          const float4 uj4 = __ldg(lv_in + 2 * size_t(j) + 1);
          if (has_rho) {
            const float diff = h2 - r2;
            xsb = in ? mad3(xsb, c_rho * diff * diff * (rhat_q + uj4.w), r) : xsb;
          }
          if (has_p) {
            // evaluated for every hit, kept for 1e-12 < r^2 < h^2
            const bool ns = in && r2 > MIN_R2;
            const float cij = cq + xj4.w;
            const float rr = sqrtf(ns ? r2 : 1.0f);
            const float inv_rr = 1.0f / rr;
            const float3 e = r * inv_rr;
            const float dg = h - rr;
            const float g = scale_g * dg * dg;
            const float gp = -2.0f * scale_g * dg;
            const float3 du = uq - f3of(uj4);
            const float edu = dot3(e, du);
            // J du = g' (e.du) e + (g / r)(du - (e.du) e)
            const float3 Jdu = e * (gp * edu) + (du - e * edu) * (g * inv_rr);
            xsb = ns ? mad3(xsb, mass * cij, Jdu) : xsb;
            phisum += ns ? mass * g * edu : 0.0f;
          }
        },
        t.hits);
  }
  xsb = group_sum3<L>(xsb);
  phisum = group_sum<L>(phisum);
  if (!active || sub != 0u) return;
  const float pb = phisum / (rt_q * rt_q);
  const float rb = rho_q > 1.0f ? (-2.0f * pq / (rt_q * rt_q * rt_q)) * phisum : 0.0f;
  const float p_bar = a.gp[q] + pb;  // p^{k+1} = p^k + ...: identity part
  const float3 vstar_b = dt * xsb;   // x*^k = x + dt v*^k
  a.gx[q] = f4(add3(f3of(a.gx[q]), xsb), 0.f);
  a.gvhat[q] = f4(add3(f3of(a.gvhat[q]), vstar_b), 0.f);
  a.ga[q] = f4(add3(f3of(a.ga[q]), dt * vstar_b), 0.f);
  if (k >= 1) {
    // elementwise half of iteration k-1's reverse: its outputs are level k
    const float max_accel = 0.25f * h / (dt * dt);
    const float3 apb = clamp_adjoint(f3of(ap_prev[q]), dt * vstar_b, max_accel);
    const float rhat = rb + (rho_q > P.rest_density ? P.pcisph_delta * p_bar : 0.0f);
    put_level_record(lv_out, q, t, k - 1, apb, rhat);
    a.gp[q] = p_bar;
    // p^k = p^(k-1) + delta max(0, rho*^k - rho0): the particle's share of
    // d/d delta at this level (pcisph_solve.wgsl's density_error)
    const float density_error = fmaxf(0.0f, rho_q - P.rest_density);
    a.gpart2[t.s2o[q]].y += double(p_bar) * double(density_error);
  }
  // k == 0: predict, x*^0 = x + dt v*^0, v*^0 = vhat + dt a (done above);
  // the non-pressure acceleration's cotangent is final: the force reverse's
  // record of q
  if (k == 0) {
    const float2 d = t.dens[q];
    float4 *fr = a.frec + 5 * size_t(q);
    fr[0] = f4(f3of(t.pos[q]), fmaxf(d.x, 1.0f));
    fr[1] = f4(f3of(t.vhat[q]), fmaxf(d.y, 1.0f));
    fr[2] = t.vel[q];
    fr[3] = t.nrm[q];
    fr[4] = a.ga[q];
  }
}

template <int L>
__global__ void __launch_bounds__(128)
    k_adj_solve(TaskQueue tq, SceneView v, TapeView t, AdjView a, const float4 *__restrict__ xpk,
                const float *__restrict__ rhok, const float4 *__restrict__ ap_prev,
                const float4 *__restrict__ lv_in, float4 *__restrict__ lv_out, int k, int K) {
  for_warp_tasks_sub<L>(tq, [&](uint32_t q, uint32_t sub) {
    adj_solve_one<L>(q, sub, v, t, a, xpk, rhok, ap_prev, lv_in, lv_out, k, K);
  });
}

// ---- force (non-pressure acceleration) -----------------------------------------------
struct ForceConst {
  float h, mass, scale_g, scale_c, near_k, visc, rho0, st, min_dist, eps_h2, h_half, h6_64,
      sep_k;
};
__device__ __forceinline__ ForceConst force_const(const GpuSphParams3D &P) {
  ForceConst c;
  c.h = P.kernel_radius;
  c.mass = P.mass;
  c.scale_g = 45.0f / (PI_F * P.kernel_radius_pow6);
  c.scale_c = 32.0f / (PI_F * P.kernel_radius_pow9);
  c.near_k = P.near_stiffness;
  c.visc = P.viscosity;
  c.rho0 = P.rest_density;
  c.st = P.surface_tension;
  c.min_dist = c.h * 0.1f;
  c.eps_h2 = 0.01f * P.kernel_radius_sq;
  c.h_half = c.h * 0.5f;
  c.h6_64 = P.kernel_radius_pow6 / 64.0f;
  c.sep_k = 200.0f / c.min_dist;
  return c;
}

// One particle of a force pair: recorded inputs with the density clamps of
// sph_force_3d_grid.wgsl (max(rho, 1)) and their derivative masks.
struct ForceSide {
  float3 x, vhat, vpre, n;
  float rb, rnb;  // max(rho, 1), max(rho_near, 1)
  bool m, mn;     // rho > 1, rho_near > 1
};
// Geometry shared by both orientations of a pair, r = x_q - x_j.
struct PairGeom {
  float3 r, u;  // u = r / |r|
  float r2, rr, inv_rr, dg, G, Gp, D, C, Cp;
  bool close;
};
__device__ __forceinline__ PairGeom pair_geom(float3 r, float r2, const ForceConst &c) {
  PairGeom g;
  g.r = r;
  g.r2 = r2;
  g.rr = sqrtf(r2);
  g.inv_rr = 1.0f / g.rr;
  g.u = r * g.inv_rr;
  g.close = g.rr < c.min_dist;
  g.dg = c.h - g.rr;
  const float dg2 = g.dg * g.dg, dg3 = dg2 * g.dg;
  g.G = c.scale_g * dg2;
  g.Gp = -2.0f * c.scale_g * g.dg;
  g.D = r2 + c.eps_h2;
  const float r3 = g.rr * r2;
  const bool far_c = g.rr >= c.h_half;
  g.C = far_c ? c.scale_c * dg3 * r3 : c.scale_c * (2.0f * dg3 * r3 - c.h6_64);
  g.Cp = (far_c ? 1.0f : 2.0f) * c.scale_c * (-3.0f * dg2 * r3 + 3.0f * dg3 * r2);
  return g;
}

struct ForceAcc {
  float3 gx, gvh, gv, gn;
  float grho, grhon, sv, ss, sn;
};

// w . T_{i<-j} reversed (T from sph_force_3d_grid.wgsl:127-220, forward in
// force_predict_one), accumulated into particle q's adjoints. JSIDE = false:
// q is i (the pair (q, j) with q's cotangent w = abar_q; q's i-side
// derivatives and the parameter gradients); JSIDE = true: q is j (the pair
// (j, q) with w = abar_j; q's j-side derivatives). e_close is the pair's
// tabulated fallback direction (constant in the positions); the cohesion
// part is scaled by the surface tension as in the forward (a_c *= st).
template <bool JSIDE>
__device__ __forceinline__ void force_half(const ForceSide &I, const ForceSide &J,
                                           const PairGeom &g, float3 w, float3 e_close,
                                           const ForceConst &c, ForceAcc &acc) {
  // every branch of the forward is evaluated and the sums are updated with
  // selects, so the lanes of a warp stay together through the pair
  const float3 zero = f3(0.f, 0.f, 0.f);
  const float3 r_ij = JSIDE ? -g.r : g.r;
  const float3 u_ij = JSIDE ? -g.u : g.u;
  const float3 e = g.close ? e_close : -u_ij;
  const float we = dot3(w, e);
  const float3 dwe = g.close ? zero : (w - e * we) * (-g.inv_rr);
  // near pressure: alpha G e
  const float Pn_i = c.near_k * I.rnb, Pn_j = c.near_k * J.rnb;
  const float inv2 = 1.0f / (2.0f * I.rb * J.rnb);
  const float alpha = -c.mass * (Pn_i + Pn_j) * inv2;
  float3 g_r = (u_ij * (g.Gp * we) + dwe * g.G) * alpha;
  const float Gwe = g.G * we;
  if (!JSIDE) {
    acc.grho += I.m ? (-alpha / I.rb) * Gwe : 0.0f;
    acc.grhon += I.mn ? (-c.mass * c.near_k * inv2) * Gwe : 0.0f;
    // d alpha / d near_stiffness = -m (rho_near_i + rho_near_j) / (2 rho_i rho_near_j)
    acc.sn += (-c.mass * (I.rnb + J.rnb) * inv2) * Gwe;
  } else {
    acc.grhon += J.mn ? (c.mass * Pn_i * inv2 / J.rnb) * Gwe : 0.0f;
  }
  // separation (close pairs): -200 (1 - r / min_dist) e
  g_r = g_r + (g.close ? u_ij * (c.sep_k * we) : zero);
  // viscosity where v_ij . x_ij < 0: beta G e, beta = m visc h vdx / (D avg)
  const float3 vij = I.vhat - J.vpre;
  const float vdx = dot3(vij, r_ij);
  const bool vis = vdx < 0.0f;
  const float avg = (I.rb + J.rb) * 0.5f;
  const float inv_Davg = 1.0f / (g.D * avg);
  const float bG = c.mass * c.h * vdx * inv_Davg;
  const float beta = c.visc * bG * g.G;
  const float dbdv = c.visc * c.mass * c.h * g.G * inv_Davg;
  const float3 g_vis = (vij * dbdv + u_ij * (c.visc * bG * g.Gp) - r_ij * (2.0f * beta / g.D)) * we +
                       dwe * beta;
  g_r = g_r + (vis ? g_vis : zero);
  const float drho = -beta / (2.0f * avg) * we;
  if (!JSIDE) {
    acc.gvh = acc.gvh + (vis ? r_ij * (we * dbdv) : zero);
    acc.grho += (vis && I.m) ? drho : 0.0f;
    acc.sv += vis ? bG * Gwe : 0.0f;
  } else {
    acc.gv = acc.gv + (vis ? r_ij * (-we * dbdv) : zero);
    acc.grho += (vis && J.m) ? drho : 0.0f;
  }
  // cohesion, scaled by st: m K C e - m K (n_i - n_j)
  const float3 wc = w * c.st;
  const float wce = dot3(wc, e);
  const float3 dwce = g.close ? zero : (wc - e * wce) * (-g.inv_rr);
  const float rs = I.rb + J.rb;
  const float Kij = 2.0f * c.rho0 / rs;
  const float mK = c.mass * Kij;
  g_r = g_r + (u_ij * (g.Cp * wce) + dwce * g.C) * mK;
  const float3 nij = I.n - J.n;
  const float dKterm = (-Kij / rs) * (c.mass * g.C * wce - c.mass * dot3(wc, nij));
  if (!JSIDE) {
    acc.gn = acc.gn + wc * (-mK);
    acc.grho += I.m ? dKterm : 0.0f;
    acc.ss += mK * g.C * we - mK * dot3(w, nij);
    acc.gx = acc.gx + g_r;
  } else {
    acc.gn = acc.gn + wc * mK;
    acc.grho += J.m ? dKterm : 0.0f;
    acc.gx = acc.gx - g_r;
  }
}

__device__ __forceinline__ float3 close_dir(const float4 *dir_tab, int dir_half, uint32_t si,
                                            uint32_t sj, uint32_t s_off) {
  const int d = int(si) - int(sj);
  if (d >= -dir_half && d <= dir_half) return f3of(__ldg(dir_tab + d + dir_half));
  return fallback_dir_eval(float(si - s_off) - float(sj - s_off));
}

// Particle i's side from its record (AdjView::frec); rho > 1 exactly when
// max(rho, 1) > 1. w receives its cotangent of the non-pressure acceleration.
__device__ __forceinline__ ForceSide force_side(const float4 *frec, uint32_t i, float3 &w) {
  const float4 *fr = frec + 5 * size_t(i);
  const float4 r0 = __ldg(fr), r1 = __ldg(fr + 1), r2 = __ldg(fr + 2), r3 = __ldg(fr + 3),
               r4 = __ldg(fr + 4);
  ForceSide S;
  S.x = f3of(r0);
  S.vhat = f3of(r1);
  S.vpre = f3of(r2);
  S.n = f3of(r3);
  S.rb = r0.w;
  S.rnb = r1.w;
  S.m = r0.w > 1.0f;
  S.mn = r1.w > 1.0f;
  w = f3of(r4);
  return S;
}

template <int L>
__device__ __forceinline__ void adj_force_one(uint32_t q, uint32_t sub, const SceneView &v,
                                              const TapeView &t, const AdjView &a,
                                              const float4 *dir_tab, int dir_half) {
  const bool active = q < v.b->n_sorted;
  const uint32_t scene = active ? t.scene_of_slot[q] : 0u;
  (void)scene;
  ForceAcc acc;
  acc.gx = acc.gvh = acc.gv = acc.gn = f3(0.f, 0.f, 0.f);
  acc.grho = acc.grhon = acc.sv = acc.ss = acc.sn = 0.f;
  if (active) {
    const DevUniforms *U = v.u + scene;
    const ForceConst c = force_const(U->sph);
    const float h2 = U->sph.kernel_radius_sq;
    float3 wq;
    const ForceSide Q = force_side(a.frec, q, wq);
    Runs R;
    flag_outside(a.err, runs_checked(Q.x, U->grid, t.cell_begin + U->c_offset, R));
    for_hits_sub<L>(
        R, t, q, sub,
        [&](uint32_t j) {
          const float3 r = Q.x - f3of(__ldg(t.pos + j));
          const float r2 = dot3(r, r);
          return r2 < h2 && r2 > MIN_R2;
        },
        [&](uint32_t j) {
          float3 wj;
          const ForceSide Jn = force_side(a.frec, j, wj);
          const float3 r = Q.x - Jn.x;
          const float r2 = dot3(r, r);
          const PairGeom g = pair_geom(r, r2, c);
          float3 ec_qj = f3(0.f, 0.f, 0.f), ec_jq = f3(0.f, 0.f, 0.f);
          if (g.close) {
            ec_qj = close_dir(dir_tab, dir_half, q, j, U->s_offset);
            ec_jq = close_dir(dir_tab, dir_half, j, q, U->s_offset);
          }
          force_half<false>(Q, Jn, g, wq, ec_qj, c, acc);
          force_half<true>(Jn, Q, g, wj, ec_jq, c, acc);
        });
  }
  acc.sv = group_sum<L>(acc.sv);
  acc.ss = group_sum<L>(acc.ss);
  acc.sn = group_sum<L>(acc.sn);
  acc.gx = group_sum3<L>(acc.gx);
  acc.gvh = group_sum3<L>(acc.gvh);
  acc.gv = group_sum3<L>(acc.gv);
  acc.gn = group_sum3<L>(acc.gn);
  acc.grho = group_sum<L>(acc.grho);
  acc.grhon = group_sum<L>(acc.grhon);
  if (!active || sub != 0u) return;
  a.gx[q] = f4(add3(f3of(a.gx[q]), acc.gx), 0.f);
  a.gvhat[q] = f4(add3(f3of(a.gvhat[q]), acc.gvh), 0.f);
  a.gv[q] = f4(acc.gv, 0.f);
  a.grho[q] = make_float2(acc.grho, acc.grhon);
  a.gn[q] = f4(acc.gn, 0.f);
  // the particle's share of d/d viscosity, d/d surface tension and d/d near
  // stiffness, summed over steps in canonical order (FP64), reduced per
  // scene at the end
  const uint32_t o = t.s2o[q];
  double2 &gp = a.gpart[o];
  gp = make_double2(gp.x + double(acc.sv), gp.y + double(acc.ss));
  a.gpart2[o].x += double(acc.sn);
}

template <int L>
__global__ void __launch_bounds__(128)
    k_adj_force(TaskQueue tq, SceneView v, TapeView t, AdjView a, const float4 *__restrict__ dir_tab,
                int dir_half) {
  for_warp_tasks_sub<L>(tq, [&](uint32_t q, uint32_t sub) {
    adj_force_one<L>(q, sub, v, t, a, dir_tab, dir_half);
  });
}

// ---- XSPH -------------------------------------------------------------------------
template <int L>
__device__ __forceinline__ void adj_xsph_one(uint32_t q, uint32_t sub, const SceneView &v,
                                             const TapeView &t, const AdjView &a) {
  const bool active = q < v.b->n_sorted;
  const uint32_t qq = active ? q : 0u;
  const DevUniforms *U = v.u + t.scene_of_slot[qq];
  const GpuSphParams3D &P = U->sph;
  const float h2 = P.kernel_radius_sq, mass = P.mass, eps = P.xsph_epsilon;
  const float3 xq = f3of(t.pos[qq]);
  const float rho_q = t.dens[qq].x;
  const float3 wq = f3of(a.gvhat[qq]);
  float3 gvp = f3(0.f, 0.f, 0.f), gx = f3(0.f, 0.f, 0.f);
  float grhop = 0.f;
  if (active && eps > 0.0f) {
    const float scale_d = 315.0f / (64.0f * PI_F * P.kernel_radius_pow9);
    const float3 vq = f3of(t.vel[q]);
    const float rb_q = fmaxf(rho_q, 1.0f);
    const float fq = eps * mass / rb_q;
    const float grho_k = rho_q > 1.0f ? -eps * mass / (rb_q * rb_q) : 0.0f;
    Runs R;
    flag_outside(a.err, runs_checked(xq, U->grid, t.cell_begin + U->c_offset, R));
    auto in_range = [&](uint32_t j) {
      const float3 r = xq - f3of(__ldg(t.pos + j));
      const float r2 = dot3(r, r);
      return r2 < h2 && r2 > MIN_R2;
    };
    for_hits_sub<L>(R, t, q, sub, in_range, [&](uint32_t j) {
      const float3 xj = f3of(__ldg(t.pos + j));
      const float3 r = xq - xj;  // r_qj
      const float r2 = dot3(r, r);
      const float diff = h2 - r2;
      const float W = scale_d * diff * diff * diff;
      const float dWs = -6.0f * scale_d * diff * diff;  // dW/dr = dWs * r
      const float3 vj = f3of(__ldg(t.vel + j));
      const float fj = eps * mass / fmaxf(__ldg(&t.dens[j].x), 1.0f);
      const float3 wj = f3of(__ldg(a.gvhat + j));
      const float3 dv = vj - vq;
      // (A) term_{q<-j} = fj W (v_j - v_q) with wq; (B) term_{j<-q} = fq W (v_q - v_j) with wj
      gvp = gvp + (wj * fq - wq * fj) * W;
      const float wdv = -dot3(wj, dv);
      grhop += grho_k * W * wdv;
      gx = gx + r * ((fj * dot3(wq, dv) + fq * wdv) * dWs);
    });
  }
  gvp = group_sum3<L>(gvp);
  gx = group_sum3<L>(gx);
  grhop = group_sum<L>(grhop);
  if (!active || sub != 0u) return;
  a.gv[q] = f4(add3(add3(f3of(a.gv[q]), wq), gvp), 0.f);  // vhat = v + eps * sum
  const float grho = a.grho[q].x + grhop;
  // rho = rho_raw / gamma: store the raw density's cotangent and fold the
  // gamma derivative here (d gamma / d x is local to q)
  const GpuContainerGeometry &c = U->geom;
  const float h = P.kernel_radius;
  const float3 l = world_to_local(c, xq);
  const float dw[6] = {l.x + c.half_width, c.half_width - l.x, l.y + c.half_height,
                       c.half_height - l.y, l.z + c.half_depth, c.half_depth - l.z};
  float fw[6], prod = 1.0f;
#pragma unroll
  for (int w = 0; w < 6; w++) {
    fw[w] = dw[w] < h ? 0.5f + 0.5f * clampf(dw[w] / h, 0.0f, 1.0f) : 1.0f;
    prod *= fw[w];
  }
  const float gamma_q = fmaxf(prod, 0.1f);
  const float rb_raw = grho / gamma_q;
  a.grho[q] = make_float2(rb_raw, a.grho[q].y);
  if (prod > 0.1f && grho != 0.0f) {
    const float gamma_b = -rb_raw * rho_q;  // d rho / d gamma = -rho_raw / gamma^2
    float lg[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int w = 0; w < 6; w++) {
      if (!(dw[w] < h && dw[w] > 0.0f)) continue;  // clamp saturated or inactive
      float others = 1.0f;
#pragma unroll
      for (int o = 0; o < 6; o++)
        if (o != w) others *= fw[o];
      lg[w >> 1] += gamma_b * others * (0.5f / h) * ((w & 1) ? -1.0f : 1.0f);
    }
    gx = gx + local_dir_to_world(c, f3(lg[0], lg[1], lg[2]));  // Ri^T
  }
  a.gx[q] = f4(add3(f3of(a.gx[q]), gx), 0.f);
}

template <int L>
__global__ void __launch_bounds__(128) k_adj_xsph(TaskQueue tq, SceneView v, TapeView t, AdjView a) {
  for_warp_tasks_sub<L>(tq, [&](uint32_t q, uint32_t sub) { adj_xsph_one<L>(q, sub, v, t, a); });
}

// ---- density, near density, normal ------------------------------------------------------
template <int L>
__device__ __forceinline__ void adj_density_one(uint32_t q, uint32_t sub, const SceneView &v,
                                                const TapeView &t, const AdjView &a) {
  const bool active = q < v.b->n_sorted;
  float3 gx = f3(0.f, 0.f, 0.f);
  if (active) {
    const DevUniforms *U = v.u + t.scene_of_slot[q];
    const GpuSphParams3D &P = U->sph;
    const float h = P.kernel_radius, h2 = P.kernel_radius_sq, mass = P.mass;
    const float scale_d = 315.0f / (64.0f * PI_F * P.kernel_radius_pow9);
    const float scale_n = 15.0f / (PI_F * P.kernel_radius_pow6);
    const float h8 = P.kernel_radius_pow6 * h * h;
    const float cnorm = 945.0f / (32.0f * PI_F * h8) * (mass / P.rest_density);
    const float c_rho = -6.0f * mass * scale_d, c_near = -3.0f * mass * scale_n;
    const float3 xq = f3of(t.pos[q]);
    const float2 gq = a.grho[q];
    const float3 nq = f3of(a.gn[q]);
    Runs R;
    flag_outside(a.err, runs_checked(xq, U->grid, t.cell_begin + U->c_offset, R));
    auto in_range = [&](uint32_t j) {
      const float3 r = xq - f3of(__ldg(t.pos + j));
      const float r2 = dot3(r, r);
      return r2 < h2 && r2 > MIN_R2;
    };
    for_hits_sub<L>(R, t, q, sub, in_range, [&](uint32_t j) {
      const float3 xj = f3of(__ldg(t.pos + j));
      const float3 r = xq - xj;  // r_qj; the pair (j, q) has r_jq = -r
      const float r2 = dot3(r, r);
      const float2 gj = __ldg(a.grho + j);
      const float3 nj = f3of(__ldg(a.gn + j));
      const float diff = h2 - r2;
      const float rr = sqrtf(r2);
      const float dn = h - rr;
      // d/dr_qj of q's terms minus d/dr_jq of j's terms (both odd in r except
      // the normal's, which is even): the radial parts add, the normal parts
      // subtract
      const float radial =
          c_rho * diff * diff * (gq.x + gj.x) + c_near * dn * dn * (gq.y + gj.y) / rr;
      const float3 dnrm = nq - nj;
      gx = gx + r * radial + (dnrm * (diff * diff) - r * (4.0f * diff * dot3(dnrm, r))) * cnorm;
    });
  }
  gx = group_sum3<L>(gx);
  if (!active || sub != 0u) return;
  a.gx[q] = f4(add3(f3of(a.gx[q]), gx), 0.f);
}

template <int L>
__global__ void __launch_bounds__(128) k_adj_density(TaskQueue tq, SceneView v, TapeView t, AdjView a) {
  for_warp_tasks_sub<L>(tq, [&](uint32_t q, uint32_t sub) { adj_density_one<L>(q, sub, v, t, a); });
}

// ---- back to canonical order ---------------------------------------------------------------
__global__ void __launch_bounds__(256)
    k_adj_to_canonical(SceneView v, TapeView t, AdjView a, float4 *__restrict__ xbar_out,
                       float4 *__restrict__ vbar_out) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.b->n_sorted) return;
  const uint32_t orig = t.s2o[s];
  xbar_out[orig] = a.gx[s];
  vbar_out[orig] = a.gv[s];
}

// ---- the density-splat MSE loss ---------------------------------------------------------------
// L = (1/V) sum_v (rho_v - target_v)^2 over the V voxels; gg_v = dL/drho_v /
// gamma_v (0 for clipped voxels). The loss sums in FP64 in a fixed order:
// a shared-memory tree per block, then k_sum_partials over the blocks.
__global__ void __launch_bounds__(256)
    k_splat_mse(SplatArgs sa, const float *__restrict__ field, const float *__restrict__ target,
                float *__restrict__ gg, double *__restrict__ partial) {
  const uint32_t gs = sa.mc.grid_size;
  const uint32_t nvox = gs * gs * gs;
  const uint32_t vx = blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (vx < nvox) {
    const float d = field[vx] - target[vx];
    l = double(d) * double(d);
    const uint32_t x = vx % gs, y = (vx / gs) % gs, z = vx / (gs * gs);
    const float cs = sa.mc.cell_size;
    const float3 wp = f3(sa.mc.grid_min[0] + (float(x) + 0.5f) * cs,
                         sa.mc.grid_min[1] + (float(y) + 0.5f) * cs,
                         sa.mc.grid_min[2] + (float(z) + 0.5f) * cs);
    const GpuContainerGeometry &c = sa.geom;
    const float3 lo = world_to_local(c, wp);
    const bool clipped =
        c.clip_enabled != 0u &&
        !(lo.x >= -c.half_width && lo.x <= c.half_width && lo.y >= -c.half_height &&
          lo.y <= c.half_height && lo.z >= -c.half_depth && lo.z <= c.half_depth);
    float gamma = 1.0f;
    const float h = sa.mc.kernel_radius;
    const float dd[5] = {lo.x + c.half_width, c.half_width - lo.x, lo.y + c.half_height,
                         lo.z + c.half_depth, c.half_depth - lo.z};
    for (int w = 0; w < 5; w++)
      if (dd[w] < h) gamma *= 0.5f + 0.5f * clampf(dd[w] / h, 0.0f, 1.0f);
    gamma = fmaxf(gamma, 0.15f);
    gg[vx] = clipped ? 0.0f : (2.0f * d / float(nvox)) / gamma;
  }
  __shared__ double part[256];
  part[threadIdx.x] = l / double(nvox);
  __syncthreads();
  for (unsigned o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = part[0];
}

// out = sum of n partials, fixed order (one block).
__global__ void __launch_bounds__(1024)
    k_sum_partials(const double *__restrict__ partial, uint32_t n, double *__restrict__ out) {
  __shared__ double part[1024];
  double acc = 0.0;
  for (uint32_t i = threadIdx.x; i < n; i += 1024u) acc += partial[i];
  part[threadIdx.x] = acc;
  __syncthreads();
  for (unsigned o = 512; o > 0; o >>= 1) {
    if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = part[0];
}

// dL/dx_j = sum_v gg_v * 6 coeff (h^2 - r^2)^2 (w_v - x_j), over the voxels
// within the splat radius of particle j (canonical order).
__global__ void __launch_bounds__(128)
    k_splat_adjoint(SplatArgs sa, uint32_t n, const float4 *__restrict__ pos,
                    const float *__restrict__ gg, float4 *__restrict__ xbar) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float3 x = f3of(pos[i]);
  const float h = sa.mc.kernel_radius, h2 = h * h, cs = sa.mc.cell_size;
  const int gs = int(sa.mc.grid_size);
  int lo[3], hi[3];
  const float xa[3] = {x.x, x.y, x.z};
  for (int ax = 0; ax < 3; ax++) {
    const float g0 = sa.mc.grid_min[ax];
    lo[ax] = max(0, int(floorf((xa[ax] - h - g0) / cs - 0.5f)));
    hi[ax] = min(gs - 1, int(ceilf((xa[ax] + h - g0) / cs - 0.5f)));
  }
  float3 g = f3(0.f, 0.f, 0.f);
  for (int z = lo[2]; z <= hi[2]; z++)
    for (int y = lo[1]; y <= hi[1]; y++)
      for (int xx = lo[0]; xx <= hi[0]; xx++) {
        const float3 wp = f3(sa.mc.grid_min[0] + (float(xx) + 0.5f) * cs,
                             sa.mc.grid_min[1] + (float(y) + 0.5f) * cs,
                             sa.mc.grid_min[2] + (float(z) + 0.5f) * cs);
        const float3 d = wp - x;
        const float r2 = dot3(d, d);
        if (!(r2 < h2)) continue;
        const float diff = h2 - r2;
        const float w = __ldg(gg + size_t(xx) + size_t(gs) * (size_t(y) + size_t(gs) * z));
        g = mad3(g, w * 6.0f * sa.coeff * diff * diff, d);
      }
  xbar[i] = f4(g, 0.f);
}

// Per-scene sums of the particles' parameter-gradient shares in a fixed
// order: one block per scene, strided partial sums then a shared-memory tree.
__global__ void __launch_bounds__(256)
    k_reduce_params(const double2 *__restrict__ gpart, const double2 *__restrict__ gpart2,
                    const uint32_t *__restrict__ scene_first,
                    const uint32_t *__restrict__ scene_count, double *__restrict__ gparam,
                    double *__restrict__ gparam2) {
  __shared__ double sv[256], ss[256], sn[256], sd[256];
  const uint32_t sc = blockIdx.x;
  const uint32_t first = scene_first[sc], count = scene_count[sc];
  double v = 0.0, w = 0.0, x = 0.0, y = 0.0;
  for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) {
    const double2 g = gpart[first + i];
    const double2 g2 = gpart2[first + i];
    v += g.x;
    w += g.y;
    x += g2.x;
    y += g2.y;
  }
  sv[threadIdx.x] = v;
  ss[threadIdx.x] = w;
  sn[threadIdx.x] = x;
  sd[threadIdx.x] = y;
  __syncthreads();
  for (unsigned o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sv[threadIdx.x] += sv[threadIdx.x + o];
      ss[threadIdx.x] += ss[threadIdx.x + o];
      sn[threadIdx.x] += sn[threadIdx.x + o];
      sd[threadIdx.x] += sd[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    gparam[3 * sc + 0] = sv[0];
    gparam[3 * sc + 1] = 0.0;  // stiffness: read by no stage of the step
    gparam[3 * sc + 2] = ss[0];
    gparam2[2 * sc + 0] = sn[0];
    gparam2[2 * sc + 1] = sd[0];
  }
}

// (N, 3) float rows <-> float4 records (w = 0)
__global__ void __launch_bounds__(256)
    k_rows_to_f4(uint32_t n, const float *__restrict__ rows, float4 *__restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_float4(rows[3 * size_t(i)], rows[3 * size_t(i) + 1], rows[3 * size_t(i) + 2], 0.f);
}
__global__ void __launch_bounds__(256)
    k_f4_to_rows(uint32_t n, const float4 *__restrict__ in, float *__restrict__ rows) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 x = in[i];
  rows[3 * size_t(i)] = x.x;
  rows[3 * size_t(i) + 1] = x.y;
  rows[3 * size_t(i) + 2] = x.z;
}

inline unsigned blocks_for(uint32_t n, unsigned threads) { return (n + threads - 1) / threads; }

}  // namespace

cudaError_t launch_reduce_params(const double2 *gpart, const double2 *gpart2,
                                 const uint32_t *scene_first, const uint32_t *scene_count,
                                 uint32_t scenes, double *gparam, double *gparam2,
                                 cudaStream_t st) {
  if (scenes == 0) return cudaSuccess;
  k_reduce_params<<<scenes, 256, 0, st>>>(gpart, gpart2, scene_first, scene_count, gparam,
                                          gparam2);
  return cudaGetLastError();
}

cudaError_t launch_rows_to_f4(uint32_t n, const float *rows, float4 *out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_rows_to_f4<<<blocks_for(n, 256), 256, 0, st>>>(n, rows, out);
  return cudaGetLastError();
}
cudaError_t launch_f4_to_rows(uint32_t n, const float4 *in, float *rows, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_f4_to_rows<<<blocks_for(n, 256), 256, 0, st>>>(n, in, rows);
  return cudaGetLastError();
}

template <class K>
unsigned resident_blocks(K kernel, int sm_count) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0) != cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  return unsigned(per_sm * sm_count);
}

namespace {
template <int L>
struct AdjBlocks {
  unsigned solve = 0, force = 0, xsph = 0, density = 0;
};

template <int L>
cudaError_t adj_gathers(const SceneView &v, const TapeView &t, const AdjView &a,
                        const float4 *dir_tab, int dir_half, uint32_t n, int K, int sm_count,
                        cudaStream_t st) {
  static AdjBlocks<L> b;
  if (!b.solve) {
    b.solve = resident_blocks(k_adj_solve<L>, sm_count);
    b.force = resident_blocks(k_adj_force<L>, sm_count);
    b.xsph = resident_blocks(k_adj_xsph<L>, sm_count);
    b.density = resident_blocks(k_adj_density<L>, sm_count);
  }
  const uint32_t nwarps = (n + 31u) / 32u;
  // the force reverse (long per-hit body) takes the hit-sorted slots, so its
  // lanes finish together; the others (short bodies) keep the recorded warp
  // order, whose neighbouring particles share their neighbours' loads in L1
  auto queue = [&](int slot) { return TaskQueue{t.order, a.counters + slot, n, nwarps, false}; };
  auto hit_queue = [&](int slot) {
    return TaskQueue{t.perm_hit, a.counters + slot, n, nwarps, true};
  };
  for (int k = K - 1; k >= 0; k--)
    k_adj_solve<L><<<b.solve, 128, 0, st>>>(queue(k), v, t, a, t.xp[k], t.rho[k],
                                            k >= 1 ? t.ap[k - 1] : nullptr, a.lv[k & 1],
                                            a.lv[(k + 1) & 1], k, K);
  k_adj_force<L><<<b.force, 128, 0, st>>>(hit_queue(K), v, t, a, dir_tab, dir_half);
  k_adj_xsph<L><<<b.xsph, 128, 0, st>>>(queue(K + 1), v, t, a);
  k_adj_density<L><<<b.density, 128, 0, st>>>(queue(K + 2), v, t, a);
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_adj_step(const SceneView &v, const TapeView &t, const AdjView &a,
                            const float4 *xbar_in, const float4 *vbar_in, float4 *xbar_out,
                            float4 *vbar_out, const float4 *dir_tab, int dir_half, uint32_t n,
                            int K, int lanes, int sm_count, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  // one task counter per gather launch: K solves, force, XSPH, density
  cudaError_t e = cudaMemsetAsync(a.counters, 0, sizeof(uint32_t) * (K + 3), st);
  if (e != cudaSuccess) return e;
  k_adj_integrate<<<blocks_for(n, 128), 128, 0, st>>>(v, t, a, xbar_in, vbar_in, t.ap[K - 1], K);
  switch (lanes) {
    case 8: e = adj_gathers<8>(v, t, a, dir_tab, dir_half, n, K, sm_count, st); break;
    case 4: e = adj_gathers<4>(v, t, a, dir_tab, dir_half, n, K, sm_count, st); break;
    case 2: e = adj_gathers<2>(v, t, a, dir_tab, dir_half, n, K, sm_count, st); break;
    default: e = adj_gathers<1>(v, t, a, dir_tab, dir_half, n, K, sm_count, st); break;
  }
  if (e != cudaSuccess) return e;
  k_adj_to_canonical<<<blocks_for(n, 256), 256, 0, st>>>(v, t, a, xbar_out, vbar_out);
  return cudaGetLastError();
}

cudaError_t launch_splat_mse(const SplatArgs &sa, const float *field, const float *target,
                             float *gg, double *partial, double *loss, cudaStream_t st) {
  const uint32_t gs = sa.mc.grid_size;
  const uint32_t nvox = gs * gs * gs;
  if (nvox == 0) return cudaSuccess;
  const unsigned blocks = blocks_for(nvox, 256);
  k_splat_mse<<<blocks, 256, 0, st>>>(sa, field, target, gg, partial);
  k_sum_partials<<<1, 1024, 0, st>>>(partial, blocks, loss);
  return cudaGetLastError();
}

cudaError_t launch_splat_adjoint(const SplatArgs &sa, uint32_t n, const float4 *pos,
                                 const float *gg, float4 *xbar, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_splat_adjoint<<<blocks_for(n, 128), 128, 0, st>>>(sa, n, pos, gg, xbar);
  return cudaGetLastError();
}

}  // namespace fs
