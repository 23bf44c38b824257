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
// surface tension) are reduced in FP64.
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

template <class F>
__device__ __forceinline__ void for_candidates(const Runs &R, F &&f) {
  for (int r = 0; r < R.count; r++)
    for (uint32_t j = R.lo[r]; j < R.hi[r]; j++) f(j);
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

__device__ __forceinline__ void warp_add_params(double *gparam, uint32_t scene, double gv,
                                                double gs) {
  // FP64 reduction of the scalar-parameter gradients: warp sums, one atomic
  // per warp when its lanes share a scene, else per lane
  const unsigned full = 0xffffffffu;
  const uint32_t s0 = __shfl_sync(full, scene, 0);
  if (__all_sync(full, scene == s0)) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      gv += __shfl_xor_sync(full, gv, o);
      gs += __shfl_xor_sync(full, gs, o);
    }
    if ((threadIdx.x & 31u) == 0u && (gv != 0.0 || gs != 0.0)) {
      atomicAdd(gparam + 3 * s0 + 0, gv);
      atomicAdd(gparam + 3 * s0 + 2, gs);
    }
  } else if (gv != 0.0 || gs != 0.0) {
    atomicAdd(gparam + 3 * scene + 0, gv);
    atomicAdd(gparam + 3 * scene + 2, gs);
  }
}

// ---- integrate + finalize --------------------------------------------------------
__global__ void __launch_bounds__(128)
    k_adj_integrate(SceneView v, TapeView t, AdjView a, const float4 *__restrict__ xbar_in,
                    const float4 *__restrict__ vbar_in, int K) {
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
  const float3 apb = clamp_adjoint(f3of(t.ap[K - 1][s]), dt * vfb, max_accel);
  a.gx[s] = f4(xb, 0.f);
  a.gvhat[s] = f4(vfb, 0.f);
  a.ga[s] = f4(dt * vfb, 0.f);
  a.gu[(K - 1) & 1][s] = f4(apb, 0.f);
  a.gp[s] = 0.f;
  a.gv[s] = make_float4(0.f, 0.f, 0.f, 0.f);
  a.grho[s] = make_float2(0.f, 0.f);
  a.gn[s] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// ---- one PCISPH iteration (level k) ------------------------------------------------
__global__ void __launch_bounds__(128)
    k_adj_solve(SceneView v, TapeView t, AdjView a, int k, int K) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= v.b->n_sorted) return;
  const DevUniforms *U = v.u + t.scene_of_slot[q];
  const GpuSphParams3D &P = U->sph;
  const float h = P.kernel_radius, h2 = P.kernel_radius_sq, mass = P.mass, dt = P.dt;
  const float scale_d = 315.0f / (64.0f * PI_F * P.kernel_radius_pow9);
  const float scale_g = 45.0f / (PI_F * P.kernel_radius_pow6);
  const float4 xq4 = t.xp[k][q];
  const float3 xq = f3of(xq4);
  const float pq = xq4.w;
  const float rho_q = t.rho[k][q];
  const float rt_q = fmaxf(rho_q, 1.0f);
  const float4 uq4 = a.gu[k & 1][q];
  const float3 uq = f3of(uq4);
  const float rhat_q = uq4.w;
  const bool has_rho = k < K - 1;  // level K's density and pressure are unused
  const bool has_p = k >= 1;       // level 0 holds zero pressures
  Runs R;
  flag_outside(a.err, runs_checked(f3of(t.pos[q]), U->grid, t.cell_begin + U->c_offset, R));
  float3 xsb = f3(0.f, 0.f, 0.f);
  float pb = 0.f, rb = 0.f;
  for_candidates(R, [&](uint32_t j) {
    const float4 xj4 = __ldg(t.xp[k] + j);
    const float3 r = xq - f3of(xj4);
    const float r2 = dot3(r, r);
    if (!(r2 < h2)) return;
    const float4 uj4 = __ldg(a.gu[k & 1] + j);
    const float diff = h2 - r2;
    if (has_rho) xsb = mad3(xsb, -6.0f * mass * scale_d * diff * diff * (rhat_q + uj4.w), r);
    if (has_p && r2 > MIN_R2) {
      const float rt_j = fmaxf(__ldg(t.rho[k] + j), 1.0f);
      const float cij = pq / (rt_q * rt_q) + xj4.w / (rt_j * rt_j);
      const float rr = sqrtf(r2);
      const float3 e = r * (1.0f / rr);
      const float dg = h - rr;
      const float g = scale_g * dg * dg;
      const float gp = -2.0f * scale_g * dg;
      const float3 du = uq - f3of(uj4);
      const float edu = dot3(e, du);
      // J du = g' (e.du) e + (g / r)(du - (e.du) e)
      const float3 Jdu = e * (gp * edu) + (du - e * edu) * (g / rr);
      xsb = mad3(xsb, mass * cij, Jdu);
      const float phidu = g * edu;  // phi . du with phi = g e
      pb += mass / (rt_q * rt_q) * phidu;
      if (rho_q > 1.0f) rb += mass * (-2.0f * pq / (rt_q * rt_q * rt_q)) * phidu;
    }
  });
  const float p_bar = a.gp[q] + pb;  // p^{k+1} = p^k + ...: identity part
  const float3 vstar_b = dt * xsb;   // x*^k = x + dt v*^k
  float4 gx = a.gx[q], gvh = a.gvhat[q], ga = a.ga[q];
  gx = f4(add3(f3of(gx), xsb), 0.f);
  gvh = f4(add3(f3of(gvh), vstar_b), 0.f);
  ga = f4(add3(f3of(ga), dt * vstar_b), 0.f);
  a.gx[q] = gx;
  a.gvhat[q] = gvh;
  a.ga[q] = ga;
  if (k >= 1) {
    // elementwise half of iteration k-1's reverse: its outputs are level k
    const float max_accel = 0.25f * h / (dt * dt);
    const float3 apb = clamp_adjoint(f3of(t.ap[k - 1][q]), dt * vstar_b, max_accel);
    const float rhat = rb + (rho_q > P.rest_density ? P.pcisph_delta * p_bar : 0.0f);
    a.gu[(k - 1) & 1][q] = f4(apb, rhat);
    a.gp[q] = p_bar;
  }
  // k == 0: predict, x*^0 = x + dt v*^0, v*^0 = vhat + dt a (done above)
}

// ---- force (non-pressure acceleration) -----------------------------------------------
struct ForceSide {
  float3 x, vhat, vpre, n;
  float rho, rhon;
};
struct ForcePair {  // reverse outputs of one pair term T_{i<-j}
  float3 g_r;       // d/d(x_i - x_j)
  float3 g_vhat_i, g_vpre_j, g_n_i, g_n_j;
  float g_rho_i, g_rho_j, g_rhon_i, g_rhon_j, g_visc, g_st;
};

// w . T_{i<-j} reversed, T from sph_force_3d_grid.wgsl:127-220 (see
// force_predict_one for the forward). e_close is the tabulated fallback
// direction of the pair (constant in the positions). The cohesion part of
// the pair is scaled by the surface tension in the forward (a_c *= st).
__device__ __forceinline__ ForcePair force_pair_vjp(const ForceSide &I, const ForceSide &J,
                                                    float3 w, float3 e_close,
                                                    const GpuSphParams3D &P) {
  ForcePair o;
  const float h = P.kernel_radius, h2 = P.kernel_radius_sq, mass = P.mass;
  const float scale_g = 45.0f / (PI_F * P.kernel_radius_pow6);
  const float scale_c = 32.0f / (PI_F * P.kernel_radius_pow9);
  const float near_k = P.near_stiffness, visc = P.viscosity, rho0 = P.rest_density;
  const float st = P.surface_tension;
  const float min_dist = h * 0.1f;
  const float3 r = I.x - J.x;
  const float r2 = dot3(r, r);
  const float rr = sqrtf(r2);
  const float3 u = r * (1.0f / rr);  // d rr / d r
  const bool close = rr < min_dist;
  const float3 e = close ? e_close : -u;
  const float rho_i = fmaxf(I.rho, 1.0f), rho_j = fmaxf(J.rho, 1.0f);
  const float rhon_i = fmaxf(I.rhon, 1.0f), rhon_j = fmaxf(J.rhon, 1.0f);
  const bool mi = I.rho > 1.0f, mj = J.rho > 1.0f, mni = I.rhon > 1.0f, mnj = J.rhon > 1.0f;
  const float Pn_i = near_k * rhon_i, Pn_j = near_k * rhon_j;
  const float dg = h - rr;
  const float G = scale_g * dg * dg;
  const float Gp = -2.0f * scale_g * dg;
  const float we = dot3(w, e);
  const float3 dwe = close ? f3(0.f, 0.f, 0.f) : (w - e * we) * (-1.0f / rr);
  float3 g_r = f3(0.f, 0.f, 0.f);
  // near pressure: alpha G e
  const float alpha = -mass * (Pn_i + Pn_j) / (2.0f * rho_i * rhon_j);
  g_r = g_r + (u * (Gp * we) + dwe * G) * alpha;
  o.g_rho_i = mi ? (-alpha / rho_i) * G * we : 0.f;
  o.g_rhon_i = mni ? (-mass * near_k / (2.0f * rho_i * rhon_j)) * G * we : 0.f;
  o.g_rhon_j = mnj ? (mass * Pn_i / (2.0f * rho_i * rhon_j * rhon_j)) * G * we : 0.f;
  o.g_rho_j = 0.f;
  // separation (close pairs): -200 (1 - r / min_dist) e
  if (close) g_r = g_r + u * ((200.0f / min_dist) * we);
  // viscosity (v_ij . x_ij < 0): beta G e, beta = m visc h vdx / (D avg)
  const float3 vij = I.vhat - J.vpre;
  const float vdx = dot3(vij, r);
  o.g_vhat_i = f3(0.f, 0.f, 0.f);
  o.g_vpre_j = f3(0.f, 0.f, 0.f);
  o.g_visc = 0.f;
  if (vdx < 0.0f) {
    const float D = r2 + 0.01f * h2;
    const float avg = (rho_i + rho_j) * 0.5f;
    const float bG = mass * h * vdx / (D * avg);  // per unit viscosity and G
    const float beta = visc * bG * G;
    const float dbeta_dvdx = visc * mass * h * G / (D * avg);
    g_r = g_r + (vij * dbeta_dvdx + u * (visc * bG * Gp) - r * (2.0f * beta / D)) * we + dwe * beta;
    o.g_vhat_i = r * (we * dbeta_dvdx);
    o.g_vpre_j = r * (-we * dbeta_dvdx);
    const float drho = -beta / (2.0f * avg) * we;
    o.g_rho_i += mi ? drho : 0.f;
    o.g_rho_j += mj ? drho : 0.f;
    o.g_visc = bG * G * we;
  }
  // cohesion, scaled by st: m K C e - m K (n_i - n_j)
  const float3 wc = w * st;
  const float wce = dot3(wc, e);
  const float3 dwce = close ? f3(0.f, 0.f, 0.f) : (wc - e * wce) * (-1.0f / rr);
  const float rs = rho_i + rho_j;
  const float Kij = 2.0f * rho0 / rs;
  const float dK = -Kij / rs;
  const float r3 = rr * rr * rr;
  const float dg2 = dg * dg, dg3 = dg2 * dg;
  const bool far_c = rr >= h * 0.5f;
  const float C = far_c ? scale_c * dg3 * r3
                        : scale_c * (2.0f * dg3 * r3 - P.kernel_radius_pow6 / 64.0f);
  const float Cp = (far_c ? 1.0f : 2.0f) * scale_c * (-3.0f * dg2 * r3 + 3.0f * dg3 * rr * rr);
  g_r = g_r + (u * (Cp * wce) + dwce * C) * (mass * Kij);
  const float3 nij = I.n - J.n;
  o.g_n_i = wc * (-mass * Kij);
  o.g_n_j = wc * (mass * Kij);
  const float dKterm = dK * (mass * C * wce - mass * dot3(wc, nij));
  o.g_rho_i += mi ? dKterm : 0.f;
  o.g_rho_j += mj ? dKterm : 0.f;
  o.g_st = mass * Kij * C * we - mass * Kij * dot3(w, nij);
  o.g_r = g_r;
  return o;
}

__device__ __forceinline__ float3 close_dir(const float4 *dir_tab, int dir_half, uint32_t si,
                                            uint32_t sj, uint32_t s_off) {
  const int d = int(si) - int(sj);
  if (d >= -dir_half && d <= dir_half) return f3of(__ldg(dir_tab + d + dir_half));
  return fallback_dir_eval(float(si - s_off) - float(sj - s_off));
}

__global__ void __launch_bounds__(128)
    k_adj_force(SceneView v, TapeView t, AdjView a, const float4 *__restrict__ dir_tab,
                int dir_half) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = q < v.b->n_sorted;
  const uint32_t scene = active ? t.scene_of_slot[q] : 0u;
  double acc_visc = 0.0, acc_st = 0.0;
  if (active) {
    const DevUniforms *U = v.u + scene;
    const GpuSphParams3D &P = U->sph;
    const float h2 = P.kernel_radius_sq;
    auto side = [&](uint32_t i) {
      ForceSide S;
      S.x = f3of(__ldg(t.pos + i));
      S.vhat = f3of(__ldg(t.vhat + i));
      S.vpre = f3of(__ldg(t.vel + i));
      S.n = f3of(__ldg(t.nrm + i));
      const float2 d = __ldg(t.dens + i);
      S.rho = d.x;
      S.rhon = d.y;
      return S;
    };
    const ForceSide Q = side(q);
    const float3 wq = f3of(a.ga[q]);
    Runs R;
    flag_outside(a.err, runs_checked(Q.x, U->grid, t.cell_begin + U->c_offset, R));
    float3 gx = f3(0.f, 0.f, 0.f), gvh = f3(0.f, 0.f, 0.f), gv = f3(0.f, 0.f, 0.f);
    float3 gn = f3(0.f, 0.f, 0.f);
    float grho = 0.f, grhon = 0.f;
    float sv = 0.f, ss = 0.f;
    for_candidates(R, [&](uint32_t j) {
      const float3 xj = f3of(__ldg(t.pos + j));
      const float3 r = Q.x - xj;
      const float r2 = dot3(r, r);
      if (!(r2 < h2 && r2 > MIN_R2)) return;
      const ForceSide Jn = side(j);
      // (A) T_{q<-j} with q's cotangent: q's i-side
      const ForcePair A = force_pair_vjp(Q, Jn, wq, close_dir(dir_tab, dir_half, q, j, U->s_offset), P);
      gx = gx + A.g_r;
      gvh = gvh + A.g_vhat_i;
      grho += A.g_rho_i;
      grhon += A.g_rhon_i;
      gn = gn + A.g_n_i;
      sv += A.g_visc;
      ss += A.g_st;
      // (B) T_{j<-q} with j's cotangent: q's j-side
      const float3 wj = f3of(__ldg(a.ga + j));
      const ForcePair B = force_pair_vjp(Jn, Q, wj, close_dir(dir_tab, dir_half, j, q, U->s_offset), P);
      gx = gx - B.g_r;
      gv = gv + B.g_vpre_j;
      grho += B.g_rho_j;
      grhon += B.g_rhon_j;
      gn = gn + B.g_n_j;
    });
    a.gx[q] = f4(add3(f3of(a.gx[q]), gx), 0.f);
    a.gvhat[q] = f4(add3(f3of(a.gvhat[q]), gvh), 0.f);
    a.gv[q] = f4(gv, 0.f);
    a.grho[q] = make_float2(grho, grhon);
    a.gn[q] = f4(gn, 0.f);
    // a_c *= st and a = ... + a_c: d/d st = w . sum of raw cohesion terms
    acc_visc = double(sv);
    acc_st = double(ss);
  }
  warp_add_params(a.gparam, scene, acc_visc, acc_st);
}

// ---- XSPH -------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_adj_xsph(SceneView v, TapeView t, AdjView a) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= v.b->n_sorted) return;
  const DevUniforms *U = v.u + t.scene_of_slot[q];
  const GpuSphParams3D &P = U->sph;
  const float h2 = P.kernel_radius_sq, mass = P.mass, eps = P.xsph_epsilon;
  const float scale_d = 315.0f / (64.0f * PI_F * P.kernel_radius_pow9);
  const float3 wq = f3of(a.gvhat[q]);
  float3 gv = add3(f3of(a.gv[q]), wq);  // vhat = v + eps * sum
  float3 gx = f3(0.f, 0.f, 0.f);
  float grho = a.grho[q].x;
  const float3 xq = f3of(t.pos[q]);
  const float rho_q = t.dens[q].x;
  const float gamma_q = boundary_gamma(U->geom, P.kernel_radius, xq);
  if (eps > 0.0f) {
    const float3 vq = f3of(t.vel[q]);
    const float rb_q = fmaxf(rho_q, 1.0f);
    const float fq = eps * mass / rb_q;
    Runs R;
    flag_outside(a.err, runs_checked(xq, U->grid, t.cell_begin + U->c_offset, R));
    for_candidates(R, [&](uint32_t j) {
      const float3 xj = f3of(__ldg(t.pos + j));
      const float3 r = xq - xj;  // r_qj
      const float r2 = dot3(r, r);
      if (!(r2 < h2 && r2 > MIN_R2)) return;
      const float diff = h2 - r2;
      const float W = scale_d * diff * diff * diff;
      const float dWs = -6.0f * scale_d * diff * diff;  // dW/dr = dWs * r
      const float3 vj = f3of(__ldg(t.vel + j));
      const float rho_j = __ldg(&t.dens[j].x);
      const float fj = eps * mass / fmaxf(rho_j, 1.0f);
      // (A) term_{q<-j} = fj W (v_j - v_q), cotangent wq
      gv = gv - wq * (fj * W);
      gx = gx + r * (fj * dot3(wq, vj - vq) * dWs);
      // (B) term_{j<-q} = fq W (v_q - v_j), cotangent wj; dW/dr_jq = dWs * (-r)
      const float3 wj = f3of(__ldg(a.gvhat + j));
      const float wdv = dot3(wj, vq - vj);
      gv = gv + wj * (fq * W);
      if (rho_q > 1.0f) grho += (-eps * mass / (rb_q * rb_q)) * W * wdv;
      gx = gx + r * (fq * wdv * dWs);  // -(fq wdv dWs (-r))
    });
  }
  a.gv[q] = f4(gv, 0.f);
  a.gx[q] = f4(add3(f3of(a.gx[q]), gx), 0.f);
  // rho = rho_raw / gamma: store the raw density's cotangent and fold the
  // gamma derivative here (d gamma / d x is local to q)
  const float rb_raw = grho / gamma_q;
  a.grho[q] = make_float2(rb_raw, a.grho[q].y);
  // gamma = max(prod_w f_w, 0.1), f_w = 0.5 + 0.5 clamp(d_w / h, 0, 1)
  const GpuContainerGeometry &c = U->geom;
  const float h = P.kernel_radius;
  const float3 l = world_to_local(c, xq);
  const float dw[6] = {l.x + c.half_width, c.half_width - l.x, l.y + c.half_height,
                       c.half_height - l.y, l.z + c.half_depth, c.half_depth - l.z};
  const float sgn[6] = {1.f, -1.f, 1.f, -1.f, 1.f, -1.f};
  float fw[6], prod = 1.0f;
  for (int w = 0; w < 6; w++) {
    fw[w] = dw[w] < h ? 0.5f + 0.5f * clampf(dw[w] / h, 0.0f, 1.0f) : 1.0f;
    prod *= fw[w];
  }
  if (prod > 0.1f && grho != 0.0f) {
    const float gamma_b = -rb_raw * rho_q;  // d rho / d gamma = -rho_raw / gamma^2
    float lg[3] = {0.f, 0.f, 0.f};
    for (int w = 0; w < 6; w++) {
      if (!(dw[w] < h && dw[w] > 0.0f)) continue;  // clamp saturated or inactive
      float others = 1.0f;
      for (int o = 0; o < 6; o++)
        if (o != w) others *= fw[o];
      lg[w >> 1] += gamma_b * others * (0.5f / h) * sgn[w];
    }
    const float3 xg = local_dir_to_world(c, f3(lg[0], lg[1], lg[2]));  // Ri^T
    a.gx[q] = f4(add3(f3of(a.gx[q]), xg), 0.f);
  }
}

// ---- density, near density, normal ------------------------------------------------------
__global__ void __launch_bounds__(128) k_adj_density(SceneView v, TapeView t, AdjView a) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= v.b->n_sorted) return;
  const DevUniforms *U = v.u + t.scene_of_slot[q];
  const GpuSphParams3D &P = U->sph;
  const float h = P.kernel_radius, h2 = P.kernel_radius_sq, mass = P.mass;
  const float scale_d = 315.0f / (64.0f * PI_F * P.kernel_radius_pow9);
  const float scale_n = 15.0f / (PI_F * P.kernel_radius_pow6);
  const float h8 = P.kernel_radius_pow6 * h * h;
  const float cnorm = 945.0f / (32.0f * PI_F * h8) * (mass / P.rest_density);
  const float3 xq = f3of(t.pos[q]);
  const float2 gq = a.grho[q];
  const float3 nq = f3of(a.gn[q]);
  Runs R;
  flag_outside(a.err, runs_checked(xq, U->grid, t.cell_begin + U->c_offset, R));
  float3 gx = f3(0.f, 0.f, 0.f);
  // d/dr of one ordered pair's terms, r = x_i - x_j, with i's cotangents
  auto pair = [&](float3 r, float r2, float2 gi, float3 ni) {
    const float diff = h2 - r2;
    const float rr = sqrtf(r2);
    const float dn = h - rr;
    float3 g = r * (-6.0f * mass * scale_d * diff * diff * gi.x);
    g = g + r * (-3.0f * mass * scale_n * dn * dn * gi.y / rr);
    g = g + (ni * (diff * diff) - r * (4.0f * diff * dot3(ni, r))) * cnorm;
    return g;
  };
  for_candidates(R, [&](uint32_t j) {
    const float3 xj = f3of(__ldg(t.pos + j));
    const float3 r = xq - xj;
    const float r2 = dot3(r, r);
    if (!(r2 < h2 && r2 > MIN_R2)) return;
    gx = gx + pair(r, r2, gq, nq);
    gx = gx - pair(-r, r2, __ldg(a.grho + j), f3of(__ldg(a.gn + j)));
  });
  a.gx[q] = f4(add3(f3of(a.gx[q]), gx), 0.f);
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
// gamma_v (0 for clipped voxels), loss partial sums in FP64.
__global__ void __launch_bounds__(256)
    k_splat_mse(SplatArgs sa, const float *__restrict__ field, const float *__restrict__ target,
                float *__restrict__ gg, double *__restrict__ loss) {
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
  l /= double(nvox);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31u) == 0u && l != 0.0) atomicAdd(loss, l);
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

cudaError_t launch_adj_step(const SceneView &v, const TapeView &t, const AdjView &a,
                            const float4 *xbar_in, const float4 *vbar_in, float4 *xbar_out,
                            float4 *vbar_out, const float4 *dir_tab, int dir_half, uint32_t n,
                            int K, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const unsigned b = blocks_for(n, 128);
  k_adj_integrate<<<b, 128, 0, st>>>(v, t, a, xbar_in, vbar_in, K);
  for (int k = K - 1; k >= 0; k--) k_adj_solve<<<b, 128, 0, st>>>(v, t, a, k, K);
  k_adj_force<<<b, 128, 0, st>>>(v, t, a, dir_tab, dir_half);
  k_adj_xsph<<<b, 128, 0, st>>>(v, t, a);
  k_adj_density<<<b, 128, 0, st>>>(v, t, a);
  k_adj_to_canonical<<<blocks_for(n, 256), 256, 0, st>>>(v, t, a, xbar_out, vbar_out);
  return cudaGetLastError();
}

cudaError_t launch_splat_mse(const SplatArgs &sa, const float *field, const float *target,
                             float *gg, double *loss, cudaStream_t st) {
  const uint32_t gs = sa.mc.grid_size;
  const uint32_t nvox = gs * gs * gs;
  if (nvox == 0) return cudaSuccess;
  k_splat_mse<<<blocks_for(nvox, 256), 256, 0, st>>>(sa, field, target, gg, loss);
  return cudaGetLastError();
}

cudaError_t launch_splat_adjoint(const SplatArgs &sa, uint32_t n, const float4 *pos,
                                 const float *gg, float4 *xbar, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_splat_adjoint<<<blocks_for(n, 128), 128, 0, st>>>(sa, n, pos, gg, xbar);
  return cudaGetLastError();
}

}  // namespace fs
