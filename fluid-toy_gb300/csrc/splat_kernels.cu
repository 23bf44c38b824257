// splat_kernels.cu — the marching-cubes density pass on sm_103a.
//
// mc_density.wgsl:130-231 with anisotropy off: one thread per voxel, x
// fastest. The voxel's SPH cell (unclamped) and its neighbours within
// cell_radius are visited in the shader's order (dz, dy, dx, slot); cells
// adjacent in x are adjacent in the sorted arrays, so each (dy, dz) row is
// one contiguous slot range, as in the neighbour passes. Compiled with
// -fmad=false: every expression keeps the shader's operation order, so the
// field is bit-identical to the FP32 restatement.
#include <cmath>

#include "sph_device.cuh"

namespace fs {
namespace {

// mc_density.wgsl:110-128: five walls (no ceiling), floor 0.15
__device__ __forceinline__ float mc_boundary_gamma(const GpuContainerGeometry &c, float3 local,
                                                   float h) {
  float gamma = 1.0f;
  const float d_nx = local.x + c.half_width;
  const float d_px = c.half_width - local.x;
  const float d_fl = local.y + c.half_height;
  const float d_nz = local.z + c.half_depth;
  const float d_pz = c.half_depth - local.z;
  if (d_nx < h) gamma *= 0.5f + 0.5f * clampf(d_nx / h, 0.0f, 1.0f);
  if (d_px < h) gamma *= 0.5f + 0.5f * clampf(d_px / h, 0.0f, 1.0f);
  if (d_fl < h) gamma *= 0.5f + 0.5f * clampf(d_fl / h, 0.0f, 1.0f);
  if (d_nz < h) gamma *= 0.5f + 0.5f * clampf(d_nz / h, 0.0f, 1.0f);
  if (d_pz < h) gamma *= 0.5f + 0.5f * clampf(d_pz / h, 0.0f, 1.0f);
  return fmaxf(gamma, 0.15f);
}

__global__ void __launch_bounds__(128)
    k_density_splat(SplatArgs a, const float4 *__restrict__ s_pos,
                    const uint32_t *__restrict__ begin, float *__restrict__ out) {
  const uint32_t gs = a.mc.grid_size;
  const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= gs * gs * gs) return;
  const uint32_t x = v % gs, y = (v / gs) % gs, z = v / (gs * gs);
  const float cs = a.mc.cell_size;
  const float3 wp = f3(a.mc.grid_min[0] + (float(x) + 0.5f) * cs,
                       a.mc.grid_min[1] + (float(y) + 0.5f) * cs,
                       a.mc.grid_min[2] + (float(z) + 0.5f) * cs);
  const float h = a.mc.kernel_radius;
  const float h_sq = h * h;
  const GpuGridParams &g = a.sph;
  const long long cx = __float2int_rd((wp.x - g.grid_origin_x) * g.inv_cell_size);
  const long long cy = __float2int_rd((wp.y - g.grid_origin_y) * g.inv_cell_size);
  const long long cz = __float2int_rd((wp.z - g.grid_origin_z) * g.inv_cell_size);
  const long long r = a.cell_radius;
  const long long gx = g.grid_size_x, gy = g.grid_size_y, gz = g.grid_size_z;
  const long long x0 = cx - r < 0 ? 0 : cx - r;
  const long long x1 = cx + r > gx - 1 ? gx - 1 : cx + r;
  float density = 0.0f;
  if (x0 <= x1) {
    for (long long dz = -r; dz <= r; dz++) {
      const long long zz = cz + dz;
      if (zz < 0 || zz >= gz) continue;
      for (long long dy = -r; dy <= r; dy++) {
        const long long yy = cy + dy;
        if (yy < 0 || yy >= gy) continue;
        const uint32_t row = uint32_t(yy) * g.grid_size_x + uint32_t(zz) * g.grid_size_x * g.grid_size_y;
        const uint32_t lo = __ldg(begin + row + uint32_t(x0));
        const uint32_t hi = __ldg(begin + row + uint32_t(x1) + 1u);
#pragma unroll 4
        for (uint32_t j = lo; j < hi; j++) {
          const float4 p = __ldg(s_pos + j);
          const float3 d = f3(wp.x - p.x, wp.y - p.y, wp.z - p.z);
          const float r_sq = dot3(d, d);
          if (r_sq < h_sq) {
            const float diff = h_sq - r_sq;
            density += a.coeff * diff * diff * diff;
          }
        }
      }
    }
  }
  const GpuContainerGeometry &c = a.geom;
  const float3 local = world_to_local(c, wp);
  if (c.clip_enabled != 0u &&
      !(local.x >= -c.half_width && local.x <= c.half_width && local.y >= -c.half_height &&
        local.y <= c.half_height && local.z >= -c.half_depth && local.z <= c.half_depth)) {
    out[v] = -1.0f;
    return;
  }
  out[v] = density / mc_boundary_gamma(c, local, h);
}

}  // namespace

SplatArgs make_splat_args(const GpuMcGridParams &mc, const GpuContainerGeometry &geom,
                          const GpuGridParams &sph) {
  SplatArgs a;
  a.mc = mc;
  a.geom = geom;
  a.sph = sph;
  const float h = mc.kernel_radius;
  a.coeff = 315.0f / (64.0f * PI_F * pow_int_f32(h, 9u));
  a.cell_radius = int(std::ceil(h * sph.inv_cell_size));
  return a;
}

cudaError_t launch_density_splat(const SplatArgs &a, const float4 *s_pos, const uint32_t *begin,
                                 float *out, cudaStream_t st) {
  const uint32_t gs = a.mc.grid_size;
  const uint32_t voxels = gs * gs * gs;
  if (voxels == 0) return cudaSuccess;
  k_density_splat<<<(voxels + 127u) / 128u, 128, 0, st>>>(a, s_pos, begin, out);
  return cudaGetLastError();
}

}  // namespace fs
