// rigid_kernels.cu — the device-resident rigid-body coupling: after a frame's
// substeps, each coupled scene's body is integrated from the frame's reaction
// accumulator (integrate_rigid_body, src/state/rigid_body.rs:277-365) or, if
// held, clamped to its container (:415-479), and the scene's GpuRigidBody is
// rewritten for the next frame (to_gpu_rigid_body, :131-146). One thread per
// scene; the arithmetic is rigid_math.h's, shared with the host entry points.
#include "fs_internal.h"
#include "rigid_math.h"

namespace fs {
namespace {

__global__ void k_rigid_frame(DevUniforms *__restrict__ u, FsRigidBodyState *__restrict__ st,
                              const GpuRigidBodyAccum *__restrict__ accum,
                              const uint8_t *__restrict__ coupled, uint32_t n_scenes,
                              uint32_t substeps) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_scenes || !coupled[k]) return;
  FsRigidBodyState s = st[k];
  DevUniforms &U = u[k];
  if (s.enabled) {
    if (!s.held) rb::integrate(s, U.geom, U.sph.dt, substeps, U.gravity.direction, accum[k]);
    else rb::clamp_to_container(s, U.geom, false);
  }
  st[k] = s;
  rb::to_gpu(s, U.rigid);
}

// Rewrite the coupled scenes' GpuRigidBody from their states (after a host
// upload of the parameter blocks).
__global__ void k_rigid_sync(DevUniforms *__restrict__ u, const FsRigidBodyState *__restrict__ st,
                             const uint8_t *__restrict__ coupled, uint32_t n_scenes) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_scenes || !coupled[k]) return;
  rb::to_gpu(st[k], u[k].rigid);
}

}  // namespace

cudaError_t launch_rigid_frame(const DevState &d, uint32_t n_scenes, uint32_t substeps,
                               cudaStream_t st) {
  k_rigid_frame<<<(n_scenes + 127) / 128, 128, 0, st>>>(d.u, d.rb_state, d.accum, d.rb_coupled,
                                                        n_scenes, substeps);
  return cudaGetLastError();
}

cudaError_t launch_rigid_sync(const DevState &d, uint32_t n_scenes, cudaStream_t st) {
  k_rigid_sync<<<(n_scenes + 127) / 128, 128, 0, st>>>(d.u, d.rb_state, d.rb_coupled, n_scenes);
  return cudaGetLastError();
}

}  // namespace fs
