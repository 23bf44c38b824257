// spray_internal.h — types shared by the whitewater host side (spray.cu) and
// its kernels (spray_kernels.cu).
#pragma once

#include "fs_internal.h"

namespace fs {

// One scene's inputs and the spray system's device state.
struct SprayView {
  const DevUniforms *u;         // the scene's parameter block
  const float4 *s_pos, *s_vel;  // sorted positions, pre-XSPH velocities (all scenes)
  const float2 *s_dens;         // sorted density (post boundary gamma), near density
  const float4 *s_nrm;          // sorted Akinci normals
  const uint32_t *begin;        // the scene's cell_begin (global slot numbers)
  uint32_t s_offset;            // the scene's first sorted slot
  uint32_t *write_head;         // ring write head
  float *limits;                // potential ceilings: trapped air, wave crest
  uint32_t *emit_stats;         // [4] per-frame potential maxima (f32 bits), then
                                // live_stats [4]: total, spray, foam, bubble
  uint32_t *live_stats;
};

struct SprayFrame {
  GpuSprayParams params;
};

inline uint32_t scan_tiles_for(uint32_t n) { return scan_tiles(n); }

cudaError_t launch_spray_frame(const SprayView &sv, const SprayFrame &f, uint32_t n,
                               uint32_t *counts, uint32_t *ends, unsigned long long *scan_tiles,
                               uint32_t *err, GpuSprayParticle *ring, cudaStream_t st);

}  // namespace fs
