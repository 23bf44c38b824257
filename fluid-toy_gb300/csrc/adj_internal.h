// adj_internal.h — types shared by the reverse pass's host side (adjoint.cu)
// and its kernels (adj_kernels.cu).
#pragma once

#include "fs_internal.h"

namespace fs {

constexpr int kMaxAdjIters = 16;  // PCISPH iterations a recorded step may hold

// One recorded forward step, grid-sorted order (the buffers the step's
// kernels wrote, see enqueue_step with a DevState override).
struct TapeView {
  const uint32_t *s2o;
  const uint16_t *scene_of_slot;
  const uint32_t *cell_begin;  // [cells + 1], global slot numbers
  const float4 *pos, *vel, *nrm, *vhat, *anp, *vfin;
  const float2 *dens;
  const float4 *xp[kMaxAdjIters + 1];  // predicted (x*, p) per level
  const float *rho[kMaxAdjIters + 1];  // predicted densities per level
  const float4 *ap[kMaxAdjIters];      // pressure acceleration before the clamp
  const uint32_t *order;               // the step's task order (warp ids, heaviest first)
  const uint32_t *mask_words;          // the step's hit masks (density pass)
  const uint32_t *mask_off;            // word offset of each slot's mask, or MASK_NONE
  const uint32_t *perm_hit;            // slots ordered by hit count, heaviest first
  const uint32_t *hits;                // union over the levels of the in-range masks at x*
};

// Reverse accumulators, grid-sorted order.
struct AdjView {
  float4 *gx;     // d/d position
  float4 *gvhat;  // d/d post-XSPH velocity
  float4 *gv;     // d/d pre-XSPH velocity (the step's input velocity)
  float4 *ga;     // d/d non-pressure acceleration
  float4 *gn;     // d/d Akinci normal
  float2 *grho;   // d/d density (raw, after the XSPH reverse), d/d near density
  float *gp;      // d/d pressure carried between PCISPH levels
  // per level, two float4 per particle (ping-pong between levels): the
  // level's (x*, p / max(rho*, 1)^2), then (d/d pressure acceleration
  // (pre-clamp), d/d next density); a neighbour's pair of records is one
  // 32-byte load site in the level's reverse
  float4 *lv[2];
  // [5 N]: each particle's inputs to the force reverse (x, max(rho, 1);
  // vhat, max(rho_near, 1); v; n; d/d non-pressure acceleration), written by
  // level 0's reverse so that a neighbour is one 80-byte load site
  float4 *frec;
  double *gparam; // [scenes][3]: viscosity, stiffness, surface_tension (FP64)
  double *gparam2;  // [scenes][2]: near_stiffness, pcisph_delta (FP64)
  double2 *gpart; // [N] canonical: each particle's share of d/d (viscosity, surface tension)
  double2 *gpart2;  // [N] canonical: each particle's share of d/d (near_stiffness, pcisph_delta)
  uint32_t *counters;  // task counters of the gather launches [kMaxAdjIters + 3]
  uint32_t *err;
};

cudaError_t launch_adj_step(const SceneView &v, const TapeView &t, const AdjView &a,
                            const float4 *xbar_in, const float4 *vbar_in, float4 *xbar_out,
                            float4 *vbar_out, const float4 *dir_tab, int dir_half, uint32_t n,
                            int K, int lanes, int sm_count, cudaStream_t st);
// partial: one double per 256 voxels
cudaError_t launch_splat_mse(const SplatArgs &sa, const float *field, const float *target,
                             float *gg, double *partial, double *loss, cudaStream_t st);
cudaError_t launch_reduce_params(const double2 *gpart, const double2 *gpart2,
                                 const uint32_t *scene_first, const uint32_t *scene_count,
                                 uint32_t scenes, double *gparam, double *gparam2,
                                 cudaStream_t st);
cudaError_t launch_rows_to_f4(uint32_t n, const float *rows, float4 *out, cudaStream_t st);
cudaError_t launch_f4_to_rows(uint32_t n, const float4 *in, float *rows, cudaStream_t st);
cudaError_t launch_splat_adjoint(const SplatArgs &sa, uint32_t n, const float4 *pos,
                                 const float *gg, float4 *xbar, cudaStream_t st);

}  // namespace fs
