// fs_internal.h — internal types shared by the host orchestration (sim.cu)
// and the sm_103a kernels (grid_kernels.cu, sph_kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fluidsph.h"

namespace fs {

// Load depths (candidate records in flight per lane) each neighbour pass is
// instantiated for; see kLoadDepths / kXsphDepths in sph_kernels.cu. 32 is the
// staged form of XSPH (a warp's chunk of 32 records in shared memory); the
// density and solve passes have no staged form and are tuned over the first
// four only.
constexpr int kNumLoadDepths = 5;
constexpr int kPlainCandidates = 4;
constexpr uint32_t kDensityDepths[kNumLoadDepths] = {0, 4, 8, 16, 32};
constexpr uint32_t kXsphDepthList[kNumLoadDepths] = {1, 4, 8, 16, 32};

// Work-order scratch words (DevState::order_hist), zeroed each step: the
// bucket counts and cursors of the 33 work buckets, the positions'
// small-coordinate flag, a pad word, then the step's in-range pair count
// (64 bits, 8-byte aligned; the density pass sums it).
constexpr int ORDER_HIST_WORDS = 2 * 33 + 1 + 1 + 2;
constexpr int ORDER_HIST_STEP_HITS = 2 * 33 + 2;

// The neighbour passes' load-depth choice of a simulation (indices into the
// lists above).
struct KernelForms {
  uint8_t density = 0, solve = 0, xsph = 1;
  uint32_t key() const { return uint32_t(density) | uint32_t(solve) << 8 | uint32_t(xsph) << 16; }
};

// Parameter block resident in device memory. The update_* entry points copy
// their struct here with cudaMemcpyAsync on the simulation's stream, which
// orders them before later steps exactly like the reference's
// queue.write_buffer uploads (sph_3d_grid.rs:1446-1473), and lets captured
// step graphs stay valid across parameter changes.
// One block per scene: a simulation holds one scene, a batch many.
struct DevUniforms {
  GpuSphParams3D sph;
  GpuGridParams grid;
  GpuContainerGeometry geom;
  GpuGravity gravity;
  GpuMouseForce mouse;
  GpuRigidBody rigid;
  uint32_t n;         // effective particle count of the scene for every stage
  uint32_t sdf_res;   // SDF texture edge length (1 = the reference's dummy)
  uint32_t p_offset;  // first canonical particle of the scene
  uint32_t c_offset;  // first cell of the scene in the global cell arrays
  uint32_t s_offset;  // first sorted slot of the scene
  uint32_t pad[3];
};

// Counts over all scenes of a simulation (device copy).
struct DevBatch {
  uint32_t n_scenes;
  uint32_t n_canon;      // canonical particles in the buffer
  uint32_t n_sorted;     // hashed particles (sum of the scenes' effective counts)
  uint32_t cells_total;  // sum of the scenes' cell counts
};

// What a kernel needs to find the scene of a particle or sorted slot.
struct SceneView {
  const DevUniforms *u;         // [n_scenes]
  const DevBatch *b;
  const uint16_t *scene_of;     // canonical particle -> scene
  const uint16_t *scene_of_slot;  // sorted slot -> scene
};

// Neighbour-statistics counters written by the density and solve kernels.
enum StatIndex : int {
  STAT_CAND_DENSITY = 0,  // candidate pair tests in the density pass
  STAT_HIT_DENSITY = 1,   // pairs with r^2 < h^2 (self included)
  STAT_HIT_NONSELF = 2,   // pairs with 1e-12 < r^2 < h^2
  STAT_CAND_SOLVE = 3,    // candidate tests summed over solve iterations
  STAT_HIT_SOLVE = 4,     // predicted-position pairs with r^2 < h^2
  STAT_COOP_FORCE = 5,    // particles whose force pass ran cooperatively
  STAT_COUNT = 8
};

// Device error word bits.
enum ErrorBits : uint32_t {
  ERR_SCAN_TIMEOUT = 1u,      // decoupled-lookback poll limit reached
  ERR_ADJ_OUTSIDE_GRID = 2u,  // reverse pass: a particle's cell outside the grid
};

// Particle state in HBM: structure-of-arrays, one 16-byte record per particle
// per field so every particle read is one coalesced 128-bit load.
struct DevState {
  // canonical order (index = particle identity, the reference's particle_buffer)
  float4 *p_pos;    // x, y, z, _pad0
  float4 *p_vel;    // vx, vy, vz, _pad1
  float4 *p_force;  // fx, fy, fz, 0  (a_np during the step, dv after it)
  float4 *p_aux;    // 2 per particle: (density, near, nx, ny), (nz, 0, 0, 0)
  // grid-sorted order (index = sorted slot, the reference's sorted buffer)
  float4 *s_pos;    // x, y, z, _pad0
  float4 *s_vel;    // pre-XSPH velocity, _pad1
  float4 *s_frc;    // force field copied at reorder (sorted-view fidelity)
  float2 *s_dens;   // density (boundary-corrected), near density
  float4 *s_nrm;    // Akinci normal, 0
  float4 *vel_x;    // post-XSPH velocity (the canonical velocity mid-step)
  float4 *nb_pos;   // neighbour records (density pass): position, max(density, 1)
  float4 *nb_vel;   //   pre-XSPH velocity, mass / max(density, 1)
  float4 *nb_nrm;   //   Akinci normal, max(near density, 1)
  float *pterm[2];  // solve: p / max(rho, 1)^2 per particle, ping-pong with pred_xp
  // density dedupe (particles at bit-identical positions within a 32-slot warp)
  uint32_t *rep_of;     // representative slot of each sorted slot
  uint32_t *dd_list;    // representatives, compacted in slot order
  uint32_t *dd_warp;    // per 32-slot warp: representatives
  uint32_t *dd_incl;    // inclusive scan of dd_warp (the last entry: size of dd_list)
  unsigned long long *dd_tiles;  // scan descriptors for dd_incl + ticket word
  uint8_t *dd_bucket;   // per 32-entry task of dd_list: candidate bucket
  uint32_t *dd_order;   // tasks of dd_list, heaviest first
  uint32_t *dd_hist;    // bucket histogram + cursors
  uint32_t *dens_cand;  // candidates of each sorted slot (k_warp_work)
  uint32_t *dens_hits;  // its pairs with r^2 < h^2
  float4 *anp;      // non-pressure acceleration a_np
  float4 *pred_xp[2];  // predicted position, pressure (ping-pong)
  float *pred_rho[2];  // predicted density (ping-pong)
  float4 *pred_v;      // final predicted (corrected) velocity
  // grid
  uint32_t *cell_of;     // particle -> cell (hash output)
  uint32_t *rank_of;     // particle -> arrival rank within its cell
  uint32_t *t_tmp;       // unsorted slot -> particle
  uint32_t *big_cells;   // [4 + 2 big_item_cap(M)]: items, 2 tickets, pad, (cell, chunk) items
  uint32_t *s2o;         // sorted slot -> particle (sorted_to_orig)
  uint32_t *cidx;        // particle -> sorted slot (particle_cell_indices)
  uint32_t *counts;      // cell_counts[total_cells]
  uint32_t *cell_begin;  // [total_cells + 1]; cell_begin + 1 = cell_starts
  unsigned long long *tile_status;  // decoupled-lookback descriptors
  uint32_t *tile_ticket;
  float *sdf;
  uint32_t *mask_words;            // per-particle hit bitmasks (see sph_kernels.cu)
  uint32_t *mask_off;              // word offset of each sorted slot's mask
  uint32_t *mask_hits;             // set bits in each sorted slot's mask
  // Neighbour-pass work order (heaviest first): warps of 32 sorted slots for
  // density, XSPH and solve; a slot permutation by hit count for force.
  uint32_t *warp_order;            // [M / 32] warp ids
  uint8_t *warp_bucket;            // [M / 32] work bucket of each warp
  uint32_t *order_hist;            // [ORDER_HIST_WORDS] bucket counts, bucket cursors,
                                   // the step's small-coordinate flag and pair count
  uint32_t *perm_hit;              // [M] sorted slots by decreasing hit count
  uint16_t *work_key;              // [M] hit-count bucket of each sorted slot
  uint32_t *key_hist;              // [3 * KEY_BUCKETS]: counts, bases, cursors
  uint32_t *task_counters;         // one task counter per neighbour-pass launch
  int sm_count;                    // streaming multiprocessors of the device
  unsigned long long *mask_alloc;  // bump allocator of mask words
  unsigned long long mask_cap;     // mask capacity in words
  float4 *dir_tab;  // close-pair fallback directions for slot differences
  int dir_half;     // table covers d in [-dir_half, dir_half]
  GpuRigidBodyAccum *accum;  // [n_scenes]
  FsRigidBodyState *rb_state;  // [n_scenes] device-resident coupled bodies
  uint8_t *rb_coupled;         // [n_scenes] 1 = coupled
  uint32_t *err;
  unsigned long long *stats;
  DevUniforms *u;           // [n_scenes]
  DevBatch *b;
  uint16_t *scene_of;       // canonical particle -> scene
  uint16_t *scene_of_slot;  // sorted slot -> scene
  SceneView view() const { return SceneView{u, b, scene_of, scene_of_slot}; }
  // Recording of the PCISPH levels for the reverse pass; null = ping-pong in
  // pred_xp/pred_rho. Host arrays of device pointers: level k holds the
  // predicted (x*, p) and densities read by iteration k (level 0 = predict).
  float4 *const *rec_xp = nullptr;   // [iterations + 1]
  float *const *rec_rho = nullptr;   // [iterations + 1]
  float4 *const *rec_ap = nullptr;   // [iterations] pressure acceleration before the clamp
  uint32_t *rec_hits = nullptr;  // union over the PCISPH levels of their hit masks (density mask layout)
  // neighbour-pass instantiations: indices into the passes' load-depth lists
  // (kLoadDepths for density and solve, kXsphDepths for XSPH, sph_kernels.cu);
  // the same results whatever they are, chosen per workload by speed
  uint8_t load_density = 0, load_solve = 0, load_xsph = 1;
};

// Set the thread-local text fs_last_error() returns (sim.cu).
void set_last_error(const char *msg);

// x^n for an integral n >= 1: binary exponentiation in double, rounded once
// to float (host_params.cpp). The library's value of WGSL pow(x, n.0).
float pow_int_f32(float x, unsigned n);

// The MC density pass (splat_kernels.cu). begin: the scene's cell_begin
// (global slot numbers), s_pos: the sorted positions of all scenes.
struct SplatArgs {
  GpuMcGridParams mc;
  GpuContainerGeometry geom;
  GpuGridParams sph;
  float coeff;      // 315 / (64 pi pow(h, 9))
  int cell_radius;  // ceil(h * sph.inv_cell_size)
};
SplatArgs make_splat_args(const GpuMcGridParams &mc, const GpuContainerGeometry &geom,
                          const GpuGridParams &sph);
cudaError_t launch_density_splat(const SplatArgs &a, const float4 *s_pos, const uint32_t *begin,
                                 float *out, cudaStream_t st);

// ---- kernel launchers (grid_kernels.cu / sph_kernels.cu) --------------------
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// Cells with more than SORT_SMALL particles are ordered in chunks of
// SORT_CHUNK slots (each sorted by one block in shared memory, then each
// particle ranked by binary searches in the cell's other chunks); smaller
// ones by per-slot counting (O(count^2) per cell, every slot in parallel).
constexpr uint32_t SORT_SMALL = 512, SORT_CHUNK = 4096;
// work items (cell, chunk) the reorder can list: at most one partial chunk
// per big cell beyond the full chunks
inline uint32_t big_item_cap(uint32_t max_particles) {
  return max_particles / SORT_CHUNK + max_particles / (SORT_SMALL + 1) + 1;
}

inline uint32_t scan_tiles(uint32_t total_cells) {
  return (total_cells + SCAN_TILE - 1) / SCAN_TILE;
}

// n_canon: canonical particles of all scenes; n_sorted: hashed particles.
cudaError_t launch_hash(const DevState &d, uint32_t n_canon, cudaStream_t st);
cudaError_t launch_scan(const DevState &d, uint32_t total_cells, cudaStream_t st);
// The scan kernel on caller-provided scratch: tile_status holds
// scan_tiles(total_cells) descriptors followed by the ticket word, all zero.
cudaError_t launch_scan_with_scratch(const uint32_t *counts, uint32_t *ends, uint32_t total_cells,
                                     unsigned long long *tile_status, uint32_t *err,
                                     cudaStream_t st);
// The scan on caller-provided scratch of scan_tiles(total_cells) + 2 zeroed
// words; inject = every look-back wait runs out (the failure-detection
// self-test, fs_selftest_scan_wait).
cudaError_t launch_scan_selftest(const uint32_t *counts, uint32_t *ends, uint32_t total_cells,
                                 unsigned long long *tile_status, uint32_t *err, bool inject,
                                 cudaStream_t st);
cudaError_t launch_scatter(const DevState &d, uint32_t n_canon, cudaStream_t st);
cudaError_t launch_sort_gather(const DevState &d, uint32_t n_sorted, cudaStream_t st);
// 64-byte AoS records of canonical particles or sorted slots [first, first + count)
cudaError_t launch_export_aos(const DevState &d, bool sorted, uint32_t first, uint32_t count,
                              void *out, cudaStream_t st);
cudaError_t launch_dir_table(const DevState &d, cudaStream_t st);
cudaError_t launch_density(const DevState &d, uint32_t n, cudaStream_t st);
constexpr int TASK_COUNTERS = 16;
constexpr int KEY_BUCKETS = 8192;
// Warp order (before density) and the force pass's hit permutation (after it).
cudaError_t launch_order_warps(const DevState &d, uint32_t n, cudaStream_t st);
cudaError_t launch_order_hits(const DevState &d, uint32_t n, cudaStream_t st);
cudaError_t launch_xsph(const DevState &d, uint32_t n, cudaStream_t st);
cudaError_t launch_force_predict(const DevState &d, uint32_t n, cudaStream_t st);
cudaError_t launch_solve(const DevState &d, uint32_t n, int iter, int last,
                         cudaStream_t st);
cudaError_t launch_rigid_frame(const DevState &d, uint32_t n_scenes, uint32_t substeps,
                               cudaStream_t st);
cudaError_t launch_rigid_sync(const DevState &d, uint32_t n_scenes, cudaStream_t st);
cudaError_t launch_finalize_integrate(const DevState &d, uint32_t n, int final_buf,
                                      cudaStream_t st);

}  // namespace fs
