// grid_kernels.cu — uniform-grid build for the SPH step on sm_103a:
// hash + count, single-pass decoupled-lookback scan, and a stable counting
// sort that gathers the particle records into grid order.
//
// Reference stages (WGSL, src/shaders/): grid_clear.wgsl:23-29,
// grid_build.wgsl:33-62, prefix_scan.wgsl:38-122 (+ the counts->starts copy at
// sph_3d_grid.rs:1295-1301), grid_reorder.wgsl:37-63.
//
// Output conventions match the reference buffers bit for bit:
//   cell_counts[c]            particles hashed into cell c
//   cell_starts[c]            INCLUSIVE prefix end of cell c; this library
//                             stores cell_begin[0..total] with cell_begin[0]=0
//                             so that cell_starts == cell_begin + 1
//   particle_cell_indices[i]  sorted slot of particle i (after reorder)
//   sorted_to_orig[s]         particle in sorted slot s
// Slot order inside a cell is ascending particle index (stable). The
// reference's atomicAdd slot makes that order unspecified; a stable order makes
// every later summation deterministic.
#include <cuda/atomic>

#include "fs_internal.h"

namespace fs {
namespace {

// position_to_cell + clamped cell_to_index, grid_build.wgsl:33-44.
// floor((p - origin) * inv) converted with saturation (cvt.rmi), then clamped.
__device__ __forceinline__ uint32_t hash_cell(float4 p, const GpuGridParams &g) {
  int cx = __float2int_rd((p.x - g.grid_origin_x) * g.inv_cell_size);
  int cy = __float2int_rd((p.y - g.grid_origin_y) * g.inv_cell_size);
  int cz = __float2int_rd((p.z - g.grid_origin_z) * g.inv_cell_size);
  cx = min(max(cx, 0), int(g.grid_size_x) - 1);
  cy = min(max(cy, 0), int(g.grid_size_y) - 1);
  cz = min(max(cz, 0), int(g.grid_size_z) - 1);
  return uint32_t(cx) + uint32_t(cy) * g.grid_size_x +
         uint32_t(cz) * g.grid_size_x * g.grid_size_y;
}

// Hash + count with warp-aggregated atomics: lanes holding the same cell
// (found with __match_any_sync) elect one leader that adds the group's size;
// every lane keeps its arrival rank (leader's old count + rank among peers).
// Each scene owns a block of the global cell arrays (c_offset), so one pass
// hashes every scene; particles beyond a scene's effective count stay out.
__global__ void __launch_bounds__(256) k_hash(const float4 *__restrict__ pos, SceneView v,
                                              uint32_t *__restrict__ cell_of,
                                              uint32_t *__restrict__ rank_of,
                                              uint32_t *__restrict__ counts) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool active = i < v.b->n_canon;
  uint32_t cell = 0;
  if (active) {
    const DevUniforms *U = v.u + v.scene_of[i];
    active = i - U->p_offset < U->n;
    if (active) cell = U->c_offset + hash_cell(pos[i], U->grid);
  }
  const unsigned act = __ballot_sync(0xffffffffu, active);
  if (!active) return;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned peers = __match_any_sync(act, cell);
  const int leader = __ffs(peers) - 1;
  const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
  uint32_t base = 0;
  if (int(lane) == leader) base = atomicAdd(&counts[cell], uint32_t(__popc(peers)));
  base = __shfl_sync(peers, base, leader);
  cell_of[i] = cell;
  rank_of[i] = base + rank;
}

// ---- single-pass scan (decoupled look-back) --------------------------------
// Tile descriptor: bits 32-33 flag (0 none, 1 tile aggregate, 2 inclusive
// prefix), bits 0-31 value. Tiles are processed in ticket order, so a tile
// only waits for predecessors that are already running and publish their
// aggregate before they wait on anyone: no deadlock. Each poll loop is still
// bounded; on expiry the kernel records ERR_SCAN_TIMEOUT and continues.
constexpr unsigned long long FLAG_AGG = 1ull << 32;
constexpr unsigned long long FLAG_PRE = 2ull << 32;
constexpr int LOOKBACK_POLL_LIMIT = 1 << 22;
// Failure-detection self-test (fs_selftest_scan_wait): the look-back polls a
// word that nothing ever publishes, with this short bound, so every wait of a
// tile after the first runs out on every call; the kernel then finishes as
// after a real expiry (a wrong prefix, the expiry recorded in the error word).
constexpr int INJECTED_POLL_LIMIT = 64;

__device__ __forceinline__ void publish(unsigned long long *slot, unsigned long long v) {
  cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> r(*slot);
  r.store(v, cuda::memory_order_release);
}
__device__ __forceinline__ unsigned long long peek(unsigned long long *slot) {
  cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> r(*slot);
  return r.load(cuda::memory_order_acquire);
}

template <bool kInjectExpiry>
__global__ void __launch_bounds__(SCAN_THREADS)
    k_scan(const uint32_t *__restrict__ counts, uint32_t *__restrict__ ends,
           uint32_t total, unsigned long long *tile_status, uint32_t *tile_ticket,
           uint32_t *err, unsigned long long *never_published) {
  // items staged through shared memory; padded to avoid bank conflicts when
  // each thread walks its 16 consecutive items.
  __shared__ uint32_t sm[SCAN_TILE + SCAN_TILE / 32];
  __shared__ uint32_t s_warp[SCAN_THREADS / 32];
  __shared__ uint32_t s_tile, s_exclusive;
  const int t = threadIdx.x;
  const int lane = t & 31, warp = t >> 5;
  if (t == 0) s_tile = atomicAdd(tile_ticket, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const size_t base = size_t(tile) * SCAN_TILE;

#define PAD(k) ((k) + ((k) >> 5))
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    const size_t g = base + size_t(k) * SCAN_THREADS + t;
    const int li = k * SCAN_THREADS + t;
    sm[PAD(li)] = g < total ? counts[g] : 0u;
  }
  __syncthreads();
  uint32_t v[SCAN_ITEMS];
  uint32_t run = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    run += sm[PAD(t * SCAN_ITEMS + k)];
    v[k] = run;
  }
  // block-wide exclusive scan of the per-thread totals
  uint32_t x = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < SCAN_THREADS / 32 ? s_warp[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < SCAN_THREADS / 32) s_warp[lane] = w;  // inclusive warp sums
  }
  __syncthreads();
  const uint32_t warp_excl = warp > 0 ? s_warp[warp - 1] : 0u;
  const uint32_t thread_excl = warp_excl + x - run;
  const uint32_t tile_sum = s_warp[SCAN_THREADS / 32 - 1];

  // look-back by warp 0
  if (warp == 0) {
    if (tile == 0) {
      if (lane == 0) {
        publish(&tile_status[0], FLAG_PRE | tile_sum);
        s_exclusive = 0;
      }
    } else {
      if (lane == 0) publish(&tile_status[tile], FLAG_AGG | tile_sum);
      uint32_t exclusive = 0;
      int window_end = int(tile) - 1;  // closest predecessor
      bool done = false;
      bool timed_out = false;
      while (!done) {
        const int idx = window_end - lane;
        unsigned long long d = FLAG_PRE;  // lanes before tile 0 read "prefix 0"
        if (idx >= 0) {
          int polls = 0;
          unsigned long long *slot = kInjectExpiry ? never_published : &tile_status[idx];
          const int limit = kInjectExpiry ? INJECTED_POLL_LIMIT : LOOKBACK_POLL_LIMIT;
          d = peek(slot);
          while ((d >> 32) == 0ull) {
            if (++polls > limit) {
              timed_out = true;
              d = FLAG_PRE;  // give up: treat as zero prefix
              break;
            }
            __nanosleep(64);
            d = peek(slot);
          }
        }
        const unsigned pre_mask = __ballot_sync(0xffffffffu, (d >> 32) == 2ull);
        const uint32_t val = idx >= 0 ? uint32_t(d & 0xffffffffull) : 0u;
        if (pre_mask) {
          const int first = __ffs(pre_mask) - 1;  // nearest inclusive prefix
          uint32_t contrib = lane <= first ? val : 0u;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(0xffffffffu, contrib, o);
          exclusive += contrib;
          done = true;
        } else {
          uint32_t contrib = val;
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(0xffffffffu, contrib, o);
          exclusive += contrib;
          window_end -= 32;
        }
      }
      if (__any_sync(0xffffffffu, timed_out) && lane == 0) atomicOr(err, ERR_SCAN_TIMEOUT);
      if (lane == 0) {
        publish(&tile_status[tile], FLAG_PRE | (exclusive + tile_sum));
        s_exclusive = exclusive;
      }
    }
  }
  __syncthreads();
  const uint32_t off = s_exclusive + thread_excl;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) sm[PAD(t * SCAN_ITEMS + k)] = off + v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    const size_t g = base + size_t(k) * SCAN_THREADS + t;
    if (g < total) ends[g] = sm[PAD(k * SCAN_THREADS + t)];
  }
#undef PAD
}

// Scatter every hashed particle to its unsorted slot: begin[cell] + arrival rank.
__global__ void __launch_bounds__(256) k_scatter(SceneView v, const uint32_t *__restrict__ cell_of,
                                                 const uint32_t *__restrict__ rank_of,
                                                 const uint32_t *__restrict__ begin,
                                                 uint32_t *__restrict__ t_tmp) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.b->n_canon) return;
  const DevUniforms *U = v.u + v.scene_of[i];
  if (i - U->p_offset >= U->n) return;
  t_tmp[begin[cell_of[i]] + rank_of[i]] = i;
}

// Stable counting sort, second half: slot s of the unsorted order holds
// particle v; its final slot is begin[cell] + #{particles of the cell with a
// smaller index}. The record is gathered into grid order (grid_reorder.wgsl:
// 54-62) and both index maps and the slot's scene are written.
__device__ __forceinline__ void gather_slot(const SceneView &sv, uint32_t v, uint32_t d,
                                            const float4 *__restrict__ p_pos,
                                            const float4 *__restrict__ p_vel,
                                            const float4 *__restrict__ p_force,
                                            float4 *__restrict__ s_pos, float4 *__restrict__ s_vel,
                                            float4 *__restrict__ s_frc, uint32_t *__restrict__ s2o,
                                            uint32_t *__restrict__ cidx,
                                            uint16_t *__restrict__ scene_of_slot) {
  s2o[d] = v;
  cidx[v] = d;
  scene_of_slot[d] = sv.scene_of[v];
  s_pos[d] = p_pos[v];
  s_vel[d] = p_vel[v];
  s_frc[d] = p_force[v];
}

// Per slot, counting the cell's smaller indices (O(count^2) per cell); the
// cells with more than SORT_SMALL particles are listed instead, as one work
// item per chunk of SORT_CHUNK slots, for k_big_sort and k_big_rank.
__global__ void __launch_bounds__(256)
    k_sort_gather(SceneView sv, const uint32_t *__restrict__ t_tmp,
                  const uint32_t *__restrict__ cell_of, const uint32_t *__restrict__ begin,
                  const float4 *__restrict__ p_pos, const float4 *__restrict__ p_vel,
                  const float4 *__restrict__ p_force, float4 *__restrict__ s_pos,
                  float4 *__restrict__ s_vel, float4 *__restrict__ s_frc,
                  uint32_t *__restrict__ s2o, uint32_t *__restrict__ cidx,
                  uint16_t *__restrict__ scene_of_slot, uint32_t *__restrict__ big) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= sv.b->n_sorted) return;
  const uint32_t v = t_tmp[s];
  const uint32_t c = cell_of[v];
  const uint32_t b = begin[c], e = begin[c + 1];
  if (e - b > SORT_SMALL) {
    if (s == b) {
      const uint32_t chunks = (e - b + SORT_CHUNK - 1u) / SORT_CHUNK;
      const uint32_t first = atomicAdd(&big[0], chunks);
      for (uint32_t q = 0; q < chunks; q++) {
        big[4 + 2 * (first + q)] = c;
        big[4 + 2 * (first + q) + 1] = q;
      }
    }
    return;
  }
  uint32_t rank = 0;
  for (uint32_t k = b; k < e; k++) rank += (t_tmp[k] < v) ? 1u : 0u;
  gather_slot(sv, v, b + rank, p_pos, p_vel, p_force, s_pos, s_vel, s_frc, s2o, cidx,
              scene_of_slot);
}

// Takes the next listed item for the whole block from ticket counter `t`;
// false when none is left. Sets the item's cell range and chunk.
__device__ __forceinline__ bool next_big_item(uint32_t *big, int t, const uint32_t *begin,
                                              uint32_t &b, uint32_t &m, uint32_t &q) {
  __shared__ uint32_t s_item;
  __syncthreads();  // the block is done with the previous item
  if (threadIdx.x == 0) s_item = atomicAdd(&big[t], 1u);
  __syncthreads();
  const uint32_t item = s_item;
  if (item >= big[0]) return false;
  const uint32_t c = big[4 + 2 * item];
  q = big[4 + 2 * item + 1];
  b = begin[c];
  m = begin[c + 1] - b;
  return true;
}

// Sorts each listed chunk of t_tmp ascending in place (bitonic network in
// shared memory, padded to a power of two with 0xffffffff; the particle
// indices are distinct).
constexpr unsigned BIG_THREADS = 512;
__global__ void __launch_bounds__(BIG_THREADS) k_big_sort(uint32_t *__restrict__ t_tmp,
                                                          const uint32_t *__restrict__ begin,
                                                          uint32_t *__restrict__ big) {
  __shared__ uint32_t ids[SORT_CHUNK];
  const unsigned t = threadIdx.x;
  uint32_t b, m, q;
  while (next_big_item(big, 1, begin, b, m, q)) {
    const uint32_t lo = b + q * SORT_CHUNK, len = min(SORT_CHUNK, m - q * SORT_CHUNK);
    uint32_t P = 1u;
    while (P < len) P <<= 1;
    for (uint32_t i = t; i < P; i += BIG_THREADS) ids[i] = i < len ? t_tmp[lo + i] : 0xffffffffu;
    __syncthreads();
    for (uint32_t k = 2; k <= P; k <<= 1) {
      for (uint32_t j = k >> 1; j > 0; j >>= 1) {
        for (uint32_t r = t; r < P / 2; r += BIG_THREADS) {
          const uint32_t i0 = ((r & ~(j - 1u)) << 1) | (r & (j - 1u));  // bit j clear
          const uint32_t i1 = i0 | j;
          const uint32_t x = ids[i0], y = ids[i1];
          if ((x > y) == ((i0 & k) == 0u)) {
            ids[i0] = y;
            ids[i1] = x;
          }
        }
        __syncthreads();
      }
    }
    for (uint32_t i = t; i < len; i += BIG_THREADS) t_tmp[lo + i] = ids[i];
  }
}

// Number of entries of the ascending run a[0, len) below v.
__device__ __forceinline__ uint32_t count_below(const uint32_t *__restrict__ a, uint32_t len,
                                                uint32_t v) {
  uint32_t lo = 0u, hi = len;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < v) lo = mid + 1u;
    else hi = mid;
  }
  return lo;
}

// The particles of each listed chunk: rank = position in its sorted chunk +
// the entries below it in the cell's other chunks; gathered into grid order.
__global__ void __launch_bounds__(BIG_THREADS)
    k_big_rank(SceneView sv, const uint32_t *__restrict__ t_tmp,
               const uint32_t *__restrict__ begin, const float4 *__restrict__ p_pos,
               const float4 *__restrict__ p_vel, const float4 *__restrict__ p_force,
               float4 *__restrict__ s_pos, float4 *__restrict__ s_vel,
               float4 *__restrict__ s_frc, uint32_t *__restrict__ s2o,
               uint32_t *__restrict__ cidx, uint16_t *__restrict__ scene_of_slot,
               uint32_t *__restrict__ big) {
  uint32_t b, m, q;
  while (next_big_item(big, 2, begin, b, m, q)) {
    const uint32_t lo = b + q * SORT_CHUNK, len = min(SORT_CHUNK, m - q * SORT_CHUNK);
    const uint32_t chunks = (m + SORT_CHUNK - 1u) / SORT_CHUNK;
    for (uint32_t i = threadIdx.x; i < len; i += BIG_THREADS) {
      const uint32_t v = t_tmp[lo + i];
      uint32_t rank = i;
      for (uint32_t r = 0; r < chunks; r++)
        if (r != q)
          rank += count_below(t_tmp + b + r * SORT_CHUNK, min(SORT_CHUNK, m - r * SORT_CHUNK), v);
      gather_slot(sv, v, b + rank, p_pos, p_vel, p_force, s_pos, s_vel, s_frc, s2o, cidx,
                  scene_of_slot);
    }
  }
}

inline unsigned blocks_for(uint32_t n, unsigned threads) {
  return unsigned((n + threads - 1) / threads);
}

}  // namespace

// counts must be zeroed by the caller (the grid_clear stage).
cudaError_t launch_hash(const DevState &d, uint32_t n_canon, cudaStream_t st) {
  if (n_canon == 0) return cudaSuccess;
  k_hash<<<blocks_for(n_canon, 256), 256, 0, st>>>(d.p_pos, d.view(), d.cell_of, d.rank_of,
                                                   d.counts);
  return cudaGetLastError();
}

cudaError_t launch_scan(const DevState &d, uint32_t total_cells, cudaStream_t st) {
  const uint32_t tiles = scan_tiles(total_cells);
  // descriptors and the ticket counter (stored right after them) start at 0
  cudaError_t e = cudaMemsetAsync(d.tile_status, 0,
                                  sizeof(unsigned long long) * (size_t(tiles) + 1), st);
  if (e != cudaSuccess) return e;
  k_scan<false><<<tiles, SCAN_THREADS, 0, st>>>(d.counts, d.cell_begin + 1, total_cells,
                                                d.tile_status, d.tile_ticket, d.err, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_scan_with_scratch(const uint32_t *counts, uint32_t *ends, uint32_t total_cells,
                                     unsigned long long *tile_status, uint32_t *err,
                                     cudaStream_t st) {
  if (total_cells == 0) return cudaSuccess;
  const uint32_t tiles = scan_tiles(total_cells);
  k_scan<false><<<tiles, SCAN_THREADS, 0, st>>>(
      counts, ends, total_cells, tile_status, reinterpret_cast<uint32_t *>(tile_status + tiles),
      err, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_scan_selftest(const uint32_t *counts, uint32_t *ends, uint32_t total_cells,
                                 unsigned long long *tile_status, uint32_t *err, bool inject,
                                 cudaStream_t st) {
  if (total_cells == 0) return cudaSuccess;
  const uint32_t tiles = scan_tiles(total_cells);
  // tile_status: tiles descriptors, the ticket word, then the word that the
  // injected form polls and nothing writes (all cleared by the caller)
  uint32_t *ticket = reinterpret_cast<uint32_t *>(tile_status + tiles);
  if (inject)
    k_scan<true><<<tiles, SCAN_THREADS, 0, st>>>(counts, ends, total_cells, tile_status, ticket,
                                                 err, tile_status + tiles + 1);
  else
    k_scan<false><<<tiles, SCAN_THREADS, 0, st>>>(counts, ends, total_cells, tile_status, ticket,
                                                  err, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_scatter(const DevState &d, uint32_t n_canon, cudaStream_t st) {
  if (n_canon == 0) return cudaSuccess;
  k_scatter<<<blocks_for(n_canon, 256), 256, 0, st>>>(d.view(), d.cell_of, d.rank_of,
                                                      d.cell_begin, d.t_tmp);
  return cudaGetLastError();
}

namespace {
// 64-byte SphParticle3D records (particle.rs:8-17) packed from the SoA
// arrays into caller device memory: position + pad, velocity + pad,
// force + density, near density + normal. Four threads per record, one
// 16-byte quarter each, so consecutive threads store consecutive quarters.
__global__ void __launch_bounds__(256)
    k_export_aos(uint32_t count, bool sorted, const float4 *__restrict__ pos,
                 const float4 *__restrict__ vel, const float4 *__restrict__ frc,
                 const float4 *__restrict__ aux, const float2 *__restrict__ dens,
                 const float4 *__restrict__ nrm, float4 *__restrict__ out) {
  const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= uint64_t(count) * 4u) return;
  const uint32_t i = uint32_t(t >> 2), q = uint32_t(t & 3u);
  float4 v;
  if (q == 0u) {
    v = pos[i];
  } else if (q == 1u) {
    v = vel[i];
  } else if (sorted) {
    const float2 d = dens[i];
    if (q == 2u) {
      const float4 f = frc[i];
      v = make_float4(f.x, f.y, f.z, d.x);
    } else {
      const float4 n = nrm[i];
      v = make_float4(d.y, n.x, n.y, n.z);
    }
  } else {
    const float4 a0 = aux[2 * size_t(i)];
    if (q == 2u) {
      const float4 f = frc[i];
      v = make_float4(f.x, f.y, f.z, a0.x);
    } else {
      v = make_float4(a0.y, a0.z, a0.w, aux[2 * size_t(i) + 1].x);
    }
  }
  out[t] = v;
}
}  // namespace

cudaError_t launch_export_aos(const DevState &d, bool sorted, uint32_t first, uint32_t count,
                              void *out, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  const uint64_t threads = uint64_t(count) * 4u;
  const unsigned blocks = unsigned((threads + 255u) / 256u);
  if (sorted)
    k_export_aos<<<blocks, 256, 0, st>>>(count, true, d.s_pos + first, d.s_vel + first,
                                         d.s_frc + first, nullptr, d.s_dens + first,
                                         d.s_nrm + first, static_cast<float4 *>(out));
  else
    k_export_aos<<<blocks, 256, 0, st>>>(count, false, d.p_pos + first, d.p_vel + first,
                                         d.p_force + first, d.p_aux + 2 * size_t(first), nullptr,
                                         nullptr, static_cast<float4 *>(out));
  return cudaGetLastError();
}

cudaError_t launch_sort_gather(const DevState &d, uint32_t n_sorted, cudaStream_t st) {
  if (n_sorted == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(d.big_cells, 0, 4 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  k_sort_gather<<<blocks_for(n_sorted, 256), 256, 0, st>>>(
      d.view(), d.t_tmp, d.cell_of, d.cell_begin, d.p_pos, d.p_vel, d.p_force, d.s_pos, d.s_vel,
      d.s_frc, d.s2o, d.cidx, d.scene_of_slot, d.big_cells);
  const unsigned blocks = 4u * unsigned(d.sm_count);
  k_big_sort<<<blocks, BIG_THREADS, 0, st>>>(d.t_tmp, d.cell_begin, d.big_cells);
  k_big_rank<<<blocks, BIG_THREADS, 0, st>>>(d.view(), d.t_tmp, d.cell_begin, d.p_pos, d.p_vel,
                                             d.p_force, d.s_pos, d.s_vel, d.s_frc, d.s2o, d.cidx,
                                             d.scene_of_slot, d.big_cells);
  return cudaGetLastError();
}

}  // namespace fs
