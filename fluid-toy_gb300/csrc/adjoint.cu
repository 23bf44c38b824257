// adjoint.cu — the differentiable rollout behind fs_adj_* (include/fluidsph.h).
//
// No counterpart in the reference: it differentiates SphSimulation3DGrid's
// step (sph_3d_grid.rs:1261-1444) with respect to the initial state and the
// viscosity / surface-tension parameters. Forward records: it runs the steps
// on the simulation's graphs and keeps the canonical state (x, v) every
// `checkpoint_every` steps. Backward consumes cotangents of the final state:
// segment by segment from the last, it restores the segment's checkpoint,
// re-runs its steps once more while recording each step's intermediates (the
// sorted state, densities, normals, XSPH velocities, accelerations and every
// PCISPH level) into a tape, then reverses the recorded steps one by one
// with the kernels of adj_kernels.cu. Memory: the checkpoints, one segment of
// tape and the reverse accumulators.
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <vector>

#include "adj_internal.h"
#include "fs_sim.h"

using namespace fs;

namespace {

struct TapeSlot {
  uint32_t *s2o;
  uint16_t *sos;
  uint32_t *cell_begin;
  float4 *pos, *vel, *nrm, *vhat, *anp, *vfin;
  float2 *dens;
  float4 *xp[kMaxAdjIters + 1];
  float *rho[kMaxAdjIters + 1];
  float4 *ap[kMaxAdjIters];
  uint32_t *order;
  uint32_t *mask_words, *mask_off, *perm_hit;
  uint32_t *hits;  // union of the PCISPH levels' hit masks, same layout as mask_words
  size_t mask_cap;
};

// Hit-mask words a tape slot holds: 96 per particle on average (3,072
// candidates) plus a floor; particles beyond the capacity fall back to
// testing their candidates, in the forward and in the reverse pass alike.
size_t tape_mask_cap(size_t n) { return 96 * n + (size_t(1) << 16); }

size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

struct Carve {
  char *base;
  size_t off = 0;
  template <class T>
  T *take(size_t count) {
    T *p = reinterpret_cast<T *>(base ? base + off : nullptr);
    off += a256(sizeof(T) * std::max<size_t>(count, 1));
    return p;
  }
};

}  // namespace

struct FsAdj {
  FsSim *sim = nullptr;
  uint32_t every = 1;
  // shape at recording
  uint32_t K = 0, N = 0, G = 0, scenes = 0;
  uint32_t steps = 0;
  std::vector<DevUniforms> hu_snapshot;
  // checkpoints [nck][2][N] and the final state [2][N]
  float4 *ck = nullptr;
  size_t ck_slots = 0;
  float4 *final_state = nullptr;
  // one segment of tape + reverse accumulators + cotangents
  void *work = nullptr;
  size_t work_bytes = 0;
  uint32_t work_N = 0, work_G = 0, work_K = 0, work_every = 0, work_scenes = 0, work_segs = 0,
           work_bufs = 0;
  // tape buffers: bufs buffers of `every` recorded steps, slot b * every + t
  std::vector<TapeSlot> tape;
  uint32_t segs = 1;             // segments the forward records (the last segs)
  // With strict checkpointing (segs == 1) and two or more segments, a second
  // buffer lets the backward re-run segment s-1 on `side` while segment s is
  // reversed on the simulation's stream (bufs = 2); else bufs = segs.
  uint32_t bufs = 1;
  bool pipe_wanted = false;      // the next workspace should hold the second buffer
  bool pipe_failed = false;      // it did not fit once: no second buffer
  cudaStream_t side = nullptr;
  cudaEvent_t ev_start = nullptr, ev_rec[2] = {}, ev_free[2] = {};
  uint64_t tape_budget = 0;      // bytes the caller allows for tape buffers (0: one segment)
  uint32_t seg_limit = ~0u;      // 1 after the budget's buffers failed to allocate
  std::vector<int64_t> buf_seg;  // checkpoint segment each buffer holds (-1: none)
  AdjView av{};
  float4 *cot[2][2] = {};  // [buffer][0 = d/d pos, 1 = d/d vel], canonical
  int cur = 0;
  bool seeded = false;
  std::vector<double> param_grads;  // last backward: FS_ADJ_NUM_PARAMS per scene
  // loss scratch
  float *field = nullptr, *target = nullptr, *gg = nullptr;
  double *loss = nullptr, *partial = nullptr;
  size_t vox_cap = 0, loss_cap = 0;
  int lanes = 0;  // lanes per particle of the reverse gathers (autotuned)
  uint32_t *scene_first = nullptr, *scene_count = nullptr;  // device, canonical ranges
};

namespace {

void free_adj(FsAdj *a) {
  if (a->ck) cudaFree(a->ck);
  if (a->final_state) cudaFree(a->final_state);
  if (a->work) cudaFree(a->work);
  if (a->field) cudaFree(a->field);
  a->ck = a->final_state = nullptr;
  a->work = nullptr;
  a->field = nullptr;
}

// One recorded step's buffers.
void carve_slot(Carve &c, TapeSlot &t, size_t N, size_t G, uint32_t K) {
  {
    t.s2o = c.take<uint32_t>(N);
    t.sos = c.take<uint16_t>(N);
    t.cell_begin = c.take<uint32_t>(G + 1);
    t.pos = c.take<float4>(N);
    t.vel = c.take<float4>(N);
    t.nrm = c.take<float4>(N);
    t.vhat = c.take<float4>(N);
    t.anp = c.take<float4>(N);
    t.vfin = c.take<float4>(N);
    t.dens = c.take<float2>(N);
    for (uint32_t k = 0; k <= K; k++) {
      t.xp[k] = c.take<float4>(N);
      t.rho[k] = c.take<float>(N);
    }
    for (uint32_t k = 0; k < K; k++) t.ap[k] = c.take<float4>(N);
    t.order = c.take<uint32_t>((N + 31) / 32);
    t.mask_cap = tape_mask_cap(N);
    t.mask_words = c.take<uint32_t>(t.mask_cap);
    t.mask_off = c.take<uint32_t>(N);
    t.perm_hit = c.take<uint32_t>(N);
    t.hits = c.take<uint32_t>(t.mask_cap);
  }
}

// Bytes of one checkpoint segment's tape (`every` recorded steps).
uint64_t segment_bytes(const FsAdj *a) {
  Carve c{nullptr};
  TapeSlot t{};
  carve_slot(c, t, a->N, a->G, a->K);
  return uint64_t(c.off) * a->every;
}

// Lay out (or size, when base == nullptr) the tape, accumulators and cotangents.
void carve_work(FsAdj *a, char *base, size_t *bytes) {
  Carve c{base};
  const size_t N = a->N, G = a->G;
  a->tape.assign(size_t(a->bufs) * a->every, TapeSlot{});
  for (TapeSlot &t : a->tape) carve_slot(c, t, N, G, a->K);
  AdjView &v = a->av;
  v.gx = c.take<float4>(N);
  v.gvhat = c.take<float4>(N);
  v.gv = c.take<float4>(N);
  v.ga = c.take<float4>(N);
  v.gn = c.take<float4>(N);
  v.grho = c.take<float2>(N);
  v.gp = c.take<float>(N);
  v.lv[0] = c.take<float4>(2 * size_t(N));
  v.lv[1] = c.take<float4>(2 * size_t(N));
  v.frec = c.take<float4>(5 * size_t(N));
  v.gparam = c.take<double>(3 * size_t(a->scenes));
  v.gparam2 = c.take<double>(2 * size_t(a->scenes));
  v.gpart = c.take<double2>(N);
  v.gpart2 = c.take<double2>(N);
  a->scene_first = c.take<uint32_t>(a->scenes);
  a->scene_count = c.take<uint32_t>(a->scenes);
  v.counters = c.take<uint32_t>(kMaxAdjIters + 3);
  for (auto &b : a->cot)
    for (auto &p : b) p = c.take<float4>(N);
  *bytes = c.off;
}

int ensure_work(FsAdj *a) {
  const uint32_t want_bufs =
      a->segs + ((a->segs == 1 && a->pipe_wanted && !a->pipe_failed) ? 1u : 0u);
  if (a->work && a->work_N == a->N && a->work_G == a->G && a->work_K == a->K &&
      a->work_every == a->every && a->work_scenes == a->scenes && a->work_segs == a->segs &&
      a->work_bufs == want_bufs)
    return FS_OK;
  FsSim *s = a->sim;
  if (a->work) {
    FS_CUDA(cudaStreamSynchronize(s->stream), "adjoint workspace");
    cudaFree(a->work);
    a->work = nullptr;
  }
  a->bufs = want_bufs;
  carve_work(a, nullptr, &a->work_bytes);
  if (cudaMalloc(&a->work, a->work_bytes) != cudaSuccess && a->bufs > 1) {
    // the budget's extra tape segments, or the pipelining buffer, do not
    // fit: fall back to one (until the budget changes)
    cudaGetLastError();
    a->work = nullptr;
    if (a->segs > 1) a->seg_limit = 1;
    else a->pipe_failed = true;
    a->segs = 1;
    a->bufs = 1;
    carve_work(a, nullptr, &a->work_bytes);
  }
  if (!a->work) FS_CUDA(cudaMalloc(&a->work, a->work_bytes), "allocate adjoint workspace");
  carve_work(a, static_cast<char *>(a->work), &a->work_bytes);
  // cell_begin[0] of every slot must read 0 (the scan writes from index 1)
  FS_CUDA(cudaMemsetAsync(a->work, 0, a->work_bytes, s->stream), "clear adjoint workspace");
  a->av.err = s->d.err;
  a->work_N = a->N;
  a->work_G = a->G;
  a->work_K = a->K;
  a->work_every = a->every;
  a->work_segs = a->segs;
  a->work_bufs = a->bufs;
  a->buf_seg.assign(a->bufs, -1);
  a->work_scenes = a->scenes;
  return FS_OK;
}

// The simulation's buffers with the step's outputs redirected into slot t.
DevState recording_state(const FsAdj *a, const TapeSlot &t) {
  DevState dv = a->sim->d;
  dv.s2o = t.s2o;
  dv.scene_of_slot = t.sos;
  dv.cell_begin = t.cell_begin;
  dv.s_pos = t.pos;
  dv.s_vel = t.vel;
  dv.s_nrm = t.nrm;
  dv.s_dens = t.dens;
  dv.vel_x = t.vhat;
  dv.anp = t.anp;
  dv.pred_v = t.vfin;
  dv.rec_xp = t.xp;
  dv.rec_rho = t.rho;
  dv.rec_ap = t.ap;
  dv.warp_order = t.order;
  dv.mask_words = t.mask_words;
  dv.mask_off = t.mask_off;
  dv.mask_cap = t.mask_cap;
  dv.perm_hit = t.perm_hit;
  dv.rec_hits = t.hits;
  return dv;
}

TapeView tape_view(const TapeSlot &t, uint32_t K) {
  TapeView v{};
  v.s2o = t.s2o;
  v.scene_of_slot = t.sos;
  v.cell_begin = t.cell_begin;
  v.pos = t.pos;
  v.vel = t.vel;
  v.nrm = t.nrm;
  v.vhat = t.vhat;
  v.anp = t.anp;
  v.vfin = t.vfin;
  v.dens = t.dens;
  for (uint32_t k = 0; k <= K; k++) {
    v.xp[k] = t.xp[k];
    v.rho[k] = t.rho[k];
  }
  for (uint32_t k = 0; k < K; k++) v.ap[k] = t.ap[k];
  v.order = t.order;
  v.mask_words = t.mask_words;
  v.mask_off = t.mask_off;
  v.perm_hit = t.perm_hit;
  v.hits = t.hits;
  return v;
}

int copy_state(FsSim *s, float4 *dst_pos, float4 *dst_vel, const float4 *src_pos,
               const float4 *src_vel, uint32_t n) {
  FS_CUDA(cudaMemcpyAsync(dst_pos, src_pos, sizeof(float4) * n, cudaMemcpyDeviceToDevice,
                          s->stream),
          "copy state");
  FS_CUDA(cudaMemcpyAsync(dst_vel, src_vel, sizeof(float4) * n, cudaMemcpyDeviceToDevice,
                          s->stream),
          "copy state");
  return FS_OK;
}

// What the reverse pass differentiates: every particle active, mouse force
// and rigid body off, at most kMaxAdjIters PCISPH iterations.
int check_supported(const char *who, FsSim *s) {
  if (s->iterations > uint32_t(kMaxAdjIters))
    return fail(FS_E_STATE, "%s: %u PCISPH iterations (at most %d are differentiated)", who,
                s->iterations, kMaxAdjIters);
  if (s->hb.n_sorted != s->hb.n_canon)
    return fail(FS_E_STATE, "%s: every particle must be active (num_particles >= count)", who);
  for (uint32_t k = 0; k < s->scenes(); k++) {
    if (s->hu[k].mouse.is_active == 1u)
      return fail(FS_E_STATE, "%s: scene %u: the mouse force is not differentiated", who, k);
    if (s->hu[k].rigid.is_active != 0u)
      return fail(FS_E_STATE, "%s: scene %u: the rigid-body coupling is not differentiated", who,
                  k);
  }
  return FS_OK;
}

// Autotuner of the reverse gathers' lanes per particle, per particle-count
// bucket (floor(log2 N)) and iteration count: on the first backward of a
// bucket every candidate runs the last recorded step's reverse once (the
// reverse of a step is idempotent apart from the parameter sums, which are
// cleared afterwards) and the fastest is kept for the process.
std::mutex g_tune_mu;
std::map<uint64_t, int> g_tuned_lanes;

int tune_lanes(FsAdj *a, const SceneView &v, const TapeView &tv) {
  FsSim *s = a->sim;
  uint32_t bucket = 0;
  while ((2u << bucket) <= a->N && bucket < 31) bucket++;
  const uint64_t key = (uint64_t(bucket) << 32) | a->K;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned_lanes.find(key);
    if (it != g_tuned_lanes.end()) return it->second;
  }
  cudaEvent_t e0, e1;
  FS_CUDA(cudaEventCreate(&e0), "tuner event");
  FS_CUDA(cudaEventCreate(&e1), "tuner event");
  int best = 1;
  float best_ms = 0.0f;
  const int cand[4] = {1, 2, 4, 8};
  for (int rep = 0; rep < 2; rep++)  // the first pass warms every variant up
    for (int L : cand) {
      cudaEventRecord(e0, s->stream);
      cudaError_t e = launch_adj_step(v, tv, a->av, a->cot[a->cur][0], a->cot[a->cur][1],
                                      a->cot[a->cur ^ 1][0], a->cot[a->cur ^ 1][1], s->d.dir_tab,
                                      s->d.dir_half, a->N, int(a->K), L, s->d.sm_count, s->stream);
      cudaEventRecord(e1, s->stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0.0f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return cuda_fail(e, "reverse-pass tuning");
      }
      if (rep == 1 && (best_ms == 0.0f || ms < best_ms)) {
        best_ms = ms;
        best = L;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  FS_CUDA(cudaMemsetAsync(a->av.gpart, 0, sizeof(double2) * a->N, s->stream),
          "clear parameter gradients");
  FS_CUDA(cudaMemsetAsync(a->av.gpart2, 0, sizeof(double2) * a->N, s->stream),
          "clear parameter gradients");
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tuned_lanes[key] = best;
  return best;
}

// The splat-MSE losses of `count` scenes of the recorded rollout's final
// state: one grid build of the final positions, then per scene the density
// splat, the loss against its target (grid_size^3 floats, host or device) and
// the seeded cotangents of its particles (velocity cotangent 0); the losses
// land in device memory and are read once.
int splat_mse_losses(FsAdj *a, uint32_t count, const uint32_t *scenes,
                     const GpuMcGridParams *grids, const GpuContainerGeometry *geoms,
                     const float *const *targets, int on_device, double *losses,
                     const char *fn) {
  FsSim *s = a->sim;
  if (!a->work) return fail(FS_E_STATE, "%s: no recorded rollout", fn);
  size_t vox_max = 0;
  for (uint32_t k = 0; k < count; k++) {
    if (scenes[k] >= s->scenes())
      return fail(FS_E_INVALID_ARGUMENT, "%s: scene %u of %u", fn, scenes[k], s->scenes());
    if (!targets[k]) return fail(FS_E_INVALID_ARGUMENT, "%s: null target", fn);
    const uint32_t gs = grids[k].grid_size;
    if (gs == 0 || gs > 1024)
      return fail(FS_E_INVALID_ARGUMENT, "%s: grid_size %u outside [1, 1024]", fn, gs);
    const SplatArgs sa = make_splat_args(grids[k], geoms[k], s->hu[scenes[k]].grid);
    if (sa.cell_radius < 1 || sa.cell_radius > 8)
      return fail(FS_E_INVALID_ARGUMENT, "%s: splat radius spans %d cells", fn, sa.cell_radius);
    vox_max = std::max(vox_max, size_t(gs) * gs * gs);
  }
  int rc;
  if ((rc = set_device(s))) return rc;
  if (a->vox_cap < vox_max || a->loss_cap < count) {
    const size_t vox = std::max(vox_max, a->vox_cap);
    const size_t nl = std::max<size_t>({size_t(count), size_t(s->scenes()), a->loss_cap});
    FS_CUDA(cudaStreamSynchronize(s->stream), "loss scratch");
    if (a->field) cudaFree(a->field);
    a->field = nullptr;
    a->vox_cap = a->loss_cap = 0;
    const size_t bytes = a256(sizeof(float) * vox) * 3 + a256(sizeof(double) * nl) +
                         a256(sizeof(double) * (vox / 256 + 1));
    char *p = nullptr;
    FS_CUDA(cudaMalloc(&p, bytes), "allocate loss scratch");
    a->field = reinterpret_cast<float *>(p);
    a->target = reinterpret_cast<float *>(p + a256(sizeof(float) * vox));
    a->gg = reinterpret_cast<float *>(p + 2 * a256(sizeof(float) * vox));
    a->loss = reinterpret_cast<double *>(p + 3 * a256(sizeof(float) * vox));
    a->partial = reinterpret_cast<double *>(p + 3 * a256(sizeof(float) * vox) +
                                            a256(sizeof(double) * nl));
    a->vox_cap = vox;
    a->loss_cap = nl;
  }
  // the final positions, grid-sorted, then per scene its splat and loss
  if ((rc = enqueue_grid_build(s))) return rc;
  for (uint32_t k = 0; k < count; k++) {
    const uint32_t scene = scenes[k];
    const DevUniforms &u = s->hu[scene];
    const SplatArgs sa = make_splat_args(grids[k], geoms[k], u.grid);
    const size_t vox = size_t(grids[k].grid_size) * grids[k].grid_size * grids[k].grid_size;
    FS_CUDA(launch_density_splat(sa, s->d.s_pos, s->d.cell_begin + u.c_offset, a->field,
                                 s->stream),
            "loss splat");
    const float *target = targets[k];
    if (!on_device) {
      FS_CUDA(cudaMemcpyAsync(a->target, targets[k], sizeof(float) * vox,
                              cudaMemcpyHostToDevice, s->stream),
              "upload target");
      target = a->target;
    }
    FS_CUDA(launch_splat_mse(sa, a->field, target, a->gg, a->partial, a->loss + k, s->stream),
            "loss");
    FS_CUDA(launch_splat_adjoint(sa, s->scene_n[scene], s->d.p_pos + u.p_offset, a->gg,
                                 a->cot[a->cur][0] + u.p_offset, s->stream),
            "loss adjoint");
    FS_CUDA(cudaMemsetAsync(a->cot[a->cur][1] + u.p_offset, 0,
                            sizeof(float4) * s->scene_n[scene], s->stream),
            "clear velocity cotangent");
  }
  FS_CUDA(cudaMemcpyAsync(losses, a->loss, sizeof(double) * count, cudaMemcpyDeviceToHost,
                          s->stream),
          "read losses");
  if ((rc = check_device_error(s))) return rc;
  a->seeded = true;
  return FS_OK;
}

#define CHECK_ADJ(a) \
  if (!(a) || !(a)->sim) return fail(FS_E_INVALID_ARGUMENT, "%s: null handle", __func__)

}  // namespace

extern "C" {

int fs_adj_create(FsSim *sim, uint32_t checkpoint_every, FsAdj **out) {
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_adj_create: out is null");
  *out = nullptr;
  if (!sim) return fail(FS_E_INVALID_ARGUMENT, "fs_adj_create: null simulation");
  if (checkpoint_every == 0 || checkpoint_every > 4096)
    return fail(FS_E_INVALID_ARGUMENT, "fs_adj_create: checkpoint_every %u outside [1, 4096]",
                checkpoint_every);
  FsAdj *a = new (std::nothrow) FsAdj();
  if (!a) return fail(FS_E_CAPACITY, "fs_adj_create: out of host memory");
  a->sim = sim;
  a->every = checkpoint_every;
  if (cudaSetDevice(sim->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&a->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&a->ev_start, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&a->ev_rec[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&a->ev_rec[1], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&a->ev_free[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&a->ev_free[1], cudaEventDisableTiming) != cudaSuccess) {
    const cudaError_t e = cudaGetLastError();
    fs_adj_destroy(a);
    return cuda_fail(e, "fs_adj_create: side stream and events");
  }
  *out = a;
  return FS_OK;
}

int fs_adj_set_tape_budget(FsAdj *a, uint64_t bytes) {
  CHECK_ADJ(a);
  a->tape_budget = bytes;
  a->seg_limit = ~0u;
  return FS_OK;
}

int fs_adj_tape_info(FsAdj *a, uint32_t *segments, uint64_t *segment_bytes_out) {
  CHECK_ADJ(a);
  if (segments) *segments = a->work ? a->segs : 0u;
  if (segment_bytes_out) *segment_bytes_out = a->work ? segment_bytes(a) : 0u;
  return FS_OK;
}

int fs_adj_destroy(FsAdj *a) {
  if (!a) return FS_OK;
  if (a->sim) {
    cudaSetDevice(a->sim->device);
    cudaStreamSynchronize(a->sim->stream);
  }
  if (a->side) {
    cudaStreamSynchronize(a->side);
    cudaStreamDestroy(a->side);
  }
  for (cudaEvent_t e : {a->ev_start, a->ev_rec[0], a->ev_rec[1], a->ev_free[0], a->ev_free[1]})
    if (e) cudaEventDestroy(e);
  free_adj(a);
  delete a;
  return FS_OK;
}

int fs_adj_forward(FsAdj *a, uint32_t nsteps) {
  CHECK_ADJ(a);
  FsSim *s = a->sim;
  int rc;
  if ((rc = set_device(s))) return rc;
  if ((rc = check_supported(__func__, s))) return rc;
  if (a->K != s->iterations || a->N != s->hb.n_canon) a->lanes = 0;
  a->K = s->iterations;
  a->N = s->hb.n_canon;
  a->G = s->cells_total;
  a->scenes = s->scenes();
  a->hu_snapshot = s->hu;
  a->steps = 0;
  a->seeded = false;
  const uint32_t nck = (nsteps + a->every - 1) / a->every;
  const size_t need = std::max<size_t>(nck, 1) * 2 * size_t(a->N);
  if (a->ck_slots < need) {
    if (a->ck) {
      FS_CUDA(cudaStreamSynchronize(s->stream), "checkpoints");
      cudaFree(a->ck);
      a->ck = nullptr;
    }
    FS_CUDA(cudaMalloc(&a->ck, sizeof(float4) * need), "allocate checkpoints");
    a->ck_slots = need;
    if (a->final_state) cudaFree(a->final_state);
    a->final_state = nullptr;
  }
  if (!a->final_state)
    FS_CUDA(cudaMalloc(&a->final_state, sizeof(float4) * 2 * std::max<size_t>(a->N, 1)),
            "allocate final state");
  // tape segment buffers: one, or as many as the caller's budget holds (up
  // to the rollout's segments)
  {
    const uint64_t seg = segment_bytes(a);
    uint64_t want = seg ? a->tape_budget / seg : 1;
    want = std::max<uint64_t>(1, std::min<uint64_t>({want, uint64_t(std::max<uint32_t>(nck, 1)),
                                                      uint64_t(a->seg_limit)}));
    a->segs = uint32_t(want);
  }
  a->pipe_wanted = a->segs == 1 && nck >= 2;
  if ((rc = ensure_work(a))) return rc;
  a->buf_seg.assign(a->bufs, -1);
  // the reverse pass starts with the last segments: the last `segs` record
  // their tapes on the way instead of being re-run there
  const uint32_t first_rec = nck > a->segs ? nck - a->segs : 0u;
  for (uint32_t c = 0; c < nck; c++) {
    float4 *ck = a->ck + size_t(c) * 2 * a->N;
    if ((rc = copy_state(s, ck, ck + a->N, s->d.p_pos, s->d.p_vel, a->N))) return rc;
    const uint32_t len = std::min(a->every, nsteps - c * a->every);
    if (c < first_rec) {
      if ((rc = fs_step(s, len))) return rc;
    } else {
      const uint32_t b = c - first_rec;
      for (uint32_t t = 0; t < len; t++) {
        const DevState dv = recording_state(a, a->tape[size_t(b) * a->every + t]);
        if ((rc = enqueue_step(s, false, &dv))) return rc;
      }
      a->buf_seg[b] = int64_t(c);
    }
  }
  if ((rc = copy_state(s, a->final_state, a->final_state + a->N, s->d.p_pos, s->d.p_vel, a->N)))
    return rc;
  for (int b = 0; b < 2; b++)
    FS_CUDA(cudaMemsetAsync(a->cot[a->cur][b], 0, sizeof(float4) * a->N, s->stream),
            "clear cotangents");
  a->steps = nsteps;
  return FS_OK;
}

int fs_adj_set_cotangents(FsAdj *a, const float *dl_dpos, const float *dl_dvel, int on_device) {
  CHECK_ADJ(a);
  FsSim *s = a->sim;
  int rc;
  if ((rc = set_device(s))) return rc;
  if (!a->work) return fail(FS_E_STATE, "fs_adj_set_cotangents: no recorded rollout");
  const float *src[2] = {dl_dpos, dl_dvel};
  for (int b = 0; b < 2; b++) {
    float4 *dst = a->cot[a->cur][b];
    if (!src[b]) {
      FS_CUDA(cudaMemsetAsync(dst, 0, sizeof(float4) * a->N, s->stream), "clear cotangent");
    } else if (on_device) {
      FS_CUDA(launch_rows_to_f4(a->N, src[b], dst, s->stream), "cotangent rows");
    } else {
      std::vector<float4> h(a->N);
      for (uint32_t i = 0; i < a->N; i++)
        h[i] = make_float4(src[b][3 * size_t(i)], src[b][3 * size_t(i) + 1],
                           src[b][3 * size_t(i) + 2], 0.0f);
      FS_CUDA(cudaMemcpyAsync(dst, h.data(), sizeof(float4) * a->N, cudaMemcpyHostToDevice,
                              s->stream),
              "upload cotangent");
      FS_CUDA(cudaStreamSynchronize(s->stream), "upload cotangent");
    }
  }
  a->seeded = true;
  return FS_OK;
}

int fs_adj_final_splat(FsAdj *a, uint32_t scene, const GpuMcGridParams *grid,
                       const GpuContainerGeometry *geom, float *out, int out_on_device) {
  CHECK_ADJ(a);
  FsSim *s = a->sim;
  if (!grid || !geom || !out) return fail(FS_E_INVALID_ARGUMENT, "fs_adj_final_splat: null argument");
  if (scene >= s->scenes())
    return fail(FS_E_INVALID_ARGUMENT, "fs_adj_final_splat: scene %u of %u", scene, s->scenes());
  if (grid->grid_size == 0 || grid->grid_size > 1024)
    return fail(FS_E_INVALID_ARGUMENT, "fs_adj_final_splat: grid_size %u outside [1, 1024]",
                grid->grid_size);
  int rc;
  if ((rc = set_device(s))) return rc;
  const DevUniforms &u = s->hu[scene];
  const SplatArgs sa = make_splat_args(*grid, *geom, u.grid);
  if (sa.cell_radius < 1 || sa.cell_radius > 8)
    return fail(FS_E_INVALID_ARGUMENT, "fs_adj_final_splat: splat radius spans %d cells",
                sa.cell_radius);
  if ((rc = enqueue_grid_build(s))) return rc;
  const size_t vox = size_t(grid->grid_size) * grid->grid_size * grid->grid_size;
  if (out_on_device) {
    FS_CUDA(launch_density_splat(sa, s->d.s_pos, s->d.cell_begin + u.c_offset, out, s->stream),
            "final splat");
    return FS_OK;
  }
  float *tmp = nullptr;
  FS_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&tmp), sizeof(float) * vox, s->stream),
          "final splat scratch");
  cudaError_t e = launch_density_splat(sa, s->d.s_pos, s->d.cell_begin + u.c_offset, tmp, s->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, tmp, sizeof(float) * vox, cudaMemcpyDeviceToHost, s->stream);
  cudaFreeAsync(tmp, s->stream);
  if (e != cudaSuccess) return cuda_fail(e, "final splat");
  return check_device_error(s);
}

int fs_adj_splat_mse_loss(FsAdj *a, uint32_t scene, const GpuMcGridParams *grid,
                          const GpuContainerGeometry *geom, const float *target,
                          int target_on_device, double *loss_out) {
  CHECK_ADJ(a);
  if (!grid || !geom || !target || !loss_out)
    return fail(FS_E_INVALID_ARGUMENT, "fs_adj_splat_mse_loss: null argument");
  return splat_mse_losses(a, 1, &scene, grid, geom, &target, target_on_device, loss_out,
                          "fs_adj_splat_mse_loss");
}

int fs_adj_splat_mse_losses(FsAdj *a, uint32_t count, const uint32_t *scenes,
                            const GpuMcGridParams *grids, const GpuContainerGeometry *geoms,
                            const float *const *targets, int targets_on_device,
                            double *losses) {
  CHECK_ADJ(a);
  if (count == 0) return FS_OK;
  if (!scenes || !grids || !geoms || !targets || !losses)
    return fail(FS_E_INVALID_ARGUMENT, "fs_adj_splat_mse_losses: null argument");
  return splat_mse_losses(a, count, scenes, grids, geoms, targets, targets_on_device, losses,
                          "fs_adj_splat_mse_losses");
}

int fs_adj_param_gradients(FsAdj *a, double *out, uint32_t scenes) {
  CHECK_ADJ(a);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_adj_param_gradients: null output");
  if (a->param_grads.empty())
    return fail(FS_E_STATE, "fs_adj_param_gradients: no fs_adj_backward has run");
  if (scenes != a->scenes)
    return fail(FS_E_INVALID_ARGUMENT, "fs_adj_param_gradients: scene count %u, expected %u",
                scenes, a->scenes);
  std::memcpy(out, a->param_grads.data(), sizeof(double) * a->param_grads.size());
  return FS_OK;
}

int fs_adj_backward(FsAdj *a, float *dl_dpos0, float *dl_dvel0, int on_device,
                    double *dl_dparams) {
  CHECK_ADJ(a);
  FsSim *s = a->sim;
  int rc;
  if ((rc = set_device(s))) return rc;
  if (!a->work) return fail(FS_E_STATE, "fs_adj_backward: no recorded rollout");
  if (!a->seeded) return fail(FS_E_STATE, "fs_adj_backward: no cotangents (set them or a loss)");
  if (s->iterations != a->K || s->hb.n_canon != a->N || s->scenes() != a->scenes ||
      std::memcmp(s->hu.data(), a->hu_snapshot.data(), sizeof(DevUniforms) * a->scenes) != 0)
    return fail(FS_E_STATE, "fs_adj_backward: parameters changed since fs_adj_forward");
  const uint32_t N = a->N, K = a->K;
  FS_CUDA(cudaMemsetAsync(a->av.gpart, 0, sizeof(double2) * N, s->stream),
          "clear parameter gradients");
  FS_CUDA(cudaMemsetAsync(a->av.gpart2, 0, sizeof(double2) * N, s->stream),
          "clear parameter gradients");
  {
    std::vector<uint32_t> first(a->scenes), count(a->scenes);
    for (uint32_t k = 0; k < a->scenes; k++) {
      first[k] = s->hu[k].p_offset;
      count[k] = s->scene_n[k];
    }
    FS_CUDA(cudaMemcpyAsync(a->scene_first, first.data(), sizeof(uint32_t) * a->scenes,
                            cudaMemcpyHostToDevice, s->stream),
            "scene ranges");
    FS_CUDA(cudaMemcpyAsync(a->scene_count, count.data(), sizeof(uint32_t) * a->scenes,
                            cudaMemcpyHostToDevice, s->stream),
            "scene ranges");
    FS_CUDA(cudaStreamSynchronize(s->stream), "scene ranges");
  }
  const uint32_t nck = (a->steps + a->every - 1) / a->every;
  const SceneView base = s->d.view();
  // restore segment seg's checkpoint and re-run it, recording into buffer b
  auto rerun = [&](uint32_t seg, uint32_t b) -> int {
    const uint32_t len = std::min(a->every, a->steps - seg * a->every);
    a->buf_seg[b] = -1;
    const float4 *ck = a->ck + size_t(seg) * 2 * N;
    int r;
    if ((r = copy_state(s, s->d.p_pos, s->d.p_vel, ck, ck + N, N))) return r;
    for (uint32_t t = 0; t < len; t++) {
      const DevState dv = recording_state(a, a->tape[size_t(b) * a->every + t]);
      if ((r = enqueue_step(s, false, &dv))) return r;
    }
    a->buf_seg[b] = int64_t(seg);
    return FS_OK;
  };
  // Pipelined (strict checkpointing with the second buffer): segment seg-1 is
  // re-run on the side stream into the other buffer while seg is reversed on
  // the simulation's stream. The re-run touches only the simulation's state
  // and step buffers and its own tape buffer; the reversal reads only its tape
  // buffer, the cotangents and the accumulators, so the two are independent
  // apart from the buffer hand-over, which events order: the reversal of a
  // buffer waits for its re-run (ev_rec), and a re-run into a buffer waits for
  // the reversal that last read it (ev_free).
  const bool pipe = a->bufs == 2 && a->segs == 1 && nck >= 2;
  cudaStream_t main_stream = s->stream;
  auto rerun_side = [&](uint32_t seg, uint32_t b) -> int {
    FS_CUDA(cudaStreamWaitEvent(a->side, a->ev_free[b], 0), "order the re-run");
    s->stream = a->side;
    const int r = rerun(seg, b);
    s->stream = main_stream;
    if (r) return r;
    FS_CUDA(cudaEventRecord(a->ev_rec[b], a->side), "order the re-run");
    return FS_OK;
  };
  bool on_side[2] = {false, false};
  if (pipe) {
    // the side stream starts after everything queued before the backward
    // (the loss reads the final state the first re-run overwrites)
    FS_CUDA(cudaEventRecord(a->ev_start, main_stream), "order the re-run");
    FS_CUDA(cudaStreamWaitEvent(a->side, a->ev_start, 0), "order the re-run");
    // buffers carry no pending reversal yet
    FS_CUDA(cudaEventRecord(a->ev_free[0], main_stream), "order the re-run");
    FS_CUDA(cudaEventRecord(a->ev_free[1], main_stream), "order the re-run");
  }
  for (uint32_t seg = nck; seg-- > 0;) {
    const uint32_t len = std::min(a->every, a->steps - seg * a->every);
    uint32_t b = 0;
    while (b < a->bufs && a->buf_seg[b] != int64_t(seg)) b++;
    if (b == a->bufs) {
      if (pipe) {
        // only the last segment can be missing here (the forward did not
        // record it); the others were started on the side stream below
        b = 0;
        if ((rc = rerun_side(seg, b))) return rc;
        on_side[b] = true;
      } else {
        // buffer 0's segment, if any, has been reversed already
        b = 0;
        if ((rc = rerun(seg, b))) return rc;
      }
    }
    if (pipe && on_side[b]) {
      FS_CUDA(cudaStreamWaitEvent(main_stream, a->ev_rec[b], 0), "order the reversal");
      on_side[b] = false;
    }
    const TapeSlot *seg_tape = a->tape.data() + size_t(b) * a->every;
    if (a->lanes == 0) {
      // tuned on the segment's last step before the next re-run is queued,
      // so that nothing else runs while the candidates are timed
      SceneView v = base;
      v.scene_of_slot = seg_tape[len - 1].sos;
      const int L = tune_lanes(a, v, tape_view(seg_tape[len - 1], K));
      if (L < 0) return L;
      a->lanes = L;
    }
    if (pipe && seg >= 1) {
      // start the next segment's re-run into the other buffer
      const uint32_t o = b ^ 1u;
      if ((rc = rerun_side(seg - 1, o))) return rc;
      on_side[o] = true;
    }
    for (uint32_t t = len; t-- > 0;) {
      const TapeSlot &slot = seg_tape[t];
      SceneView v = base;
      v.scene_of_slot = slot.sos;
      const int nxt = a->cur ^ 1;
      FS_CUDA(launch_adj_step(v, tape_view(slot, K), a->av, a->cot[a->cur][0], a->cot[a->cur][1],
                              a->cot[nxt][0], a->cot[nxt][1], s->d.dir_tab, s->d.dir_half, N,
                              int(K), a->lanes, s->d.sm_count, s->stream),
              "reverse step");
      a->cur = nxt;
    }
    if (pipe) FS_CUDA(cudaEventRecord(a->ev_free[b], main_stream), "order the re-run");
  }
  // outputs
  const float4 *g[2] = {a->cot[a->cur][0], a->cot[a->cur][1]};
  float *outs[2] = {dl_dpos0, dl_dvel0};
  std::vector<float4> host(N);
  for (int b = 0; b < 2; b++) {
    if (!outs[b]) continue;
    if (on_device) {
      FS_CUDA(launch_f4_to_rows(N, g[b], outs[b], s->stream), "gradient rows");
    } else {
      FS_CUDA(cudaMemcpyAsync(host.data(), g[b], sizeof(float4) * N, cudaMemcpyDeviceToHost,
                              s->stream),
              "download gradient");
      FS_CUDA(cudaStreamSynchronize(s->stream), "download gradient");
      for (uint32_t i = 0; i < N; i++) {
        outs[b][3 * size_t(i)] = host[i].x;
        outs[b][3 * size_t(i) + 1] = host[i].y;
        outs[b][3 * size_t(i) + 2] = host[i].z;
      }
    }
  }
  FS_CUDA(launch_reduce_params(a->av.gpart, a->av.gpart2, a->scene_first, a->scene_count,
                               a->scenes, a->av.gparam, a->av.gparam2, s->stream),
          "parameter gradients");
  if (dl_dparams)
    FS_CUDA(cudaMemcpyAsync(dl_dparams, a->av.gparam, sizeof(double) * 3 * a->scenes,
                            cudaMemcpyDeviceToHost, s->stream),
            "download parameter gradients");
  a->param_grads.resize(size_t(FS_ADJ_NUM_PARAMS) * a->scenes);
  {
    std::vector<double> g3(3 * size_t(a->scenes)), g2(2 * size_t(a->scenes));
    FS_CUDA(cudaMemcpyAsync(g3.data(), a->av.gparam, sizeof(double) * g3.size(),
                            cudaMemcpyDeviceToHost, s->stream),
            "download parameter gradients");
    FS_CUDA(cudaMemcpyAsync(g2.data(), a->av.gparam2, sizeof(double) * g2.size(),
                            cudaMemcpyDeviceToHost, s->stream),
            "download parameter gradients");
    FS_CUDA(cudaStreamSynchronize(s->stream), "download parameter gradients");
    for (uint32_t k = 0; k < a->scenes; k++) {
      double *o = a->param_grads.data() + size_t(FS_ADJ_NUM_PARAMS) * k;
      o[0] = g3[3 * size_t(k)];
      o[1] = g3[3 * size_t(k) + 1];
      o[2] = g3[3 * size_t(k) + 2];
      o[3] = g2[2 * size_t(k)];
      o[4] = g2[2 * size_t(k) + 1];
    }
  }
  // leave the simulation at the rollout's final state
  if ((rc = copy_state(s, s->d.p_pos, s->d.p_vel, a->final_state, a->final_state + N, N)))
    return rc;
  uint32_t err = 0;
  FS_CUDA(cudaMemcpyAsync(&err, s->d.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream),
          "read error word");
  FS_CUDA(cudaStreamSynchronize(s->stream), "backward");
  if (err & ERR_ADJ_OUTSIDE_GRID) {
    FS_CUDA(cudaMemset(s->d.err, 0, sizeof(uint32_t)), "clear error word");
    return fail(FS_E_STATE, "fs_adj_backward: a particle left the grid (neighbour sets are "
                            "then not symmetric); the gradient is not valid");
  }
  if ((rc = check_device_error(s))) return rc;
  a->seeded = false;
  return FS_OK;
}

}  // extern "C"
