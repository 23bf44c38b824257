// sim.cu — SphSimulation3DGrid behind the C ABI (include/fluidsph.h).
//
// Mirrors the reference's simulation object (src/simulation/sph_3d_grid.rs):
// construction and buffer allocation (:104-305), step() dispatch sequence
// (:1261-1444), parameter uploads (:1446-1477), rigid-body accumulator
// clear/readback (:1479-1498), buffer getters (:1500-1530) and spawning
// (:1534-1569). All device memory lives in one arena allocated at creation.
//
// A simulation holds one or more scenes. fs_create makes one; fs_batch_create
// makes many independent scenes stepped together, every stage one launch over
// all of them. Scene k owns canonical particles [p_offset, p_offset + n_k),
// cells [c_offset, c_offset + G_k) of the global cell arrays and sorted slots
// [s_offset, s_offset + active_k), so the global prefix scan over all cells is
// every scene's own scan shifted by s_offset.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "fs_sim.h"

using namespace fs;

namespace {
thread_local std::string g_last_error = "no error";
}  // namespace

int fs::fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int fs::cuda_fail(cudaError_t e, const char *what) {
  return fail(FS_E_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

namespace {

static_assert(sizeof(SphParticle3D) == 64, "SphParticle3D layout");
static_assert(sizeof(GpuSphParams3D) == 64, "GpuSphParams3D layout");
static_assert(sizeof(GpuContainerGeometry) == 128, "GpuContainerGeometry layout");
static_assert(sizeof(GpuGravity) == 16, "GpuGravity layout");
static_assert(sizeof(GpuMouseForce) == 48, "GpuMouseForce layout");
static_assert(sizeof(GpuRigidBody) == 96, "GpuRigidBody layout");
static_assert(sizeof(GpuRigidBodyAccum) == 32, "GpuRigidBodyAccum layout");
static_assert(sizeof(GpuGridParams) == 48, "GpuGridParams layout");
static_assert(offsetof(SphParticle3D, density) == 44, "density offset");
static_assert(offsetof(SphParticle3D, normal) == 52, "normal offset");
static_assert(offsetof(GpuContainerGeometry, wall_stiffness) == 112, "geometry offset");
static_assert(offsetof(GpuRigidBody, rot_row0) == 48, "rigid offset");
static_assert(sizeof(FsSceneInfo) == 80, "FsSceneInfo layout");
static_assert(sizeof(GpuMcGridParams) == 48, "GpuMcGridParams layout");
static_assert(sizeof(FsRigidBodyState) == 80, "FsRigidBodyState layout");
static_assert(sizeof(GpuSprayParams) == 80, "GpuSprayParams layout");
static_assert(sizeof(GpuSprayParticle) == 48, "GpuSprayParticle layout");
static_assert(FS_BATCH_MAX_SCENES <= 65535u, "scene ids are 16-bit");

}  // namespace

void fs::set_last_error(const char *msg) { g_last_error = msg; }

namespace {

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Carve the arena: every buffer 256-byte aligned.
struct Carver {
  char *base;
  size_t off = 0;
  template <class T>
  T *take(size_t count) {
    T *p = reinterpret_cast<T *>(base ? base + off : nullptr);
    off += align256(sizeof(T) * std::max<size_t>(count, 1));
    return p;
  }
};

void carve(FsSim *s, char *base, size_t *bytes) {
  Carver c{base};
  const size_t M = s->max_n;
  const size_t G = s->cells_total;
  DevState &d = s->d;
  d.p_pos = c.take<float4>(M);
  d.p_vel = c.take<float4>(M);
  d.p_force = c.take<float4>(M);
  d.p_aux = c.take<float4>(2 * M);
  d.s_pos = c.take<float4>(M);
  d.s_vel = c.take<float4>(M);
  d.s_frc = c.take<float4>(M);
  d.s_dens = c.take<float2>(M);
  d.s_nrm = c.take<float4>(M);
  d.vel_x = c.take<float4>(M);
  d.nb_pos = c.take<float4>(M);
  d.nb_vel = c.take<float4>(M);
  d.nb_nrm = c.take<float4>(M);
  d.anp = c.take<float4>(M);
  d.pred_xp[0] = c.take<float4>(M);
  d.pred_xp[1] = c.take<float4>(M);
  d.pred_rho[0] = c.take<float>(M);
  d.pred_rho[1] = c.take<float>(M);
  d.pterm[0] = c.take<float>(M);
  d.pterm[1] = c.take<float>(M);
  d.rep_of = c.take<uint32_t>(M);
  d.dd_list = c.take<uint32_t>(M);
  d.dd_warp = c.take<uint32_t>((M + 31) / 32 + 1);
  d.dd_incl = c.take<uint32_t>((M + 31) / 32 + 1);
  d.dd_tiles = c.take<unsigned long long>(scan_tiles((M + 31) / 32) + 1);
  d.dd_bucket = c.take<uint8_t>((M + 31) / 32);
  d.dd_order = c.take<uint32_t>((M + 31) / 32);
  d.dd_hist = c.take<uint32_t>(2 * 33);
  d.dens_cand = c.take<uint32_t>(M);
  d.dens_hits = c.take<uint32_t>(M);
  d.pred_v = c.take<float4>(M);
  d.cell_of = c.take<uint32_t>(M);
  d.rank_of = c.take<uint32_t>(M);
  d.t_tmp = c.take<uint32_t>(M);
  d.big_cells = c.take<uint32_t>(4 + 2 * size_t(big_item_cap(M)));
  d.s2o = c.take<uint32_t>(M);
  d.cidx = c.take<uint32_t>(M);
  d.counts = c.take<uint32_t>(G);
  d.cell_begin = c.take<uint32_t>(G + 1);
  const size_t tiles = scan_tiles(uint32_t(G));
  d.tile_status = c.take<unsigned long long>(tiles + 1);
  d.tile_ticket = reinterpret_cast<uint32_t *>(d.tile_status ? d.tile_status + tiles : nullptr);
  d.sdf = c.take<float>(size_t(s->sdf_res) * s->sdf_res * s->sdf_res);
  // hit masks: one bit per candidate; 128 words (4096 candidates) per
  // particle of capacity, at least 2^22 words; overflow falls back to testing
  d.mask_cap = std::max<size_t>(size_t(1) << 22, 128 * M);
  d.mask_words = c.take<uint32_t>(d.mask_cap);
  d.mask_off = c.take<uint32_t>(M);
  d.mask_hits = c.take<uint32_t>(M);
  d.warp_order = c.take<uint32_t>((M + 31) / 32);
  d.warp_bucket = c.take<uint8_t>((M + 31) / 32);
  d.order_hist = c.take<uint32_t>(ORDER_HIST_WORDS);
  d.perm_hit = c.take<uint32_t>(M);
  d.work_key = c.take<uint16_t>(M);
  d.key_hist = c.take<uint32_t>(3 * KEY_BUCKETS);
  d.task_counters = c.take<uint32_t>(TASK_COUNTERS);
  d.mask_alloc = c.take<unsigned long long>(1);
  d.dir_half = int(std::min<size_t>(M, size_t(1) << 20));
  d.dir_tab = c.take<float4>(2 * size_t(d.dir_half) + 1);
  const size_t S = s->scenes();
  d.accum = c.take<GpuRigidBodyAccum>(S);
  d.rb_state = c.take<FsRigidBodyState>(S);
  d.rb_coupled = c.take<uint8_t>(S);
  d.err = c.take<uint32_t>(4);
  d.stats = c.take<unsigned long long>(STAT_COUNT);
  d.u = c.take<DevUniforms>(S);
  d.b = c.take<DevBatch>(1);
  d.scene_of = c.take<uint16_t>(M);
  d.scene_of_slot = c.take<uint16_t>(M);
  *bytes = c.off;
}

void destroy_graphs(FsSim *s) {
  for (StepGraph &g : s->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = StepGraph{};
  }
}

// Offsets and counts of every scene from the scene sizes and the current
// num_particles parameters.
void layout(FsSim *s) {
  uint32_t p = 0, c = 0, so = 0;
  for (uint32_t k = 0; k < s->scenes(); k++) {
    DevUniforms &u = s->hu[k];
    u.n = s->active(k);
    u.grid.num_particles = u.n;
    u.sdf_res = s->sdf_res;
    u.p_offset = p;
    u.c_offset = c;
    u.s_offset = so;
    p += s->scene_n[k];
    c += u.grid.total_cells;
    so += u.n;
  }
  s->hb.n_scenes = s->scenes();
  s->hb.n_canon = p;
  s->hb.n_sorted = so;
  s->hb.cells_total = c;
}

// Upload every scene's parameter block and the batch header.
int upload_uniforms(FsSim *s) {
  layout(s);
  FS_CUDA(cudaMemcpyAsync(s->d.u, s->hu.data(), sizeof(DevUniforms) * s->scenes(),
                          cudaMemcpyHostToDevice, s->stream),
          "upload parameters");
  FS_CUDA(cudaMemcpyAsync(s->d.b, &s->hb, sizeof(DevBatch), cudaMemcpyHostToDevice, s->stream),
          "upload batch header");
  if (s->any_coupled())
    FS_CUDA(launch_rigid_sync(s->d, s->scenes(), s->stream), "coupled rigid bodies");
  return FS_OK;
}

// Upload scene k's block after a change to it; a change of its active count
// moves the later scenes' slots, so then every block goes up.
int upload_scene(FsSim *s, uint32_t k) {
  const uint32_t before = s->hb.n_sorted;
  layout(s);
  if (s->hb.n_sorted != before) return upload_uniforms(s);
  FS_CUDA(cudaMemcpyAsync(s->d.u + k, &s->hu[k], sizeof(DevUniforms), cudaMemcpyHostToDevice,
                          s->stream),
          "upload scene parameters");
  if (s->any_coupled())
    FS_CUDA(launch_rigid_sync(s->d, s->scenes(), s->stream), "coupled rigid bodies");
  return FS_OK;
}

}  // namespace

int fs::check_device_error(FsSim *s) {
  uint32_t err = 0;
  FS_CUDA(cudaStreamSynchronize(s->stream), "synchronize");
  FS_CUDA(cudaMemcpy(&err, s->d.err, sizeof(uint32_t), cudaMemcpyDeviceToHost), "read error word");
  if (err) {
    FS_CUDA(cudaMemset(s->d.err, 0, sizeof(uint32_t)), "clear error word");
    if (err & ERR_SCAN_TIMEOUT)
      return fail(FS_E_DEVICE_TIMEOUT, "device-side wait gave up (scan look-back, code %u)", err);
    return fail(FS_E_DEVICE_TIMEOUT, "device error word %u", err);
  }
  return FS_OK;
}

namespace {

// AoS <-> SoA conversion of canonical records on the host.
void aos_to_soa(const SphParticle3D *in, uint32_t count, std::vector<float4> &pos,
                std::vector<float4> &vel, std::vector<float4> &frc, std::vector<float4> &aux) {
  pos.resize(count);
  vel.resize(count);
  frc.resize(count);
  aux.resize(2 * size_t(count));
  for (uint32_t i = 0; i < count; i++) {
    const SphParticle3D &p = in[i];
    pos[i] = make_float4(p.position[0], p.position[1], p.position[2], p._pad0);
    vel[i] = make_float4(p.velocity[0], p.velocity[1], p.velocity[2], p._pad1);
    frc[i] = make_float4(p.force[0], p.force[1], p.force[2], 0.0f);
    aux[2 * size_t(i)] = make_float4(p.density, p.near_density, p.normal[0], p.normal[1]);
    aux[2 * size_t(i) + 1] = make_float4(p.normal[2], 0.0f, 0.0f, 0.0f);
  }
}

int write_particles(FsSim *s, const SphParticle3D *parts, uint32_t offset, uint32_t count) {
  if (count == 0) return FS_OK;
  std::vector<float4> pos, vel, frc, aux;
  aos_to_soa(parts, count, pos, vel, frc, aux);
  const size_t b = sizeof(float4) * count;
  FS_CUDA(cudaMemcpyAsync(s->d.p_pos + offset, pos.data(), b, cudaMemcpyHostToDevice, s->stream), "upload positions");
  FS_CUDA(cudaMemcpyAsync(s->d.p_vel + offset, vel.data(), b, cudaMemcpyHostToDevice, s->stream), "upload velocities");
  FS_CUDA(cudaMemcpyAsync(s->d.p_force + offset, frc.data(), b, cudaMemcpyHostToDevice, s->stream), "upload forces");
  FS_CUDA(cudaMemcpyAsync(s->d.p_aux + 2 * size_t(offset), aux.data(), 2 * b, cudaMemcpyHostToDevice, s->stream), "upload aux");
  // pageable-source copies may return before completion; keep the staging
  // vectors alive until the copies are done
  FS_CUDA(cudaStreamSynchronize(s->stream), "upload particles");
  return FS_OK;
}

}  // namespace

// One step: the stage sequence of step(), sph_3d_grid.rs:1261-1444, over all
// scenes at once, on the simulation's buffers or on `dv` (the same buffers
// with some replaced, e.g. by a recording for the reverse pass).
int fs::enqueue_step(FsSim *s, bool timed, const DevState *dv, const KernelForms *forms,
                     cudaEvent_t *marks, int xsph_all) {
  const uint32_t n = s->hb.n_sorted;
  const uint32_t n_canon = s->hb.n_canon;
  const uint32_t G = s->cells_total;
  cudaStream_t st = s->stream;
  DevState d = dv ? *dv : s->d;
  const KernelForms &f = forms ? *forms : s->forms;
  d.load_density = f.density;
  d.load_solve = f.solve;
  d.load_xsph = f.xsph;
  auto mark = [&](int i) -> int {
    if (marks) {
      if (i < FS_STAGE_COUNT) FS_CUDA(cudaEventRecord(marks[i], st), "record stage event");
    } else if (timed) {
      FS_CUDA(cudaEventRecord(s->ev[i], st), "record stage event");
    }
    return FS_OK;
  };
  int rc;
  if ((rc = mark(0))) return rc;
  FS_CUDA(cudaMemsetAsync(d.counts, 0, sizeof(uint32_t) * G, st), "grid clear");
  if ((rc = mark(1))) return rc;
  FS_CUDA(launch_hash(d, n_canon, st), "grid build (hash)");
  if ((rc = mark(2))) return rc;
  FS_CUDA(launch_scan(d, G, st), "prefix scan");
  if ((rc = mark(3))) return rc;
  FS_CUDA(launch_scatter(d, n_canon, st), "reorder (scatter)");
  FS_CUDA(launch_sort_gather(d, n, st), "reorder (sort/gather)");
  if ((rc = mark(4))) return rc;
  FS_CUDA(launch_order_warps(d, n, st), "neighbour-pass work order");
  FS_CUDA(launch_density(d, n, st), "density");
  FS_CUDA(launch_order_hits(d, n, st), "neighbour-pass work order (hits)");
  if ((rc = mark(5))) return rc;
  if (xsph_all >= 0 && marks) {
    for (int i = 0; i < kNumLoadDepths; i++) {
      FS_CUDA(cudaEventRecord(marks[FS_STAGE_COUNT + i], st), "record XSPH event");
      d.load_xsph = uint8_t((xsph_all + i) % kNumLoadDepths);
      FS_CUDA(launch_xsph(d, n, st), "xsph");
    }
    FS_CUDA(cudaEventRecord(marks[FS_STAGE_COUNT + kNumLoadDepths], st), "record XSPH event");
    d.load_xsph = f.xsph;
  } else {
    FS_CUDA(launch_xsph(d, n, st), "xsph");
  }
  if ((rc = mark(6))) return rc;
  FS_CUDA(launch_force_predict(d, n, st), "force + predict");
  if ((rc = mark(7))) return rc;
  const int K = int(s->iterations);
  for (int k = 0; k < K; k++) FS_CUDA(launch_solve(d, n, k, k == K - 1, st), "pcisph solve");
  if ((rc = mark(8))) return rc;
  FS_CUDA(launch_finalize_integrate(d, n, K & 1, st), "finalize + integrate");
  if ((rc = mark(9))) return rc;
  return FS_OK;
}

// The grid build of the current canonical state alone (grid_clear, hash,
// scan, reorder: the first stages of a step).
int fs::enqueue_grid_build(FsSim *s) {
  const DevState &d = s->d;
  cudaStream_t st = s->stream;
  FS_CUDA(cudaMemsetAsync(d.counts, 0, sizeof(uint32_t) * s->cells_total, st), "grid clear");
  FS_CUDA(launch_hash(d, s->hb.n_canon, st), "grid build (hash)");
  FS_CUDA(launch_scan(d, s->cells_total, st), "prefix scan");
  FS_CUDA(launch_scatter(d, s->hb.n_canon, st), "reorder (scatter)");
  FS_CUDA(launch_sort_gather(d, s->hb.n_sorted, st), "reorder (sort/gather)");
  return FS_OK;
}

namespace {

// The graph of `steps` back-to-back steps for the current counts, captured
// on first use (least recently used slot replaced).
// The neighbour passes' load depths (FsSim::forms): a simulation's bucket
// is looked up in the process-wide table first; if it is not there, the
// depths are measured once the simulation has run this many steps (the clumps
// of an over-compressed start have formed by then).
constexpr uint64_t kTuneAfterSteps = 8;
constexpr int kTuneSteps = 2 * kNumLoadDepths;

bool capturing(FsSim *s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(s->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
}

// The process-wide table: bucket -> depths and the times they were chosen by.
struct TuneEntry {
  KernelForms forms;
  float ms[3][kNumLoadDepths];
};
std::mutex g_forms_mu;
std::map<std::tuple<int, uint32_t, uint32_t, uint32_t>, TuneEntry> g_forms_table;

std::tuple<int, uint32_t, uint32_t, uint32_t> tune_key(const FsSim *s) {
  const uint32_t n = std::max(s->hb.n_sorted, 1u);
  uint32_t bucket = 0;
  while ((n >> (bucket + 1)) != 0u) bucket++;
  return {s->device, bucket, s->scenes() > 1 ? 1u : 0u, s->iterations};
}

// Adopt the table's depths for this simulation's bucket, if it holds them.
void tune_lookup(FsSim *s) {
  if (s->tune_state != 0 || s->tune_phase != 0) return;
  std::lock_guard<std::mutex> lk(g_forms_mu);
  const auto it = g_forms_table.find(tune_key(s));
  if (it == g_forms_table.end()) return;
  s->forms = it->second.forms;
  s->tune_state = 2;
  s->tune_source = 2;
}

// Candidate c of measured step p: 0, 1, .., n-1, n-1, .., 0.
int tune_candidate(int p) { return p < kNumLoadDepths ? p : kTuneSteps - 1 - p; }

// Wait for the measured steps and keep each pass's fastest depth.
int tune_decide(FsSim *s) {
  if (s->tune_state != 1 || capturing(s)) return FS_OK;
  FS_CUDA(cudaEventSynchronize(s->tune_ev[kTuneSteps - 1][8]), "kernel-form measurement");
  float ms[3][kNumLoadDepths] = {};
  float xs[kNumLoadDepths][kTuneSteps];
  for (int p = 0; p < kTuneSteps; p++) {
    const int c = tune_candidate(p);
    float t[2];
    // density (with the work-order kernels around it: the same for every
    // depth) and the PCISPH solve iterations: one sample per step, two per
    // depth, averaged
    FS_CUDA(cudaEventElapsedTime(&t[0], s->tune_ev[p][4], s->tune_ev[p][5]), "kernel-form measurement");
    FS_CUDA(cudaEventElapsedTime(&t[1], s->tune_ev[p][7], s->tune_ev[p][8]), "kernel-form measurement");
    ms[0][c] += 0.5f * t[0];
    ms[2][c] += 0.5f * t[1];
    // XSPH: every depth in every step
    for (int i = 0; i < kNumLoadDepths; i++) {
      const int cx = (p + i) % kNumLoadDepths;
      FS_CUDA(cudaEventElapsedTime(&xs[cx][p], s->tune_ev[p][FS_STAGE_COUNT + i],
                                   s->tune_ev[p][FS_STAGE_COUNT + i + 1]),
              "kernel-form measurement");
    }
  }
  // XSPH: the median of each depth's samples (a disturbed step does not
  // decide)
  for (int c = 0; c < kNumLoadDepths; c++) {
    std::sort(xs[c], xs[c] + kTuneSteps);
    ms[1][c] = 0.5f * (xs[c][kTuneSteps / 2 - 1] + xs[c][kTuneSteps / 2]);
  }
  uint8_t best[3] = {0, 0, 0};
  for (int k = 0; k < 3; k++)
    for (int c = 1; c < (k == 1 ? kNumLoadDepths : kPlainCandidates); c++)  // XSPH: staged too
      if (ms[k][c] < ms[k][best[k]]) best[k] = uint8_t(c);
  s->forms.density = best[0];
  s->forms.xsph = best[1];
  s->forms.solve = best[2];
  std::memcpy(s->tune_ms, ms, sizeof(ms));
  s->tune_state = 2;
  s->tune_source = 1;
  std::lock_guard<std::mutex> lk(g_forms_mu);
  TuneEntry e;
  e.forms = s->forms;
  std::memcpy(e.ms, ms, sizeof(ms));
  g_forms_table[tune_key(s)] = e;
  return FS_OK;
}

// Run the measured steps that are due, consuming them from nsteps.
int tune_steps(FsSim *s, uint32_t &nsteps) {
  while (nsteps > 0 && s->tune_state == 0 && s->steps_done >= kTuneAfterSteps) {
    const int p = s->tune_phase;
    const int c = tune_candidate(p);
    KernelForms f;  // depth 32 (the last candidate) is XSPH's alone
    f.xsph = uint8_t(c);
    f.density = f.solve = uint8_t(c < kPlainCandidates ? c : kPlainCandidates - 1);
    const int rc = enqueue_step(s, false, nullptr, &f, s->tune_ev[p], p % kNumLoadDepths);
    if (rc) return rc;
    s->steps_done++;
    nsteps--;
    if (++s->tune_phase == kTuneSteps) s->tune_state = 1;
  }
  return FS_OK;
}

int graph_for(FsSim *s, uint32_t steps, cudaGraphExec_t *out) {
  StepGraph *slot = nullptr;
  for (StepGraph &g : s->graphs) {
    if (g.exec && g.steps == steps && g.n_canon == s->hb.n_canon &&
        g.n_sorted == s->hb.n_sorted && g.iters == s->iterations && g.stream == s->stream &&
        g.forms == s->forms.key()) {
      g.last_use = ++s->graph_clock;
      *out = g.exec;
      return FS_OK;
    }
  }
  for (StepGraph &g : s->graphs) {  // an empty slot, else the least recently used
    if (!g.exec) {
      slot = &g;
      break;
    }
    if (!slot || g.last_use < slot->last_use) slot = &g;
  }
  if (slot->exec) cudaGraphExecDestroy(slot->exec);
  *slot = StepGraph{};
  cudaGraph_t g = nullptr;
  FS_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
  int rc = FS_OK;
  for (uint32_t k = 0; k < steps && rc == FS_OK; k++) rc = enqueue_step(s, false);
  cudaError_t e = cudaStreamEndCapture(s->stream, &g);
  if (rc != FS_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "end capture");
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "instantiate step graph");
  slot->exec = exec;
  slot->steps = steps;
  slot->n_canon = s->hb.n_canon;
  slot->n_sorted = s->hb.n_sorted;
  slot->iters = s->iterations;
  slot->stream = s->stream;
  slot->forms = s->forms.key();
  slot->last_use = ++s->graph_clock;
  *out = exec;
  return FS_OK;
}

#define CHECK_SIM(s) \
  if (!(s)) return fail(FS_E_INVALID_ARGUMENT, "%s: null simulation", __func__)

}  // namespace

int fs::set_device(FsSim *s) {
  FS_CUDA(cudaSetDevice(s->device), "cudaSetDevice");
  return FS_OK;
}

namespace {

// Plain entry points act on a simulation's single scene.
#define CHECK_PLAIN(s)                                                                        \
  if ((s)->scenes() != 1)                                                                    \
  return fail(FS_E_STATE, "%s: the simulation holds %u scenes (use the fs_batch_* calls)", \
              __func__, (s)->scenes())

#define CHECK_SCENE(s, k)                                                              \
  if ((k) >= (s)->scenes())                                                           \
  return fail(FS_E_INVALID_ARGUMENT, "%s: scene %u of %u", __func__, unsigned(k),     \
              (s)->scenes())

// Initial uniforms of SphSimulation3DGrid::new (sph_3d_grid.rs:257-300).
void default_scene(DevUniforms &u, const GpuSphParams3D &params, const GpuContainerGeometry &geom) {
  std::memset(&u, 0, sizeof(u));
  u.sph = params;
  u.geom = geom;
  u.gravity = GpuGravity{{0.0f, -9.8f, 0.0f}, 0.0f};
  u.mouse = GpuMouseForce{{0.0f, 0.0f, 0.0f}, 0.5f, 30.0f, 0u, 0u, 0.0f, {0.0f, 0.0f, -1.0f}, 0.0f};
  u.rigid = GpuRigidBody{{0.0f, 0.0f, 0.0f}, 0.15f, {0.0f, 0.0f, 0.0f}, 0u, 200.0f, 0u, 0.0f, 0.0f,
                         {1.0f, 0.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 1.0f, 0.0f}};
}

// Shared body of fs_create and fs_batch_create.
int create_sim(const char *who, const SphParticle3D *particles, const uint32_t *counts,
               uint32_t num_scenes, const GpuSphParams3D *params, const GpuContainerGeometry *geoms,
               uint32_t max_particles, const float *sdf, uint32_t sdf_res, int device,
               uint32_t abi_version, bool batch, FsSim **out) {
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "%s: out is null", who);
  *out = nullptr;
  if (abi_version != FS_ABI_VERSION)
    return fail(FS_E_ABI_MISMATCH, "%s: caller ABI 0x%08x, library ABI 0x%08x", who, abi_version,
                FS_ABI_VERSION);
  if (!params || !geoms) return fail(FS_E_INVALID_ARGUMENT, "%s: params/geometry is null", who);
  if (num_scenes == 0 || num_scenes > FS_BATCH_MAX_SCENES)
    return fail(FS_E_INVALID_ARGUMENT, "%s: %u scenes outside [1, %u]", who, num_scenes,
                FS_BATCH_MAX_SCENES);
  uint64_t total = 0;
  for (uint32_t k = 0; k < num_scenes; k++) total += counts[k];
  if (total > 0 && !particles) return fail(FS_E_INVALID_ARGUMENT, "%s: particles is null", who);
  if (sdf && (sdf_res == 0 || sdf_res > 512))
    return fail(FS_E_INVALID_ARGUMENT, "%s: sdf_res %u outside [1, 512]", who, sdf_res);
  for (uint32_t k = 0; k < num_scenes; k++) {
    const float h = params[k].kernel_radius;
    if (!(h > 0.0f) || !std::isfinite(h))
      return fail(FS_E_INVALID_ARGUMENT, "%s: scene %u kernel_radius must be finite and > 0", who, k);
  }
  const uint64_t max_n = std::max<uint64_t>(max_particles, total);
  if (max_n > (1u << 30))
    return fail(FS_E_CAPACITY, "%s: %llu particles > 2^30", who, (unsigned long long)max_n);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(FS_E_NO_DEVICE, "%s: no CUDA device", who);
  if (device < 0 || device >= ndev)
    return fail(FS_E_INVALID_ARGUMENT, "%s: device %d of %d", who, device, ndev);

  FsSim *s = new (std::nothrow) FsSim();
  if (!s) return fail(FS_E_CAPACITY, "%s: out of host memory", who);
  s->device = device;
  s->batch = batch;
  s->max_n = uint32_t(max_n);
  s->sdf_res = sdf ? sdf_res : 1u;
  s->scene_n.assign(counts, counts + num_scenes);
  s->coupled.assign(num_scenes, 0);
  s->hu.resize(num_scenes);
  uint64_t cells = 0;
  for (uint32_t k = 0; k < num_scenes; k++) {
    default_scene(s->hu[k], params[k], geoms[k]);
    GpuGridParams grid;
    int rc = fs_grid_params_for(params[k].kernel_radius, counts[k], &grid);
    if (rc != FS_OK) {
      delete s;
      return fail(rc, "%s: scene %u grid for kernel_radius %g does not fit", who, k,
                  double(params[k].kernel_radius));
    }
    s->hu[k].grid = grid;
    cells += grid.total_cells;
  }
  if (cells >= (uint64_t(1) << 32) - 1) {
    delete s;
    return fail(FS_E_CAPACITY, "%s: %llu cells over all scenes", who, (unsigned long long)cells);
  }
  s->cells_total = uint32_t(cells);
  layout(s);

  auto bail = [&](int code) {
    if (s->arena) cudaFree(s->arena);
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
    for (auto &e : s->ev)
      if (e) cudaEventDestroy(e);
    for (auto &row : s->tune_ev)
      for (auto &e : row)
        if (e) cudaEventDestroy(e);
    delete s;
    return code;
  };
  int rc;
  if ((rc = set_device(s))) return bail(rc);
  cudaError_t e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bail(cuda_fail(e, "create stream"));
  s->stream = s->own_stream;
  for (auto &ev : s->ev) {
    e = cudaEventCreate(&ev);
    if (e != cudaSuccess) return bail(cuda_fail(e, "create event"));
  }
  for (auto &row : s->tune_ev)
    for (auto &ev : row) {
      e = cudaEventCreate(&ev);
      if (e != cudaSuccess) return bail(cuda_fail(e, "create event"));
    }
  carve(s, nullptr, &s->arena_bytes);
  {
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return bail(cuda_fail(e, "query SM count"));
    s->d.sm_count = sms;
  }
  e = cudaMalloc(&s->arena, s->arena_bytes);
  if (e != cudaSuccess) return bail(cuda_fail(e, "allocate device arena"));
  carve(s, static_cast<char *>(s->arena), &s->arena_bytes);
  e = cudaMemsetAsync(s->arena, 0, s->arena_bytes, s->stream);
  if (e != cudaSuccess) return bail(cuda_fail(e, "clear device arena"));
  const float one = 1.0f;
  e = cudaMemcpyAsync(s->d.sdf, sdf ? sdf : &one,
                      sizeof(float) * size_t(s->sdf_res) * s->sdf_res * s->sdf_res,
                      cudaMemcpyHostToDevice, s->stream);
  if (e != cudaSuccess) return bail(cuda_fail(e, "upload SDF"));
  if (num_scenes > 1) {  // scene ids of the canonical particles (a single scene is all zero)
    std::vector<uint16_t> ids(s->hb.n_canon);
    for (uint32_t k = 0; k < num_scenes; k++)
      std::fill(ids.begin() + s->hu[k].p_offset, ids.begin() + s->hu[k].p_offset + counts[k],
                uint16_t(k));
    e = cudaMemcpyAsync(s->d.scene_of, ids.data(), sizeof(uint16_t) * ids.size(),
                        cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "upload scene ids"));
  }
  if ((rc = upload_uniforms(s))) return bail(rc);
  e = launch_dir_table(s->d, s->stream);
  if (e != cudaSuccess) return bail(cuda_fail(e, "close-pair direction table"));
  if ((rc = write_particles(s, particles, 0, uint32_t(total)))) return bail(rc);
  e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return bail(cuda_fail(e, who));
  *out = s;
  return FS_OK;
}

// Scene k's canonical records [first, first + count) as 64-byte AoS.
int read_canonical(FsSim *s, uint32_t first, SphParticle3D *out, uint32_t count) {
  std::vector<float4> pos(count), vel(count), frc(count), aux(2 * size_t(count));
  const size_t b = sizeof(float4) * count;
  if (count) {
    FS_CUDA(cudaMemcpyAsync(pos.data(), s->d.p_pos + first, b, cudaMemcpyDeviceToHost, s->stream), "download");
    FS_CUDA(cudaMemcpyAsync(vel.data(), s->d.p_vel + first, b, cudaMemcpyDeviceToHost, s->stream), "download");
    FS_CUDA(cudaMemcpyAsync(frc.data(), s->d.p_force + first, b, cudaMemcpyDeviceToHost, s->stream), "download");
    FS_CUDA(cudaMemcpyAsync(aux.data(), s->d.p_aux + 2 * size_t(first), 2 * b, cudaMemcpyDeviceToHost, s->stream), "download");
  }
  int rc;
  if ((rc = check_device_error(s))) return rc;
  for (uint32_t i = 0; i < count; i++) {
    SphParticle3D &p = out[i];
    p.position[0] = pos[i].x; p.position[1] = pos[i].y; p.position[2] = pos[i].z; p._pad0 = pos[i].w;
    p.velocity[0] = vel[i].x; p.velocity[1] = vel[i].y; p.velocity[2] = vel[i].z; p._pad1 = vel[i].w;
    p.force[0] = frc[i].x; p.force[1] = frc[i].y; p.force[2] = frc[i].z;
    const float4 a0 = aux[2 * size_t(i)], a1 = aux[2 * size_t(i) + 1];
    p.density = a0.x; p.near_density = a0.y;
    p.normal[0] = a0.z; p.normal[1] = a0.w; p.normal[2] = a1.x;
  }
  return FS_OK;
}

// Sorted slots [first, first + count) as 64-byte AoS.
int read_sorted(FsSim *s, uint32_t first, SphParticle3D *out, uint32_t count) {
  std::vector<float4> pos(count), vel(count), frc(count), nrm(count);
  std::vector<float2> dens(count);
  const size_t b = sizeof(float4) * count;
  if (count) {
    FS_CUDA(cudaMemcpyAsync(pos.data(), s->d.s_pos + first, b, cudaMemcpyDeviceToHost, s->stream), "download");
    FS_CUDA(cudaMemcpyAsync(vel.data(), s->d.s_vel + first, b, cudaMemcpyDeviceToHost, s->stream), "download");
    FS_CUDA(cudaMemcpyAsync(frc.data(), s->d.s_frc + first, b, cudaMemcpyDeviceToHost, s->stream), "download");
    FS_CUDA(cudaMemcpyAsync(nrm.data(), s->d.s_nrm + first, b, cudaMemcpyDeviceToHost, s->stream), "download");
    FS_CUDA(cudaMemcpyAsync(dens.data(), s->d.s_dens + first, sizeof(float2) * count, cudaMemcpyDeviceToHost, s->stream), "download");
  }
  int rc;
  if ((rc = check_device_error(s))) return rc;
  for (uint32_t i = 0; i < count; i++) {
    SphParticle3D &p = out[i];
    p.position[0] = pos[i].x; p.position[1] = pos[i].y; p.position[2] = pos[i].z; p._pad0 = pos[i].w;
    p.velocity[0] = vel[i].x; p.velocity[1] = vel[i].y; p.velocity[2] = vel[i].z; p._pad1 = vel[i].w;
    p.force[0] = frc[i].x; p.force[1] = frc[i].y; p.force[2] = frc[i].z;
    p.density = dens[i].x; p.near_density = dens[i].y;
    p.normal[0] = nrm[i].x; p.normal[1] = nrm[i].y; p.normal[2] = nrm[i].z;
  }
  return FS_OK;
}

// Scene k's cell counts and inclusive ends, relative to the scene's first slot.
int read_cells(FsSim *s, uint32_t k, uint32_t *counts, uint32_t *starts) {
  const DevUniforms &u = s->hu[k];
  const uint32_t G = u.grid.total_cells;
  const size_t b = sizeof(uint32_t) * G;
  if (counts) FS_CUDA(cudaMemcpyAsync(counts, s->d.counts + u.c_offset, b, cudaMemcpyDeviceToHost, s->stream), "download counts");
  if (starts) FS_CUDA(cudaMemcpyAsync(starts, s->d.cell_begin + 1 + u.c_offset, b, cudaMemcpyDeviceToHost, s->stream), "download starts");
  int rc;
  if ((rc = check_device_error(s))) return rc;
  if (starts && u.s_offset)
    for (uint32_t c = 0; c < G; c++) starts[c] -= u.s_offset;
  return FS_OK;
}

// Scene k's index maps in scene-local numbering: particle -> slot for its
// first `count` particles, slot -> particle for its first `count` slots.
int read_index_maps(FsSim *s, uint32_t k, uint32_t *cell_indices, uint32_t *sorted_to_orig,
                    uint32_t count) {
  const DevUniforms &u = s->hu[k];
  const size_t b = sizeof(uint32_t) * count;
  if (cell_indices && count) FS_CUDA(cudaMemcpyAsync(cell_indices, s->d.cidx + u.p_offset, b, cudaMemcpyDeviceToHost, s->stream), "download cell indices");
  if (sorted_to_orig && count) FS_CUDA(cudaMemcpyAsync(sorted_to_orig, s->d.s2o + u.s_offset, b, cudaMemcpyDeviceToHost, s->stream), "download sorted_to_orig");
  int rc;
  if ((rc = check_device_error(s))) return rc;
  for (uint32_t i = 0; i < count; i++) {
    if (cell_indices) cell_indices[i] -= u.s_offset;
    if (sorted_to_orig) sorted_to_orig[i] -= u.p_offset;
  }
  return FS_OK;
}

}  // namespace

extern "C" {

const char *fs_last_error(void) { return g_last_error.c_str(); }
uint32_t fs_abi_version(void) { return FS_ABI_VERSION; }

int fs_create(const SphParticle3D *particles, uint32_t num_particles, const GpuSphParams3D *params,
              const GpuContainerGeometry *geom, uint32_t max_particles, const float *sdf,
              uint32_t sdf_res, int device, uint32_t abi_version, FsSim **out) {
  return create_sim("fs_create", particles, &num_particles, 1, params, geom, max_particles, sdf,
                    sdf_res, device, abi_version, false, out);
}

int fs_destroy(FsSim *s) {
  if (!s) return FS_OK;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  destroy_graphs(s);
  if (s->frame_graph.exec) cudaGraphExecDestroy(s->frame_graph.exec);
  for (auto &e : s->ev)
    if (e) cudaEventDestroy(e);
  for (auto &row : s->tune_ev)
    for (auto &e : row)
      if (e) cudaEventDestroy(e);
  if (s->splat_buf) cudaFree(s->splat_buf);
  if (s->arena) cudaFree(s->arena);
  if (s->own_stream) cudaStreamDestroy(s->own_stream);
  delete s;
  return FS_OK;
}

namespace {
int run_steps(FsSim *s, uint32_t nsteps);
}

int fs_step(FsSim *s, uint32_t nsteps) {
  CHECK_SIM(s);
  int rc;
  if ((rc = set_device(s))) return rc;
  if (nsteps == 0) return FS_OK;
  if (!capturing(s)) {
    tune_lookup(s);
    if ((rc = tune_decide(s))) return rc;
    // stage-timed steps are never measurement steps
    if (!s->timing && s->tune_state == 0 && s->steps_done < kTuneAfterSteps &&
        s->steps_done + nsteps > kTuneAfterSteps) {
      const uint32_t pre = uint32_t(kTuneAfterSteps - s->steps_done);
      if ((rc = run_steps(s, pre))) return rc;
      s->steps_done += pre;
      nsteps -= pre;
    }
    if (!s->timing && (rc = tune_steps(s, nsteps))) return rc;
    if (nsteps == 0) return FS_OK;
  }
  s->steps_done += nsteps;
  return run_steps(s, nsteps);
}

namespace {
// The step loop: stage-timed steps, one step, or graphs of up to
// kMaxGraphSteps steps.
int run_steps(FsSim *s, uint32_t nsteps) {
  int rc;
  if (s->timing) {
    for (uint32_t k = 0; k < nsteps; k++) {
      if ((rc = enqueue_step(s, true))) return rc;
      FS_CUDA(cudaEventSynchronize(s->ev[FS_STAGE_COUNT - 1]), "timed step");
      for (int i = 0; i < FS_STAGE_COUNT - 1; i++) {
        float ms = 0.0f;
        FS_CUDA(cudaEventElapsedTime(&ms, s->ev[i], s->ev[i + 1]), "stage time");
        s->stage_ms[i] += ms;
      }
      float total = 0.0f;
      FS_CUDA(cudaEventElapsedTime(&total, s->ev[0], s->ev[FS_STAGE_COUNT - 1]), "step time");
      s->stage_ms[FS_STAGE_COUNT - 1] += total;
      s->timed_steps++;
    }
    return FS_OK;
  }
  if (nsteps == 1) return enqueue_step(s, false);
  // nsteps = chunks * chunk + rest: a graph of `chunk` steps (at most
  // kMaxGraphSteps) replayed, then single-step graphs for the rest
  const uint32_t chunks = (nsteps + kMaxGraphSteps - 1) / kMaxGraphSteps;
  const uint32_t chunk = nsteps / chunks;
  const uint32_t rest = nsteps - chunks * chunk;
  cudaGraphExec_t g = nullptr;
  if ((rc = graph_for(s, chunk, &g))) return rc;
  for (uint32_t k = 0; k < chunks; k++)
    FS_CUDA(cudaGraphLaunch(g, s->stream), "launch step graph");
  if (rest) {
    if ((rc = graph_for(s, 1, &g))) return rc;
    for (uint32_t k = 0; k < rest; k++) FS_CUDA(cudaGraphLaunch(g, s->stream), "launch step graph");
  }
  return FS_OK;
}
}  // namespace

int fs_load_batching(FsSim *s, int *batched, int *decided) {
  CHECK_SIM(s);
  int rc;
  if ((rc = set_device(s))) return rc;
  if (!capturing(s)) tune_lookup(s);
  if ((rc = tune_decide(s))) return rc;
  if (batched) *batched = (s->forms.density > 0 || s->forms.solve > 0) ? 1 : 0;
  if (decided) *decided = s->tune_state == 2 ? 1 : 0;
  return FS_OK;
}

int fs_kernel_forms(FsSim *s, FsKernelForms *out) {
  CHECK_SIM(s);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_kernel_forms: null output");
  int rc;
  if ((rc = set_device(s))) return rc;
  if (!capturing(s)) tune_lookup(s);
  if ((rc = tune_decide(s))) return rc;
  std::memset(out, 0, sizeof(*out));
  out->density_loads = kDensityDepths[s->forms.density];
  out->solve_loads = kDensityDepths[s->forms.solve];
  out->xsph_loads = kXsphDepthList[s->forms.xsph];
  out->decided = s->tune_state == 2 ? uint32_t(s->tune_source) : 0u;
  out->bucket = std::get<1>(tune_key(s));
  for (int k = 0; k < 3; k++)
    for (int c = 0; c < kNumLoadDepths; c++) out->ms[k][c] = s->tune_ms[k][c];
  return FS_OK;
}

int fs_set_kernel_forms(FsSim *s, int density_loads, int solve_loads, int xsph_loads) {
  CHECK_SIM(s);
  if (density_loads < 0 && solve_loads < 0 && xsph_loads < 0) {
    s->tune_state = 0;
    s->tune_phase = 0;
    s->tune_source = 0;
    s->forms = KernelForms{};
    return FS_OK;
  }
  auto index_of = [](const uint32_t *list, int v) {
    for (int c = 0; c < kNumLoadDepths; c++)
      if (int(list[c]) == v) return c;
    return -1;
  };
  const int d = index_of(kDensityDepths, density_loads), so = index_of(kDensityDepths, solve_loads),
            x = index_of(kXsphDepthList, xsph_loads);
  if (d < 0 || so < 0 || x < 0)
    return fail(FS_E_INVALID_ARGUMENT,
                "fs_set_kernel_forms: depths must be in {0, 4, 8, 16} (density, solve) "
                "and {1, 4, 8, 16, 32} (xsph), or all -1");
  int rc;
  if ((rc = set_device(s))) return rc;
  if (s->tune_state == 1 && !capturing(s)) {
    // measured steps in flight: let them finish before their events are reused
    FS_CUDA(cudaEventSynchronize(s->tune_ev[kTuneSteps - 1][8]), "kernel-form measurement");
  }
  if (d >= kPlainCandidates || so >= kPlainCandidates)
    return fail(FS_E_INVALID_ARGUMENT,
                "fs_set_kernel_forms: the density and solve passes have no staged form");
  s->forms.density = uint8_t(d);
  s->forms.solve = uint8_t(so);
  s->forms.xsph = uint8_t(x);
  s->tune_state = 2;
  s->tune_source = 3;
  return FS_OK;
}

int fs_kernel_forms_table(FsKernelFormsEntry *out, uint32_t capacity, uint32_t *count) {
  if (!count) return fail(FS_E_INVALID_ARGUMENT, "fs_kernel_forms_table: null count");
  std::lock_guard<std::mutex> lk(g_forms_mu);
  *count = uint32_t(g_forms_table.size());
  if (!out) return FS_OK;
  uint32_t k = 0;
  for (const auto &kv : g_forms_table) {
    if (k >= capacity) break;
    FsKernelFormsEntry &e = out[k++];
    std::memset(&e, 0, sizeof(e));
    e.device = uint32_t(std::get<0>(kv.first));
    e.bucket = std::get<1>(kv.first);
    e.many_scenes = std::get<2>(kv.first);
    e.iterations = std::get<3>(kv.first);
    e.density_loads = kDensityDepths[kv.second.forms.density];
    e.solve_loads = kDensityDepths[kv.second.forms.solve];
    e.xsph_loads = kXsphDepthList[kv.second.forms.xsph];
    for (int p = 0; p < 3; p++)
      for (int c = 0; c < kNumLoadDepths; c++) e.ms[p][c] = kv.second.ms[p][c];
  }
  return FS_OK;
}

int fs_prepare_steps(FsSim *s, uint32_t nsteps) {
  CHECK_SIM(s);
  int rc;
  if ((rc = set_device(s))) return rc;
  if (!capturing(s)) tune_lookup(s);
  if ((rc = tune_decide(s))) return rc;  // capture with the final choice
  if (nsteps < 2 || s->timing) return FS_OK;
  const uint32_t chunks = (nsteps + kMaxGraphSteps - 1) / kMaxGraphSteps;
  const uint32_t chunk = nsteps / chunks;
  cudaGraphExec_t g = nullptr;
  if ((rc = graph_for(s, chunk, &g))) return rc;
  if (nsteps != chunks * chunk && (rc = graph_for(s, 1, &g))) return rc;
  return FS_OK;
}

int fs_update_sph_params(FsSim *s, const GpuSphParams3D *p) {
  CHECK_SIM(s);
  CHECK_PLAIN(s);
  return fs_batch_update_scene(s, 0, p, nullptr, nullptr, nullptr, nullptr);
}
int fs_update_container_geometry(FsSim *s, const GpuContainerGeometry *g) {
  CHECK_SIM(s);
  CHECK_PLAIN(s);
  return fs_batch_update_scene(s, 0, nullptr, g, nullptr, nullptr, nullptr);
}
int fs_update_mouse_force(FsSim *s, const GpuMouseForce *m) {
  CHECK_SIM(s);
  CHECK_PLAIN(s);
  return fs_batch_update_scene(s, 0, nullptr, nullptr, nullptr, m, nullptr);
}
int fs_update_gravity(FsSim *s, const GpuGravity *g) {
  CHECK_SIM(s);
  CHECK_PLAIN(s);
  return fs_batch_update_scene(s, 0, nullptr, nullptr, g, nullptr, nullptr);
}
int fs_update_rigid_body(FsSim *s, const GpuRigidBody *b) {
  CHECK_SIM(s);
  CHECK_PLAIN(s);
  return fs_batch_update_scene(s, 0, nullptr, nullptr, nullptr, nullptr, b);
}
int fs_set_pcisph_iterations(FsSim *s, uint32_t iterations) {
  CHECK_SIM(s);
  s->iterations = std::max(iterations, 1u);
  return FS_OK;
}

int fs_clear_rigid_body_accum(FsSim *s) {
  CHECK_SIM(s);
  int rc;
  if ((rc = set_device(s))) return rc;
  FS_CUDA(cudaMemsetAsync(s->d.accum, 0, sizeof(GpuRigidBodyAccum) * s->scenes(), s->stream),
          "clear accumulator");
  return FS_OK;
}
int fs_read_rigid_body_accum(FsSim *s, GpuRigidBodyAccum *out) {
  CHECK_SIM(s);
  CHECK_PLAIN(s);
  return fs_batch_read_rigid_body_accum(s, out, 1);
}

int fs_num_particles(const FsSim *s, uint32_t *out) {
  CHECK_SIM(s);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_num_particles: null out");
  *out = s->hb.n_canon;
  return FS_OK;
}

int fs_grid_params(const FsSim *s, GpuGridParams *out) {
  CHECK_SIM(s);
  CHECK_PLAIN(s);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_grid_params: null out");
  *out = s->hu[0].grid;
  return FS_OK;
}

int fs_spawn_particles(FsSim *s, const float position[3], uint32_t count, float spread,
                       uint32_t *spawned) {
  CHECK_SIM(s);
  CHECK_PLAIN(s);
  if (!position || !spawned) return fail(FS_E_INVALID_ARGUMENT, "fs_spawn_particles: null argument");
  *spawned = 0;
  const uint32_t n = s->scene_n[0];
  const uint32_t available = s->max_n - n;
  const uint32_t spawn = std::min(count, available);
  if (spawn == 0) return FS_OK;
  int rc;
  if ((rc = set_device(s))) return rc;
  // the records of sph_3d_grid.rs:1543-1557 (fs_spawn_positions)
  std::vector<SphParticle3D> np(spawn);
  uint32_t made = 0;
  if ((rc = fs_spawn_positions(position, count, spread, n, s->max_n, np.data(), &made)))
    return fail(rc, "fs_spawn_particles: spawn positions");
  if ((rc = write_particles(s, np.data(), n, spawn))) return rc;
  s->scene_n[0] = n + spawn;
  if ((rc = upload_uniforms(s))) return rc;
  *spawned = spawn;
  return FS_OK;
}

int fs_download_particles(FsSim *s, SphParticle3D *out, uint32_t count) {
  CHECK_SIM(s);
  CHECK_PLAIN(s);
  return fs_batch_download_scene(s, 0, out, count);
}

int fs_download_sorted(FsSim *s, SphParticle3D *out, uint32_t count) {
  CHECK_SIM(s);
  CHECK_PLAIN(s);
  if (count > s->scene_n[0])
    return fail(FS_E_CAPACITY, "fs_download_sorted: %u > %u particles", count, s->scene_n[0]);
  if (count && !out) return fail(FS_E_INVALID_ARGUMENT, "fs_download_sorted: null out");
  int rc;
  if ((rc = set_device(s))) return rc;
  return read_sorted(s, 0, out, count);
}

int fs_download_cells(FsSim *s, uint32_t *counts, uint32_t *starts, uint32_t total_cells) {
  CHECK_SIM(s);
  CHECK_PLAIN(s);
  return fs_batch_download_scene_cells(s, 0, counts, starts, total_cells);
}

int fs_download_index_maps(FsSim *s, uint32_t *cell_indices, uint32_t *sorted_to_orig, uint32_t count) {
  CHECK_SIM(s);
  CHECK_PLAIN(s);
  if (count > s->scene_n[0]) return fail(FS_E_CAPACITY, "fs_download_index_maps: %u > %u", count, s->scene_n[0]);
  int rc;
  if ((rc = set_device(s))) return rc;
  return read_index_maps(s, 0, cell_indices, sorted_to_orig, count);
}

int fs_upload_particles(FsSim *s, const SphParticle3D *particles, uint32_t count) {
  CHECK_SIM(s);
  CHECK_PLAIN(s);
  return fs_batch_upload_scene(s, 0, particles, count);
}

int fs_rigid_coupling_set_state(FsSim *s, uint32_t scene, const FsRigidBodyState *state) {
  CHECK_SIM(s);
  CHECK_SCENE(s, scene);
  int rc;
  if ((rc = set_device(s))) return rc;
  const uint8_t flag = state ? 1 : 0;
  if (state)
    FS_CUDA(cudaMemcpyAsync(s->d.rb_state + scene, state, sizeof(FsRigidBodyState),
                            cudaMemcpyHostToDevice, s->stream),
            "upload rigid-body state");
  FS_CUDA(cudaMemcpyAsync(s->d.rb_coupled + scene, &flag, 1, cudaMemcpyHostToDevice, s->stream),
          "rigid-body coupling flag");
  FS_CUDA(cudaStreamSynchronize(s->stream), "rigid-body coupling");
  s->coupled[scene] = flag;
  if (state) FS_CUDA(launch_rigid_sync(s->d, s->scenes(), s->stream), "coupled rigid bodies");
  return FS_OK;
}

int fs_rigid_coupling_get_state(FsSim *s, uint32_t scene, FsRigidBodyState *out) {
  CHECK_SIM(s);
  CHECK_SCENE(s, scene);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_rigid_coupling_get_state: null out");
  if (!s->coupled[scene])
    return fail(FS_E_STATE, "fs_rigid_coupling_get_state: scene %u is not coupled", scene);
  int rc;
  if ((rc = set_device(s))) return rc;
  FS_CUDA(cudaMemcpyAsync(out, s->d.rb_state + scene, sizeof(FsRigidBodyState),
                          cudaMemcpyDeviceToHost, s->stream),
          "download rigid-body state");
  return check_device_error(s);
}

int fs_frames(FsSim *s, uint32_t substeps, uint32_t frames) {
  CHECK_SIM(s);
  if (substeps == 0 || substeps > kMaxGraphSteps)
    return fail(FS_E_INVALID_ARGUMENT, "fs_frames: substeps %u outside [1, %u]", substeps,
                kMaxGraphSteps);
  int rc;
  if ((rc = set_device(s))) return rc;
  if (frames == 0) return FS_OK;
  if (!capturing(s)) tune_lookup(s);
  if ((rc = tune_decide(s))) return rc;
  s->steps_done += uint64_t(substeps) * frames;
  StepGraph &g = s->frame_graph;
  if (!(g.exec && g.steps == substeps && g.n_canon == s->hb.n_canon &&
        g.n_sorted == s->hb.n_sorted && g.iters == s->iterations && g.stream == s->stream &&
        g.forms == s->forms.key())) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = StepGraph{};
    cudaGraph_t graph = nullptr;
    FS_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaError_t e = cudaMemsetAsync(s->d.accum, 0, sizeof(GpuRigidBodyAccum) * s->scenes(),
                                    s->stream);
    rc = e == cudaSuccess ? FS_OK : cuda_fail(e, "clear accumulators");
    for (uint32_t k = 0; k < substeps && rc == FS_OK; k++) rc = enqueue_step(s, false);
    if (rc == FS_OK) {
      e = launch_rigid_frame(s->d, s->scenes(), substeps, s->stream);
      if (e != cudaSuccess) rc = cuda_fail(e, "rigid-body integration");
    }
    e = cudaStreamEndCapture(s->stream, &graph);
    if (rc != FS_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "end capture");
    e = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      g.exec = nullptr;
      return cuda_fail(e, "instantiate frame graph");
    }
    g.steps = substeps;
    g.n_canon = s->hb.n_canon;
    g.n_sorted = s->hb.n_sorted;
    g.iters = s->iterations;
    g.stream = s->stream;
    g.forms = s->forms.key();
  }
  for (uint32_t f = 0; f < frames; f++)
    FS_CUDA(cudaGraphLaunch(g.exec, s->stream), "launch frame graph");
  return FS_OK;
}

int fs_density_splat(FsSim *s, uint32_t scene, const GpuMcGridParams *grid,
                     const GpuContainerGeometry *geom, float *density, int density_on_device) {
  CHECK_SIM(s);
  CHECK_SCENE(s, scene);
  if (!grid || !geom || !density)
    return fail(FS_E_INVALID_ARGUMENT, "fs_density_splat: null argument");
  if (grid->grid_size == 0 || grid->grid_size > 1024)
    return fail(FS_E_INVALID_ARGUMENT, "fs_density_splat: grid_size %u outside [1, 1024]",
                grid->grid_size);
  if (!(grid->kernel_radius > 0.0f) || !std::isfinite(grid->kernel_radius) ||
      !(grid->cell_size > 0.0f) || !std::isfinite(grid->cell_size))
    return fail(FS_E_INVALID_ARGUMENT, "fs_density_splat: kernel_radius and cell_size must be "
                                       "finite and > 0");
  const SplatArgs a = make_splat_args(*grid, *geom, s->hu[scene].grid);
  if (a.cell_radius < 1 || a.cell_radius > 8)
    return fail(FS_E_INVALID_ARGUMENT, "fs_density_splat: splat radius spans %d SPH cells (1..8)",
                a.cell_radius);
  int rc;
  if ((rc = set_device(s))) return rc;
  const size_t voxels = size_t(grid->grid_size) * grid->grid_size * grid->grid_size;
  const uint32_t *begin = s->d.cell_begin + s->hu[scene].c_offset;
  if (density_on_device) {
    FS_CUDA(launch_density_splat(a, s->d.s_pos, begin, density, s->stream), "density splat");
    return FS_OK;
  }
  if (s->splat_cap < voxels) {
    if (s->splat_buf) {
      FS_CUDA(cudaStreamSynchronize(s->stream), "density splat");
      cudaFree(s->splat_buf);
      s->splat_buf = nullptr;
      s->splat_cap = 0;
    }
    FS_CUDA(cudaMalloc(&s->splat_buf, sizeof(float) * voxels), "allocate density field");
    s->splat_cap = voxels;
  }
  FS_CUDA(launch_density_splat(a, s->d.s_pos, begin, s->splat_buf, s->stream), "density splat");
  FS_CUDA(cudaMemcpyAsync(density, s->splat_buf, sizeof(float) * voxels, cudaMemcpyDeviceToHost,
                          s->stream),
          "download density field");
  return check_device_error(s);
}

int fs_device_pointers(FsSim *s, FsDevicePointers *out) {
  CHECK_SIM(s);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_device_pointers: null out");
  out->pos = s->d.p_pos;
  out->vel = s->d.p_vel;
  out->force = s->d.p_force;
  out->sorted_pos = s->d.s_pos;
  out->sorted_vel = s->d.s_vel;
  out->sorted_density = s->d.s_dens;
  out->sorted_normal = s->d.s_nrm;
  out->cell_counts = s->d.counts;
  out->cell_starts = s->d.cell_begin + 1;
  out->cell_begin = s->d.cell_begin;
  out->particle_cell_indices = s->d.cidx;
  out->sorted_to_orig = s->d.s2o;
  out->stream = s->stream;
  return FS_OK;
}

int fs_set_stream(FsSim *s, void *cuda_stream) {
  CHECK_SIM(s);
  int rc;
  if ((rc = set_device(s))) return rc;
  FS_CUDA(cudaStreamSynchronize(s->stream), "drain previous stream");
  s->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : s->own_stream;
  return FS_OK;
}

int fs_sync(FsSim *s) {
  CHECK_SIM(s);
  int rc;
  if ((rc = set_device(s))) return rc;
  return check_device_error(s);
}

int fs_selftest_scan_wait(FsSim *s, int inject, uint32_t *starts_out) {
  CHECK_SIM(s);
  int rc;
  if ((rc = set_device(s))) return rc;
  if (capturing(s)) return fail(FS_E_STATE, "fs_selftest_scan_wait: stream is capturing");
  const uint32_t G = s->cells_total;
  const uint32_t tiles = scan_tiles(G);
  // scratch of its own: the simulation's cell tables stay as the last step
  // left them; only the device error word is shared with the step
  uint32_t *ends = nullptr;
  unsigned long long *desc = nullptr;
  FS_CUDA(cudaMalloc(&ends, sizeof(uint32_t) * size_t(G)), "self-test scratch");
  cudaError_t e = cudaMalloc(&desc, sizeof(unsigned long long) * (size_t(tiles) + 2));
  if (e == cudaSuccess)
    e = cudaMemsetAsync(desc, 0, sizeof(unsigned long long) * (size_t(tiles) + 2), s->stream);
  if (e == cudaSuccess)
    e = launch_scan_selftest(s->d.counts, ends, G, desc, s->d.err, inject != 0, s->stream);
  if (e == cudaSuccess && starts_out)
    e = cudaMemcpyAsync(starts_out, ends, sizeof(uint32_t) * size_t(G), cudaMemcpyDeviceToHost,
                        s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  cudaFree(desc);
  cudaFree(ends);
  FS_CUDA(e, "fs_selftest_scan_wait");
  return FS_OK;
}

int fs_enable_stage_timing(FsSim *s, int enable) {
  CHECK_SIM(s);
  s->timing = enable != 0;
  return FS_OK;
}

int fs_stage_times(FsSim *s, double ms[FS_STAGE_COUNT], uint32_t *steps, int reset) {
  CHECK_SIM(s);
  int rc;
  if ((rc = set_device(s))) return rc;
  if ((rc = check_device_error(s))) return rc;
  if (ms)
    for (int i = 0; i < FS_STAGE_COUNT; i++) ms[i] = s->stage_ms[i];
  if (steps) *steps = s->timed_steps;
  if (reset) {
    for (int i = 0; i < FS_STAGE_COUNT; i++) s->stage_ms[i] = 0.0;
    s->timed_steps = 0;
  }
  return FS_OK;
}

int fs_neighbor_stats(FsSim *s, uint64_t out[FS_STAT_COUNT], int reset) {
  CHECK_SIM(s);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_neighbor_stats: null out");
  int rc;
  if ((rc = set_device(s))) return rc;
  unsigned long long v[STAT_COUNT] = {};
  FS_CUDA(cudaMemcpyAsync(v, s->d.stats, sizeof(v), cudaMemcpyDeviceToHost, s->stream), "read stats");
  if ((rc = check_device_error(s))) return rc;
  for (int i = 0; i < FS_STAT_COUNT; i++) out[i] = v[i];
  if (reset) FS_CUDA(cudaMemset(s->d.stats, 0, sizeof(v)), "reset stats");
  return FS_OK;
}

// ---- batched form ---------------------------------------------------------------

int fs_batch_create(const SphParticle3D *particles, const uint32_t *scene_counts,
                    uint32_t num_scenes, const GpuSphParams3D *params,
                    const GpuContainerGeometry *geoms, const float *sdf, uint32_t sdf_res,
                    int device, uint32_t abi_version, FsSim **out) {
  if (!scene_counts) return fail(FS_E_INVALID_ARGUMENT, "fs_batch_create: scene_counts is null");
  return create_sim("fs_batch_create", particles, scene_counts, num_scenes, params, geoms, 0, sdf,
                    sdf_res, device, abi_version, true, out);
}

int fs_batch_num_scenes(const FsSim *s, uint32_t *out) {
  CHECK_SIM(s);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_batch_num_scenes: null out");
  *out = s->scenes();
  return FS_OK;
}

int fs_batch_scene_info(const FsSim *s, uint32_t scene, FsSceneInfo *out) {
  CHECK_SIM(s);
  CHECK_SCENE(s, scene);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_batch_scene_info: null out");
  const DevUniforms &u = s->hu[scene];
  std::memset(out, 0, sizeof(*out));
  out->particle_offset = u.p_offset;
  out->num_particles = s->scene_n[scene];
  out->active_particles = u.n;
  out->sorted_offset = u.s_offset;
  out->cell_offset = u.c_offset;
  out->total_cells = u.grid.total_cells;
  out->grid = u.grid;
  return FS_OK;
}

int fs_batch_update_scene(FsSim *s, uint32_t scene, const GpuSphParams3D *params,
                          const GpuContainerGeometry *geom, const GpuGravity *gravity,
                          const GpuMouseForce *mouse, const GpuRigidBody *body) {
  CHECK_SIM(s);
  CHECK_SCENE(s, scene);
  if (!params && !geom && !gravity && !mouse && !body)
    return fail(FS_E_INVALID_ARGUMENT, "%s: nothing to update", __func__);
  int rc;
  if ((rc = set_device(s))) return rc;
  DevUniforms &u = s->hu[scene];
  if (params) u.sph = *params;
  if (geom) u.geom = *geom;
  if (gravity) u.gravity = *gravity;
  if (mouse) u.mouse = *mouse;
  if (body) u.rigid = *body;
  return upload_scene(s, scene);
}

int fs_batch_read_rigid_body_accum(FsSim *s, GpuRigidBodyAccum *out, uint32_t num_scenes) {
  CHECK_SIM(s);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_batch_read_rigid_body_accum: null out");
  if (num_scenes > s->scenes())
    return fail(FS_E_INVALID_ARGUMENT, "fs_batch_read_rigid_body_accum: %u > %u scenes",
                num_scenes, s->scenes());
  int rc;
  if ((rc = set_device(s))) return rc;
  if (num_scenes)
    FS_CUDA(cudaMemcpyAsync(out, s->d.accum, sizeof(GpuRigidBodyAccum) * num_scenes,
                            cudaMemcpyDeviceToHost, s->stream),
            "read accumulators");
  return check_device_error(s);
}

int fs_batch_download_scene(FsSim *s, uint32_t scene, SphParticle3D *out, uint32_t count) {
  CHECK_SIM(s);
  CHECK_SCENE(s, scene);
  if (count > s->scene_n[scene])
    return fail(FS_E_CAPACITY, "%s: %u > %u particles", __func__, count, s->scene_n[scene]);
  if (count && !out) return fail(FS_E_INVALID_ARGUMENT, "%s: null out", __func__);
  int rc;
  if ((rc = set_device(s))) return rc;
  return read_canonical(s, s->hu[scene].p_offset, out, count);
}

int fs_export_particles_aos(FsSim *s, uint32_t scene, int sorted, SphParticle3D *device_out,
                            uint32_t count) {
  CHECK_SIM(s);
  CHECK_SCENE(s, scene);
  const uint32_t avail = sorted ? s->hu[scene].n : s->scene_n[scene];
  if (count > avail)
    return fail(FS_E_CAPACITY, "%s: %u > %u particles", __func__, count, avail);
  if (count == 0) return FS_OK;
  if (!device_out) return fail(FS_E_INVALID_ARGUMENT, "%s: null device_out", __func__);
  if (reinterpret_cast<uintptr_t>(device_out) % 16 != 0)
    return fail(FS_E_INVALID_ARGUMENT, "%s: device_out must be 16-byte aligned", __func__);
  int rc;
  if ((rc = set_device(s))) return rc;
  cudaPointerAttributes attr{};
  if (cudaPointerGetAttributes(&attr, device_out) != cudaSuccess ||
      (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)) {
    cudaGetLastError();  // clear the query's error state
    return fail(FS_E_INVALID_ARGUMENT, "%s: device_out is not CUDA device or managed memory",
                __func__);
  }
  if (attr.type == cudaMemoryTypeDevice && attr.device != s->device)
    return fail(FS_E_INVALID_ARGUMENT, "%s: device_out is on device %d, the simulation on %d",
                __func__, attr.device, s->device);
  const DevUniforms &u = s->hu[scene];
  FS_CUDA(launch_export_aos(s->d, sorted != 0, sorted ? u.s_offset : u.p_offset, count,
                            device_out, s->stream),
          "AoS export");
  return FS_OK;
}

int fs_batch_download_scene_sorted(FsSim *s, uint32_t scene, SphParticle3D *out, uint32_t count) {
  CHECK_SIM(s);
  CHECK_SCENE(s, scene);
  if (count > s->hu[scene].n)
    return fail(FS_E_CAPACITY, "%s: %u > %u active particles", __func__, count, s->hu[scene].n);
  if (count && !out) return fail(FS_E_INVALID_ARGUMENT, "%s: null out", __func__);
  int rc;
  if ((rc = set_device(s))) return rc;
  return read_sorted(s, s->hu[scene].s_offset, out, count);
}

int fs_batch_download_scene_cells(FsSim *s, uint32_t scene, uint32_t *counts, uint32_t *starts,
                                  uint32_t total_cells) {
  CHECK_SIM(s);
  CHECK_SCENE(s, scene);
  if (total_cells != s->hu[scene].grid.total_cells)
    return fail(FS_E_INVALID_ARGUMENT, "%s: total_cells %u != grid %u", __func__, total_cells,
                s->hu[scene].grid.total_cells);
  int rc;
  if ((rc = set_device(s))) return rc;
  return read_cells(s, scene, counts, starts);
}

int fs_batch_download_scene_index_maps(FsSim *s, uint32_t scene, uint32_t *cell_indices,
                                       uint32_t *sorted_to_orig, uint32_t count) {
  CHECK_SIM(s);
  CHECK_SCENE(s, scene);
  if (count > s->hu[scene].n)
    return fail(FS_E_CAPACITY, "%s: %u > %u active particles", __func__, count, s->hu[scene].n);
  int rc;
  if ((rc = set_device(s))) return rc;
  return read_index_maps(s, scene, cell_indices, sorted_to_orig, count);
}

int fs_batch_upload_scene(FsSim *s, uint32_t scene, const SphParticle3D *particles,
                          uint32_t count) {
  CHECK_SIM(s);
  CHECK_SCENE(s, scene);
  if (count > s->scene_n[scene])
    return fail(FS_E_CAPACITY, "%s: %u > %u particles", __func__, count, s->scene_n[scene]);
  if (count && !particles) return fail(FS_E_INVALID_ARGUMENT, "%s: null particles", __func__);
  int rc;
  if ((rc = set_device(s))) return rc;
  return write_particles(s, particles, s->hu[scene].p_offset, count);
}

}  // extern "C"
