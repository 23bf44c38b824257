// fs_sim.h — the simulation object behind the C ABI (sim.cu) and the host
// helpers shared with the reverse pass (adjoint.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "fs_internal.h"

namespace fs {

// Record fs_last_error's text and return `code`.
int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

#define FS_CUDA(call, what)                                   \
  do {                                                        \
    cudaError_t e__ = (call);                                 \
    if (e__ != cudaSuccess) return ::fs::cuda_fail(e__, what); \
  } while (0)

// Step graphs: one captured graph per step count, a few kept.
constexpr uint32_t kMaxGraphSteps = 256;
constexpr int kGraphSlots = 4;

struct StepGraph {
  cudaGraphExec_t exec = nullptr;
  uint32_t steps = 0, n_canon = 0, n_sorted = 0, iters = 0;
  uint32_t forms = 0;  // KernelForms::key() the graph was captured with
  cudaStream_t stream = nullptr;
  uint64_t last_use = 0;
};

}  // namespace fs

struct FsSim {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  bool batch = false;       // made by fs_batch_create
  uint32_t max_n = 0;       // canonical capacity
  uint32_t iterations = 5;  // sph_3d_grid.rs:1253 default
  uint32_t sdf_res = 1;
  std::vector<uint32_t> scene_n;  // canonical particles of each scene
  std::vector<fs::DevUniforms> hu;    // host mirror of the per-scene parameter blocks
  fs::DevBatch hb{};                  // host mirror of the batch header
  uint32_t cells_total = 0;
  fs::DevState d{};
  void *arena = nullptr;
  size_t arena_bytes = 0;
  fs::StepGraph graphs[fs::kGraphSlots];
  uint64_t graph_clock = 0;
  fs::StepGraph frame_graph;    // one frame of fs_frames (steps + rigid-body integration)
  std::vector<uint8_t> coupled;  // scenes whose rigid body is device-coupled
  float *splat_buf = nullptr;  // device staging of host-bound density fields
  size_t splat_cap = 0;
  // Load depths of the neighbour passes (DevState::load_*, the same results
  // whatever they are), tuned per particle-count bucket: a simulation whose
  // bucket (floor(log2 hashed particles), one or many scenes, PCISPH
  // iterations) is in the process-wide table takes its entry; otherwise,
  // once it has run kTuneAfterSteps steps, its next kTuneSteps steps run each
  // candidate depth of the density and solve passes twice (palindromic
  // order) and every XSPH depth in every one of those steps (rotating order;
  // XSPH rewrites the same velocities from the same inputs), with events
  // around the passes, whatever the fs_step call sizes; the next call waits
  // for them once, and each pass keeps its fastest depth (density and solve
  // by the mean of their two samples, XSPH by the median of its ten), which
  // also enters the table.
  fs::KernelForms forms;
  int tune_state = 0;   // 0 measuring (phase), 1 measured (events pending), 2 decided
  int tune_source = 0;  // how the forms were decided: 1 measured, 2 table, 3 set by the caller
  int tune_phase = 0;   // measured steps so far
  // per measured step: the stage marks, then the boundaries of the XSPH
  // launches (one per depth)
  cudaEvent_t tune_ev[2 * fs::kNumLoadDepths][FS_STAGE_COUNT + fs::kNumLoadDepths + 1] = {};
  float tune_ms[3][fs::kNumLoadDepths] = {};  // measured ms per step per pass (density, XSPH, solve) and depth
  uint64_t steps_done = 0;
  // stage timing
  bool timing = false;
  cudaEvent_t ev[FS_STAGE_COUNT + 1] = {};
  double stage_ms[FS_STAGE_COUNT] = {};
  uint32_t timed_steps = 0;

  uint32_t scenes() const { return uint32_t(scene_n.size()); }
  bool any_coupled() const {
    for (uint8_t c : coupled)
      if (c) return true;
    return false;
  }
  uint32_t active(uint32_t k) const { return std::min(hu[k].sph.num_particles, scene_n[k]); }
};

namespace fs {

int set_device(FsSim *s);
// Synchronise the stream and report a device-side error word, if set.
int check_device_error(FsSim *s);
// Enqueue one step on the simulation's stream (on `dv`'s buffers if given;
// batched loads as decided for the simulation, or as `batched` when 0 / 1).
// One step on the simulation's stream. timed: stage events into s->ev;
// marks (if not null): stage events into marks[0..FS_STAGE_COUNT) instead;
// forms (if not null): these load depths instead of the simulation's.
// xsph_all >= 0 (a measured step, with marks): every XSPH depth is launched,
// starting at depth index xsph_all, marks[FS_STAGE_COUNT + i] before launch i
// and marks[FS_STAGE_COUNT + kNumLoadDepths] after the last.
int enqueue_step(FsSim *s, bool timed, const DevState *dv = nullptr,
                 const KernelForms *forms = nullptr, cudaEvent_t *marks = nullptr,
                 int xsph_all = -1);
// Enqueue only the grid build (clear, hash, scan, reorder) of the current state.
int enqueue_grid_build(FsSim *s);

}  // namespace fs
