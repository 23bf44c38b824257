// sim.cu — SphSimulation3DGrid behind the C ABI (include/fluidsph.h).
//
// Mirrors the reference's simulation object (src/simulation/sph_3d_grid.rs):
// construction and buffer allocation (:104-305), step() dispatch sequence
// (:1261-1444), parameter uploads (:1446-1477), rigid-body accumulator
// clear/readback (:1479-1498), buffer getters (:1500-1530) and spawning
// (:1534-1569). All device memory lives in one arena allocated at creation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "fs_internal.h"

using namespace fs;

namespace {

thread_local std::string g_last_error = "no error";

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(FS_E_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

#define FS_CUDA(call, what)                         \
  do {                                              \
    cudaError_t e__ = (call);                       \
    if (e__ != cudaSuccess) return cuda_fail(e__, what); \
  } while (0)

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

}  // namespace

void fs::set_last_error(const char *msg) { g_last_error = msg; }

struct FsSim {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  uint32_t n = 0;      // particles in the canonical buffer (num_particles())
  uint32_t max_n = 0;  // capacity
  uint32_t iterations = 5;  // sph_3d_grid.rs:1253 default
  uint32_t sdf_res = 1;
  GpuGridParams grid{};
  DevUniforms host_u{};  // host mirror of the device parameter block
  DevState d{};
  void *arena = nullptr;
  size_t arena_bytes = 0;
  // CUDA graph of one step (replayed for nsteps > 1)
  cudaGraphExec_t graph_exec = nullptr;
  uint32_t graph_n = 0, graph_iters = 0;
  cudaStream_t graph_stream = nullptr;
  // stage timing
  bool timing = false;
  cudaEvent_t ev[FS_STAGE_COUNT + 1] = {};
  double stage_ms[FS_STAGE_COUNT] = {};
  uint32_t timed_steps = 0;

  uint32_t effective_n() const { return std::min(host_u.sph.num_particles, n); }
};

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
  const size_t G = s->grid.total_cells;
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
  d.anp = c.take<float4>(M);
  d.pred_xp[0] = c.take<float4>(M);
  d.pred_xp[1] = c.take<float4>(M);
  d.pred_rho[0] = c.take<float>(M);
  d.pred_rho[1] = c.take<float>(M);
  d.pred_v = c.take<float4>(M);
  d.cell_of = c.take<uint32_t>(M);
  d.rank_of = c.take<uint32_t>(M);
  d.t_tmp = c.take<uint32_t>(M);
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
  d.task_counters = c.take<uint32_t>(TASK_COUNTERS);
  d.warp_bucket = c.take<uint8_t>((M + 31) / 32);
  d.order_hist = c.take<uint32_t>(2 * 33);
  d.mask_alloc = c.take<unsigned long long>(1);
  d.dir_half = int(std::min<size_t>(M, size_t(1) << 20));
  d.dir_tab = c.take<float4>(2 * size_t(d.dir_half) + 1);
  d.accum = c.take<GpuRigidBodyAccum>(1);
  d.err = c.take<uint32_t>(4);
  d.stats = c.take<unsigned long long>(STAT_COUNT);
  d.u = c.take<DevUniforms>(1);
  *bytes = c.off;
}

void destroy_graph(FsSim *s) {
  if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
  s->graph_exec = nullptr;
}

int upload_uniforms(FsSim *s) {
  s->host_u.n = s->effective_n();
  s->host_u.grid = s->grid;
  s->host_u.grid.num_particles = s->host_u.n;
  s->host_u.sdf_res = s->sdf_res;
  FS_CUDA(cudaMemcpyAsync(s->d.u, &s->host_u, sizeof(DevUniforms), cudaMemcpyHostToDevice,
                          s->stream),
          "upload parameters");
  return FS_OK;
}

int check_device_error(FsSim *s) {
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

// One step: the stage sequence of step(), sph_3d_grid.rs:1261-1444.
int enqueue_step(FsSim *s, bool timed) {
  const uint32_t n = s->effective_n();
  const uint32_t G = s->grid.total_cells;
  cudaStream_t st = s->stream;
  const DevState &d = s->d;
  auto mark = [&](int i) -> int {
    if (timed) FS_CUDA(cudaEventRecord(s->ev[i], st), "record stage event");
    return FS_OK;
  };
  int rc;
  if ((rc = mark(0))) return rc;
  FS_CUDA(cudaMemsetAsync(d.counts, 0, sizeof(uint32_t) * G, st), "grid clear");
  if ((rc = mark(1))) return rc;
  FS_CUDA(launch_hash(d, n, st), "grid build (hash)");
  if ((rc = mark(2))) return rc;
  FS_CUDA(launch_scan(d, G, st), "prefix scan");
  if ((rc = mark(3))) return rc;
  FS_CUDA(launch_scatter(d, n, st), "reorder (scatter)");
  FS_CUDA(launch_sort_gather(d, n, st), "reorder (sort/gather)");
  if ((rc = mark(4))) return rc;
  FS_CUDA(launch_order_warps(d, n, st), "neighbour-pass work order");
  FS_CUDA(launch_density(d, n, st), "density");
  if ((rc = mark(5))) return rc;
  FS_CUDA(launch_xsph(d, n, st), "xsph");
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

int ensure_graph(FsSim *s) {
  const uint32_t n = s->effective_n();
  if (s->graph_exec && s->graph_n == n && s->graph_iters == s->iterations &&
      s->graph_stream == s->stream)
    return FS_OK;
  destroy_graph(s);
  cudaGraph_t g = nullptr;
  FS_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
  int rc = enqueue_step(s, false);
  cudaError_t e = cudaStreamEndCapture(s->stream, &g);
  if (rc != FS_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "end capture");
  e = cudaGraphInstantiate(&s->graph_exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    s->graph_exec = nullptr;
    return cuda_fail(e, "instantiate step graph");
  }
  s->graph_n = n;
  s->graph_iters = s->iterations;
  s->graph_stream = s->stream;
  return FS_OK;
}

#define CHECK_SIM(s) \
  if (!(s)) return fail(FS_E_INVALID_ARGUMENT, "%s: null simulation", __func__)

int set_device(FsSim *s) {
  FS_CUDA(cudaSetDevice(s->device), "cudaSetDevice");
  return FS_OK;
}

}  // namespace

extern "C" {

const char *fs_last_error(void) { return g_last_error.c_str(); }
uint32_t fs_abi_version(void) { return FS_ABI_VERSION; }

int fs_create(const SphParticle3D *particles, uint32_t num_particles, const GpuSphParams3D *params,
              const GpuContainerGeometry *geom, uint32_t max_particles, const float *sdf,
              uint32_t sdf_res, int device, uint32_t abi_version, FsSim **out) {
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_create: out is null");
  *out = nullptr;
  if (abi_version != FS_ABI_VERSION)
    return fail(FS_E_ABI_MISMATCH, "fs_create: caller ABI 0x%08x, library ABI 0x%08x", abi_version,
                FS_ABI_VERSION);
  if (!params || !geom) return fail(FS_E_INVALID_ARGUMENT, "fs_create: params/geometry is null");
  if (num_particles > 0 && !particles)
    return fail(FS_E_INVALID_ARGUMENT, "fs_create: particles is null");
  if (sdf && (sdf_res == 0 || sdf_res > 512))
    return fail(FS_E_INVALID_ARGUMENT, "fs_create: sdf_res %u outside [1, 512]", sdf_res);
  const float h = params->kernel_radius;
  if (!(h > 0.0f) || !std::isfinite(h))
    return fail(FS_E_INVALID_ARGUMENT, "fs_create: kernel_radius must be finite and > 0");
  const uint32_t max_n = std::max(max_particles, num_particles);
  if (max_n > (1u << 30)) return fail(FS_E_CAPACITY, "fs_create: max_particles %u > 2^30", max_n);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(FS_E_NO_DEVICE, "fs_create: no CUDA device");
  if (device < 0 || device >= ndev)
    return fail(FS_E_INVALID_ARGUMENT, "fs_create: device %d of %d", device, ndev);

  FsSim *s = new (std::nothrow) FsSim();
  if (!s) return fail(FS_E_CAPACITY, "fs_create: out of host memory");
  s->device = device;
  s->n = num_particles;
  s->max_n = max_n;
  GpuGridParams grid;
  int rc = fs_grid_params_for(h, num_particles, &grid);
  if (rc != FS_OK) {
    delete s;
    return fail(rc, "fs_create: grid for kernel_radius %g does not fit", double(h));
  }
  s->grid = grid;
  s->sdf_res = sdf ? sdf_res : 1u;
  s->host_u.sph = *params;
  s->host_u.geom = *geom;
  // initial uniforms of SphSimulation3DGrid::new (sph_3d_grid.rs:257-300)
  s->host_u.gravity = GpuGravity{{0.0f, -9.8f, 0.0f}, 0.0f};
  s->host_u.mouse = GpuMouseForce{{0.0f, 0.0f, 0.0f}, 0.5f, 30.0f, 0u, 0u, 0.0f, {0.0f, 0.0f, -1.0f}, 0.0f};
  s->host_u.rigid = GpuRigidBody{{0.0f, 0.0f, 0.0f}, 0.15f, {0.0f, 0.0f, 0.0f}, 0u, 200.0f, 0u, 0.0f, 0.0f,
                                 {1.0f, 0.0f, 0.0f, 0.0f}, {0.0f, 1.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 1.0f, 0.0f}};

  auto bail = [&](int code) {
    if (s->arena) cudaFree(s->arena);
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
    for (auto &e : s->ev)
      if (e) cudaEventDestroy(e);
    delete s;
    return code;
  };
  if ((rc = set_device(s))) return bail(rc);
  cudaError_t e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bail(cuda_fail(e, "create stream"));
  s->stream = s->own_stream;
  for (auto &ev : s->ev) {
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
  if ((rc = upload_uniforms(s))) return bail(rc);
  e = launch_dir_table(s->d, s->stream);
  if (e != cudaSuccess) return bail(cuda_fail(e, "close-pair direction table"));
  if ((rc = write_particles(s, particles, 0, num_particles))) return bail(rc);
  e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return bail(cuda_fail(e, "fs_create"));
  *out = s;
  return FS_OK;
}

int fs_destroy(FsSim *s) {
  if (!s) return FS_OK;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  destroy_graph(s);
  for (auto &e : s->ev)
    if (e) cudaEventDestroy(e);
  if (s->arena) cudaFree(s->arena);
  if (s->own_stream) cudaStreamDestroy(s->own_stream);
  delete s;
  return FS_OK;
}

int fs_step(FsSim *s, uint32_t nsteps) {
  CHECK_SIM(s);
  int rc;
  if ((rc = set_device(s))) return rc;
  if (nsteps == 0) return FS_OK;
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
  if ((rc = ensure_graph(s))) return rc;
  for (uint32_t k = 0; k < nsteps; k++)
    FS_CUDA(cudaGraphLaunch(s->graph_exec, s->stream), "launch step graph");
  return FS_OK;
}

int fs_update_sph_params(FsSim *s, const GpuSphParams3D *p) {
  CHECK_SIM(s);
  if (!p) return fail(FS_E_INVALID_ARGUMENT, "fs_update_sph_params: null params");
  int rc;
  if ((rc = set_device(s))) return rc;
  s->host_u.sph = *p;
  return upload_uniforms(s);
}
int fs_update_container_geometry(FsSim *s, const GpuContainerGeometry *g) {
  CHECK_SIM(s);
  if (!g) return fail(FS_E_INVALID_ARGUMENT, "fs_update_container_geometry: null geometry");
  int rc;
  if ((rc = set_device(s))) return rc;
  s->host_u.geom = *g;
  return upload_uniforms(s);
}
int fs_update_mouse_force(FsSim *s, const GpuMouseForce *m) {
  CHECK_SIM(s);
  if (!m) return fail(FS_E_INVALID_ARGUMENT, "fs_update_mouse_force: null mouse force");
  int rc;
  if ((rc = set_device(s))) return rc;
  s->host_u.mouse = *m;
  return upload_uniforms(s);
}
int fs_update_gravity(FsSim *s, const GpuGravity *g) {
  CHECK_SIM(s);
  if (!g) return fail(FS_E_INVALID_ARGUMENT, "fs_update_gravity: null gravity");
  int rc;
  if ((rc = set_device(s))) return rc;
  s->host_u.gravity = *g;
  return upload_uniforms(s);
}
int fs_update_rigid_body(FsSim *s, const GpuRigidBody *b) {
  CHECK_SIM(s);
  if (!b) return fail(FS_E_INVALID_ARGUMENT, "fs_update_rigid_body: null rigid body");
  int rc;
  if ((rc = set_device(s))) return rc;
  s->host_u.rigid = *b;
  return upload_uniforms(s);
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
  FS_CUDA(cudaMemsetAsync(s->d.accum, 0, sizeof(GpuRigidBodyAccum), s->stream), "clear accumulator");
  return FS_OK;
}
int fs_read_rigid_body_accum(FsSim *s, GpuRigidBodyAccum *out) {
  CHECK_SIM(s);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_read_rigid_body_accum: null out");
  int rc;
  if ((rc = set_device(s))) return rc;
  FS_CUDA(cudaMemcpyAsync(out, s->d.accum, sizeof(GpuRigidBodyAccum), cudaMemcpyDeviceToHost,
                          s->stream),
          "read accumulator");
  return check_device_error(s);
}

int fs_num_particles(const FsSim *s, uint32_t *out) {
  CHECK_SIM(s);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_num_particles: null out");
  *out = s->n;
  return FS_OK;
}

int fs_grid_params(const FsSim *s, GpuGridParams *out) {
  CHECK_SIM(s);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_grid_params: null out");
  *out = s->grid;
  out->num_particles = std::min(s->host_u.sph.num_particles, s->n);
  return FS_OK;
}

int fs_spawn_particles(FsSim *s, const float position[3], uint32_t count, float spread,
                       uint32_t *spawned) {
  CHECK_SIM(s);
  if (!position || !spawned) return fail(FS_E_INVALID_ARGUMENT, "fs_spawn_particles: null argument");
  *spawned = 0;
  const uint32_t available = s->max_n - s->n;
  const uint32_t spawn = std::min(count, available);
  if (spawn == 0) return FS_OK;
  int rc;
  if ((rc = set_device(s))) return rc;
  // golden-angle spiral in layers of 20, sph_3d_grid.rs:1546-1557
  std::vector<SphParticle3D> np(spawn);
  for (uint32_t i = 0; i < spawn; i++) {
    const float angle = float(i) * 2.39996f;
    const float r = spread * std::sqrt(float(i) / float(spawn));
    const uint32_t layer = i / 20u;
    std::memset(&np[i], 0, sizeof(SphParticle3D));
    np[i].position[0] = position[0] + r * std::cos(angle);
    np[i].position[1] = position[1] + float(layer) * spread * 0.3f;
    np[i].position[2] = position[2] + r * std::sin(angle);
  }
  if ((rc = write_particles(s, np.data(), s->n, spawn))) return rc;
  s->n += spawn;
  if ((rc = upload_uniforms(s))) return rc;
  *spawned = spawn;
  return FS_OK;
}

int fs_download_particles(FsSim *s, SphParticle3D *out, uint32_t count) {
  CHECK_SIM(s);
  if (count > s->n) return fail(FS_E_CAPACITY, "fs_download_particles: %u > %u particles", count, s->n);
  if (count && !out) return fail(FS_E_INVALID_ARGUMENT, "fs_download_particles: null out");
  int rc;
  if ((rc = set_device(s))) return rc;
  std::vector<float4> pos(count), vel(count), frc(count), aux(2 * size_t(count));
  const size_t b = sizeof(float4) * count;
  if (count) {
    FS_CUDA(cudaMemcpyAsync(pos.data(), s->d.p_pos, b, cudaMemcpyDeviceToHost, s->stream), "download");
    FS_CUDA(cudaMemcpyAsync(vel.data(), s->d.p_vel, b, cudaMemcpyDeviceToHost, s->stream), "download");
    FS_CUDA(cudaMemcpyAsync(frc.data(), s->d.p_force, b, cudaMemcpyDeviceToHost, s->stream), "download");
    FS_CUDA(cudaMemcpyAsync(aux.data(), s->d.p_aux, 2 * b, cudaMemcpyDeviceToHost, s->stream), "download");
  }
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

int fs_download_sorted(FsSim *s, SphParticle3D *out, uint32_t count) {
  CHECK_SIM(s);
  if (count > s->n) return fail(FS_E_CAPACITY, "fs_download_sorted: %u > %u particles", count, s->n);
  if (count && !out) return fail(FS_E_INVALID_ARGUMENT, "fs_download_sorted: null out");
  int rc;
  if ((rc = set_device(s))) return rc;
  std::vector<float4> pos(count), vel(count), frc(count), nrm(count);
  std::vector<float2> dens(count);
  const size_t b = sizeof(float4) * count;
  if (count) {
    FS_CUDA(cudaMemcpyAsync(pos.data(), s->d.s_pos, b, cudaMemcpyDeviceToHost, s->stream), "download");
    FS_CUDA(cudaMemcpyAsync(vel.data(), s->d.s_vel, b, cudaMemcpyDeviceToHost, s->stream), "download");
    FS_CUDA(cudaMemcpyAsync(frc.data(), s->d.s_frc, b, cudaMemcpyDeviceToHost, s->stream), "download");
    FS_CUDA(cudaMemcpyAsync(nrm.data(), s->d.s_nrm, b, cudaMemcpyDeviceToHost, s->stream), "download");
    FS_CUDA(cudaMemcpyAsync(dens.data(), s->d.s_dens, sizeof(float2) * count, cudaMemcpyDeviceToHost, s->stream), "download");
  }
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

int fs_download_cells(FsSim *s, uint32_t *counts, uint32_t *starts, uint32_t total_cells) {
  CHECK_SIM(s);
  if (total_cells != s->grid.total_cells)
    return fail(FS_E_INVALID_ARGUMENT, "fs_download_cells: total_cells %u != grid %u", total_cells,
                s->grid.total_cells);
  int rc;
  if ((rc = set_device(s))) return rc;
  const size_t b = sizeof(uint32_t) * total_cells;
  if (counts) FS_CUDA(cudaMemcpyAsync(counts, s->d.counts, b, cudaMemcpyDeviceToHost, s->stream), "download counts");
  if (starts) FS_CUDA(cudaMemcpyAsync(starts, s->d.cell_begin + 1, b, cudaMemcpyDeviceToHost, s->stream), "download starts");
  return check_device_error(s);
}

int fs_download_index_maps(FsSim *s, uint32_t *cell_indices, uint32_t *sorted_to_orig, uint32_t count) {
  CHECK_SIM(s);
  if (count > s->n) return fail(FS_E_CAPACITY, "fs_download_index_maps: %u > %u", count, s->n);
  int rc;
  if ((rc = set_device(s))) return rc;
  const size_t b = sizeof(uint32_t) * count;
  if (cell_indices && count) FS_CUDA(cudaMemcpyAsync(cell_indices, s->d.cidx, b, cudaMemcpyDeviceToHost, s->stream), "download cell indices");
  if (sorted_to_orig && count) FS_CUDA(cudaMemcpyAsync(sorted_to_orig, s->d.s2o, b, cudaMemcpyDeviceToHost, s->stream), "download sorted_to_orig");
  return check_device_error(s);
}

int fs_upload_particles(FsSim *s, const SphParticle3D *particles, uint32_t count) {
  CHECK_SIM(s);
  if (count > s->n) return fail(FS_E_CAPACITY, "fs_upload_particles: %u > %u particles", count, s->n);
  if (count && !particles) return fail(FS_E_INVALID_ARGUMENT, "fs_upload_particles: null particles");
  int rc;
  if ((rc = set_device(s))) return rc;
  return write_particles(s, particles, 0, count);
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

}  // extern "C"
