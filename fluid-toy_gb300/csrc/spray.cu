// spray.cu — the whitewater system behind fs_spray_* (include/fluidsph.h),
// the counterpart of SpraySystem (src/simulation/spray.rs:96-491) attached to
// one scene of a simulation. Its device state: the ring buffer of diffuse
// particles, the write head, the two potential ceilings, the per-frame
// maxima and live counts, and the emission scratch (per-particle spawn
// counts and their scan).
#include <cstring>
#include <new>
#include <vector>

#include "fs_sim.h"
#include "spray_internal.h"

using namespace fs;

struct FsSpray {
  FsSim *sim = nullptr;
  uint32_t scene = 0;
  uint32_t max_particles = 0;
  void *mem = nullptr;
  GpuSprayParticle *ring = nullptr;
  uint32_t *head = nullptr;      // write head
  float *limits = nullptr;       // [2]
  uint32_t *stats = nullptr;     // [8]: emit maxima [4], live counts [4]
  uint32_t *counts = nullptr;    // [cap]
  uint32_t *ends = nullptr;      // [cap]
  unsigned long long *tiles = nullptr;
  uint32_t cap = 0;              // emitters the scratch holds
};

namespace {

size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

#define CHECK_SPRAY(p) \
  if (!(p) || !(p)->sim) return fail(FS_E_INVALID_ARGUMENT, "%s: null handle", __func__)

// initial ceilings, spray.rs:29-30
constexpr float AUTO_TA_INIT = 3.0f, AUTO_WC_INIT = 1.0f;

int reset_state(FsSpray *p) {
  FsSim *s = p->sim;
  FS_CUDA(cudaMemsetAsync(p->ring, 0, sizeof(GpuSprayParticle) * p->max_particles, s->stream),
          "clear spray ring");
  FS_CUDA(cudaMemsetAsync(p->head, 0, sizeof(uint32_t), s->stream), "clear write head");
  FS_CUDA(cudaMemsetAsync(p->stats, 0, sizeof(uint32_t) * 8, s->stream), "clear spray stats");
  const float lim[2] = {AUTO_TA_INIT, AUTO_WC_INIT};
  FS_CUDA(cudaMemcpyAsync(p->limits, lim, sizeof(lim), cudaMemcpyHostToDevice, s->stream),
          "spray ceilings");
  FS_CUDA(cudaStreamSynchronize(s->stream), "spray reset");
  return FS_OK;
}

}  // namespace

extern "C" {

int fs_spray_create(FsSim *sim, uint32_t scene, uint32_t max_particles, FsSpray **out) {
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_spray_create: out is null");
  *out = nullptr;
  if (!sim) return fail(FS_E_INVALID_ARGUMENT, "fs_spray_create: null simulation");
  if (scene >= sim->scenes())
    return fail(FS_E_INVALID_ARGUMENT, "fs_spray_create: scene %u of %u", scene, sim->scenes());
  if (max_particles == 0 || max_particles > (1u << 28))
    return fail(FS_E_INVALID_ARGUMENT, "fs_spray_create: max_particles %u outside [1, 2^28]",
                max_particles);
  int rc;
  if ((rc = set_device(sim))) return rc;
  FsSpray *p = new (std::nothrow) FsSpray();
  if (!p) return fail(FS_E_CAPACITY, "fs_spray_create: out of host memory");
  p->sim = sim;
  p->scene = scene;
  p->max_particles = max_particles;
  p->cap = std::max<uint32_t>(sim->scene_n[scene], 1u);
  const size_t tiles = scan_tiles(p->cap) + 1;
  const size_t bytes = a256(sizeof(GpuSprayParticle) * max_particles) + a256(4) + a256(8) +
                       a256(32) + 2 * a256(sizeof(uint32_t) * p->cap) + a256(8 * tiles);
  cudaError_t e = cudaMalloc(&p->mem, bytes);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(e, "allocate spray buffers");
  }
  char *c = static_cast<char *>(p->mem);
  p->ring = reinterpret_cast<GpuSprayParticle *>(c);
  c += a256(sizeof(GpuSprayParticle) * max_particles);
  p->head = reinterpret_cast<uint32_t *>(c);
  c += a256(4);
  p->limits = reinterpret_cast<float *>(c);
  c += a256(8);
  p->stats = reinterpret_cast<uint32_t *>(c);
  c += a256(32);
  p->counts = reinterpret_cast<uint32_t *>(c);
  c += a256(sizeof(uint32_t) * p->cap);
  p->ends = reinterpret_cast<uint32_t *>(c);
  c += a256(sizeof(uint32_t) * p->cap);
  p->tiles = reinterpret_cast<unsigned long long *>(c);
  if ((rc = reset_state(p))) {
    cudaFree(p->mem);
    delete p;
    return rc;
  }
  *out = p;
  return FS_OK;
}

int fs_spray_destroy(FsSpray *p) {
  if (!p) return FS_OK;
  if (p->sim) {
    cudaSetDevice(p->sim->device);
    cudaStreamSynchronize(p->sim->stream);
  }
  if (p->mem) cudaFree(p->mem);
  delete p;
  return FS_OK;
}

int fs_spray_reset(FsSpray *p) {
  CHECK_SPRAY(p);
  int rc;
  if ((rc = set_device(p->sim))) return rc;
  return reset_state(p);
}

int fs_spray_step(FsSpray *p, const GpuSprayParams *params) {
  CHECK_SPRAY(p);
  if (!params) return fail(FS_E_INVALID_ARGUMENT, "fs_spray_step: null params");
  if (params->max_particles != p->max_particles)
    return fail(FS_E_INVALID_ARGUMENT, "fs_spray_step: params.max_particles %u != ring %u",
                params->max_particles, p->max_particles);
  FsSim *s = p->sim;
  int rc;
  if ((rc = set_device(s))) return rc;
  const DevUniforms &u = s->hu[p->scene];
  const uint32_t n = std::min(std::min(params->num_sph_particles, u.n), p->cap);
  SprayView sv;
  sv.u = s->d.u + p->scene;
  sv.s_pos = s->d.s_pos;
  sv.s_vel = s->d.s_vel;
  sv.s_dens = s->d.s_dens;
  sv.s_nrm = s->d.s_nrm;
  sv.begin = s->d.cell_begin + u.c_offset;
  sv.s_offset = u.s_offset;
  sv.write_head = p->head;
  sv.limits = p->limits;
  sv.emit_stats = p->stats;
  sv.live_stats = p->stats + 4;
  SprayFrame f;
  f.params = *params;
  FS_CUDA(launch_spray_frame(sv, f, n, p->counts, p->ends, p->tiles, s->d.err, p->ring, s->stream),
          "spray frame");
  return FS_OK;
}

int fs_spray_stats(FsSpray *p, uint32_t out[4]) {
  CHECK_SPRAY(p);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_spray_stats: null out");
  int rc;
  if ((rc = set_device(p->sim))) return rc;
  FS_CUDA(cudaMemcpyAsync(out, p->stats + 4, sizeof(uint32_t) * 4, cudaMemcpyDeviceToHost,
                          p->sim->stream),
          "read spray stats");
  return check_device_error(p->sim);
}

int fs_spray_limits(FsSpray *p, float limits[2], uint32_t *write_head) {
  CHECK_SPRAY(p);
  int rc;
  if ((rc = set_device(p->sim))) return rc;
  if (limits)
    FS_CUDA(cudaMemcpyAsync(limits, p->limits, sizeof(float) * 2, cudaMemcpyDeviceToHost,
                            p->sim->stream),
            "read spray ceilings");
  if (write_head)
    FS_CUDA(cudaMemcpyAsync(write_head, p->head, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                            p->sim->stream),
            "read write head");
  return check_device_error(p->sim);
}

int fs_spray_download(FsSpray *p, GpuSprayParticle *out, uint32_t count) {
  CHECK_SPRAY(p);
  if (count > p->max_particles)
    return fail(FS_E_CAPACITY, "fs_spray_download: %u > %u slots", count, p->max_particles);
  if (count && !out) return fail(FS_E_INVALID_ARGUMENT, "fs_spray_download: null out");
  int rc;
  if ((rc = set_device(p->sim))) return rc;
  if (count)
    FS_CUDA(cudaMemcpyAsync(out, p->ring, sizeof(GpuSprayParticle) * count,
                            cudaMemcpyDeviceToHost, p->sim->stream),
            "download spray ring");
  return check_device_error(p->sim);
}

int fs_spray_device_buffer(FsSpray *p, void **out) {
  CHECK_SPRAY(p);
  if (!out) return fail(FS_E_INVALID_ARGUMENT, "fs_spray_device_buffer: null out");
  *out = p->ring;
  return FS_OK;
}

}  // extern "C"
