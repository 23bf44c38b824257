// noalloc_scan.cu — the cell prefix scan for callers that cannot allocate
// device memory.
//
// Some callers of this library cannot call cudaMalloc: code running inside a
// CUDA stream capture that must not add allocation nodes, real-time loops
// that forbid allocator calls (and their implicit synchronisation) after
// start-up, and hosts whose memory pools are owned by another runtime. For
// them fs_prefix_scan_noalloc runs the single-pass decoupled-lookback scan
// with its tile descriptors in a fixed file-scope device array instead of in
// memory the library allocates.
//
// Limits and sharing rules:
//   - at most FS_NOALLOC_SCAN_MAX_CELLS cells per call (the array holds one
//     8-byte descriptor per 4096-cell tile: 128 KiB, resident on every GPU
//     that loads the library until the process exits);
//   - every call on a device uses the same array, which keeps the last call's
//     contents; each call clears the part it uses on its stream first, so
//     calls ordered on the GPU are independent, but calls that overlap on the
//     GPU (different streams without ordering) race on the descriptors;
//   - the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current); make that first call
//     before any stream capture. Every later call made while its stream is
//     not capturing looks the address up again, so a context that was torn
//     down and rebuilt (cudaDeviceReset, or another runtime resetting the
//     primary context) is followed; a call inside a capture uses the address
//     of the last call outside one.
#include <cuda_runtime.h>

#include <mutex>

#include "fs_internal.h"

namespace {

constexpr uint32_t kMaxTiles = FS_NOALLOC_SCAN_MAX_CELLS / fs::SCAN_TILE;
constexpr int kMaxDevices = 64;

// descriptors [0, tiles), the ticket word at [tiles], a status word for
// callers that pass no status pointer at [kMaxTiles + 1]
static __device__ __align__(256) unsigned long long g_scan_scratch[kMaxTiles + 2];

std::mutex g_setup_mutex;
unsigned long long *g_scratch_addr[kMaxDevices] = {};

// Device address of g_scan_scratch on the current device (host code may not
// take the address of a __device__ symbol directly). Looked up again on every
// call with `refresh` set: after a context reset the module is loaded anew and
// the array can sit at another address.
cudaError_t scratch_address(int device, bool refresh, unsigned long long **out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (refresh || !g_scratch_addr[device]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scan_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[device] = static_cast<unsigned long long *>(p);
  }
  *out = g_scratch_addr[device];
  return cudaSuccess;
}

}  // namespace

static_assert(FS_NOALLOC_SCAN_MAX_CELLS % fs::SCAN_TILE == 0, "whole tiles");

extern "C" int fs_prefix_scan_noalloc(const uint32_t *cell_counts, uint32_t *cell_starts,
                                      uint32_t total_cells, uint32_t *device_status,
                                      void *stream) {
  if (total_cells == 0) return FS_OK;
  if (!cell_counts || !cell_starts) {
    fs::set_last_error("fs_prefix_scan_noalloc: null counts or starts");
    return FS_E_INVALID_ARGUMENT;
  }
  if (total_cells > FS_NOALLOC_SCAN_MAX_CELLS) {
    fs::set_last_error("fs_prefix_scan_noalloc: total_cells exceeds FS_NOALLOC_SCAN_MAX_CELLS");
    return FS_E_CAPACITY;
  }
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess || device < 0 || device >= kMaxDevices) {
    fs::set_last_error("fs_prefix_scan_noalloc: no usable current CUDA device");
    return FS_E_NO_DEVICE;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // outside a capture the lookup is an ordinary runtime call; inside one the
  // cached address is used (a lookup there could load the module)
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &capture) != cudaSuccess) {
    (void)cudaGetLastError();
    capture = cudaStreamCaptureStatusActive;
  }
  unsigned long long *scratch = nullptr;
  e = scratch_address(device, capture == cudaStreamCaptureStatusNone, &scratch);
  if (e != cudaSuccess) {
    fs::set_last_error("fs_prefix_scan_noalloc: cudaGetSymbolAddress failed");
    return FS_E_CUDA;
  }
  const uint32_t tiles = fs::scan_tiles(total_cells);
  // descriptors and ticket start at zero for every call
  e = cudaMemsetAsync(scratch, 0, sizeof(unsigned long long) * (size_t(tiles) + 1), st);
  if (e != cudaSuccess) {
    fs::set_last_error("fs_prefix_scan_noalloc: clearing the scratch array failed");
    return FS_E_CUDA;
  }
  uint32_t *status = device_status
                         ? device_status
                         : reinterpret_cast<uint32_t *>(scratch + kMaxTiles + 1);
  if (!device_status) {
    // the internal status word starts clear too, like the descriptors
    e = cudaMemsetAsync(status, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) {
      fs::set_last_error("fs_prefix_scan_noalloc: clearing the status word failed");
      return FS_E_CUDA;
    }
  }
  // the reference's cell_starts are the inclusive prefix sums
  e = fs::launch_scan_with_scratch(cell_counts, cell_starts, total_cells, scratch, status, st);
  if (e != cudaSuccess) {
    fs::set_last_error("fs_prefix_scan_noalloc: kernel launch failed");
    return FS_E_CUDA;
  }
  return FS_OK;
}
