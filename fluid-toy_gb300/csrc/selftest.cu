// selftest.cu — exhaustive check of the correctly rounded arithmetic that
// the force and solve passes use in place of IEEE division, reciprocal and
// square root (rcp_fast, sqrt_fast, markstein with the fast_ok / fast_num_ok
// range checks, sph_device.cuh).
//
// rcp_fast and sqrt_fast refine the hardware approximations rcp.approx and
// rsqrt.approx, whose exact outputs no document fixes, so their bit-identity
// with __frcp_rn and sqrtf is established here on every one of the 2^32
// input bit patterns, through the same pattern the kernels use (the fast
// result where the operand passes fast_ok, the IEEE operation otherwise).
// Quotients (a Markstein correction from rcp_fast) are compared with IEEE
// division on 2^32 pseudo-random operand pairs (random bit patterns: every
// sign, exponent and special value) the same way. NaN results compare equal
// to NaN.
#include <cuda_runtime.h>

#include "sph_device.cuh"

namespace fs {
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {  // SplitMix64 finaliser
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ bool same(float a, float b) {
  return (a != a && b != b) || __float_as_uint(a) == __float_as_uint(b);
}

__global__ void __launch_bounds__(256) k_check_unary(unsigned long long *bad) {
  unsigned long long n_rcp = 0, n_sqrt = 0;
  const uint64_t total = 1ull << 32;
  for (uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; t < total;
       t += uint64_t(gridDim.x) * blockDim.x) {
    const float x = __uint_as_float(uint32_t(t));
    const bool ok = fast_ok(x);
    if (!same(ok ? rcp_fast(x) : __frcp_rn(x), __frcp_rn(x))) n_rcp++;
    if (!same(ok ? sqrt_fast(x) : sqrtf(x), sqrtf(x))) n_sqrt++;
  }
  if (n_rcp) atomicAdd(bad + 0, n_rcp);
  if (n_sqrt) atomicAdd(bad + 1, n_sqrt);
}

__global__ void __launch_bounds__(256) k_check_div(unsigned long long *bad) {
  unsigned long long n_div = 0, n_in = 0;
  const uint64_t total = 1ull << 32;
  for (uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; t < total;
       t += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t r = mix64(t);
    float a = __uint_as_float(uint32_t(r));
    float b = __uint_as_float(uint32_t(r >> 32));
    if ((t & 1u) == 0u) {
      // half of the pairs drawn inside the fast range (exponents uniform in
      // [-60, 59], random significands and signs), where the fast path runs
      const uint32_t ea = uint32_t((r >> 8) % 120u) + 67u, eb = uint32_t((r >> 20) % 120u) + 67u;
      a = __uint_as_float((uint32_t(r) & 0x807fffffu) | (ea << 23));
      b = __uint_as_float((uint32_t(r >> 32) & 0x807fffffu) | (eb << 23));
    }
    const bool ok = fast_num_ok(a) && fast_ok(b);
    if (ok) n_in++;
    const float q = ok ? markstein(a, b, rcp_fast(b)) : a / b;
    if (!same(q, a / b)) n_div++;
  }
  if (n_div) atomicAdd(bad + 2, n_div);
  atomicAdd(bad + 3, n_in);
}

// ---- FP32 pipe throughput ---------------------------------------------------
// Eight independent dependency chains per thread, kFp32Unroll steps each per
// loop iteration. FUSED: one fma.rn per step (2 FLOP); otherwise one FMUL
// and one FADD per step (2 FLOP in two instructions: the non-contracted
// arithmetic the bit-exact kernels compile to under -fmad=false). The
// result is written so that nothing is eliminated.
constexpr int kFp32Unroll = 16;

template <bool FUSED>
__global__ void __launch_bounds__(256) k_fp32_rate(float *__restrict__ out, float b, float c,
                                                  int iters) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; k++) a[k] = float(t & 1023u) * 1e-3f + float(k);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int u = 0; u < kFp32Unroll; u++) {
#pragma unroll
      for (int k = 0; k < 8; k++) {
        if (FUSED) {
          a[k] = __fmaf_rn(a[k], b, c);
        } else {
          a[k] = __fmul_rn(a[k], b);
          a[k] = __fadd_rn(a[k], c);
        }
      }
    }
  }
  float sum = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; k++) sum += a[k];
  out[t] = sum;
}

}  // namespace
}  // namespace fs

extern "C" int fs_selftest_fp32_rate(int device, double tflops[2]) {
  if (!tflops) return FS_E_INVALID_ARGUMENT;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return FS_E_NO_DEVICE;
  if (device < 0 || device >= count) return FS_E_INVALID_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) return FS_E_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return FS_E_CUDA;
  const int blocks = sms * 4, threads = 256;  // 32 warps per SM
  const int iters = 16384;
  float *out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * size_t(blocks) * threads) != cudaSuccess) return FS_E_CUDA;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  const double flop = 2.0 * 8.0 * fs::kFp32Unroll * double(iters) * blocks * threads;
  for (int fused = 1; fused >= 0 && e == cudaSuccess; fused--) {
    float best = 0.0f;
    for (int rep = 0; rep < 6 && e == cudaSuccess; rep++) {  // first launch warms up
      e = cudaEventRecord(e0);
      if (fused)
        fs::k_fp32_rate<true><<<blocks, threads>>>(out, 0.999999f, 1e-7f, iters);
      else
        fs::k_fp32_rate<false><<<blocks, threads>>>(out, 0.999999f, 1e-7f, iters);
      if (e == cudaSuccess) e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaEventRecord(e1);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0.0f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0 && (best == 0.0f || ms < best)) best = ms;
    }
    tflops[fused ? 0 : 1] = best > 0.0f ? flop / (double(best) * 1e-3) / 1e12 : 0.0;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  return e == cudaSuccess ? FS_OK : FS_E_CUDA;
}

extern "C" int fs_selftest_arithmetic(int device, unsigned long long results[4]) {
  if (!results) return FS_E_INVALID_ARGUMENT;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return FS_E_NO_DEVICE;
  if (device < 0 || device >= count) return FS_E_INVALID_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) return FS_E_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return FS_E_CUDA;
  unsigned long long *bad = nullptr;
  if (cudaMalloc(&bad, 4 * sizeof(unsigned long long)) != cudaSuccess) return FS_E_CUDA;
  cudaError_t e = cudaMemset(bad, 0, 4 * sizeof(unsigned long long));
  if (e == cudaSuccess) {
    fs::k_check_unary<<<sms * 8, 256>>>(bad);
    fs::k_check_div<<<sms * 8, 256>>>(bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpy(results, bad, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(bad);
  return e == cudaSuccess ? FS_OK : FS_E_CUDA;
}
