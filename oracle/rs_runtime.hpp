// rs_runtime.hpp — the C++ meaning of the Rust builtins that
// oracle/rs2cpp.py's translations of fluid-toy's host functions use.
//
// TEST INFRASTRUCTURE ONLY (see rs2cpp.py). Each item states the Rust
// semantics it reproduces:
//   f32::sqrt / abs / ceil / floor / sin / cos   the C library's float
//                                                functions (what rustc's
//                                                llvm.* intrinsics call)
//   f32::sin_cos                                 (sin(x), cos(x))
//   f32::powi(n)                                 square-and-multiply from the
//                                                lowest bit (LLVM's expansion
//                                                of llvm.powi for a constant
//                                                exponent, and compiler-rt's
//                                                __powisf2, agree on it)
//   f32::min / max                               IEEE minNum / maxNum (fminf)
//   integer min / max                            std::min / std::max
//   x as T                                       float -> int saturates, NaN
//                                                -> 0; enum -> its value;
//                                                otherwise static_cast
//   [a, b, ...] / [x; N]                         std::array
//   iter().map(f).sum()                          left fold from -0.0
// plus host stand-ins for the wgpu calls spawn_particles makes (a buffer is
// a byte vector; write_buffer copies the bytes at the offset).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <tuple>
#include <type_traits>
#include <vector>

namespace rs {

constexpr float PI_F32 = 3.14159265358979323846f;  // std::f32::consts::PI

template <class T, class U>
inline T as(U x) {
  if constexpr (std::is_enum_v<U>) {
    return static_cast<T>(static_cast<std::underlying_type_t<U>>(x));
  } else if constexpr (std::is_floating_point_v<U> && std::is_integral_v<T>) {
    if (x != x) return T(0);
    if (x <= U(std::numeric_limits<T>::min())) return std::numeric_limits<T>::min();
    if (x >= U(std::numeric_limits<T>::max())) return std::numeric_limits<T>::max();
    return static_cast<T>(x);
  } else {
    return static_cast<T>(x);
  }
}

template <class... A>
inline auto arr(A... a) {
  return std::array<std::common_type_t<A...>, sizeof...(A)>{a...};
}
template <size_t N, class T>
inline std::array<T, N> rep(T x) {
  std::array<T, N> out;
  out.fill(x);
  return out;
}

inline float sqrt(float x) { return std::sqrt(x); }
inline float abs(float x) { return std::fabs(x); }
inline float ceil(float x) { return std::ceil(x); }
inline float floor(float x) { return std::floor(x); }
inline float sin(float x) { return std::sin(x); }
inline float cos(float x) { return std::cos(x); }
inline std::tuple<float, float> sin_cos(float x) { return {std::sin(x), std::cos(x)}; }

inline float powi(float x, int n) {
  if (n == 0) return 1.0f;
  const bool recip = n < 0;
  unsigned b = recip ? unsigned(-n) : unsigned(n);
  float r = 0.0f, a = x;
  bool have = false;
  while (b) {
    if (b & 1u) {
      r = have ? r * a : a;
      have = true;
    }
    b >>= 1;
    if (b) a = a * a;
  }
  return recip ? 1.0f / r : r;
}

inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
template <class T, std::enable_if_t<std::is_integral_v<T>, int> = 0>
inline T min(T a, T b) { return std::min(a, b); }
template <class T, std::enable_if_t<std::is_integral_v<T>, int> = 0>
inline T max(T a, T b) { return std::max(a, b); }

template <class C, class F>
inline auto sum_map(const C &c, F f) {
  using R = decltype(f(*std::begin(c)));
  R acc = R(-0.0);
  for (const auto &v : c) acc = acc + f(v);
  return acc;
}

template <class T>
inline size_t size_of() { return sizeof(T); }

// ---- wgpu / bytemuck / Vec stand-ins (spawn_particles) ----------------------------
struct Bytes {
  const uint8_t *data;
  size_t size;
};
struct AnyVec {  // Vec<T> of plain records, kept as bytes
  std::vector<uint8_t> bytes;
  template <class T>
  void push_back(const T &x) {
    const auto *p = reinterpret_cast<const uint8_t *>(&x);
    bytes.insert(bytes.end(), p, p + sizeof(T));
  }
};
inline AnyVec Vec_with_capacity(size_t) { return AnyVec{}; }
inline Bytes bytemuck_cast_slice(const AnyVec &v) { return {v.bytes.data(), v.bytes.size()}; }
template <class T>
inline Bytes bytemuck_bytes_of(const T &x) {
  return {reinterpret_cast<const uint8_t *>(&x), sizeof(T)};
}
struct wgpu_Queue {};
struct Buffer {
  mutable std::vector<uint8_t> bytes;
};
inline void method_write_buffer(const wgpu_Queue &, const Buffer &b, uint64_t offset, Bytes src) {
  if (b.bytes.size() < offset + src.size) b.bytes.resize(offset + src.size);
  std::memcpy(b.bytes.data() + offset, src.data, src.size);
}

}  // namespace rs
