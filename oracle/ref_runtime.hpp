// ref_runtime.hpp — C++ meanings for the WGSL subset used by fluid-toy's step
// shaders, so that oracle/wgsl2cpp.py can translate those shaders mechanically
// and run them on the CPU (TEST INFRASTRUCTURE ONLY: the translation pins the
// oracle restatement; it is never part of the product).
//
// Semantics chosen to match WGSL on an IEEE-754 binary32 machine with no
// operation fusion (compile with -ffp-contract=off):
//   - f32 arithmetic is single IEEE ops; vec ops act per component;
//   - dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z, length = sqrt(dot(v, v)),
//     normalize(v) = v / length(v);
//   - f32 -> i32/u32 conversion truncates toward zero and saturates (NaN -> 0);
//   - atomics act immediately (invocations run one at a time, in index order);
//   - textureSampleLevel is clamp-to-edge trilinear filtering with exact f32
//     weights (hardware samplers use reduced-precision weights).
#pragma once

#include <cmath>
#include <coroutine>
#include <cstdint>
#include <cstring>
#include <functional>
#include <thread>
#include <type_traits>
#include <vector>

namespace wgsl {

using f32 = float;
using u32 = uint32_t;
using i32 = int32_t;

template <class T>
struct vec2 {
  T x{}, y{};
  vec2() = default;
  explicit vec2(T s) : x(s), y(s) {}
  vec2(T a, T b) : x(a), y(b) {}
};

template <class T>
struct vec3 {
  T x{}, y{}, z{};
  vec3() = default;
  explicit vec3(T s) : x(s), y(s), z(s) {}
  vec3(T a, T b, T c) : x(a), y(b), z(c) {}
  template <class U, class = std::enable_if_t<!std::is_same_v<U, T>>>
  explicit vec3(const vec3<U> &o);
  vec2<T> xz() const { return vec2<T>(x, z); }
  vec2<T> xy() const { return vec2<T>(x, y); }
  T &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  const T &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <class T>
struct vec4 {
  T x{}, y{}, z{}, w{};
  vec4() = default;
  explicit vec4(T s) : x(s), y(s), z(s), w(s) {}
  vec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
  vec3<T> xyz() const { return vec3<T>(x, y, z); }
};

static_assert(sizeof(vec3<float>) == 12, "vec3 must be 12 bytes");
static_assert(sizeof(vec4<float>) == 16, "vec4 must be 16 bytes");

// scalar conversions (WGSL value constructors)
inline i32 to_i32(float v) {
  if (std::isnan(v)) return 0;
  if (v >= 2147483647.0f) return INT32_MAX;
  if (v <= -2147483648.0f) return INT32_MIN;
  return i32(v);
}
inline i32 to_i32(double v) { return to_i32(float(v)); }
inline i32 to_i32(i32 v) { return v; }
inline i32 to_i32(u32 v) { return i32(v); }
inline u32 to_u32(float v) {
  if (std::isnan(v) || v <= 0.0f) return 0u;
  if (v >= 4294967295.0f) return UINT32_MAX;
  return u32(v);
}
inline u32 to_u32(i32 v) { return u32(v); }
inline u32 to_u32(u32 v) { return v; }
inline f32 to_f32(f32 v) { return v; }
inline f32 to_f32(i32 v) { return f32(v); }
inline f32 to_f32(u32 v) { return f32(v); }

template <class T, class U>
inline T convert(U v) {
  if constexpr (std::is_same_v<T, i32>) return to_i32(v);
  else if constexpr (std::is_same_v<T, u32>) return to_u32(v);
  else return to_f32(v);
}

template <class T>
template <class U, class>
vec3<T>::vec3(const vec3<U> &o) : x(convert<T>(o.x)), y(convert<T>(o.y)), z(convert<T>(o.z)) {}

// ---- operators -------------------------------------------------------------
#define WGSL_V3_BINOP(op)                                                               \
  template <class T> inline vec3<T> operator op(vec3<T> a, vec3<T> b) {               \
    return vec3<T>(a.x op b.x, a.y op b.y, a.z op b.z);                                \
  }                                                                                     \
  template <class T> inline vec3<T> operator op(vec3<T> a, T s) {                      \
    return vec3<T>(a.x op s, a.y op s, a.z op s);                                      \
  }                                                                                     \
  template <class T> inline vec3<T> operator op(T s, vec3<T> a) {                      \
    return vec3<T>(s op a.x, s op a.y, s op a.z);                                      \
  }                                                                                     \
  template <class T> inline vec3<T> &operator op##=(vec3<T> & a, vec3<T> b) {          \
    a = a op b;                                                                         \
    return a;                                                                           \
  }                                                                                     \
  template <class T> inline vec3<T> &operator op##=(vec3<T> & a, T s) {                \
    a = a op s;                                                                         \
    return a;                                                                           \
  }
WGSL_V3_BINOP(+)
WGSL_V3_BINOP(-)
WGSL_V3_BINOP(*)
WGSL_V3_BINOP(/)
#undef WGSL_V3_BINOP
template <class T> inline vec3<T> operator-(vec3<T> a) { return vec3<T>(-a.x, -a.y, -a.z); }
template <class T> inline vec2<T> operator/(vec2<T> a, T s) { return vec2<T>(a.x / s, a.y / s); }

// ---- builtins ----------------------------------------------------------------
template <class T> inline T dot(vec3<T> a, vec3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline T dot(vec2<T> a, vec2<T> b) { return a.x * b.x + a.y * b.y; }
inline f32 length(vec3<f32> v) { return std::sqrt(dot(v, v)); }
inline f32 length(vec2<f32> v) { return std::sqrt(dot(v, v)); }
inline vec3<f32> normalize(vec3<f32> v) { return v / length(v); }
inline vec3<f32> cross(vec3<f32> a, vec3<f32> b) {
  return vec3<f32>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline f32 sqrt(f32 x) { return std::sqrt(x); }
// sin/cos: the same fixed FP32 evaluation the oracle restatement uses for the
// close-pair direction (WGSL leaves the accuracy to the implementation).
inline float reduce_half_pi(float x, int *q) {
  const float k = std::rint(x * 0.636619747f);
  float r = std::fma(-k, 1.57079637f, x);
  r = std::fma(-k, -4.37113883e-08f, r);
  r = std::fma(-k, -1.71512451e-15f, r);
  *q = int(k) & 3;
  return r;
}
inline float sin_poly(float r) {
  const float r2 = r * r;
  float p = std::fma(r2, 2.75573188e-06f, -1.98412701e-04f);
  p = std::fma(r2, p, 8.33333377e-03f);
  p = std::fma(r2, p, -0.166666672f);
  return std::fma(r * r2, p, r);
}
inline float cos_poly(float r) {
  const float r2 = r * r;
  float p = std::fma(r2, -2.755732e-07f, 2.48015876e-05f);
  p = std::fma(r2, p, -1.38888892e-03f);
  p = std::fma(r2, p, 4.16666679e-02f);
  p = std::fma(r2, p, -0.5f);
  return std::fma(r2, p, 1.0f);
}
inline f32 sin(f32 x) {
  int q;
  const float r = reduce_half_pi(x, &q);
  const float s = sin_poly(r), c = cos_poly(r);
  return q == 0 ? s : (q == 1 ? c : (q == 2 ? -s : -c));
}
inline f32 cos(f32 x) {
  int q;
  const float r = reduce_half_pi(x, &q);
  const float s = sin_poly(r), c = cos_poly(r);
  return q == 0 ? c : (q == 1 ? -s : (q == 2 ? -c : s));
}
inline f32 abs(f32 x) { return std::fabs(x); }
inline vec3<f32> abs(vec3<f32> v) { return vec3<f32>(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }
inline f32 floor(f32 x) { return std::floor(x); }
inline f32 ceil(f32 x) { return std::ceil(x); }
inline f32 fract(f32 x) { return x - std::floor(x); }
inline f32 round(f32 x) { return std::nearbyint(x); }  // WGSL: half to even
inline vec3<f32> mix(vec3<f32> a, vec3<f32> b, f32 t) { return a * (1.0f - t) + b * t; }
template <class T> inline T bitcast(f32 v) {
  static_assert(sizeof(T) == 4, "32-bit bitcast");
  T out;
  std::memcpy(&out, &v, 4);
  return out;
}
// pow: WGSL leaves its precision to the implementation. A positive integral
// exponent up to 64 is evaluated as binary exponentiation in double, rounded
// once to f32 (the library's own definition, fs_pow_f32); other exponents use
// std::pow in double.
inline f32 pow(f32 x, f32 y) {
  if (y >= 1.0f && y <= 64.0f && y == std::floor(y)) {
    double r = 1.0, b = double(x);
    for (unsigned n = unsigned(y); n; n >>= 1) {
      if (n & 1u) r *= b;
      b *= b;
    }
    return f32(r);
  }
  return f32(std::pow(double(x), double(y)));
}
inline vec3<f32> floor(vec3<f32> v) { return vec3<f32>(std::floor(v.x), std::floor(v.y), std::floor(v.z)); }
inline f32 max(f32 a, f32 b) { return std::fmax(a, b); }
inline f32 min(f32 a, f32 b) { return std::fmin(a, b); }
inline i32 max(i32 a, i32 b) { return a > b ? a : b; }
inline i32 min(i32 a, i32 b) { return a < b ? a : b; }
inline u32 max(u32 a, u32 b) { return a > b ? a : b; }
inline u32 min(u32 a, u32 b) { return a < b ? a : b; }
inline f32 clamp(f32 e, f32 lo, f32 hi) { return min(max(e, lo), hi); }
inline i32 clamp(i32 e, i32 lo, i32 hi) { return min(max(e, lo), hi); }
inline f32 sign(f32 x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }

// atomics: invocations run one at a time
template <class T, class U> inline T atomicAdd(T *p, U v) {
  T old = *p;
  *p = T(old + T(v));
  return old;
}
template <class T, class U> inline void atomicStore(T *p, U v) { *p = T(v); }
template <class T, class U> inline T atomicMax(T *p, U v) {
  const T old = *p;
  if (T(v) > old) *p = T(v);
  return old;
}

// fixed-size arrays (workgroup memory)
template <class T, int N>
struct array {
  T v[N];
  T &operator[](u32 i) { return v[i]; }
  const T &operator[](u32 i) const { return v[i]; }
};

// textures: a res^3 R32Float volume, x fastest
template <class T>
struct texture_3d {
  const float *data = nullptr;
  int res = 1;
};
struct sampler {};
// write-only r32float storage volume, dim^3 texels, x fastest
struct texture_storage_3d_r32f {
  float *data = nullptr;
  u32 dim = 0;
};
inline void textureStore(texture_storage_3d_r32f &t, vec3<i32> c, vec4<f32> v) {
  t.data[size_t(c.x) + size_t(t.dim) * (size_t(c.y) + size_t(t.dim) * size_t(c.z))] = v.x;
}
struct vec4r {
  float r;
};
inline vec4r textureSampleLevel(const texture_3d<f32> &t, const sampler &, vec3<f32> uvw, f32) {
  const int res = t.res;
  auto texel = [&](int x, int y, int z) -> float {
    x = x < 0 ? 0 : (x > res - 1 ? res - 1 : x);
    y = y < 0 ? 0 : (y > res - 1 ? res - 1 : y);
    z = z < 0 ? 0 : (z > res - 1 ? res - 1 : z);
    return t.data[size_t(x) + size_t(y) * res + size_t(z) * res * res];
  };
  const float tx = uvw.x * float(res) - 0.5f;
  const float ty = uvw.y * float(res) - 0.5f;
  const float tz = uvw.z * float(res) - 0.5f;
  const float fx0 = std::floor(tx), fy0 = std::floor(ty), fz0 = std::floor(tz);
  const float ax = tx - fx0, ay = ty - fy0, az = tz - fz0;
  auto clampi = [&](int v) { return v < -1 ? -1 : (v > res ? res : v); };
  const int x0 = clampi(to_i32(fx0)), y0 = clampi(to_i32(fy0)), z0 = clampi(to_i32(fz0));
  auto mix = [](float a, float b, float w) { return a * (1.0f - w) + b * w; };
  const float c00 = mix(texel(x0, y0, z0), texel(x0 + 1, y0, z0), ax);
  const float c10 = mix(texel(x0, y0 + 1, z0), texel(x0 + 1, y0 + 1, z0), ax);
  const float c01 = mix(texel(x0, y0, z0 + 1), texel(x0 + 1, y0, z0 + 1), ax);
  const float c11 = mix(texel(x0, y0 + 1, z0 + 1), texel(x0 + 1, y0 + 1, z0 + 1), ax);
  const float c0 = mix(c00, c10, ay);
  const float c1 = mix(c01, c11, ay);
  return vec4r{mix(c0, c1, az)};
}

// ---- dispatch ------------------------------------------------------------------
using uvec3 = vec3<u32>;

// Invocations one at a time in global-index order (no barriers in the shader).
inline void dispatch_sequential(u32 groups, u32 wg_size,
                                const std::function<void(uvec3, uvec3, uvec3)> &fn) {
  for (u32 g = 0; g < groups; g++)
    for (u32 l = 0; l < wg_size; l++) fn(uvec3(g * wg_size + l, 0u, 0u), uvec3(l, 0u, 0u), uvec3(g, 0u, 0u));
}

// 3-D dispatch, invocations one at a time (no barriers in the shader).
inline void dispatch_sequential_3d(u32 gx, u32 gy, u32 gz, uvec3 wg,
                                   const std::function<void(uvec3, uvec3, uvec3)> &fn) {
  for (u32 z = 0; z < gz; z++)
    for (u32 y = 0; y < gy; y++)
      for (u32 x = 0; x < gx; x++)
        for (u32 lz = 0; lz < wg.z; lz++)
          for (u32 ly = 0; ly < wg.y; ly++)
            for (u32 lx = 0; lx < wg.x; lx++)
              fn(uvec3(x * wg.x + lx, y * wg.y + ly, z * wg.z + lz), uvec3(lx, ly, lz),
                 uvec3(x, y, z));
}

// Shaders with workgroupBarrier(): every function that reaches a barrier is
// translated into a coroutine (`task`). A barrier suspends the invocation; the
// dispatcher resumes all invocations of the workgroup in turn, so each one
// runs up to the next barrier before any passes it (WGSL requires barriers in
// uniform control flow). Workgroups run one after another.
inline thread_local std::coroutine_handle<> tl_suspended_leaf;

struct task {
  struct promise_type {
    std::coroutine_handle<> continuation;
    task get_return_object() { return task{std::coroutine_handle<promise_type>::from_promise(*this)}; }
    std::suspend_always initial_suspend() noexcept { return {}; }
    struct final_awaiter {
      bool await_ready() noexcept { return false; }
      std::coroutine_handle<> await_suspend(std::coroutine_handle<promise_type> h) noexcept {
        auto c = h.promise().continuation;
        return c ? c : std::noop_coroutine();
      }
      void await_resume() noexcept {}
    };
    final_awaiter final_suspend() noexcept { return {}; }
    void return_void() {}
    void unhandled_exception() { std::terminate(); }
  };
  std::coroutine_handle<promise_type> h;
  explicit task(std::coroutine_handle<promise_type> hh) : h(hh) {}
  task(task &&o) noexcept : h(o.h) { o.h = {}; }
  task(const task &) = delete;
  ~task() {
    if (h) h.destroy();
  }
  // awaiting a nested barrier function: run it now, come back when it ends
  bool await_ready() { return false; }
  std::coroutine_handle<> await_suspend(std::coroutine_handle<> cont) {
    h.promise().continuation = cont;
    return h;
  }
  void await_resume() {}
};

struct barrier_point {
  bool await_ready() noexcept { return false; }
  void await_suspend(std::coroutine_handle<> h) noexcept { tl_suspended_leaf = h; }
  void await_resume() noexcept {}
};

inline void dispatch_barriers(u32 groups, u32 wg_size, const std::function<void()> &reset_shared,
                              const std::function<task(uvec3, uvec3, uvec3)> &fn) {
  for (u32 g = 0; g < groups; g++) {
    reset_shared();
    std::vector<task> inv;
    std::vector<std::coroutine_handle<>> next;
    inv.reserve(wg_size);
    for (u32 l = 0; l < wg_size; l++) {
      inv.push_back(fn(uvec3(g * wg_size + l, 0u, 0u), uvec3(l, 0u, 0u), uvec3(g, 0u, 0u)));
      next.push_back(inv.back().h);
    }
    bool running = true;
    while (running) {
      running = false;
      for (u32 l = 0; l < wg_size; l++) {
        if (!next[l]) continue;
        tl_suspended_leaf = nullptr;
        next[l].resume();
        next[l] = tl_suspended_leaf;  // null once the invocation has finished
        if (next[l]) running = true;
      }
    }
  }
}

}  // namespace wgsl
