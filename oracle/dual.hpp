// dual.hpp — forward-mode (tangent) numbers for the oracle.
//
// TEST INFRASTRUCTURE ONLY. Dual<V> carries a value of type V (float: the
// FP32 restatement, double: the FP64 twin) and one directional derivative in
// double. Every value operation is the same single IEEE operation the plain
// oracle performs on V, so an Oracle<Dual<float>> follows the FP32
// restatement's trajectory bit for bit while propagating d(state)/d(seed)
// through the same branches: the exact derivative of the piecewise-smooth
// discretisation the reverse pass differentiates. Branches compare values.
#pragma once

#include <cmath>
#include <type_traits>

template <class V>
struct Dual {
  V v{};
  double d = 0.0;
  Dual() = default;
  Dual(V x) : v(x), d(0.0) {}
  Dual(V x, double dx) : v(x), d(dx) {}
  template <class U, class = std::enable_if_t<std::is_arithmetic_v<U> && !std::is_same_v<U, V>>>
  Dual(U x) : v(V(x)), d(0.0) {}
  explicit operator double() const { return double(v); }
  explicit operator float() const { return float(v); }

  friend Dual operator+(Dual a, Dual b) { return Dual(V(a.v + b.v), a.d + b.d); }
  friend Dual operator-(Dual a, Dual b) { return Dual(V(a.v - b.v), a.d - b.d); }
  friend Dual operator*(Dual a, Dual b) {
    return Dual(V(a.v * b.v), a.d * double(b.v) + double(a.v) * b.d);
  }
  friend Dual operator/(Dual a, Dual b) {
    const V q = V(a.v / b.v);
    return Dual(q, (a.d - double(q) * b.d) / double(b.v));
  }
  friend Dual operator-(Dual a) { return Dual(V(-a.v), -a.d); }
  Dual &operator+=(Dual b) { return *this = *this + b; }
  Dual &operator-=(Dual b) { return *this = *this - b; }
  Dual &operator*=(Dual b) { return *this = *this * b; }
  Dual &operator/=(Dual b) { return *this = *this / b; }
  friend bool operator<(Dual a, Dual b) { return a.v < b.v; }
  friend bool operator>(Dual a, Dual b) { return a.v > b.v; }
  friend bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
  friend bool operator>=(Dual a, Dual b) { return a.v >= b.v; }
  friend bool operator==(Dual a, Dual b) { return a.v == b.v; }
  friend bool operator!=(Dual a, Dual b) { return a.v != b.v; }
};

template <class V> inline Dual<V> sqrt_(Dual<V> a) {
  const V r = std::sqrt(a.v);
  return Dual<V>(r, r == V(0) ? 0.0 : a.d / (2.0 * double(r)));
}
template <class V> inline Dual<V> floor_(Dual<V> a) { return Dual<V>(std::floor(a.v), 0.0); }
template <class V> inline Dual<V> fabs_(Dual<V> a) {
  return Dual<V>(std::fabs(a.v), a.v < V(0) ? -a.d : a.d);
}
template <class V> inline Dual<V> fmax_(Dual<V> a, Dual<V> b) {
  if (std::isnan(a.v)) return b;
  if (std::isnan(b.v)) return a;
  return a.v >= b.v ? a : b;
}
template <class V> inline Dual<V> fmin_(Dual<V> a, Dual<V> b) {
  if (std::isnan(a.v)) return b;
  if (std::isnan(b.v)) return a;
  return a.v <= b.v ? a : b;
}
