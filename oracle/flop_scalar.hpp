// Test infrastructure: a scalar type that counts floating-point operations.
//
// Instantiating the oracle (oracle.hpp) on FlopScalar yields the algorithmic
// FLOP count of one evaluation of each function: +, -, *, / each count 1,
// sqrt counts 1, and sin/cos pairs are counted separately.  The counts are
// the per-evaluation work figures used for the roofline of the GPU kernels.
#pragma once

#include <cmath>
#include <limits>

namespace orc {

struct FlopCounter {
  static thread_local long long ops;
  static thread_local long long sincos;
};

struct FlopScalar {
  double v = 0.0;
  FlopScalar() = default;
  FlopScalar(double x) : v(x) {}  // NOLINT: implicit on purpose (literals)
  explicit operator double() const { return v; }
};

inline FlopScalar operator+(FlopScalar a, FlopScalar b) { ++FlopCounter::ops; return FlopScalar(a.v + b.v); }
inline FlopScalar operator-(FlopScalar a, FlopScalar b) { ++FlopCounter::ops; return FlopScalar(a.v - b.v); }
inline FlopScalar operator*(FlopScalar a, FlopScalar b) { ++FlopCounter::ops; return FlopScalar(a.v * b.v); }
inline FlopScalar operator/(FlopScalar a, FlopScalar b) { ++FlopCounter::ops; return FlopScalar(a.v / b.v); }
inline FlopScalar operator-(FlopScalar a) { return FlopScalar(-a.v); }
inline FlopScalar& operator+=(FlopScalar& a, FlopScalar b) { a = a + b; return a; }
inline FlopScalar& operator-=(FlopScalar& a, FlopScalar b) { a = a - b; return a; }
inline FlopScalar& operator*=(FlopScalar& a, FlopScalar b) { a = a * b; return a; }
inline FlopScalar& operator/=(FlopScalar& a, FlopScalar b) { a = a / b; return a; }
inline bool operator<(FlopScalar a, FlopScalar b) { return a.v < b.v; }
inline bool operator>(FlopScalar a, FlopScalar b) { return a.v > b.v; }
inline bool operator<=(FlopScalar a, FlopScalar b) { return a.v <= b.v; }
inline bool operator>=(FlopScalar a, FlopScalar b) { return a.v >= b.v; }
inline bool operator==(FlopScalar a, FlopScalar b) { return a.v == b.v; }
inline bool operator!=(FlopScalar a, FlopScalar b) { return a.v != b.v; }

inline FlopScalar o_sqrt(FlopScalar x) { ++FlopCounter::ops; return FlopScalar(std::sqrt(x.v)); }
inline void o_sincos(FlopScalar a, FlopScalar* s, FlopScalar* c) {
  ++FlopCounter::sincos;
  *s = FlopScalar(std::sin(a.v));
  *c = FlopScalar(std::cos(a.v));
}
template <> inline FlopScalar o_eps<FlopScalar>() { return FlopScalar(std::numeric_limits<double>::epsilon()); }

}  // namespace orc
