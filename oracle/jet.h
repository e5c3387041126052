// Test infrastructure, not product code.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg may load the oracle; the GPU library never links it.
//
// Forward-mode automatic differentiation ("jets") used by the oracle to obtain factor Jacobians
// with respect to the tangent-space perturbation, which is exactly what the reference's generated
// `with_linearization` code computes symbolically
// (symforce/codegen/codegen.py Codegen.with_linearization; e.g.
// symforce/examples/bundle_adjustment_in_the_large/gen/snavely_reprojection_factor.h:33-41).
#pragma once

#include <cmath>

namespace oracle {

template <int N>
struct Jet {
  double a;     // value
  double v[N];  // derivative with respect to the N seeded inputs

  Jet() : a(0) {
    for (int i = 0; i < N; ++i) v[i] = 0;
  }
  Jet(double x) : a(x) {  // NOLINT: implicit constants
    for (int i = 0; i < N; ++i) v[i] = 0;
  }
  static Jet Seed(double x, int k) {
    Jet j(x);
    if (k >= 0 && k < N) j.v[k] = 1.0;
    return j;
  }
};

template <int N>
inline Jet<N> operator+(const Jet<N>& x, const Jet<N>& y) {
  Jet<N> r(x.a + y.a);
  for (int i = 0; i < N; ++i) r.v[i] = x.v[i] + y.v[i];
  return r;
}
template <int N>
inline Jet<N> operator-(const Jet<N>& x, const Jet<N>& y) {
  Jet<N> r(x.a - y.a);
  for (int i = 0; i < N; ++i) r.v[i] = x.v[i] - y.v[i];
  return r;
}
template <int N>
inline Jet<N> operator-(const Jet<N>& x) {
  Jet<N> r(-x.a);
  for (int i = 0; i < N; ++i) r.v[i] = -x.v[i];
  return r;
}
template <int N>
inline Jet<N> operator*(const Jet<N>& x, const Jet<N>& y) {
  Jet<N> r(x.a * y.a);
  for (int i = 0; i < N; ++i) r.v[i] = x.a * y.v[i] + x.v[i] * y.a;
  return r;
}
template <int N>
inline Jet<N> operator/(const Jet<N>& x, const Jet<N>& y) {
  Jet<N> r(x.a / y.a);
  const double inv = 1.0 / y.a;
  for (int i = 0; i < N; ++i) r.v[i] = (x.v[i] - r.a * y.v[i]) * inv;
  return r;
}
template <int N>
inline Jet<N> operator+(const Jet<N>& x, double y) { return x + Jet<N>(y); }
template <int N>
inline Jet<N> operator+(double x, const Jet<N>& y) { return Jet<N>(x) + y; }
template <int N>
inline Jet<N> operator-(const Jet<N>& x, double y) { return x - Jet<N>(y); }
template <int N>
inline Jet<N> operator-(double x, const Jet<N>& y) { return Jet<N>(x) - y; }
template <int N>
inline Jet<N> operator*(const Jet<N>& x, double y) {
  Jet<N> r(x.a * y);
  for (int i = 0; i < N; ++i) r.v[i] = x.v[i] * y;
  return r;
}
template <int N>
inline Jet<N> operator*(double x, const Jet<N>& y) { return y * x; }
template <int N>
inline Jet<N> operator/(const Jet<N>& x, double y) { return x * (1.0 / y); }
template <int N>
inline Jet<N> operator/(double x, const Jet<N>& y) { return Jet<N>(x) / y; }

template <int N>
inline Jet<N> Chain(const Jet<N>& x, double fx, double dfx) {
  Jet<N> r(fx);
  for (int i = 0; i < N; ++i) r.v[i] = dfx * x.v[i];
  return r;
}

template <int N>
inline Jet<N> sqrt(const Jet<N>& x) {
  const double s = std::sqrt(x.a);
  return Chain(x, s, 0.5 / s);
}
template <int N>
inline Jet<N> sin(const Jet<N>& x) { return Chain(x, std::sin(x.a), std::cos(x.a)); }
template <int N>
inline Jet<N> cos(const Jet<N>& x) { return Chain(x, std::cos(x.a), -std::sin(x.a)); }
template <int N>
inline Jet<N> acos(const Jet<N>& x) {
  return Chain(x, std::acos(x.a), -1.0 / std::sqrt(1.0 - x.a * x.a));
}
template <int N>
inline Jet<N> log1p(const Jet<N>& x) { return Chain(x, std::log1p(x.a), 1.0 / (1.0 + x.a)); }
template <int N>
inline Jet<N> fabs(const Jet<N>& x) { return x.a < 0 ? -x : x; }
template <int N>
inline Jet<N> atan2(const Jet<N>& y, const Jet<N>& x) {
  Jet<N> r(std::atan2(y.a, x.a));
  const double d = x.a * x.a + y.a * y.a;
  for (int i = 0; i < N; ++i) r.v[i] = (x.a * y.v[i] - y.a * x.v[i]) / d;
  return r;
}
// x^e for a constant exponent e.
template <int N>
inline Jet<N> pow(const Jet<N>& x, double e) {
  return Chain(x, std::pow(x.a, e), e * std::pow(x.a, e - 1.0));
}
// min(x, c) with a constant c: derivative follows the selected branch.
template <int N>
inline Jet<N> fmin(const Jet<N>& x, double c) { return x.a < c ? x : Jet<N>(c); }

// Plain-double overloads so the factor templates compile for Scalar = double.
inline double Value(double x) { return x; }
template <int N>
inline double Value(const Jet<N>& x) { return x.a; }

}  // namespace oracle
