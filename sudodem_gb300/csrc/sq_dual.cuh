// Forward-mode dual numbers for the adjoint of the superellipsoid timestep.
//
// Dual<N> carries a value and N tangent components.  Every operation computes its value with
// exactly the double operation the plain (T = double) instantiation of the same templated code
// performs, in the same order, so a replay of a timestep in Dual<N> takes bit for bit the same
// branches (Levenberg-Marquardt accept/reject and stop tests, contact gates, Coulomb cap,
// damping signs) as the double run it replays.  Tangents are derivatives of the smooth
// function each branch defines ("differentiated as taken").  The translation unit that
// includes this header is compiled with --fmad=false, as the forward kernels are.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#define SQA_HD __host__ __device__ __forceinline__

namespace sqadj {

template <int N>
struct Dual {
  double v;
  double d[N];
  SQA_HD Dual() {}
  SQA_HD Dual(double x) : v(x) {
#pragma unroll
    for (int k = 0; k < N; k++) d[k] = 0.0;
  }
};

SQA_HD double val(double x) { return x; }
template <int N> SQA_HD double val(const Dual<N>& x) { return x.v; }

// seeds: x is input number k of the current chunk (tangent e_k)
template <int N> SQA_HD Dual<N> seed(double x, int k) { Dual<N> r(x); if (k >= 0 && k < N) r.d[k] = 1.0; return r; }

template <int N> SQA_HD Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r; r.v = -a.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = -a.d[k];
  return r;
}
template <int N> SQA_HD Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <int N> SQA_HD Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <int N> SQA_HD Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <int N> SQA_HD Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
// mixed with plain doubles (constants): the value is the same double operation
template <int N> SQA_HD Dual<N> operator+(const Dual<N>& a, double b) { Dual<N> r = a; r.v = a.v + b; return r; }
template <int N> SQA_HD Dual<N> operator+(double a, const Dual<N>& b) { Dual<N> r = b; r.v = a + b.v; return r; }
template <int N> SQA_HD Dual<N> operator-(const Dual<N>& a, double b) { Dual<N> r = a; r.v = a.v - b; return r; }
template <int N> SQA_HD Dual<N> operator-(double a, const Dual<N>& b) {
  Dual<N> r; r.v = a - b.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = -b.d[k];
  return r;
}
template <int N> SQA_HD Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r; r.v = a.v * b;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] * b;
  return r;
}
template <int N> SQA_HD Dual<N> operator*(double a, const Dual<N>& b) {
  Dual<N> r; r.v = a * b.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a * b.d[k];
  return r;
}
template <int N> SQA_HD Dual<N> operator/(const Dual<N>& a, double b) {
  Dual<N> r; r.v = a.v / b;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] / b;
  return r;
}
template <int N> SQA_HD Dual<N> operator/(double a, const Dual<N>& b) {
  Dual<N> r; r.v = a / b.v;
  const double f = -r.v / b.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = f * b.d[k];
  return r;
}
template <int N, class U> SQA_HD Dual<N>& operator+=(Dual<N>& a, const U& b) { a = a + b; return a; }
template <int N, class U> SQA_HD Dual<N>& operator-=(Dual<N>& a, const U& b) { a = a - b; return a; }
template <int N, class U> SQA_HD Dual<N>& operator*=(Dual<N>& a, const U& b) { a = a * b; return a; }
template <int N, class U> SQA_HD Dual<N>& operator/=(Dual<N>& a, const U& b) { a = a / b; return a; }

// ---------------------------------------------------------------------------
// Functions, overloaded for double (the forward kernels) and Dual<N> (the replay).
SQA_HD double tsqrt(double x) { return sqrt(x); }
SQA_HD double tfabs(double x) { return fabs(x); }
SQA_HD double tatan(double x) { return atan(x); }
SQA_HD double tatan2(double y, double x) { return atan2(y, x); }
SQA_HD double tpow(double a, double b) { return pow(a, b); }
SQA_HD void tsincos(double x, double* s, double* c) { sincos(x, s, c); }

template <int N> SQA_HD Dual<N> tsqrt(const Dual<N>& a) {
  Dual<N> r; r.v = sqrt(a.v);
  const double f = r.v > 0 ? 0.5 / r.v : 0.0;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] * f;
  return r;
}
template <int N> SQA_HD Dual<N> tfabs(const Dual<N>& a) {
  Dual<N> r; r.v = fabs(a.v);
  const double s = a.v < 0 ? -1.0 : 1.0;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = s * a.d[k];
  return r;
}
template <int N> SQA_HD Dual<N> tatan(const Dual<N>& a) {
  Dual<N> r; r.v = atan(a.v);
  const double f = 1.0 / (1.0 + a.v * a.v);
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] * f;
  return r;
}
template <int N> SQA_HD Dual<N> tatan2(const Dual<N>& y, const Dual<N>& x) {
  Dual<N> r; r.v = atan2(y.v, x.v);
  const double den = x.v * x.v + y.v * y.v;
  const double fx = den > 0 ? x.v / den : 0.0, fy = den > 0 ? y.v / den : 0.0;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = fx * y.d[k] - fy * x.d[k];
  return r;
}
template <int N> SQA_HD void tsincos(const Dual<N>& a, Dual<N>* s, Dual<N>* c) {
  double sv, cv;
  sincos(a.v, &sv, &cv);
  s->v = sv; c->v = cv;
#pragma unroll
  for (int k = 0; k < N; k++) { s->d[k] = cv * a.d[k]; c->d[k] = -sv * a.d[k]; }
}
// a^b for a >= 0 when the exponent varies (every such call site takes the power of an
// absolute value).  At a == 0 the tangent is set to 0: the exact derivative is 0 or
// unbounded there, and an argument that is exactly zero only arises on a coordinate plane of
// the local frame.  With a constant exponent the base may be negative (the cube in lmder2's
// damping update): d(a^b) = b a^b / a.
template <int N> SQA_HD Dual<N> tpow(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = pow(a.v, b.v);
  const bool pos = a.v > 0;
  const double fa = pos ? r.v * b.v / a.v : 0.0, fb = pos ? r.v * log(a.v) : 0.0;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = fa * a.d[k] + fb * b.d[k];
  return r;
}
template <int N> SQA_HD Dual<N> tpow(const Dual<N>& a, double b) {
  Dual<N> r; r.v = pow(a.v, b);
  const double fa = a.v != 0 ? r.v * b / a.v : 0.0;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = fa * a.d[k];
  return r;
}
template <int N> SQA_HD Dual<N> tpow(double a, const Dual<N>& b) {
  Dual<N> r; r.v = pow(a, b.v);
  const double fb = a > 0 ? r.v * log(a) : 0.0;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = fb * b.d[k];
  return r;
}

// Sign (lib/base/Math.hpp:186): piecewise constant, no tangent
template <class T> SQA_HD double tsgn(const T& f) { const double x = val(f); return x < 0 ? -1.0 : (x > 0 ? 1.0 : 0.0); }

}  // namespace sqadj
