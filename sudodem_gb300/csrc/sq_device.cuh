// Device arithmetic for the superellipsoid hot path (FP64 form).
//
// Every expression keeps the reference's operand order: Eigen 3.3.5 with vectorisation
// off reduces length-3 sums as a0 + (a1 + a2) (lib/Eigen/src/Core/Redux.h:91-105) and
// evaluates small matrix-vector products coefficient-wise (Core/ProductEvaluators.h:550).
// The translation unit that includes this header is compiled with --fmad=false so that
// a*b+c is not contracted, as in the reference's x86-64 -O2 build.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace sqdem {

struct D3 { double x, y, z; };
__host__ __device__ __forceinline__ D3 d3(double a, double b, double c) { D3 r; r.x = a; r.y = b; r.z = c; return r; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ D3 operator-(D3 a) { return d3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ D3 operator*(double s, D3 a) { return d3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ D3 operator*(D3 a, double s) { return d3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ double dot(D3 a, D3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
__device__ __forceinline__ double sqn(D3 a) { return a.x * a.x + (a.y * a.y + a.z * a.z); }
__device__ __forceinline__ double nrm(D3 a) { return sqrt(sqn(a)); }
__device__ __forceinline__ D3 cross(D3 a, D3 b) {
  return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ void normalize(D3& a) {
  double z = sqn(a);
  if (z > 0) { double n = sqrt(z); a.x /= n; a.y /= n; a.z /= n; }
}
__device__ __forceinline__ double sgn(double f) { return f < 0 ? -1.0 : (f > 0 ? 1.0 : 0.0); }
// std::max / std::min semantics (first argument wins unless the comparison is true),
// which the reference relies on when a value is NaN (Dispatching.cpp:38-44).
__device__ __forceinline__ double fmax_ref(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double fmin_ref(double a, double b) { return (b < a) ? b : a; }

// Rotation matrix of a unit quaternion (Eigen Quaternion::toRotationMatrix,
// Geometry/Quaternion.h:536-568).  The reference caches R (rot_mat2global) and
// R^T = conj(q).toRotationMatrix() (rot_mat2local) on the shape; both are bit-identical
// to what is built here from the same quaternion, so only R is kept.
struct Rot { double m[9]; };
__host__ __device__ __forceinline__ Rot quatToRot(double w, double x, double y, double z) {
  const double tx = 2.0 * x, ty = 2.0 * y, tz = 2.0 * z;
  const double twx = tx * w, twy = ty * w, twz = tz * w;
  const double txx = tx * x, txy = ty * x, txz = tz * x;
  const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
  Rot r;
  r.m[0] = 1.0 - (tyy + tzz); r.m[1] = txy - twz;         r.m[2] = txz + twy;
  r.m[3] = txy + twz;         r.m[4] = 1.0 - (txx + tzz); r.m[5] = tyz - twx;
  r.m[6] = txz - twy;         r.m[7] = tyz + twx;         r.m[8] = 1.0 - (txx + tyy);
  return r;
}
// R * v
__device__ __forceinline__ D3 mulG(const Rot& R, D3 v) {
  return d3(R.m[0] * v.x + (R.m[1] * v.y + R.m[2] * v.z),
            R.m[3] * v.x + (R.m[4] * v.y + R.m[5] * v.z),
            R.m[6] * v.x + (R.m[7] * v.y + R.m[8] * v.z));
}
// R^T * v == rot_mat2local * v (same coefficients, same order)
__device__ __forceinline__ D3 mulL(const Rot& R, D3 v) {
  return d3(R.m[0] * v.x + (R.m[3] * v.y + R.m[6] * v.z),
            R.m[1] * v.x + (R.m[4] * v.y + R.m[7] * v.z),
            R.m[2] * v.x + (R.m[5] * v.y + R.m[8] * v.z));
}

// Superellipsoid of one body with the exponents it needs per evaluation.
struct SqShape {
  double rx, ry, rz, e1, e2, rmax;
  double a1, a2;       // 2 - eps1, 2 - eps2
  double i1, i2;       // 1/(2 - eps1), 1/(2 - eps2)
  Rot R;
  D3 pos;
};
__host__ __device__ __forceinline__ void shapeInit(SqShape& s, double rx, double ry, double rz, double e1, double e2,
                                          double rmax) {
  s.rx = rx; s.ry = ry; s.rz = rz; s.e1 = e1; s.e2 = e2; s.rmax = rmax;
  s.a1 = 2. - e1; s.a2 = 2. - e2;
  s.i1 = 1 / (2. - e1); s.i2 = 1 / (2. - e2);
}

// Superquadrics::Normal2Phi (pkg/dem/Superquadrics.cpp:269-307) followed by
// Superquadrics::getSurface (:110-120): the point of the surface, in the local frame, whose
// outward normal is n.  One sincos of phi0 serves both, as one cos value does in the
// reference.  The evaluation order of every product is the reference's.
__device__ __forceinline__ D3 supportLocal(const SqShape& s, D3 n) {
  const double Y = pow(fabs(s.ry * n.y), s.i1), X = pow(fabs(s.rx * n.x), s.i1), W = pow(fabs(s.rx * n.x), s.i2);
  const double ph0 = atan2(sgn(n.y) * Y, sgn(n.x) * X);
  double s0, c0;
  sincos(ph0, &s0, &c0);
  const double t = pow(fabs(c0), s.a1), u = pow(fabs(c0), s.e1), v = pow(fabs(s0), s.e1);
  const double Z = pow(fabs(s.rz * n.z * t), s.i2);
  const double ph1 = atan2(sgn(n.z) * Z, W);
  double s1, c1;
  sincos(ph1, &s1, &c1);
  const double pc1 = pow(fabs(c1), s.e2), w = pow(fabs(s1), s.e2);
  D3 r;
  r.x = sgn(c0) * s.rx * u * pc1;
  r.y = sgn(s0) * s.ry * v * pc1;
  r.z = sgn(s1) * s.rz * w;
  return r;
}
// Superquadrics::isInside (Superquadrics.cpp:103-108); p is relative to the centre.
__device__ __forceinline__ bool isInside(const SqShape& s, D3 p) {
  p = mulL(s.R, p);
  return 1 > pow(pow(fabs(p.x / s.rx), 2.0 / s.e1) + pow(fabs(p.y / s.ry), 2.0 / s.e1), s.e1 / s.e2) +
                 pow(fabs(p.z / s.rz), 2.0 / s.e2);
}

// Disfunction, 9-argument form (pkg/dem/Superquadrics_Ig2.cpp:622-687).
__device__ __forceinline__ void disfunction(const SqShape& A, const SqShape& B, double pa0, double pa1, D3& center,
                                            D3& p1, D3& p2, bool& stop_flag) {
  double sa0, ca0, sa1, ca1;
  sincos(pa0, &sa0, &ca0);
  sincos(pa1, &sa1, &ca1);
  D3 contact = d3(ca0 * ca1, sa0 * ca1, sa1);
  p1 = mulG(A.R, supportLocal(A, mulL(A.R, contact))) + A.pos;
  p2 = mulG(B.R, supportLocal(B, (-1.0) * mulL(B.R, contact))) + B.pos;
  D3 d = p2 - p1;
  center = 0.5 * (p1 + p2);
  if (dot(contact, d) > 0) stop_flag = true;
}

__device__ __forceinline__ void centerLine(D3 pos1, D3 pos2, double para[2]) {
  D3 d0 = pos2 - pos1;
  para[0] = atan2(d0.y, d0.x);
  para[1] = atan(d0.z / sqrt(d0.x * d0.x + d0.y * d0.y));
  para[0] += 1e-5; para[1] += 1e-5;
}

}  // namespace sqdem

namespace sqdem {
// ---------------------------------------------------------------------------
// FP32 form of the shape evaluation, in the frame of body A (A at the origin).
struct SqShapeF {
  float rx, ry, rz, e1, e2, a1, i1, i2;
  float R[9];
  float px, py, pz;
};
struct F3 { float x, y, z; };
__device__ __forceinline__ F3 f3(float a, float b, float c) { F3 r; r.x = a; r.y = b; r.z = c; return r; }
__device__ __forceinline__ float dotf(F3 a, F3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
__device__ __forceinline__ float nrmf(F3 a) { return sqrtf(dotf(a, a)); }
__device__ __forceinline__ float sgnf(float f) { return f < 0 ? -1.f : (f > 0 ? 1.f : 0.f); }

__device__ __forceinline__ void shapeInitF(SqShapeF& s, double rx, double ry, double rz, double e1, double e2,
                                           const Rot& R, D3 relPos) {
  s.rx = (float)rx; s.ry = (float)ry; s.rz = (float)rz; s.e1 = (float)e1; s.e2 = (float)e2;
  s.a1 = (float)(2. - e1); s.i1 = (float)(1 / (2. - e1)); s.i2 = (float)(1 / (2. - e2));
  for (int k = 0; k < 9; k++) s.R[k] = (float)R.m[k];
  s.px = (float)relPos.x; s.py = (float)relPos.y; s.pz = (float)relPos.z;
}
// point of the surface of s whose outward normal is parallel to the global direction n
__device__ __forceinline__ F3 supportF(const SqShapeF& s, F3 n) {
  const F3 l = f3(s.R[0] * n.x + (s.R[3] * n.y + s.R[6] * n.z), s.R[1] * n.x + (s.R[4] * n.y + s.R[7] * n.z),
                  s.R[2] * n.x + (s.R[5] * n.y + s.R[8] * n.z));
  const float ph0 = atan2f(sgnf(l.y) * powf(fabsf(s.ry * l.y), s.i1), sgnf(l.x) * powf(fabsf(s.rx * l.x), s.i1));
  float s0, c0;
  sincosf(ph0, &s0, &c0);
  const float ph1 = atan2f(sgnf(l.z) * powf(fabsf(s.rz * l.z * powf(fabsf(c0), s.a1)), s.i2),
                           powf(fabsf(s.rx * l.x), s.i2));
  float s1, c1;
  sincosf(ph1, &s1, &c1);
  const float pc1 = powf(fabsf(c1), s.e2);
  const F3 q = f3(sgnf(c0) * s.rx * powf(fabsf(c0), s.e1) * pc1, sgnf(s0) * s.ry * powf(fabsf(s0), s.e1) * pc1,
                  sgnf(s1) * s.rz * powf(fabsf(s1), s.e2));
  return f3(s.R[0] * q.x + (s.R[1] * q.y + s.R[2] * q.z) + s.px, s.R[3] * q.x + (s.R[4] * q.y + s.R[5] * q.z) + s.py,
            s.R[6] * q.x + (s.R[7] * q.y + s.R[8] * q.z) + s.pz);
}
// Disfunction in FP32: support points of A along c and of B along -c; sepOut = c.(p2 - p1)
__device__ __forceinline__ void disfunctionF(const SqShapeF& A, const SqShapeF& B, float pa0, float pa1, F3& p1,
                                             F3& p2, float& sep) {
  float sa0, ca0, sa1, ca1;
  sincosf(pa0, &sa0, &ca0);
  sincosf(pa1, &sa1, &ca1);
  const F3 c = f3(ca0 * ca1, sa0 * ca1, sa1);
  p1 = supportF(A, c);
  p2 = supportF(B, f3(-c.x, -c.y, -c.z));
  sep = dotf(c, f3(p2.x - p1.x, p2.y - p1.y, p2.z - p1.z));
}
}  // namespace sqdem
