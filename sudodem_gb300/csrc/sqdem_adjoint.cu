// Adjoint of the superellipsoid timestep over a window with a frozen pair set.
//
// A window is `nsteps` timesteps of the linear contact model (Ig2_Wall_Superquadrics_
// SuperquadricsGeom + Ig2_Superquadrics_Superquadrics_SuperquadricsGeom, Ip2_Superquadrics
// Mat_SuperquadricsMat_SuperquadricsPhys, SuperquadricsLaw, NewtonIntegrator with local
// damping) in which the potential-pair set stays the one the window starts with: the collider
// does not run and the law's bound-separation erase (Superquadrics.cpp:1203-1207) is not
// applied.  Contacts still open and close within the window through the narrowphase and the
// depth gate.  Ip2 is applied afresh to every pair at the start of the window, so the contact
// stiffness and friction are functions of the current material parameters.
//
// Forward: a group of six lanes per pair runs the narrowphase (Levenberg-Marquardt restated one
// evaluation after another, lmder2 Superquadrics_Ig2.cpp:1057-1354, with its restart rules
// :2013-2053; each evaluation shared by the group), precompute (Superquadrics.cpp:1030-1050)
// and the law (:1209-1361); one thread per body gathers forces in a fixed order and integrates
// (NewtonIntegrator.cpp:99-304, 391-429).  The state is checkpointed every `checkpoint_every`
// steps.
//
// Reverse: per segment between checkpoints (last first), the segment is recomputed from its
// checkpoint with every step's state kept on a device tape, then the steps are reversed one by
// one: (1) per body, the adjoint of the integrator (translation by hand, rotation by replaying
// the leapfrog in dual numbers); (2) per pair, on a group of lanes that share its tangent
// components, the geometry and the law replayed in dual numbers from the taped state (the same
// double operations, hence the same branches: LM decisions, contact gates, Coulomb cap, damping
// signs, taken as they were), contracted with the incoming adjoints; (3) per body, a
// fixed-order gather of the pairs' contributions.  Parameter adjoints accumulate per pair and
// are mapped to bodies and materials at the end.
//
// Parameters: per-body exponents eps1, eps2 (the narrowphase shape; mass, inertia and r_max
// keep the values the bodies were built with), per-material Kn, Ks and friction coefficient
// mu = tan(frictionAngle).  Loss: sum over bodies of wF . (force of the last step) plus wX .
// (final position).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "sq_dual.cuh"
#include "../../include/sqdem.h"

namespace sqadj {

static const int NT = 17;   // tangent components per replay pass
typedef Dual<NT> DT;

// ---------------------------------------------------------------------------
// Small vector algebra on a scalar type T (double or DT), Eigen 3.3.5 operand order.
template <class T> struct V3 { T x, y, z; };
template <class T> SQA_HD V3<T> mk(const T& a, const T& b, const T& c) { V3<T> r; r.x = a; r.y = b; r.z = c; return r; }
template <class T> SQA_HD V3<T> zero3() { return mk<T>(T(0.0), T(0.0), T(0.0)); }
template <class T> SQA_HD V3<T> operator+(const V3<T>& a, const V3<T>& b) { return mk<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> SQA_HD V3<T> operator-(const V3<T>& a, const V3<T>& b) { return mk<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> SQA_HD V3<T> operator-(const V3<T>& a) { return mk<T>(-a.x, -a.y, -a.z); }
template <class S, class T> SQA_HD V3<T> operator*(const S& s, const V3<T>& a) { return mk<T>(s * a.x, s * a.y, s * a.z); }
template <class S, class T> SQA_HD V3<T> operator*(const V3<T>& a, const S& s) { return mk<T>(a.x * s, a.y * s, a.z * s); }
template <class T> SQA_HD T dot(const V3<T>& a, const V3<T>& b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
template <class T> SQA_HD T sqn(const V3<T>& a) { return a.x * a.x + (a.y * a.y + a.z * a.z); }
template <class T> SQA_HD T nrm(const V3<T>& a) { return tsqrt(sqn(a)); }
template <class T> SQA_HD V3<T> cross(const V3<T>& a, const V3<T>& b) {
  return mk<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class T> SQA_HD void normalize(V3<T>& a) {
  T z = sqn(a);
  if (val(z) > 0) { T n = tsqrt(z); a.x /= n; a.y /= n; a.z /= n; }
}
template <class T> SQA_HD V3<double> vval(const V3<T>& a) { return mk<double>(val(a.x), val(a.y), val(a.z)); }
template <class T> SQA_HD V3<T> lift(const V3<double>& a) { return mk<T>(T(a.x), T(a.y), T(a.z)); }
SQA_HD V3<double> xyz(double4 v) { return mk<double>(v.x, v.y, v.z); }
SQA_HD double4 d4(const V3<double>& a, double w) { return make_double4(a.x, a.y, a.z, w); }

// Eigen Quaternion::toRotationMatrix (Geometry/Quaternion.h:536-568)
template <class T> struct Rot { T m[9]; };
template <class T> SQA_HD Rot<T> quatToRot(const T& w, const T& x, const T& y, const T& z) {
  const T tx = 2.0 * x, ty = 2.0 * y, tz = 2.0 * z;
  const T twx = tx * w, twy = ty * w, twz = tz * w;
  const T txx = tx * x, txy = ty * x, txz = tz * x;
  const T tyy = ty * y, tyz = tz * y, tzz = tz * z;
  Rot<T> r;
  r.m[0] = 1.0 - (tyy + tzz); r.m[1] = txy - twz;         r.m[2] = txz + twy;
  r.m[3] = txy + twz;         r.m[4] = 1.0 - (txx + tzz); r.m[5] = tyz - twx;
  r.m[6] = txz - twy;         r.m[7] = tyz + twx;         r.m[8] = 1.0 - (txx + tyy);
  return r;
}
template <class T> SQA_HD V3<T> mulG(const Rot<T>& R, const V3<T>& v) {
  return mk<T>(R.m[0] * v.x + (R.m[1] * v.y + R.m[2] * v.z), R.m[3] * v.x + (R.m[4] * v.y + R.m[5] * v.z),
               R.m[6] * v.x + (R.m[7] * v.y + R.m[8] * v.z));
}
template <class T> SQA_HD V3<T> mulL(const Rot<T>& R, const V3<T>& v) {
  return mk<T>(R.m[0] * v.x + (R.m[3] * v.y + R.m[6] * v.z), R.m[1] * v.x + (R.m[4] * v.y + R.m[7] * v.z),
               R.m[2] * v.x + (R.m[5] * v.y + R.m[8] * v.z));
}

// ---------------------------------------------------------------------------
// Superellipsoid (Superquadrics.hpp:48-166) with the exponents as scalars of type T.
template <class T> struct Shape {
  double rx, ry, rz, rmax;
  T e1, e2, a1, a2, i1, i2;
  Rot<T> R;
  V3<T> pos;
};
template <class T>
SQA_HD void shapeInit(Shape<T>& s, double4 shp, const T& e1, const T& e2, const T q[4], const V3<T>& pos) {
  s.rx = shp.x; s.ry = shp.y; s.rz = shp.z; s.rmax = shp.w;
  s.e1 = e1; s.e2 = e2;
  s.a1 = 2. - e1; s.a2 = 2. - e2;
  s.i1 = 1.0 / (2. - e1); s.i2 = 1.0 / (2. - e2);
  s.R = quatToRot(q[0], q[1], q[2], q[3]);
  s.pos = pos;
}
// Normal2Phi (Superquadrics.cpp:269-307) then getSurface (:110-120), local frame
template <class T> SQA_HD V3<T> supportLocal(const Shape<T>& s, const V3<T>& n) {
  const T Y = tpow(tfabs(s.ry * n.y), s.i1), X = tpow(tfabs(s.rx * n.x), s.i1), W = tpow(tfabs(s.rx * n.x), s.i2);
  const T ph0 = tatan2(tsgn(n.y) * Y, tsgn(n.x) * X);
  T s0, c0;
  tsincos(ph0, &s0, &c0);
  const T t = tpow(tfabs(c0), s.a1), u = tpow(tfabs(c0), s.e1), v = tpow(tfabs(s0), s.e1);
  const T Z = tpow(tfabs(s.rz * n.z * t), s.i2);
  const T ph1 = tatan2(tsgn(n.z) * Z, W);
  T s1, c1;
  tsincos(ph1, &s1, &c1);
  const T pc1 = tpow(tfabs(c1), s.e2), w = tpow(tfabs(s1), s.e2);
  V3<T> r;
  r.x = tsgn(c0) * s.rx * u * pc1;
  r.y = tsgn(s0) * s.ry * v * pc1;
  r.z = tsgn(s1) * s.rz * w;
  return r;
}
// isInside (Superquadrics.cpp:103-108): a decision only, on the values
template <class T> SQA_HD bool isInside(const Shape<T>& s, const V3<double>& p0) {
  Rot<double> R;
  for (int k = 0; k < 9; k++) R.m[k] = val(s.R.m[k]);
  const V3<double> p = mulL(R, p0);
  const double e1 = val(s.e1), e2 = val(s.e2);
  return 1 > pow(pow(fabs(p.x / s.rx), 2.0 / e1) + pow(fabs(p.y / s.ry), 2.0 / e1), e1 / e2) +
                 pow(fabs(p.z / s.rz), 2.0 / e2);
}
// Disfunction (Superquadrics_Ig2.cpp:622-687)
template <class T>
__host__ __device__ __noinline__ void disfunction(const Shape<T>& A, const Shape<T>& B, const T& pa0, const T& pa1, V3<T>& center, V3<T>& p1,
                        V3<T>& p2, bool& stop_flag) {
  T sa0, ca0, sa1, ca1;
  tsincos(pa0, &sa0, &ca0);
  tsincos(pa1, &sa1, &ca1);
  const V3<T> contact = mk<T>(ca0 * ca1, sa0 * ca1, sa1);
  p1 = mulG(A.R, supportLocal(A, mulL(A.R, contact))) + A.pos;
  p2 = mulG(B.R, supportLocal(B, (-1.0) * mulL(B.R, contact))) + B.pos;
  const V3<T> d = p2 - p1;
  center = 0.5 * (p1 + p2);
  if (val(dot(contact, d)) > 0) stop_flag = true;
}
// The Disfunction evaluation lmder2 calls: in sequence on one thread (every instantiation),
// or by a group of six lanes of a warp (CoopEval, forward kernel only).
struct SeqEval {
  template <class T>
  SQA_HD void operator()(const Shape<T>& A, const Shape<T>& B, const T& pa0, const T& pa1, V3<T>& center, V3<T>& p1,
                         V3<T>& p2, bool& stop_flag) const {
    disfunction(A, B, pa0, pa1, center, p1, p2, stop_flag);
  }
};

// Disfunction by six lanes: lanes g0..g0+2 compute body A's support point, g0+3..g0+5 body
// B's, each triple running the independent pow calls of one level of Normal2Phi + getSurface
// on separate lanes (Y X W | t u v | Z | pc1 w), so that the dependency chain of one evaluation
// is 4 pow + 2 atan2 + 4 sincos instead of 18 pow + 4 atan2 + 6 sincos.  Every value is the
// result of the same operation on the same operands as in disfunction: bitwise the same.
struct CoopEval {
  unsigned mask;   // the group's six lanes
  int g0, sub;     // first lane of the group, this lane's place in it
#ifdef __CUDA_ARCH__
  __device__ double pick(double v, int src) const { return __shfl_sync(mask, v, src); }
  __device__ V3<double> support(const Shape<double>& s, const V3<double>& n, int part, int l0) const {
    double b, e;
    if (part == 0) { b = fabs(s.ry * n.y); e = s.i1; }
    else if (part == 1) { b = fabs(s.rx * n.x); e = s.i1; }
    else { b = fabs(s.rx * n.x); e = s.i2; }
    const double r1 = pow(b, e);
    const double Y = pick(r1, l0), X = pick(r1, l0 + 1), W = pick(r1, l0 + 2);
    const double ph0 = atan2(tsgn(n.y) * Y, tsgn(n.x) * X);
    double s0, c0;
    sincos(ph0, &s0, &c0);
    if (part == 0) { b = fabs(c0); e = s.a1; }
    else if (part == 1) { b = fabs(c0); e = s.e1; }
    else { b = fabs(s0); e = s.e1; }
    const double r2 = pow(b, e);
    const double t = pick(r2, l0), u = pick(r2, l0 + 1), v = pick(r2, l0 + 2);
    const double Z = pow(fabs(s.rz * n.z * t), s.i2);
    const double ph1 = atan2(tsgn(n.z) * Z, W);
    double s1, c1;
    sincos(ph1, &s1, &c1);
    if (part == 1) { b = fabs(s1); e = s.e2; } else { b = fabs(c1); e = s.e2; }
    const double r3 = pow(b, e);
    const double pc1 = pick(r3, l0), w = pick(r3, l0 + 1);
    V3<double> r;
    r.x = tsgn(c0) * s.rx * u * pc1;
    r.y = tsgn(s0) * s.ry * v * pc1;
    r.z = tsgn(s1) * s.rz * w;
    return r;
  }
#endif
  SQA_HD void operator()(const Shape<double>& A, const Shape<double>& B, const double& pa0, const double& pa1,
                         V3<double>& center, V3<double>& p1, V3<double>& p2, bool& stop_flag) const {
#ifdef __CUDA_ARCH__
    double sa0, ca0, sa1, ca1;
    sincos(pa0, &sa0, &ca0);
    sincos(pa1, &sa1, &ca1);
    const V3<double> contact = mk<double>(ca0 * ca1, sa0 * ca1, sa1);
    const int body = sub / 3, part = sub - 3 * body;
    const Shape<double>& Sh = body ? B : A;
    const V3<double> n = body ? (-1.0) * mulL(B.R, contact) : mulL(A.R, contact);
    const V3<double> pt = mulG(Sh.R, support(Sh, n, part, g0 + 3 * body)) + Sh.pos;
    p1 = mk<double>(pick(pt.x, g0), pick(pt.y, g0), pick(pt.z, g0));
    p2 = mk<double>(pick(pt.x, g0 + 3), pick(pt.y, g0 + 3), pick(pt.z, g0 + 3));
    const V3<double> d = p2 - p1;
    center = 0.5 * (p1 + p2);
    if (dot(contact, d) > 0) stop_flag = true;
#else
    disfunction(A, B, pa0, pa1, center, p1, p2, stop_flag);
#endif
  }
};

template <class T> SQA_HD void centerLine(const V3<T>& pos1, const V3<T>& pos2, T para[2]) {
  const V3<T> d0 = pos2 - pos1;
  para[0] = tatan2(d0.y, d0.x);
  para[1] = tatan(d0.z / tsqrt(d0.x * d0.x + d0.y * d0.y));
  para[0] += 1e-5; para[1] += 1e-5;
}

template <class T> struct LMOut { V3<T> p1, p2, center, contact; bool touching; int iters, stop, evals; };

// Branch tape.  The step map jumps or kinks where a decision changes: the Levenberg-Marquardt
// path (its stopping tests, step acceptances and damping updates), the narrowphase's restarts,
// the bounding-sphere and contact gates, the shear reset, the Coulomb cap and the sign of the
// local damping.  A forward run can record the outcome of every such decision (a bit per
// decision, per pair and step, in the order the pair's step takes them), and a later run can
// take the recorded outcomes instead of evaluating them: a run with perturbed parameters then
// follows the recorded branches, and its central differences are differences of one smooth
// branch, the one whose derivative the reverse pass computes.  Each forced decision whose
// natural outcome differs is counted.  The replay of the reverse pass evaluates its decisions
// (NoBranch).
//
// The superquadric surface itself is not smooth everywhere: its support point, a signed power
// sgn(x)|x|^(1/(2-e)) of the local direction's components, has an infinite derivative where a
// component crosses 0 (e < 1) and no continuation through it.  Those points are not forced;
// the tape keeps a hash of the signs of the local direction's components at every surface
// evaluation of the step (in the order evaluated), and a forced run counts the pair steps whose
// hash differs: a central difference across such a point is not a derivative.
enum { BR_OFF = 0, BR_RECORD = 1, BR_FORCE = 2 };
// per pair and step: the number of decisions, the surface-sign hash, then 7 words of outcomes
static const int BR_WORDS = 9;
static const int BR_BITS = 32 * (BR_WORDS - 2);
SQA_HD unsigned sgn3(double x, double y, double z) {
  return (x > 0 ? 1u : (x < 0 ? 2u : 0u)) | (y > 0 ? 4u : (y < 0 ? 8u : 0u)) | (z > 0 ? 16u : (z < 0 ? 32u : 0u));
}
struct NoBranch {
  SQA_HD bool operator()(bool v) { return v; }
  template <class T> SQA_HD void surf(const Shape<T>&, const Shape<T>&, const T&, const T&) {}
  template <class T> SQA_HD void surf1(const Shape<T>&, const V3<T>&) {}
};
struct BrCur {
  unsigned* w;   // this pair's words of this step
  int mode, n, dis;
  unsigned acc, cusp;
  bool writer;
  // signs of the surface evaluation's local directions: the contact direction of the angles
  // (pa0, pa1) in A's and B's frames
  template <class T> SQA_HD void surf(const Shape<T>& A, const Shape<T>& B, const T& pa0, const T& pa1) {
    if (mode == BR_OFF) return;
    double s0, c0, s1, c1;
    tsincos(val(pa0), &s0, &c0);
    tsincos(val(pa1), &s1, &c1);
    const V3<double> d = mk<double>(c0 * c1, s0 * c1, s1);
    Rot<double> R;
    for (int k = 0; k < 9; k++) R.m[k] = val(A.R.m[k]);
    const V3<double> la = mulL(R, d);
    for (int k = 0; k < 9; k++) R.m[k] = val(B.R.m[k]);
    const V3<double> lb = mulL(R, d);
    cusp = cusp * 0x9E3779B1u + (sgn3(la.x, la.y, la.z) | sgn3(lb.x, lb.y, lb.z) << 6) + 1u;
  }
  template <class T> SQA_HD void surf1(const Shape<T>& B, const V3<T>& dir) {
    if (mode == BR_OFF) return;
    Rot<double> R;
    for (int k = 0; k < 9; k++) R.m[k] = val(B.R.m[k]);
    const V3<double> lb = mulL(R, vval(dir));
    cusp = cusp * 0x9E3779B1u + sgn3(lb.x, lb.y, lb.z) + 1u;
  }
  SQA_HD bool operator()(bool v) {
    if (mode == BR_OFF) return v;
    const int k = n++;
    if (k >= BR_BITS) return v;   // beyond the tape: evaluated (counted as unforced)
    const int word = 2 + (k >> 5), bit = k & 31;
    if (mode == BR_RECORD) {
      acc |= (unsigned)v << bit;
      if (bit == 31) {
        if (writer) w[word] = acc;
        acc = 0u;
      }
      return v;
    }
    if (bit == 0) acc = w[word];
    const bool r = (acc >> bit) & 1u;
    dis += r != v;
    return r;
  }
};

// lmder2 with opts {1, 1e-15, 1e-3, 1e-20}, itmax 50 (Superquadrics_Ig2.cpp:1057-1354).  The
// Jacobian's re-evaluation at the current point (JacfunctionApp, :1033-1054) is not repeated:
// its values equal the ones stored for that point and are overwritten by the two probes.
template <class T, class E, class BR>
__host__ __device__ __noinline__ void lmder2(const Shape<T>& A, const Shape<T>& B, T p[2], LMOut<T>& o, const E& ev, BR& br) {
  const double ONE_THIRD = 0.3333333333333334;
  o.touching = true; o.evals = 1;
  bool stop_flag = false;
  T Dp0 = T(1e-7), Dp1 = T(1e-7), mu = T(0.0);
  T jt0 = T(0.0), jt1 = T(0.0), j00 = T(0.0), j01 = T(0.0), j11 = T(0.0), diag0 = T(0.0), diag1 = T(0.0), pL2 = T(0.0);
  int nu = 2, stop = 0, k;
  V3<T> P1, P2, C;
  o.contact = zero3<T>();
  ev(A, B, p[0], p[1], C, P1, P2, stop_flag);
  br.surf(A, B, p[0], p[1]);
  V3<T> pf = P2 - P1;
  T pfL2 = nrm(pf);
  if (br(!isfinite(val(pfL2)))) stop = 7;
  for (k = 0; k < 50 && !stop; ++k) {
    if (br(val(pfL2) <= 1e-20)) { stop = 6; break; }
    if (br(stop_flag)) { stop = 9; o.touching = false; break; }
    T s0, c0, s1, c1;
    tsincos(p[0], &s0, &c0);
    tsincos(p[1], &s1, &c1);
    o.contact = mk<T>(c0 * c1, s0 * c1, s1);
    const double angle = val(dot(pf, o.contact)) / (val(nrm(pf)) * val(nrm(o.contact)));
    if (br(fabs(angle) > 0.95)) { stop = 8; break; }
    ev(A, B, p[0] + Dp0, p[1], C, P1, P2, stop_flag);
    br.surf(A, B, p[0] + Dp0, p[1]);
    const V3<T> f1 = P2 - P1;
    ev(A, B, p[0], p[1] + Dp1, C, P1, P2, stop_flag);
    br.surf(A, B, p[0], p[1] + Dp1);
    const V3<T> f2 = P2 - P1;
    o.evals += 2;
    const T J00 = (f1.x - pf.x) / Dp0, J10 = (f1.y - pf.y) / Dp0, J20 = (f1.z - pf.z) / Dp0;
    const T J01 = (f2.x - pf.x) / Dp1, J11 = (f2.y - pf.y) / Dp1, J21 = (f2.z - pf.z) / Dp1;
    j00 = J00 * J00 + (J10 * J10 + J20 * J20);
    j01 = J00 * J01 + (J10 * J11 + J20 * J21);
    j11 = J01 * J01 + (J11 * J11 + J21 * J21);
    jt0 = J00 * (-1.0 * pf.x) + (J10 * (-1.0 * pf.y) + J20 * (-1.0 * pf.z));
    jt1 = J01 * (-1.0 * pf.x) + (J11 * (-1.0 * pf.y) + J21 * (-1.0 * pf.z));
    const double jinf = (fabs(val(jt0)) > fabs(val(jt1)) ? fabs(val(jt0)) : fabs(val(jt1)));
    pL2 = tsqrt(p[0] * p[0] + p[1] * p[1]);
    if (br(jinf <= 1e-15)) { stop = 1; break; }
    if (k == 0) mu = 1.0 * (br(val(j00) > val(j11)) ? j00 : j11);
    diag0 = j00; diag1 = j11;
    for (;;) {
      j00 += mu;
      j11 += mu;
      const T n_a = j00 * j11 - j01 * j01;
      Dp0 = (jt0 * j11 - jt1 * j01) / n_a;
      Dp1 = (jt1 * j00 - jt0 * j01) / n_a;
      const double DpL2 = sqrt(val(Dp0) * val(Dp0) + val(Dp1) * val(Dp1));
      if (br(DpL2 < 1e-5)) { stop = 2; break; }
      const T q0 = p[0] + Dp0, q1 = p[1] + Dp1;
      if (br(DpL2 >= (val(pL2) + 1e-3) / (1e-12 * 1e-12))) { stop = 4; break; }
      ev(A, B, q0, q1, C, P1, P2, stop_flag);
      br.surf(A, B, q0, q1);
      o.evals++;
      const V3<T> pDp_f = P2 - P1;
      const T pDp_fL2 = nrm(pDp_f);
      if (br(!isfinite(val(pDp_fL2)))) { stop = 7; break; }
      const T dL = Dp0 * (mu * Dp0 + jt0) + Dp1 * (mu * Dp1 + jt1);
      const T dF = pfL2 - pDp_fL2;
      T tmp = dF / dL;
      if (br(val(tmp) > 0.0)) {
        tmp = 1.0 - tpow(2 * tmp - 1., 3.);
        mu = mu * (br(val(tmp) >= ONE_THIRD) ? tmp : T(ONE_THIRD));
        nu = 2;
        p[0] = q0; p[1] = q1;
        pf = pDp_f; pfL2 = pDp_fL2;
        break;
      }
      mu *= (double)nu;
      const int nu2 = (int)((unsigned)nu << 1);
      if (nu2 <= nu) { stop = 5; break; }
      nu = nu2;
      j00 = diag0; j11 = diag1;
    }
  }
  if (k >= 50) stop = 3;
  o.iters = k; o.stop = stop;
  o.p1 = P1; o.p2 = P2; o.center = C;
}

// Geometry of one pair.  angMode: 0 contactAngle unchanged, 1 set to ang, 2 set to (0,0).
template <class T> struct Geom {
  bool precomputed, isShearNew;
  int angMode, evals, calls;
  T depth, ang[2];
  V3<T> normal, cp;
};

// Ig2_Superquadrics_Superquadrics_SuperquadricsGeom::go (Superquadrics_Ig2.cpp:1880-2317),
// non-sphere bodies, no periodic shift.
template <class T, class E, class BR>
__host__ __device__ __noinline__ void geomSqSq(Geom<T>& g, bool isNew, double prevDepth, const T angIn[2], const Shape<T>& A,
                                               const Shape<T>& B, const E& ev, BR& br) {
  g.precomputed = false; g.evals = 0; g.calls = 0;
  T para[2];
  if (isNew) { g.isShearNew = true; centerLine(A.pos, B.pos, para); }
  else { g.isShearNew = br(prevDepth <= 0); para[0] = angIn[0]; para[1] = angIn[1]; }
  g.angMode = isNew ? 2 : 0;
  g.depth = T(0.0);
  const double r_sum = A.rmax + B.rmax;
  if (br(val(nrm(A.pos - B.pos)) > r_sum)) { g.isShearNew = true; return; }
  LMOut<T> o;
  lmder2(A, B, para, o, ev, br);
  g.evals += o.evals; g.calls++;
  if (br((isnan(val(para[0])) || isnan(val(para[1])) || 7 == o.stop) && o.touching)) {
    centerLine(A.pos, B.pos, para);
    lmder2(A, B, para, o, ev, br);
    g.evals += o.evals; g.calls++;
  }
  T pDepth = dot(o.p1 - o.p2, o.contact);
  if (br(o.touching && 10.0 * val(nrm(o.p2 - o.p1)) > A.rmax)) {
    if (br(!isInside(A, vval(o.p2 - A.pos)) || !isInside(B, vval(o.p1 - B.pos)))) {
      centerLine(A.pos, B.pos, para);
      lmder2(A, B, para, o, ev, br);
      g.evals += o.evals; g.calls++;
      pDepth = dot(o.p1 - o.p2, o.contact);
    }
  }
  g.angMode = 1; g.ang[0] = para[0]; g.ang[1] = para[1];
  if (!o.touching) { g.isShearNew = true; return; }
  g.cp = o.center;
  g.depth = pDepth;
  V3<T> cn = o.contact;
  normalize(cn);
  g.normal = cn;
  g.precomputed = true;
}

// Ig2_Wall_Superquadrics_SuperquadricsGeom::go (Superquadrics_Ig2.cpp:2522-2611), non-sphere
template <class T, class BR>
SQA_HD void geomWallSq(Geom<T>& g, bool isNew, double prevDepth, int PA, double sense, double wallc, const Shape<T>& B,
                       BR& br) {
  g.precomputed = false; g.evals = 1; g.calls = 0; g.angMode = isNew ? 2 : 0;
  g.isShearNew = isNew ? true : br(prevDepth <= 0);
  g.depth = T(0.0);
  V3<double> nd = mk<double>(0.0, 0.0, 0.0);
  if (PA == 0) nd.x = sense; else if (PA == 1) nd.y = sense; else nd.z = sense;
  const V3<T> normal = lift<T>(nd);
  br.surf1(B, normal);
  const V3<T> point2 = mulG(B.R, supportLocal(B, -mulL(B.R, normal))) + B.pos;
  V3<T> p1 = point2;
  if (PA == 0) p1.x = T(wallc); else if (PA == 1) p1.y = T(wallc); else p1.z = T(wallc);
  const V3<T> dd = point2 - p1;
  const double ndot = PA == 0 ? nd.x * val(dd.x) : (PA == 1 ? nd.y * val(dd.y) : nd.z * val(dd.z));
  const bool apart = ndot >= 0.0;
  if (br(apart)) { g.isShearNew = true; return; }
  g.cp = 0.5 * (point2 + p1);
  // |dd|, signed where a forced contact is apart (the depth's smooth continuation)
  g.depth = apart ? -nrm(dd) : nrm(dd);
  g.normal = normal;
  g.precomputed = true;
}

// precompute (Superquadrics.cpp:1030-1050) + SuperquadricsLaw::go (:1209-1361) without
// viscous damping: Fn = kn depth n, rotated and incremented shear spring, Coulomb cap.
// Returns whether the force branch ran (depth > 1e-18); outputs the force on id1 (Fv), the
// torques on id1 and id2 and the new shear force.
template <class T> struct LawIn {
  T depth; V3<T> normal, cp, x1, x2, v1, w1, v2, w2, nPrev, sPrev; T kn, ks, tanphi;
};
template <class T> struct LawOut { V3<T> Fv, T1, T2, s; bool sliding; };
template <class T, class BR> SQA_HD bool law(const LawIn<T>& in, bool isShearNew, double dt, LawOut<T>& out, BR& br) {
  if (!br(val(in.depth) > 1E-18)) return false;
  V3<T> ortho, twist;
  if (!isShearNew) {
    ortho = cross(in.nPrev, in.normal);
    const T angle = dt * 0.5 * dot(in.normal, in.w1 + in.w2);
    twist = angle * in.normal;
  } else { ortho = zero3<T>(); twist = zero3<T>(); }
  const V3<T> c1x = in.cp - in.x1;
  const V3<T> c2x = (in.cp - in.x2) - zero3<T>();
  const V3<T> relVel = (in.v2 + cross(in.w2, c2x)) - (in.v1 + cross(in.w1, c1x));
  const V3<T> relVn = dot(in.normal, relVel) * in.normal;
  const V3<T> relVs = relVel - relVn;
  const V3<T> shearInc = relVs * dt;
  const V3<T> normalForce = in.normal * in.depth * in.kn;
  V3<T> sf;
  if (isShearNew) sf = zero3<T>();
  else {   // SuperquadricsGeom::rotate (:1053-1080)
    sf = in.sPrev;
    sf = sf - cross(sf, ortho);
    sf = sf - cross(sf, twist);
    sf = sf - dot(in.normal, sf) * in.normal;
  }
  sf = sf - in.ks * shearInc;
  const T maxFs = sqn(normalForce) * (in.tanphi * in.tanphi);
  out.sliding = false;
  if (br(val(sqn(sf)) > val(maxFs))) {
    // |Fn| tan(phi), signed where a forced contact has a negative depth (its smooth continuation)
    const T cap = val(in.depth) < 0 ? -tsqrt(maxFs) : tsqrt(maxFs);
    const T ratio = cap / nrm(sf);
    sf = sf * ratio;
    out.sliding = true;
  }
  const V3<T> Fv = ((-normalForce) - sf) + zero3<T>();
  out.Fv = Fv;
  out.T1 = -cross(in.x1 - in.cp, Fv);
  out.T2 = cross(in.x2 - in.cp, Fv);
  out.s = sf;
  return true;
}
template <class T> SQA_HD bool law(const LawIn<T>& in, bool isShearNew, double dt, LawOut<T>& out) {
  NoBranch nb;
  return law(in, isShearNew, dt, out, nb);
}

// NewtonIntegrator rotation of a superquadric: leapfrogAsphericalRotate with
// A = rot_mat2local (NewtonIntegrator.cpp:337-360, 391-429), DotQ (:470-477).  q = (w,x,y,z).
template <class T> SQA_HD void dotQ(const V3<T>& a, const T Q[4], T r[4]) {
  r[0] = ((-Q[1]) * a.x - Q[2] * a.y - Q[3] * a.z) / 2.0;
  r[1] = (Q[0] * a.x - Q[3] * a.y + Q[2] * a.z) / 2.0;
  r[2] = (Q[3] * a.x + Q[0] * a.y - Q[1] * a.z) / 2.0;
  r[3] = ((-Q[2]) * a.x + Q[1] * a.y + Q[0] * a.z) / 2.0;
}
template <class T> SQA_HD V3<T> qrotate(const T q[4], const V3<T>& v) {
  const V3<T> qv = mk<T>(q[1], q[2], q[3]);
  V3<T> uv = cross(qv, v);
  uv = uv + uv;
  const V3<T> c = cross(qv, uv);
  return mk<T>((v.x + q[0] * uv.x) + c.x, (v.y + q[0] * uv.y) + c.y, (v.z + q[0] * uv.z) + c.z);
}
template <class T>
SQA_HD void rotStep(const T q[4], const V3<T>& L, const V3<T>& M, double4 I, double dt, T qo[4], V3<T>& Lo, V3<T>& wo) {
  const Rot<T> R = quatToRot(q[0], q[1], q[2], q[3]);
  const V3<T> l_n = L + (dt / 2.) * M;
  const V3<T> l_b_n = mulL(R, l_n);
  const V3<T> w_b_n = mk<T>(l_b_n.x / I.y, l_b_n.y / I.z, l_b_n.z / I.w);
  T dq[4];
  dotQ(w_b_n, q, dq);
  const double hdt = dt / 2.;
  T Qh[4];
  for (int k = 0; k < 4; k++) Qh[k] = q[k] + dq[k] * hdt;
  Lo = L + dt * M;
  const V3<T> l_b_h = mulL(R, Lo);
  const V3<T> w_b_h = mk<T>(l_b_h.x / I.y, l_b_h.y / I.z, l_b_h.z / I.w);
  T dqh[4];
  dotQ(w_b_h, Qh, dqh);
  for (int k = 0; k < 4; k++) qo[k] = q[k] + dqh[k] * dt;
  wo = qrotate(qo, w_b_h);
  // Quaternion::normalize: squaredNorm over coefficients (x,y,z,w) = (x²+y²)+(z²+w²)
  const T z = (qo[1] * qo[1] + qo[2] * qo[2]) + (qo[3] * qo[3] + qo[0] * qo[0]);
  if (val(z) > 0) { const T n = tsqrt(z); qo[1] /= n; qo[2] /= n; qo[3] /= n; qo[0] /= n; }
}

// ---------------------------------------------------------------------------
// Device data
enum : int { CF_GEOM = 1 };                 // flag: Interaction::geom present
enum : int { CO_PRE = 1, CO_FORCE = 2, CO_ANG = 4, CO_ANG0 = 8, CO_NEW = 16, CO_SHNEW = 32, CO_SLIDE = 64 };
enum { A_MISMATCH = 0, A_EVALS, A_LMCALLS, A_REPLAYED, A_SIG, A_SIGB, A_BRDEC, A_BRDIS, A_BRUNF, A_BRCUSP, A_NCOUNT };

struct Consts {
  int nb, P;
  double dt, g[3], damping;
  const double4* shp;     // rx ry rz rmax
  const double2* eps;     // eps1 eps2 (parameters)
  const double4* massI;   // mass, inertia (3)
  const int4* binfo;      // kind, wall axis, wall sense, -
  const int2* ids;        // id1, id2 (walls are id1)
  const double4* phys;    // kn ks tanphi
  const int* bStart; const int* bList;   // per body: pair index * 2 + side (0: the body is id1)
  unsigned long long* cnt;
  // branch tape of the forward run (BR_OFF in the reverse pass's recomputation): BR_WORDS words
  // per pair and step, one word per body and step (the local damping's sign codes)
  unsigned* brPair;
  unsigned* brBody;
  int brMode;
};
// state of the scene between steps
struct State {
  double4 *pos, *ori, *vel, *angVel, *angMom;
  int* flag; double* depth; double2* angle; double4* normal; double4* shear;
};
// what a step leaves for the gather and the reverse pass
struct StepOut { double4* Fv; double4* cp; int* code; };
struct Adj {
  double4 *lPos, *lOri, *lVel, *lW, *lL, *lF, *lT;   // per body
  double2* lAng; double4 *lN, *lS;                   // per pair
  double4* con;                                       // per pair: 8 double4 (x q v w of id1, then of id2)
  double4 *accEps, *accPhys;                          // per pair parameter adjoints (e1a e2a e1b e2b | kn ks tanphi)
  const double4 *wF, *wX;
  const int* order;   // the reverse step's pair order (longest forward search first), or null
};

SQA_HD void loadQ(double4 o, double q[4]) { q[0] = o.x; q[1] = o.y; q[2] = o.z; q[3] = o.w; }

// counters: device atomics (the host instantiation is single-threaded)
#ifdef __CUDA_ARCH__
#define SQA_CNT(p, v) atomicAdd((p), (unsigned long long)(v))
#else
#define SQA_CNT(p, v) (*(p) += (unsigned long long)(v))
#endif

// ---------------------------------------------------------------------------
// One pair's inputs, read from a state (values).
struct PairVals {
  int2 id; int4 i1; bool isNew; double prevDepth; double ang[2];
  double q1[4], q2[4]; double2 e1, e2; double4 shp1, shp2, ph;
  V3<double> x1, x2, v1, w1, v2, w2, nPrev, sPrev;
};
SQA_HD void loadPair(const Consts& C, const State& S, int c, PairVals& p) {
  p.id = C.ids[c];
  p.i1 = C.binfo[p.id.x];
  p.isNew = !(S.flag[c] & CF_GEOM);
  p.prevDepth = S.depth[c];
  const double2 a = S.angle[c];
  p.ang[0] = a.x; p.ang[1] = a.y;
  loadQ(S.ori[p.id.x], p.q1); loadQ(S.ori[p.id.y], p.q2);
  p.e1 = C.eps[p.id.x]; p.e2 = C.eps[p.id.y];
  p.shp1 = C.shp[p.id.x]; p.shp2 = C.shp[p.id.y];
  p.ph = C.phys[c];
  p.x1 = xyz(S.pos[p.id.x]); p.x2 = xyz(S.pos[p.id.y]);
  p.v1 = xyz(S.vel[p.id.x]); p.w1 = xyz(S.angVel[p.id.x]);
  p.v2 = xyz(S.vel[p.id.y]); p.w2 = xyz(S.angVel[p.id.y]);
  p.nPrev = xyz(S.normal[c]); p.sPrev = xyz(S.shear[c]);
}

// tangent seeding: input k is tangent component k - base of this pass (none for double)
template <class T> struct Seeder;
template <> struct Seeder<double> { static SQA_HD double s(double x, int, int) { return x; } };
template <int N> struct Seeder<Dual<N>> { static SQA_HD Dual<N> s(double x, int k, int base) { return seed<N>(x, k - base); } };

// Geometry of a pair.  Replay slots: 0-2 position of id2, 3-6 orientation of id1, 7-10
// orientation of id2, 11-12 eps of id1, 13-14 eps of id2, 15-16 the stored contact angles.
// The position of id1 carries no tangent: the SQ-SQ outputs other than the contact point are
// invariant under a common translation, which gives their derivatives with respect to it.
template <class T, class E, class BR> SQA_HD void pairGeom(const PairVals& p, Geom<T>& g, int base, const E& ev, BR& br) {
  typedef Seeder<T> Sd;
  const V3<T> X2 = mk<T>(Sd::s(p.x2.x, 0, base), Sd::s(p.x2.y, 1, base), Sd::s(p.x2.z, 2, base));
  T q2[4];
  for (int k = 0; k < 4; k++) q2[k] = Sd::s(p.q2[k], 7 + k, base);
  Shape<T> B;
  shapeInit(B, p.shp2, Sd::s(p.e2.x, 13, base), Sd::s(p.e2.y, 14, base), q2, X2);
  if (p.i1.x == 1) {
    const double wallc = p.i1.y == 0 ? p.x1.x : (p.i1.y == 1 ? p.x1.y : p.x1.z);
    geomWallSq(g, p.isNew, p.prevDepth, p.i1.y, (double)p.i1.z, wallc, B, br);
  } else {
    T q1[4];
    for (int k = 0; k < 4; k++) q1[k] = Sd::s(p.q1[k], 3 + k, base);
    Shape<T> A;
    shapeInit(A, p.shp1, Sd::s(p.e1.x, 11, base), Sd::s(p.e1.y, 12, base), q1, lift<T>(p.x1));
    const T angIn[2] = {Sd::s(p.ang[0], 15, base), Sd::s(p.ang[1], 16, base)};
    geomSqSq(g, p.isNew, p.prevDepth, angIn, A, B, ev, br);
  }
}
template <class T, class E = SeqEval> SQA_HD void pairGeom(const PairVals& p, Geom<T>& g, int base = 0, const E& ev = E()) {
  NoBranch nb;
  pairGeom(p, g, base, ev, nb);
}

// Law inputs, 34 of them, in replay chunk `chunk` (inputs 17*chunk .. 17*chunk+16, from
// tangent component `base` of the pass on):
// 0 depth, 1-3 normal, 4-6 contact point, 7-9 x1, 10-12 x2, 13-15 v1, 16-18 w1, 19-21 v2,
// 22-24 w2, 25-27 previous normal, 28-30 previous shear force, 31 kn, 32 ks, 33 tan(phi).
template <class T> SQA_HD T lawSeed(double x, int i, int c0) { return Seeder<T>::s(x, i, c0); }
template <class T> SQA_HD V3<T> lawSeed3(const V3<double>& v, int i, int c0) {
  return mk<T>(lawSeed<T>(v.x, i, c0), lawSeed<T>(v.y, i + 1, c0), lawSeed<T>(v.z, i + 2, c0));
}
template <class T>
SQA_HD void lawInputs(const PairVals& p, double depth, const V3<double>& normal, const V3<double>& cp, int chunk,
                      LawIn<T>& in, int base = 0) {
  const int c0 = NT * chunk + base;
  in.depth = lawSeed<T>(depth, 0, c0);
  in.normal = lawSeed3<T>(normal, 1, c0);
  in.cp = lawSeed3<T>(cp, 4, c0);
  in.x1 = lawSeed3<T>(p.x1, 7, c0); in.x2 = lawSeed3<T>(p.x2, 10, c0);
  in.v1 = lawSeed3<T>(p.v1, 13, c0); in.w1 = lawSeed3<T>(p.w1, 16, c0);
  in.v2 = lawSeed3<T>(p.v2, 19, c0); in.w2 = lawSeed3<T>(p.w2, 22, c0);
  in.nPrev = lawSeed3<T>(p.nPrev, 25, c0); in.sPrev = lawSeed3<T>(p.sPrev, 28, c0);
  in.kn = lawSeed<T>(p.ph.x, 31, c0); in.ks = lawSeed<T>(p.ph.y, 32, c0); in.tanphi = lawSeed<T>(p.ph.z, 33, c0);
}

SQA_HD unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
SQA_HD unsigned long long branchHash(int item, int step, unsigned long long bits) {
  return mix64(((unsigned long long)(item + 1) * 0x9E3779B97F4A7C15ull) ^ ((unsigned long long)(step + 1) << 40) ^
               (bits * 0xC2B2AE3D27D4EB4Full));
}

// forward step of one pair (double)
template <class E = SeqEval>
SQA_HD void fwdContact(const Consts& C, const State& S, const StepOut& O, int step, int c, const E& ev = E(),
                       bool writer = true) {
  PairVals p;
  loadPair(C, S, c, p);
  Geom<double> g;
  BrCur br;
  br.mode = C.brMode; br.n = 0; br.dis = 0; br.acc = 0u; br.cusp = 0u; br.writer = writer;
  br.w = C.brMode != BR_OFF ? C.brPair + ((size_t)step * C.P + c) * BR_WORDS : nullptr;
  pairGeom<double>(p, g, 0, ev, br);
  if (!writer) return;
  int code = (g.precomputed ? CO_PRE : 0) | (p.isNew ? CO_NEW : 0) | (g.isShearNew ? CO_SHNEW : 0);
  if (g.angMode == 1) { code |= CO_ANG; S.angle[c] = make_double2(g.ang[0], g.ang[1]); }
  else if (g.angMode == 2) { code |= CO_ANG0; S.angle[c] = make_double2(0, 0); }
  double4 Fv = make_double4(0, 0, 0, 0), cp = make_double4(0, 0, 0, 0);
  V3<double> sOut = zero3<double>();
  if (g.precomputed) {
    LawIn<double> in;
    lawInputs<double>(p, g.depth, g.normal, g.cp, 0, in);
    LawOut<double> out;
    if (law(in, g.isShearNew, C.dt, out, br)) {
      code |= CO_FORCE | (out.sliding ? CO_SLIDE : 0);
      Fv = d4(out.Fv, 1.0);
      sOut = out.s;
    }
    cp = d4(g.cp, 0);
    S.normal[c] = d4(g.normal, 0);
  } else if (p.isNew) S.normal[c] = make_double4(0, 0, 0, 0);
  S.flag[c] |= CF_GEOM;
  S.depth[c] = g.depth;
  S.shear[c] = d4(sOut, 0);
  // bits 16-30: the step's Disfunction evaluations (the reverse step's cost, for its ordering)
  O.Fv[c] = Fv; O.cp[c] = cp; O.code[c] = code | (g.evals < 0x7FFF ? g.evals : 0x7FFF) << 16;
  SQA_CNT(&C.cnt[A_EVALS], g.evals);
  SQA_CNT(&C.cnt[A_LMCALLS], g.calls);
  // the decisions at which the map jumps: the Levenberg-Marquardt path (evaluations, calls).
  // The contact gate and the Coulomb cap are continuous (kinks), so they are not recorded.
  SQA_CNT(&C.cnt[A_SIG], branchHash(c, step, (unsigned long long)g.evals | ((unsigned long long)g.calls << 20)));
  if (br.mode != BR_OFF) {
    if (br.mode == BR_RECORD) {
      if ((br.n & 31) && br.n < BR_BITS) br.w[2 + (br.n >> 5)] = br.acc;
      br.w[0] = (unsigned)br.n;
      br.w[1] = br.cusp;
    } else if (br.w[1] != br.cusp) {
      SQA_CNT(&C.cnt[A_BRCUSP], 1);
    }
    SQA_CNT(&C.cnt[A_BRDEC], br.n);
    if (br.dis) SQA_CNT(&C.cnt[A_BRDIS], br.dis);
    if (br.n > BR_BITS) SQA_CNT(&C.cnt[A_BRUNF], br.n - BR_BITS);
  }
}
__global__ void __launch_bounds__(128) k_fwd_contacts(Consts C, State S, StepOut O, int step) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < C.P) fwdContact(C, S, O, step, c);
}
// The same with six lanes per pair (five pairs per warp, lanes 30 and 31 idle): each
// Disfunction evaluation is shared by the group (CoopEval); the group's first lane writes.
static const int COOP_WARPS = 4;
__global__ void __launch_bounds__(32 * COOP_WARPS) k_fwd_contacts_coop(Consts C, State S, StepOut O, int step) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = lane / 6, sub = lane - 6 * gw;
  const int c = (blockIdx.x * COOP_WARPS + warp) * 5 + gw;
  if (gw >= 5 || c >= C.P) return;
  CoopEval ev;
  ev.mask = 0x3Fu << (6 * gw);
  ev.g0 = 6 * gw;
  ev.sub = sub;
  fwdContact(C, S, O, step, c, ev, sub == 0);
}

// ForceContainer sum of one body over its pairs, in list order (NewtonIntegrator's view)
SQA_HD void gatherFT(const Consts& C, const StepOut& O, int b, const V3<double>& pos, V3<double>& f,
                                         V3<double>& m) {
  f = zero3<double>(); m = zero3<double>();
  for (int k = C.bStart[b]; k < C.bStart[b + 1]; k++) {
    const int e = C.bList[k] >> 1, side = C.bList[k] & 1;
    const double4 F4 = O.Fv[e];
    if (F4.w == 0) continue;
    const V3<double> F = xyz(F4), cp = xyz(O.cp[e]);
    if (side == 0) { f = f + F; m = m + (-cross(pos - cp, F)); }
    else { f = f + (-F); m = m + cross(pos - cp, F); }
  }
}

// translational update and the damping factors (NewtonIntegrator.cpp:99-304, cundallDamp2nd
// and cundallDamp1st :19-25) of a free, damped superquadric
struct Trans { V3<double> s, sr; };
SQA_HD Trans dampFactors(const Consts& C, const V3<double>& f, const V3<double>& m, double mass,
                                             const V3<double>& vel, const V3<double>& angVel, V3<double>& a) {
  const double dt = C.dt, d = C.damping;
  a = mk<double>(f.x / mass + C.g[0], f.y / mass + C.g[1], f.z / mass + C.g[2]);
  Trans t;
  t.s = mk<double>(1 - d * tsgn(a.x * (vel.x + 0.5 * dt * a.x)), 1 - d * tsgn(a.y * (vel.y + 0.5 * dt * a.y)),
                   1 - d * tsgn(a.z * (vel.z + 0.5 * dt * a.z)));
  t.sr = mk<double>(1 - d * tsgn(m.x * angVel.x), 1 - d * tsgn(m.y * angVel.y), 1 - d * tsgn(m.z * angVel.z));
  return t;
}

SQA_HD unsigned long long sgnBits(double x, double w, int k) {
  if (x == 0) return 0ull;
  return (w > 0 ? 1ull : (w < 0 ? 2ull : 3ull)) << (2 * k);
}
SQA_HD unsigned long long velSignBits(const V3<double>& a, const V3<double>& v, double dt, const V3<double>& m,
                                      const V3<double>& w) {
  return sgnBits(a.x, v.x + 0.5 * dt * a.x, 0) | sgnBits(a.y, v.y + 0.5 * dt * a.y, 1) |
         sgnBits(a.z, v.z + 0.5 * dt * a.z, 2) | sgnBits(m.x, w.x, 3) | sgnBits(m.y, w.y, 4) | sgnBits(m.z, w.z, 5) |
         (1ull << 12);
}
// The local damping on the branch tape: per component the sign of x w (2 bits: 1 positive, 2
// negative, 0 zero), which selects the factor 1 - d sgn(x w); x (1 - d sgn(x w)) kinks where x
// crosses 0 and jumps where w does.  Forced: the recorded factor where the natural one differs.
SQA_HD unsigned dampCode(double x, double w) {
  const double s = tsgn(x * w);
  return s > 0 ? 1u : (s < 0 ? 2u : 0u);
}
SQA_HD void dampBranches(const Consts& C, int step, int b, const V3<double>& a0, const V3<double>& vel0,
                         const V3<double>& m0, const V3<double>& angVel, Trans& t) {
  const double dt = C.dt, d = C.damping;
  const unsigned nat = dampCode(a0.x, vel0.x + 0.5 * dt * a0.x) | dampCode(a0.y, vel0.y + 0.5 * dt * a0.y) << 2 |
                       dampCode(a0.z, vel0.z + 0.5 * dt * a0.z) << 4 | dampCode(m0.x, angVel.x) << 6 |
                       dampCode(m0.y, angVel.y) << 8 | dampCode(m0.z, angVel.z) << 10;
  unsigned* slot = C.brBody + (size_t)step * C.nb + b;
  int dis = 0;
  if (C.brMode == BR_RECORD) {
    *slot = nat;
  } else if (*slot != nat) {
    const unsigned rec = *slot;
    double* f[6] = {&t.s.x, &t.s.y, &t.s.z, &t.sr.x, &t.sr.y, &t.sr.z};
    for (int k = 0; k < 6; k++) {
      const unsigned r2 = (rec >> (2 * k)) & 3u;
      if (r2 == ((nat >> (2 * k)) & 3u)) continue;
      dis++;
      *f[k] = 1 - d * (r2 == 1u ? 1.0 : (r2 == 2u ? -1.0 : 0.0));
    }
  }
  SQA_CNT(&C.cnt[A_BRDEC], 6);
  if (dis) SQA_CNT(&C.cnt[A_BRDIS], dis);
}
SQA_HD void fwdBody(const Consts& C, const State& S, const StepOut& O, int step, int b) {
  const double dt = C.dt;
  V3<double> pos = xyz(S.pos[b]);
  V3<double> vel = xyz(S.vel[b]);
  if (C.binfo[b].x == 1) {   // wall: all DOFs blocked, prescribed velocity
    pos = pos + vel * dt;
    S.pos[b] = d4(pos, 0);
    return;
  }
  V3<double> f, m, a;
  gatherFT(C, O, b, pos, f, m);
  const V3<double> angVel = xyz(S.angVel[b]);
  const double4 mI = C.massI[b];
  Trans t = dampFactors(C, f, m, mI.x, vel, angVel, a);
  const V3<double> a0 = a, vel0 = vel, m0 = m;
  // local damping x (1 - d sgn(x w)) is continuous where x crosses 0 and jumps where w does:
  // the sign of w (v + dt a / 2, resp. the angular velocity) where x is not 0
  const unsigned long long bits = velSignBits(a0, vel0, dt, m0, angVel);
  if (C.brMode != BR_OFF) dampBranches(C, step, b, a0, vel0, m0, angVel, t);
  a.x *= t.s.x; a.y *= t.s.y; a.z *= t.s.z;
  vel = vel + dt * a;
  m.x *= t.sr.x; m.y *= t.sr.y; m.z *= t.sr.z;
  double q[4], qo[4];
  loadQ(S.ori[b], q);
  V3<double> Lo, wo;
  rotStep<double>(q, xyz(S.angMom[b]), m, mI, dt, qo, Lo, wo);
  pos = pos + vel * dt;
  S.pos[b] = d4(pos, 0);
  S.ori[b] = make_double4(qo[0], qo[1], qo[2], qo[3]);
  S.vel[b] = d4(vel, 0); S.angVel[b] = d4(wo, 0); S.angMom[b] = d4(Lo, 0);
  SQA_CNT(&C.cnt[A_SIGB], branchHash(C.P + b, step, bits));
}
__global__ void __launch_bounds__(128) k_fwd_integrate(Consts C, State S, StepOut O, int step) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < C.nb) fwdBody(C, S, O, step, b);
}

// loss = sum_b wF_b . F_b (forces of the step in O) + wX_b . pos_b (state S); one block
__global__ void __launch_bounds__(256) k_loss(Consts C, State S, StepOut O, const double4* wF, const double4* wX,
                                              double* loss) {
  __shared__ double sh[256];
  double acc = 0;
  for (int b = threadIdx.x; b < C.nb; b += blockDim.x) {
    const V3<double> pos = xyz(S.pos[b]);
    V3<double> f, m;
    gatherFT(C, O, b, pos, f, m);
    acc += dot(xyz(wF[b]), f) + dot(xyz(wX[b]), pos);
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss[0] = sh[0];
}

// ---------------------------------------------------------------------------
// Reverse step, (1) the integrator of each body.  On entry the body adjoints hold
// dL/d(state after the step); on exit dL/d(state before the step) without the pairs' part,
// and lF, lT hold dL/d(force, torque) of the step.
SQA_HD void bwdBody(const Consts& C, const State& S, const StepOut& O, const Adj& A, int last, int b) {
  if (C.binfo[b].x == 1) {
    A.lF[b] = last ? A.wF[b] : make_double4(0, 0, 0, 0);
    A.lT[b] = make_double4(0, 0, 0, 0);
    return;
  }
  const double dt = C.dt;
  const V3<double> pos = xyz(S.pos[b]), vel = xyz(S.vel[b]), angVel = xyz(S.angVel[b]);
  V3<double> f, m, a;
  gatherFT(C, O, b, pos, f, m);
  const double4 mI = C.massI[b];
  const Trans t = dampFactors(C, f, m, mI.x, vel, angVel, a);
  const V3<double> lp = xyz(A.lPos[b]), lv = xyz(A.lVel[b]), lw = xyz(A.lW[b]), lL = xyz(A.lL[b]);
  const double4 lq4 = A.lOri[b];
  const double lq[4] = {lq4.x, lq4.y, lq4.z, lq4.w};
  // pos' = pos + dt vel', vel' = vel + dt s (f/mass + g)
  const V3<double> lvt = lv + dt * lp;
  V3<double> lf = mk<double>(dt * t.s.x * lvt.x / mI.x, dt * t.s.y * lvt.y / mI.x, dt * t.s.z * lvt.z / mI.x);
  // rotation, replayed with tangents on q (0-3), L (4-6) and the damped torque (7-9)
  const V3<double> md = mk<double>(m.x * t.sr.x, m.y * t.sr.y, m.z * t.sr.z);
  double q[4];
  loadQ(S.ori[b], q);
  DT qd[4], qo[4];
  for (int k = 0; k < 4; k++) qd[k] = seed<NT>(q[k], k);
  const V3<double> L = xyz(S.angMom[b]);
  const V3<DT> Ld = mk<DT>(seed<NT>(L.x, 4), seed<NT>(L.y, 5), seed<NT>(L.z, 6));
  const V3<DT> Md = mk<DT>(seed<NT>(md.x, 7), seed<NT>(md.y, 8), seed<NT>(md.z, 9));
  V3<DT> Lo, wo;
  rotStep<DT>(qd, Ld, Md, mI, dt, qo, Lo, wo);
  double gsum[10];
  for (int j = 0; j < 10; j++) {
    double s = 0;
    for (int k = 0; k < 4; k++) s += lq[k] * qo[k].d[j];
    s += lL.x * Lo.x.d[j] + lL.y * Lo.y.d[j] + lL.z * Lo.z.d[j];
    s += lw.x * wo.x.d[j] + lw.y * wo.y.d[j] + lw.z * wo.z.d[j];
    gsum[j] = s;
  }
  V3<double> lm = mk<double>(gsum[7] * t.sr.x, gsum[8] * t.sr.y, gsum[9] * t.sr.z);
  if (last) { const double4 w = A.wF[b]; lf = lf + xyz(w); }
  A.lPos[b] = d4(lp, 0);
  A.lVel[b] = d4(lvt, 0);
  A.lOri[b] = make_double4(gsum[0], gsum[1], gsum[2], gsum[3]);
  A.lL[b] = make_double4(gsum[4], gsum[5], gsum[6], 0);
  A.lW[b] = make_double4(0, 0, 0, 0);
  A.lF[b] = d4(lf, 0);
  A.lT[b] = d4(lm, 0);
}
__global__ void __launch_bounds__(128) k_bwd_integrate(Consts C, State S, StepOut O, Adj A, int last) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < C.nb) bwdBody(C, S, O, A, last, b);
}

// Reverse step, (2) one pair: replay geometry and law with tangents, contract with the
// adjoints of the pair's outputs (force and torques through lF/lT of its bodies, the stored
// contact angles, normal and shear force through lAng/lN/lS), and leave the adjoints of the
// pair's inputs: its stored history (in lAng/lN/lS), its bodies' state (in con) and the
// parameters (accumulated in accEps/accPhys).
template <int N> SQA_HD double dotd(const V3<double>& l, const V3<Dual<N>>& v, int j) {
  return l.x * v.x.d[j] + l.y * v.y.d[j] + l.z * v.z.d[j];
}
struct PairAdjIn {
  PairVals p;
  bool pre, force, needed;
  int angMode;
  V3<double> lFv, lT1, lT2, lnOut, lsOut;
  double2 la2;
};
SQA_HD void pairAdjIn(const Consts& C, const State& S, const StepOut& O, const Adj& A, int c, PairAdjIn& q) {
  loadPair(C, S, c, q.p);
  const int code = O.code[c];
  q.pre = (code & CO_PRE) != 0;
  q.force = (code & CO_FORCE) != 0;
  q.angMode = (code & CO_ANG) ? 1 : ((code & CO_ANG0) ? 2 : 0);
  q.lFv = xyz(A.lF[q.p.id.x]) - xyz(A.lF[q.p.id.y]);
  q.lT1 = xyz(A.lT[q.p.id.x]);
  q.lT2 = xyz(A.lT[q.p.id.y]);
  q.la2 = A.lAng[c];
  q.lnOut = xyz(A.lN[c]);
  q.lsOut = xyz(A.lS[c]);
  // A pair without a force whose new contact angles nothing downstream depends on (zero
  // adjoint) contributes nothing: its replay is skipped.
  q.needed = q.pre || (q.angMode == 1 && (q.la2.x != 0 || q.la2.y != 0));
}
// Contraction of one law input's tangent (component j of the replay) with the adjoints of the
// law's outputs.
template <int N> SQA_HD double lawContract(const PairAdjIn& q, const LawOut<Dual<N>>& out, int j) {
  return dotd(q.lFv, out.Fv, j) + dotd(q.lT1, out.T1, j) + dotd(q.lT2, out.T2, j) + dotd(q.lsOut, out.s, j);
}
// Contraction of one geometry input's tangent with the adjoints of the geometry's outputs
// (depth, normal, contact point from the law; stored normal and angles from the next step).
template <int N> SQA_HD double geomContract(const PairAdjIn& q, const Geom<Dual<N>>& gd, const double* lin, int j) {
  double s = 0;
  if (q.pre) {
    const V3<double> lnormal = q.lnOut + mk<double>(lin[1], lin[2], lin[3]);
    s += lin[0] * gd.depth.d[j] + dotd(lnormal, gd.normal, j) + dotd(mk<double>(lin[4], lin[5], lin[6]), gd.cp, j);
  }
  if (q.angMode == 1) s += q.la2.x * gd.ang[0].d[j] + q.la2.y * gd.ang[1].d[j];
  return s;
}
// The pair's outputs of the reverse step from lin (dL/d law inputs, zero without a force) and
// gs (contracted geometry tangents, zero without a replay).
SQA_HD void assemblePair(const Adj& A, int c, const PairAdjIn& q, const double* lin, const double* gs) {
  V3<double> lx1 = zero3<double>(), lx2 = zero3<double>(), lv1 = zero3<double>(), lw1 = zero3<double>();
  V3<double> lv2 = zero3<double>(), lw2 = zero3<double>(), lsPrev = zero3<double>();
  V3<double> lnPrev = (!q.pre && !q.p.isNew) ? q.lnOut : zero3<double>();   // passes through unchanged
  double lq1[4] = {0, 0, 0, 0}, lq2[4] = {0, 0, 0, 0}, leps[4] = {0, 0, 0, 0}, lphys[3] = {0, 0, 0};
  double langIn[2] = {q.angMode == 0 ? q.la2.x : 0.0, q.angMode == 0 ? q.la2.y : 0.0};
  if (q.force) {
    lx1 = mk<double>(lin[7], lin[8], lin[9]); lx2 = mk<double>(lin[10], lin[11], lin[12]);
    lv1 = mk<double>(lin[13], lin[14], lin[15]); lw1 = mk<double>(lin[16], lin[17], lin[18]);
    lv2 = mk<double>(lin[19], lin[20], lin[21]); lw2 = mk<double>(lin[22], lin[23], lin[24]);
    lnPrev = mk<double>(lin[25], lin[26], lin[27]); lsPrev = mk<double>(lin[28], lin[29], lin[30]);
    lphys[0] = lin[31]; lphys[1] = lin[32]; lphys[2] = lin[33];
  }
  if (q.needed) {
    lx2 = lx2 + mk<double>(gs[0], gs[1], gs[2]);
    if (q.p.i1.x != 1) lx1 = lx1 + mk<double>(lin[4], lin[5], lin[6]) - mk<double>(gs[0], gs[1], gs[2]);
    for (int k = 0; k < 4; k++) { lq1[k] = gs[3 + k]; lq2[k] = gs[7 + k]; leps[k] = gs[11 + k]; }
    langIn[0] += gs[15]; langIn[1] += gs[16];
  }
  A.lAng[c] = make_double2(langIn[0], langIn[1]);
  A.lN[c] = d4(lnPrev, 0);
  A.lS[c] = d4(lsPrev, 0);
  double4* con = A.con + (size_t)c * 8;
  con[0] = d4(lx1, 0); con[1] = make_double4(lq1[0], lq1[1], lq1[2], lq1[3]); con[2] = d4(lv1, 0); con[3] = d4(lw1, 0);
  con[4] = d4(lx2, 0); con[5] = make_double4(lq2[0], lq2[1], lq2[2], lq2[3]); con[6] = d4(lv2, 0); con[7] = d4(lw2, 0);
  const double4 ae = A.accEps[c], ap = A.accPhys[c];
  A.accEps[c] = make_double4(ae.x + leps[0], ae.y + leps[1], ae.z + leps[2], ae.w + leps[3]);
  A.accPhys[c] = make_double4(ap.x + lphys[0], ap.y + lphys[1], ap.z + lphys[2], 0);
}
// the replay's branches against the forward run's (counted, reported by the backward call)
template <int N> SQA_HD void checkReplay(const Consts& C, const StepOut& O, int c, const PairAdjIn& q,
                                         const Geom<Dual<N>>& gd) {
  if (gd.precomputed != q.pre || (gd.angMode == 1) != (q.angMode == 1)) SQA_CNT(&C.cnt[A_MISMATCH], 1);
}
template <int N> SQA_HD void checkLaw(const Consts& C, const StepOut& O, int c, bool ran, const LawOut<Dual<N>>& out) {
  if (!ran) { SQA_CNT(&C.cnt[A_MISMATCH], 1); return; }
  const double4 F4 = O.Fv[c];
  if (F4.x != out.Fv.x.v || F4.y != out.Fv.y.v || F4.z != out.Fv.z.v) SQA_CNT(&C.cnt[A_MISMATCH], 1);
}

// One thread per pair, all 17 geometry tangents and two chunks of 17 law tangents per thread.
SQA_HD void bwdContact(const Consts& C, const State& S, const StepOut& O, const Adj& A, int c) {
  PairAdjIn q;
  pairAdjIn(C, S, O, A, c, q);
  double lin[2 * NT], gs[NT];
  for (int j = 0; j < 2 * NT; j++) lin[j] = 0;
  for (int j = 0; j < NT; j++) gs[j] = 0;
  if (q.needed) {
    SQA_CNT(&C.cnt[A_REPLAYED], 1);
    Geom<DT> gd;
    pairGeom<DT>(q.p, gd);
    checkReplay(C, O, c, q, gd);
    if (q.pre && q.force) {
      const V3<double> nv = mk<double>(gd.normal.x.v, gd.normal.y.v, gd.normal.z.v);
      const V3<double> cpv = mk<double>(gd.cp.x.v, gd.cp.y.v, gd.cp.z.v);
      for (int chunk = 0; chunk < 2; chunk++) {
        LawIn<DT> in;
        lawInputs<DT>(q.p, gd.depth.v, nv, cpv, chunk, in);
        LawOut<DT> out;
        const bool ran = law(in, gd.isShearNew, C.dt, out);
        if (chunk == 0 || !ran) checkLaw(C, O, c, ran, out);
        if (ran)
          for (int j = 0; j < NT; j++) lin[chunk * NT + j] = lawContract(q, out, j);
      }
    }
    for (int j = 0; j < NT; j++) gs[j] = geomContract(q, gd, lin, j);
  }
  assemblePair(A, c, q, lin, gs);
}
__global__ void __launch_bounds__(64) k_bwd_contacts(Consts C, State S, StepOut O, Adj A) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < C.P) bwdContact(C, S, O, A, c);
}

// The same reverse step of a pair split over a group of GL lanes, lane l carrying the tangent
// components TG*l .. TG*l+TG-1 of every replay (TG*GL >= 17).  Each lane repeats the primal
// evaluations (GL-fold work) but carries fewer tangents, so the longest Levenberg-Marquardt
// replay of a step is shorter and the Dual<TG> values stay in registers.  Every tangent
// component is computed by the same operations as in k_bwd_contacts, so the results are
// bitwise the same for every shape.
static const int GRP_WARPS = 4;
template <int TG, int GL>
__global__ void __launch_bounds__(32 * GRP_WARPS) k_bwd_contacts_grp(Consts C, State S, StepOut O, Adj A) {
  constexpr int GPW = 32 / GL;
  __shared__ double shLin[GRP_WARPS * GPW][2 * NT];
  __shared__ double shGs[GRP_WARPS * GPW][NT];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = lane / GL, l = lane - gw * GL;
  const bool laneOn = gw < GPW;
  const int slot = warp * GPW + (laneOn ? gw : 0);
  const int base = TG * l;
  // grid-stride over the pairs: the launch sizes the grid so that the lanes' local memory (the
  // replayed state, a few KB per lane) of the resident blocks stays in L2
  for (int c0 = blockIdx.x * GRP_WARPS * GPW; c0 < C.P; c0 += gridDim.x * GRP_WARPS * GPW) {
  const int i = c0 + warp * GPW + gw;
  const bool active = laneOn && i < C.P;
  const int c = active && A.order ? A.order[i] : i;
  PairAdjIn q;
  Geom<Dual<TG>> gd;
  if (active) {
    pairAdjIn(C, S, O, A, c, q);
    for (int j = 0; j < TG; j++) {
      const int k = base + j;
      if (k < NT) { shLin[slot][k] = 0; shLin[slot][NT + k] = 0; }
    }
    if (q.needed) {
      if (l == 0) SQA_CNT(&C.cnt[A_REPLAYED], 1);
      pairGeom<Dual<TG>>(q.p, gd, base);
      if (l == 0) checkReplay(C, O, c, q, gd);
      if (q.pre && q.force) {
        const V3<double> nv = mk<double>(gd.normal.x.v, gd.normal.y.v, gd.normal.z.v);
        const V3<double> cpv = mk<double>(gd.cp.x.v, gd.cp.y.v, gd.cp.z.v);
        for (int chunk = 0; chunk < 2; chunk++) {
          LawIn<Dual<TG>> in;
          lawInputs<Dual<TG>>(q.p, gd.depth.v, nv, cpv, chunk, in, base);
          LawOut<Dual<TG>> out;
          const bool ran = law(in, gd.isShearNew, C.dt, out);
          if (l == 0 && (chunk == 0 || !ran)) checkLaw(C, O, c, ran, out);
          if (ran)
            for (int j = 0; j < TG; j++)
              if (base + j < NT) shLin[slot][chunk * NT + base + j] = lawContract(q, out, j);
        }
      }
    }
  }
  __syncwarp();
  if (active) {
    for (int j = 0; j < TG; j++)
      if (base + j < NT) shGs[slot][base + j] = q.needed ? geomContract(q, gd, shLin[slot], j) : 0.0;
  }
  __syncwarp();
  if (active && l == 0) assemblePair(A, c, q, shLin[slot], shGs[slot]);
  __syncwarp();
  }
}

// Reverse step, (3) each body adds its pairs' contributions, in list order.
SQA_HD void bwdGather(const Consts& C, const Adj& A, int b) {
  if (C.binfo[b].x == 1) return;
  double4 sp = A.lPos[b], so = A.lOri[b], sv = A.lVel[b], sw = A.lW[b];
  for (int k = C.bStart[b]; k < C.bStart[b + 1]; k++) {
    const int e = C.bList[k] >> 1, side = C.bList[k] & 1;
    const double4* con = A.con + (size_t)e * 8 + side * 4;
    const double4 a = con[0], q = con[1], v = con[2], w = con[3];
    sp.x += a.x; sp.y += a.y; sp.z += a.z;
    so.x += q.x; so.y += q.y; so.z += q.z; so.w += q.w;
    sv.x += v.x; sv.y += v.y; sv.z += v.z;
    sw.x += w.x; sw.y += w.y; sw.z += w.z;
  }
  A.lPos[b] = sp; A.lOri[b] = so; A.lVel[b] = sv; A.lW[b] = sw;
}
__global__ void __launch_bounds__(128) k_bwd_gather(Consts C, Adj A) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < C.nb) bwdGather(C, A, b);
}

// Order of a reverse step's pairs: a counting sort on the forward step's evaluation counts,
// longest first, so that the longest replays start in the first wave and pairs of similar
// length share a warp.  Each pair's reverse step writes only its own outputs, so the order
// changes no result.  Buckets: 64 - min(63, evals / 4), i.e. bucket 1 holds 252+ evaluations.
static const int ORD_BUCKETS = 64;
SQA_HD int ordBucket(int code) {
  const int ev = code >> 16;
  return ORD_BUCKETS - 1 - (ev / 4 < ORD_BUCKETS - 1 ? ev / 4 : ORD_BUCKETS - 1);
}
__global__ void __launch_bounds__(256) k_order_count(int P, const int* code, int* cnt) {
  __shared__ int sh[ORD_BUCKETS];
  for (int k = threadIdx.x; k < ORD_BUCKETS; k += blockDim.x) sh[k] = 0;
  __syncthreads();
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < P; c += gridDim.x * blockDim.x)
    atomicAdd(&sh[ordBucket(code[c])], 1);
  __syncthreads();
  for (int k = threadIdx.x; k < ORD_BUCKETS; k += blockDim.x)
    if (sh[k]) atomicAdd(&cnt[k], sh[k]);
}
// exclusive scan of the bucket counts into the write cursors (one warp pair of 64 threads)
__global__ void __launch_bounds__(ORD_BUCKETS) k_order_scan(int* cnt) {
  __shared__ int sh[ORD_BUCKETS];
  const int t = threadIdx.x;
  sh[t] = cnt[t];
  __syncthreads();
  if (t == 0) {
    int run = 0;
    for (int k = 0; k < ORD_BUCKETS; k++) { const int v = sh[k]; sh[k] = run; run += v; }
  }
  __syncthreads();
  cnt[t] = sh[t];
}
__global__ void __launch_bounds__(256) k_order_scatter(int P, const int* code, int* cursor, int* order) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < P; c += gridDim.x * blockDim.x)
    order[atomicAdd(&cursor[ordBucket(code[c])], 1)] = c;
}

}  // namespace sqadj

// ===========================================================================
// Host side
using namespace sqadj;

namespace {

size_t alignUp(size_t x) { return (x + 255) & ~(size_t)255; }

// byte offsets of the arrays of one State inside a single allocation
struct StateLayout {
  size_t pos, ori, vel, angVel, angMom, normal, shear, angle, depth, flag, bytes;
  void init(int nb, int P) {
    size_t o = 0;
    auto take = [&](size_t n) { size_t r = o; o = alignUp(o + n); return r; };
    pos = take(16 * 2 * (size_t)nb); ori = take(32 * (size_t)nb); vel = take(32 * (size_t)nb);
    angVel = take(32 * (size_t)nb); angMom = take(32 * (size_t)nb);
    normal = take(32 * (size_t)P); shear = take(32 * (size_t)P); angle = take(16 * (size_t)P);
    depth = take(8 * (size_t)P); flag = take(4 * (size_t)P);
    bytes = o > 0 ? o : 256;
  }
  State view(char* b) const {
    State s;
    s.pos = (double4*)(b + pos); s.ori = (double4*)(b + ori); s.vel = (double4*)(b + vel);
    s.angVel = (double4*)(b + angVel); s.angMom = (double4*)(b + angMom);
    s.normal = (double4*)(b + normal); s.shear = (double4*)(b + shear); s.angle = (double2*)(b + angle);
    s.depth = (double*)(b + depth); s.flag = (int*)(b + flag);
    return s;
  }
};

}  // namespace

struct sqdem_adj {
  int device = 0;
  cudaStream_t st = nullptr;
  std::string err;
  int nb = 0, P = 0, nmat = 0;
  double dt = 0, g[3] = {0, 0, 0}, damping = 0;
  // host copies
  std::vector<int> kind, mat;
  std::vector<int2> ids;
  std::vector<double> Kn, Ks, fa;
  // device, constant over a window
  double4 *shp = nullptr, *massI = nullptr, *phys = nullptr;
  double2* eps = nullptr;
  int4* binfo = nullptr;
  int2* idsD = nullptr;
  int *bStart = nullptr, *bList = nullptr;
  unsigned long long* cnt = nullptr;
  // states
  StateLayout L;
  char* init = nullptr;   // state at the start of the window
  char* work = nullptr;
  char* fin = nullptr;        // state after the last forward window (kept through the reverse pass)
  double4* finFv = nullptr;   // forces of that window's last step
  std::vector<char*> ckpt;
  // tape of one segment
  int tapeCap = 0;
  std::vector<char*> tapeState;
  double4 *tapeFv = nullptr, *tapeCp = nullptr;
  int* tapeCode = nullptr;
  // adjoints
  double4 *lPos = nullptr, *lOri = nullptr, *lVel = nullptr, *lW = nullptr, *lL = nullptr, *lF = nullptr, *lT = nullptr;
  double2* lAng = nullptr;
  double4 *lN = nullptr, *lS = nullptr, *con = nullptr, *accEps = nullptr, *accPhys = nullptr;
  double4 *wF = nullptr, *wX = nullptr;
  double* lossD = nullptr;
  int *order = nullptr, *orderCnt = nullptr;   // reverse-step pair order and its bucket counters
  // the last forward window
  int nsteps = 0, every = 0;
  bool haveForward = false;
  int replay = 3;   // reverse-step kernel of the pairs: 0 one thread per pair, 1.. lane-group shapes
  int replayBlocks = 1;   // grouped reverse kernels: resident blocks per SM (grid-stride); 0 = unbounded
  int numSMs = 1;
  bool coopForward = true;   // forward pairs on six-lane groups (k_fwd_contacts_coop)
  // branch tape (BR_OFF, BR_RECORD, BR_FORCE) and the steps it holds
  int brMode = BR_OFF, brSteps = 0;
  size_t brCap = 0;   // steps allocated
  unsigned *brPair = nullptr, *brBody = nullptr;
  double loss = 0;
  unsigned long long counters[A_NCOUNT] = {};
  double msForward = 0, msBackward = 0;
  std::vector<void*> allocs;
};

static sqdem_status afail(sqdem_adj* a, sqdem_status s, const std::string& m) {
  if (a) a->err = m;
  return s;
}
#define ACUDA(call)                                                                              \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return afail(a, SQDEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T> static cudaError_t aalloc(sqdem_adj* a, T** p, size_t n) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, n * sizeof(T) > 0 ? n * sizeof(T) : 16);
  if (e == cudaSuccess) { a->allocs.push_back(q); *p = (T*)q; }
  return e;
}
static void afreeAll(sqdem_adj* a) {
  for (void* p : a->allocs) cudaFree(p);
  a->allocs.clear();
  a->ckpt.clear(); a->tapeState.clear();
  a->init = a->work = a->fin = nullptr; a->finFv = nullptr; a->tapeCap = 0;
  a->brPair = a->brBody = nullptr; a->brCap = 0; a->brSteps = 0;
  a->order = a->orderCnt = nullptr;
}
static void afree(sqdem_adj* a, void* p) {
  if (!p) return;
  auto it = std::find(a->allocs.begin(), a->allocs.end(), p);
  if (it != a->allocs.end()) { cudaFree(p); a->allocs.erase(it); }
}

static Consts consts(sqdem_adj* a, bool branches = false) {
  Consts C;
  C.nb = a->nb; C.P = a->P; C.dt = a->dt; C.g[0] = a->g[0]; C.g[1] = a->g[1]; C.g[2] = a->g[2];
  C.damping = a->damping;
  C.shp = a->shp; C.eps = a->eps; C.massI = a->massI; C.binfo = a->binfo; C.ids = a->idsD; C.phys = a->phys;
  C.bStart = a->bStart; C.bList = a->bList; C.cnt = a->cnt;
  C.brMode = branches ? a->brMode : BR_OFF;
  C.brPair = a->brPair; C.brBody = a->brBody;
  return C;
}
static StepOut tapeOut(sqdem_adj* a, int slot) {
  StepOut o;
  o.Fv = a->tapeFv + (size_t)slot * a->P; o.cp = a->tapeCp + (size_t)slot * a->P; o.code = a->tapeCode + (size_t)slot * a->P;
  return o;
}
static Adj adjView(sqdem_adj* a) {
  Adj A;
  A.lPos = a->lPos; A.lOri = a->lOri; A.lVel = a->lVel; A.lW = a->lW; A.lL = a->lL; A.lF = a->lF; A.lT = a->lT;
  A.lAng = a->lAng; A.lN = a->lN; A.lS = a->lS; A.con = a->con; A.accEps = a->accEps; A.accPhys = a->accPhys;
  A.wF = a->wF; A.wX = a->wX;
  A.order = nullptr;
  return A;
}
static inline int nblk(int n, int bs) { return n > 0 ? (n + bs - 1) / bs : 1; }

// Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys::go (Superquadrics.cpp:1086-1116)
static void physOf(const sqdem_adj* a, int c, double& kn, double& ks, double& tanphi) {
  const int id1 = a->ids[c].x, id2 = a->ids[c].y;
  const int m1 = a->mat[id1], m2 = a->mat[id2];
  if (id1 > 5) {
    const double f = (a->fa[m2] < a->fa[m1]) ? a->fa[m2] : a->fa[m1];
    tanphi = tan(f);
    kn = 2.0 * a->Kn[m1] * a->Kn[m2] / (a->Kn[m1] + a->Kn[m2]);
    ks = 2.0 * a->Ks[m1] * a->Ks[m2] / (a->Ks[m1] + a->Ks[m2]);
  } else {
    tanphi = tan(a->fa[m1]); kn = a->Kn[m1]; ks = a->Ks[m1];
  }
}

static sqdem_status ensureTape(sqdem_adj* a, int K) {
  if (a->tapeCap >= K) return SQDEM_OK;
  // grow: the old tape buffers stay allocated until destroy (tapes are sized once per run)
  a->tapeState.clear();
  for (int k = 0; k < K; k++) {
    char* p = nullptr;
    ACUDA(aalloc(a, &p, a->L.bytes));
    a->tapeState.push_back(p);
  }
  ACUDA(aalloc(a, &a->tapeFv, (size_t)K * a->P));
  ACUDA(aalloc(a, &a->tapeCp, (size_t)K * a->P));
  ACUDA(aalloc(a, &a->tapeCode, (size_t)K * a->P));
  a->tapeCap = K;
  return SQDEM_OK;
}

// shapes of the pairs' reverse step: 0 one thread (17 tangents), 1: 3 lanes x 6, 2: 2 lanes x 9,
// 3: 6 lanes x 3
static void launchReplay(sqdem_adj* a, const Consts& C, const State& S, const StepOut& O, const Adj& A0) {
  const int P = a->P, bs = 32 * GRP_WARPS;
  Adj A = A0;
  if (a->order && a->replay != 0 && P > 0) {
    const int g = std::min(nblk(P, 256), 4 * a->numSMs);
    cudaMemsetAsync(a->orderCnt, 0, ORD_BUCKETS * sizeof(int), a->st);
    k_order_count<<<g, 256, 0, a->st>>>(P, O.code, a->orderCnt);
    k_order_scan<<<1, ORD_BUCKETS, 0, a->st>>>(a->orderCnt);
    k_order_scatter<<<g, 256, 0, a->st>>>(P, O.code, a->orderCnt, a->order);
    A.order = a->order;
  }
  // blocks of the grouped kernels: a->replayBlocks per SM (grid-stride), 0 = one block per
  // group of pairs (as many resident as fit: their local memory spills past L2 to DRAM)
  auto grid = [&](int perBlock) {
    const int g = nblk(P, perBlock);
    return a->replayBlocks > 0 ? std::min(g, a->numSMs * a->replayBlocks) : g;
  };
  switch (a->replay) {
    case 0: k_bwd_contacts<<<nblk(P, 64), 64, 0, a->st>>>(C, S, O, A); break;
    case 2: k_bwd_contacts_grp<9, 2><<<grid(GRP_WARPS * 16), bs, 0, a->st>>>(C, S, O, A); break;
    case 1: k_bwd_contacts_grp<6, 3><<<grid(GRP_WARPS * 10), bs, 0, a->st>>>(C, S, O, A); break;
    default: k_bwd_contacts_grp<3, 6><<<grid(GRP_WARPS * 5), bs, 0, a->st>>>(C, S, O, A); break;
  }
}

static void launchStep(sqdem_adj* a, const State& S, const StepOut& O, int step, bool branches = false) {
  const Consts C = consts(a, branches);
  if (a->coopForward)
    k_fwd_contacts_coop<<<nblk(a->P, COOP_WARPS * 5), 32 * COOP_WARPS, 0, a->st>>>(C, S, O, step);
  else
    k_fwd_contacts<<<nblk(a->P, 128), 128, 0, a->st>>>(C, S, O, step);
  k_fwd_integrate<<<nblk(a->nb, 128), 128, 0, a->st>>>(C, S, O, step);
}

extern "C" {

sqdem_status sqdem_adj_create(sqdem_adj** out, int device) {
  if (!out) return SQDEM_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return SQDEM_ERR_CUDA;
  if (device < 0 || device >= n) return SQDEM_ERR_ARG;
  sqdem_adj* a = new sqdem_adj();
  a->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&a->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaDeviceGetAttribute(&a->numSMs, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
    delete a;
    return SQDEM_ERR_CUDA;
  }
  *out = a;
  return SQDEM_OK;
}

void sqdem_adj_destroy(sqdem_adj* a) {
  if (!a) return;
  cudaSetDevice(a->device);
  if (a->st) cudaStreamSynchronize(a->st);
  afreeAll(a);
  if (a->st) cudaStreamDestroy(a->st);
  delete a;
}

const char* sqdem_adj_last_error(sqdem_adj* a) { return a ? a->err.c_str() : "null adjoint context"; }

sqdem_status sqdem_adj_load(sqdem_adj* a, int n, const int* kind, const double* shape5, const int* wall_axis_sense,
                            const int* mat, const int* isSphere, const double* state37, long npairs, const double* intr57,
                            double dt, const double* gravity3, double damping) {
  if (!a) return SQDEM_ERR_ARG;
  if (n <= 0 || !kind || !shape5 || !wall_axis_sense || !mat || !state37 || npairs < 0 || (npairs > 0 && !intr57) ||
      !gravity3 || !(dt > 0))
    return afail(a, SQDEM_ERR_ARG, "sqdem_adj_load: bad argument");
  ACUDA(cudaSetDevice(a->device));
  ACUDA(cudaStreamSynchronize(a->st));
  afreeAll(a);
  a->haveForward = false;
  a->nb = n; a->dt = dt; a->damping = damping;
  for (int k = 0; k < 3; k++) a->g[k] = gravity3[k];
  a->kind.assign(kind, kind + n);
  a->mat.assign(mat, mat + n);
  int maxMat = 0;
  for (int i = 0; i < n; i++) {
    if (kind[i] != SQDEM_SUPERQUADRIC && kind[i] != SQDEM_WALL) return afail(a, SQDEM_ERR_ARG, "unknown body kind");
    if (mat[i] < 0) return afail(a, SQDEM_ERR_ARG, "negative material id");
    maxMat = std::max(maxMat, mat[i]);
    if (kind[i] == SQDEM_SUPERQUADRIC && isSphere && isSphere[i])
      return afail(a, SQDEM_ERR_ARG, "the adjoint window supports superquadrics not flagged as spheres");
    const double* s = state37 + (size_t)i * SQDEM_BODY_STRIDE;
    if (kind[i] == SQDEM_SUPERQUADRIC && !(s[33] > 0)) return afail(a, SQDEM_ERR_ARG, "particle without mass");
  }
  a->nmat = maxMat + 1;
  // pairs: wall pairs as (wall, particle) (the dispatcher's swap, InteractionLoop.cpp:83-92); wall-wall dropped
  a->ids.clear();
  std::vector<int> hFlag; std::vector<double> hDepth; std::vector<double2> hAng; std::vector<double4> hN, hS;
  for (long r = 0; r < npairs; r++) {
    const double* o = intr57 + (size_t)r * SQDEM_INTR_STRIDE;
    int i1 = (int)o[0], i2 = (int)o[1];
    if (i1 < 0 || i2 < 0 || i1 >= n || i2 >= n || i1 == i2) return afail(a, SQDEM_ERR_ARG, "pair with a bad body id");
    if (o[44] != 0 || o[45] != 0 || o[46] != 0)
      return afail(a, SQDEM_ERR_ARG, "pair across a periodic cell boundary: the adjoint window has no periodic cell");
    if (kind[i1] == SQDEM_WALL && kind[i2] == SQDEM_WALL) continue;
    if (kind[i1] == SQDEM_SUPERQUADRIC && kind[i2] == SQDEM_WALL) std::swap(i1, i2);
    a->ids.push_back(make_int2(i1, i2));
    hFlag.push_back(o[3] != 0 ? CF_GEOM : 0);
    hDepth.push_back(o[4]);
    hAng.push_back(make_double2(o[5], o[6]));
    hN.push_back(make_double4(o[10], o[11], o[12], 0));
    hS.push_back(make_double4(o[29], o[30], o[31], 0));
  }
  a->P = (int)a->ids.size();
  const int P = a->P;
  // per-body pair lists, ascending pair index
  std::vector<int> cntB(n + 1, 0), start(n + 1, 0), list(2 * (size_t)P);
  for (int c = 0; c < P; c++) { cntB[a->ids[c].x]++; cntB[a->ids[c].y]++; }
  for (int i = 0; i < n; i++) start[i + 1] = start[i] + cntB[i];
  std::vector<int> fill(start.begin(), start.end() - 1);
  for (int c = 0; c < P; c++) { list[fill[a->ids[c].x]++] = 2 * c; list[fill[a->ids[c].y]++] = 2 * c + 1; }
  // constant body data
  std::vector<double4> hShp(n), hMI(n);
  std::vector<double2> hEps(n);
  std::vector<int4> hInfo(n);
  for (int i = 0; i < n; i++) {
    const double* s5 = shape5 + (size_t)i * 5;
    const double* s = state37 + (size_t)i * SQDEM_BODY_STRIDE;
    double rmax = 0;
    if (kind[i] == SQDEM_SUPERQUADRIC) {
      double props[5];
      sqdem_status st = sqdem_shape_props(s5[0], s5[1], s5[2], s5[3], s5[4], props);
      if (st != SQDEM_OK) return afail(a, st, "bad shape");
      rmax = props[4];
    }
    hShp[i] = make_double4(s5[0], s5[1], s5[2], rmax);
    hEps[i] = make_double2(s5[3], s5[4]);
    hMI[i] = make_double4(s[33], s[34], s[35], s[36]);
    hInfo[i] = make_int4(kind[i], wall_axis_sense[2 * i], wall_axis_sense[2 * i + 1], 0);
  }
  a->L.init(n, P);
  ACUDA(aalloc(a, &a->shp, n)); ACUDA(aalloc(a, &a->massI, n)); ACUDA(aalloc(a, &a->eps, n));
  ACUDA(aalloc(a, &a->binfo, n)); ACUDA(aalloc(a, &a->idsD, P)); ACUDA(aalloc(a, &a->phys, P));
  ACUDA(aalloc(a, &a->bStart, n + 1)); ACUDA(aalloc(a, &a->bList, 2 * (size_t)P));
  ACUDA(aalloc(a, &a->cnt, A_NCOUNT));
  ACUDA(aalloc(a, &a->init, a->L.bytes)); ACUDA(aalloc(a, &a->work, a->L.bytes)); ACUDA(aalloc(a, &a->fin, a->L.bytes));
  ACUDA(aalloc(a, &a->finFv, P));
  ACUDA(aalloc(a, &a->lPos, n)); ACUDA(aalloc(a, &a->lOri, n)); ACUDA(aalloc(a, &a->lVel, n));
  ACUDA(aalloc(a, &a->lW, n)); ACUDA(aalloc(a, &a->lL, n)); ACUDA(aalloc(a, &a->lF, n)); ACUDA(aalloc(a, &a->lT, n));
  ACUDA(aalloc(a, &a->lAng, P)); ACUDA(aalloc(a, &a->lN, P)); ACUDA(aalloc(a, &a->lS, P));
  ACUDA(aalloc(a, &a->con, 8 * (size_t)P)); ACUDA(aalloc(a, &a->accEps, P)); ACUDA(aalloc(a, &a->accPhys, P));
  ACUDA(aalloc(a, &a->wF, n)); ACUDA(aalloc(a, &a->wX, n)); ACUDA(aalloc(a, &a->lossD, 1));
  ACUDA(aalloc(a, &a->order, (size_t)P + 1)); ACUDA(aalloc(a, &a->orderCnt, ORD_BUCKETS));
  ACUDA(cudaMemcpyAsync(a->shp, hShp.data(), n * sizeof(double4), cudaMemcpyHostToDevice, a->st));
  ACUDA(cudaMemcpyAsync(a->massI, hMI.data(), n * sizeof(double4), cudaMemcpyHostToDevice, a->st));
  ACUDA(cudaMemcpyAsync(a->eps, hEps.data(), n * sizeof(double2), cudaMemcpyHostToDevice, a->st));
  ACUDA(cudaMemcpyAsync(a->binfo, hInfo.data(), n * sizeof(int4), cudaMemcpyHostToDevice, a->st));
  ACUDA(cudaMemcpyAsync(a->bStart, start.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice, a->st));
  if (P) {
    ACUDA(cudaMemcpyAsync(a->idsD, a->ids.data(), P * sizeof(int2), cudaMemcpyHostToDevice, a->st));
    ACUDA(cudaMemcpyAsync(a->bList, list.data(), 2 * (size_t)P * sizeof(int), cudaMemcpyHostToDevice, a->st));
  }
  // initial state
  std::vector<char> hs(a->L.bytes, 0);
  State hv = a->L.view(hs.data());
  for (int i = 0; i < n; i++) {
    const double* s = state37 + (size_t)i * SQDEM_BODY_STRIDE;
    hv.pos[i] = make_double4(s[0], s[1], s[2], 0);
    hv.ori[i] = make_double4(s[3], s[4], s[5], s[6]);
    hv.vel[i] = make_double4(s[7], s[8], s[9], 0);
    hv.angVel[i] = make_double4(s[10], s[11], s[12], 0);
    hv.angMom[i] = make_double4(s[13], s[14], s[15], 0);
  }
  for (int c = 0; c < P; c++) {
    hv.flag[c] = hFlag[c]; hv.depth[c] = hDepth[c]; hv.angle[c] = hAng[c]; hv.normal[c] = hN[c]; hv.shear[c] = hS[c];
  }
  ACUDA(cudaMemcpyAsync(a->init, hs.data(), a->L.bytes, cudaMemcpyHostToDevice, a->st));
  // default materials: none yet (sqdem_adj_set_materials before a forward run)
  a->Kn.clear(); a->Ks.clear(); a->fa.clear();
  ACUDA(cudaStreamSynchronize(a->st));
  return SQDEM_OK;
}

sqdem_status sqdem_adj_set_materials(sqdem_adj* a, int nmat, const double* Kn, const double* Ks, const double* frictionAngle) {
  if (!a || !Kn || !Ks || !frictionAngle) return SQDEM_ERR_ARG;
  if (nmat < a->nmat) return afail(a, SQDEM_ERR_ARG, "fewer materials than the bodies use");
  for (int m = 0; m < nmat; m++)
    if (!(Kn[m] > 0) || !(Ks[m] > 0) || !std::isfinite(frictionAngle[m]))
      return afail(a, SQDEM_ERR_ARG, "material stiffness must be positive and friction finite");
  ACUDA(cudaSetDevice(a->device));
  a->Kn.assign(Kn, Kn + nmat); a->Ks.assign(Ks, Ks + nmat); a->fa.assign(frictionAngle, frictionAngle + nmat);
  std::vector<double4> ph(a->P);
  for (int c = 0; c < a->P; c++) {
    double kn, ks, t;
    physOf(a, c, kn, ks, t);
    ph[c] = make_double4(kn, ks, t, 0);
  }
  if (a->P) ACUDA(cudaMemcpyAsync(a->phys, ph.data(), a->P * sizeof(double4), cudaMemcpyHostToDevice, a->st));
  ACUDA(cudaStreamSynchronize(a->st));
  a->haveForward = false;
  return SQDEM_OK;
}

sqdem_status sqdem_adj_set_eps(sqdem_adj* a, const double* eps2) {
  if (!a || !eps2) return SQDEM_ERR_ARG;
  for (int i = 0; i < a->nb; i++)
    if (a->kind[i] == SQDEM_SUPERQUADRIC && !(eps2[2 * i] > 0 && eps2[2 * i] < 2 && eps2[2 * i + 1] > 0 && eps2[2 * i + 1] < 2))
      return afail(a, SQDEM_ERR_ARG, "exponents must lie in (0, 2)");
  ACUDA(cudaSetDevice(a->device));
  ACUDA(cudaMemcpyAsync(a->eps, eps2, a->nb * sizeof(double2), cudaMemcpyHostToDevice, a->st));
  ACUDA(cudaStreamSynchronize(a->st));
  a->haveForward = false;
  return SQDEM_OK;
}

sqdem_status sqdem_adj_forward(sqdem_adj* a, int nsteps, int checkpoint_every, const double* wF3, const double* wX3,
                               double* loss, unsigned long long* signature) {
  if (!a || nsteps <= 0 || checkpoint_every <= 0) return SQDEM_ERR_ARG;
  if (!a->init) return afail(a, SQDEM_ERR_STATE, "sqdem_adj_load first");
  if ((int)a->Kn.size() < a->nmat) return afail(a, SQDEM_ERR_STATE, "sqdem_adj_set_materials first");
  ACUDA(cudaSetDevice(a->device));
  const int nseg = (nsteps + checkpoint_every - 1) / checkpoint_every;
  while ((int)a->ckpt.size() < nseg) {
    char* p = nullptr;
    ACUDA(aalloc(a, &p, a->L.bytes));
    a->ckpt.push_back(p);
  }
  sqdem_status s = ensureTape(a, 1);
  if (s != SQDEM_OK) return s;
  if (a->brMode == BR_FORCE && nsteps > a->brSteps)
    return afail(a, SQDEM_ERR_STATE, "forced branches: the recorded run has fewer steps than this one");
  if (a->brMode == BR_RECORD && (size_t)nsteps > a->brCap) {
    afree(a, a->brPair); afree(a, a->brBody);
    a->brPair = nullptr; a->brBody = nullptr; a->brCap = 0; a->brSteps = 0;
    ACUDA(aalloc(a, &a->brPair, (size_t)nsteps * a->P * BR_WORDS + 1));
    ACUDA(aalloc(a, &a->brBody, (size_t)nsteps * a->nb));
    a->brCap = nsteps;
  }
  if (a->brMode == BR_RECORD) a->brSteps = 0;
  std::vector<double4> hw(a->nb);
  for (int i = 0; i < a->nb; i++) hw[i] = wF3 ? make_double4(wF3[3 * i], wF3[3 * i + 1], wF3[3 * i + 2], 0) : make_double4(0, 0, 0, 0);
  ACUDA(cudaMemcpyAsync(a->wF, hw.data(), a->nb * sizeof(double4), cudaMemcpyHostToDevice, a->st));
  for (int i = 0; i < a->nb; i++) hw[i] = wX3 ? make_double4(wX3[3 * i], wX3[3 * i + 1], wX3[3 * i + 2], 0) : make_double4(0, 0, 0, 0);
  ACUDA(cudaMemcpyAsync(a->wX, hw.data(), a->nb * sizeof(double4), cudaMemcpyHostToDevice, a->st));
  ACUDA(cudaMemsetAsync(a->cnt, 0, A_NCOUNT * sizeof(unsigned long long), a->st));
  cudaEvent_t e0, e1;
  ACUDA(cudaEventCreate(&e0)); ACUDA(cudaEventCreate(&e1));
  ACUDA(cudaEventRecord(e0, a->st));
  ACUDA(cudaMemcpyAsync(a->work, a->init, a->L.bytes, cudaMemcpyDeviceToDevice, a->st));
  const State S = a->L.view(a->work);
  const StepOut O = tapeOut(a, 0);
  for (int t = 0; t < nsteps; t++) {
    if (t % checkpoint_every == 0)
      ACUDA(cudaMemcpyAsync(a->ckpt[t / checkpoint_every], a->work, a->L.bytes, cudaMemcpyDeviceToDevice, a->st));
    launchStep(a, S, O, t, true);
  }
  if (a->brMode == BR_RECORD) a->brSteps = nsteps;
  k_loss<<<1, 256, 0, a->st>>>(consts(a), S, O, a->wF, a->wX, a->lossD);
  ACUDA(cudaGetLastError());
  ACUDA(cudaMemcpyAsync(a->fin, a->work, a->L.bytes, cudaMemcpyDeviceToDevice, a->st));
  if (a->P) ACUDA(cudaMemcpyAsync(a->finFv, O.Fv, a->P * sizeof(double4), cudaMemcpyDeviceToDevice, a->st));
  ACUDA(cudaEventRecord(e1, a->st));
  ACUDA(cudaMemcpyAsync(&a->loss, a->lossD, sizeof(double), cudaMemcpyDeviceToHost, a->st));
  ACUDA(cudaMemcpyAsync(a->counters, a->cnt, A_NCOUNT * sizeof(unsigned long long), cudaMemcpyDeviceToHost, a->st));
  ACUDA(cudaStreamSynchronize(a->st));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  a->msForward = ms;
  a->nsteps = nsteps; a->every = checkpoint_every; a->haveForward = true;
  if (loss) *loss = a->loss;
  if (signature) *signature = a->counters[A_SIG];
  if (!std::isfinite(a->loss)) return afail(a, SQDEM_ERR_NUMERIC, "non-finite loss");
  return SQDEM_OK;
}

sqdem_status sqdem_adj_backward(sqdem_adj* a, double* dL_deps, double* dL_dKn, double* dL_dKs, double* dL_dmu) {
  if (!a) return SQDEM_ERR_ARG;
  if (!a->haveForward) return afail(a, SQDEM_ERR_STATE, "sqdem_adj_forward first (with the current parameters)");
  ACUDA(cudaSetDevice(a->device));
  const int K = a->every, nsteps = a->nsteps, n = a->nb, P = a->P;
  sqdem_status s = ensureTape(a, std::min(K, nsteps));
  if (s != SQDEM_OK) return s;
  cudaEvent_t e0, e1;
  ACUDA(cudaEventCreate(&e0)); ACUDA(cudaEventCreate(&e1));
  ACUDA(cudaEventRecord(e0, a->st));
  // adjoint of the final state: wX on positions, nothing else
  ACUDA(cudaMemcpyAsync(a->lPos, a->wX, n * sizeof(double4), cudaMemcpyDeviceToDevice, a->st));
  ACUDA(cudaMemsetAsync(a->lOri, 0, n * sizeof(double4), a->st)); ACUDA(cudaMemsetAsync(a->lVel, 0, n * sizeof(double4), a->st));
  ACUDA(cudaMemsetAsync(a->lW, 0, n * sizeof(double4), a->st)); ACUDA(cudaMemsetAsync(a->lL, 0, n * sizeof(double4), a->st));
  if (P) {
    ACUDA(cudaMemsetAsync(a->lAng, 0, P * sizeof(double2), a->st)); ACUDA(cudaMemsetAsync(a->lN, 0, P * sizeof(double4), a->st));
    ACUDA(cudaMemsetAsync(a->lS, 0, P * sizeof(double4), a->st));
    ACUDA(cudaMemsetAsync(a->accEps, 0, P * sizeof(double4), a->st)); ACUDA(cudaMemsetAsync(a->accPhys, 0, P * sizeof(double4), a->st));
  }
  const Consts C = consts(a);
  const Adj A = adjView(a);
  const int nseg = (nsteps + K - 1) / K;
  for (int seg = nseg - 1; seg >= 0; seg--) {
    const int t0 = seg * K, t1 = std::min(t0 + K, nsteps);
    ACUDA(cudaMemcpyAsync(a->work, a->ckpt[seg], a->L.bytes, cudaMemcpyDeviceToDevice, a->st));
    const State W = a->L.view(a->work);
    for (int t = t0; t < t1; t++) {
      ACUDA(cudaMemcpyAsync(a->tapeState[t - t0], a->work, a->L.bytes, cudaMemcpyDeviceToDevice, a->st));
      launchStep(a, W, tapeOut(a, t - t0), t);
    }
    for (int t = t1 - 1; t >= t0; t--) {
      const State S = a->L.view(a->tapeState[t - t0]);
      const StepOut O = tapeOut(a, t - t0);
      k_bwd_integrate<<<nblk(n, 128), 128, 0, a->st>>>(C, S, O, A, t == nsteps - 1 ? 1 : 0);
      if (P) launchReplay(a, C, S, O, A);
      k_bwd_gather<<<nblk(n, 128), 128, 0, a->st>>>(C, A);
    }
    ACUDA(cudaGetLastError());
  }
  ACUDA(cudaEventRecord(e1, a->st));
  std::vector<double4> ae(P), ap(P);
  if (P) {
    ACUDA(cudaMemcpyAsync(ae.data(), a->accEps, P * sizeof(double4), cudaMemcpyDeviceToHost, a->st));
    ACUDA(cudaMemcpyAsync(ap.data(), a->accPhys, P * sizeof(double4), cudaMemcpyDeviceToHost, a->st));
  }
  unsigned long long cnt[A_NCOUNT];
  ACUDA(cudaMemcpyAsync(cnt, a->cnt, A_NCOUNT * sizeof(unsigned long long), cudaMemcpyDeviceToHost, a->st));
  ACUDA(cudaStreamSynchronize(a->st));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  a->msBackward = ms;
  a->counters[A_MISMATCH] = cnt[A_MISMATCH];
  a->counters[A_REPLAYED] = cnt[A_REPLAYED];
  // map the per-pair parameter adjoints to bodies and materials (Ip2's formulas)
  std::vector<double> gE(2 * (size_t)n, 0.0), gKn(a->nmat, 0.0), gKs(a->nmat, 0.0), gMu(a->nmat, 0.0);
  for (int c = 0; c < P; c++) {
    const int id1 = a->ids[c].x, id2 = a->ids[c].y;
    if (a->kind[id1] == SQDEM_SUPERQUADRIC) { gE[2 * id1] += ae[c].x; gE[2 * id1 + 1] += ae[c].y; }
    gE[2 * id2] += ae[c].z; gE[2 * id2 + 1] += ae[c].w;
    const int m1 = a->mat[id1], m2 = a->mat[id2];
    if (id1 > 5) {
      const double s1 = a->Kn[m1] + a->Kn[m2], t1 = a->Ks[m1] + a->Ks[m2];
      gKn[m1] += ap[c].x * 2.0 * a->Kn[m2] * a->Kn[m2] / (s1 * s1);
      gKn[m2] += ap[c].x * 2.0 * a->Kn[m1] * a->Kn[m1] / (s1 * s1);
      gKs[m1] += ap[c].y * 2.0 * a->Ks[m2] * a->Ks[m2] / (t1 * t1);
      gKs[m2] += ap[c].y * 2.0 * a->Ks[m1] * a->Ks[m1] / (t1 * t1);
      gMu[(a->fa[m2] < a->fa[m1]) ? m2 : m1] += ap[c].z;   // tan(atan(mu)) = mu
    } else {
      gKn[m1] += ap[c].x; gKs[m1] += ap[c].y; gMu[m1] += ap[c].z;
    }
  }
  if (dL_deps) std::copy(gE.begin(), gE.end(), dL_deps);
  if (dL_dKn) std::copy(gKn.begin(), gKn.end(), dL_dKn);
  if (dL_dKs) std::copy(gKs.begin(), gKs.end(), dL_dKs);
  if (dL_dmu) std::copy(gMu.begin(), gMu.end(), dL_dmu);
  if (cnt[A_MISMATCH]) return afail(a, SQDEM_ERR_NUMERIC, "replay took a branch the forward run did not take");
  return SQDEM_OK;
}

sqdem_status sqdem_adj_get_state(sqdem_adj* a, double* out16) {
  if (!a || !out16) return SQDEM_ERR_ARG;
  if (!a->haveForward) return afail(a, SQDEM_ERR_STATE, "no forward run");
  ACUDA(cudaSetDevice(a->device));
  std::vector<char> hs(a->L.bytes);
  ACUDA(cudaMemcpyAsync(hs.data(), a->fin, a->L.bytes, cudaMemcpyDeviceToHost, a->st));
  ACUDA(cudaStreamSynchronize(a->st));
  const State v = a->L.view(hs.data());
  for (int i = 0; i < a->nb; i++) {
    double* o = out16 + (size_t)i * 16;
    const double4 p = v.pos[i], q = v.ori[i], ve = v.vel[i], w = v.angVel[i], L = v.angMom[i];
    o[0] = p.x; o[1] = p.y; o[2] = p.z; o[3] = q.x; o[4] = q.y; o[5] = q.z; o[6] = q.w;
    o[7] = ve.x; o[8] = ve.y; o[9] = ve.z; o[10] = w.x; o[11] = w.y; o[12] = w.z; o[13] = L.x; o[14] = L.y; o[15] = L.z;
  }
  return SQDEM_OK;
}

long sqdem_adj_num_pairs(sqdem_adj* a) { return a ? a->P : 0; }

sqdem_status sqdem_adj_set_forward(sqdem_adj* a, int cooperative) {
  if (!a) return SQDEM_ERR_ARG;
  a->coopForward = cooperative != 0;
  a->haveForward = false;
  return SQDEM_OK;
}

sqdem_status sqdem_adj_set_replay(sqdem_adj* a, int shape) {
  if (!a || shape < 0 || shape > 3) return SQDEM_ERR_ARG;
  a->replay = shape;
  return SQDEM_OK;
}

sqdem_status sqdem_adj_set_replay_blocks(sqdem_adj* a, int blocks_per_sm) {
  if (!a || blocks_per_sm < 0) return SQDEM_ERR_ARG;
  a->replayBlocks = blocks_per_sm;
  return SQDEM_OK;
}

// per pair after the forward window: id1 id2 hasGeom depth angle2 normal3 shearForce3 | force on id1 (3) of the
// last step, applied (1/0)  -> 16 doubles
sqdem_status sqdem_adj_get_pairs(sqdem_adj* a, double* out16) {
  if (!a || !out16) return SQDEM_ERR_ARG;
  if (!a->haveForward) return afail(a, SQDEM_ERR_STATE, "no forward run");
  ACUDA(cudaSetDevice(a->device));
  std::vector<char> hs(a->L.bytes);
  std::vector<double4> fv(a->P);
  ACUDA(cudaMemcpyAsync(hs.data(), a->fin, a->L.bytes, cudaMemcpyDeviceToHost, a->st));
  if (a->P) ACUDA(cudaMemcpyAsync(fv.data(), a->finFv, a->P * sizeof(double4), cudaMemcpyDeviceToHost, a->st));
  ACUDA(cudaStreamSynchronize(a->st));
  const State v = a->L.view(hs.data());
  for (int c = 0; c < a->P; c++) {
    double* o = out16 + (size_t)c * 16;
    o[0] = a->ids[c].x; o[1] = a->ids[c].y; o[2] = (v.flag[c] & CF_GEOM) ? 1 : 0; o[3] = v.depth[c];
    o[4] = v.angle[c].x; o[5] = v.angle[c].y;
    o[6] = v.normal[c].x; o[7] = v.normal[c].y; o[8] = v.normal[c].z;
    o[9] = v.shear[c].x; o[10] = v.shear[c].y; o[11] = v.shear[c].z;
    o[12] = fv[c].x; o[13] = fv[c].y; o[14] = fv[c].z; o[15] = fv[c].w;
  }
  return SQDEM_OK;
}

// counters of the last runs: replay mismatches, Disfunction evaluations (forward), LM calls
// (forward), pairs replayed (backward), forward ms, backward ms, steps, checkpoint interval
sqdem_status sqdem_adj_set_branches(sqdem_adj* a, int mode) {
  if (!a || mode < BR_OFF || mode > BR_FORCE) return SQDEM_ERR_ARG;
  if (mode == BR_FORCE && a->brSteps == 0) return afail(a, SQDEM_ERR_STATE, "forced branches: no recorded run");
  a->brMode = mode;
  return SQDEM_OK;
}

sqdem_status sqdem_adj_branch_report(sqdem_adj* a, double* out5) {
  if (!a || !out5) return SQDEM_ERR_ARG;
  out5[0] = (double)a->counters[A_BRDEC]; out5[1] = (double)a->counters[A_BRDIS];
  out5[2] = (double)a->counters[A_BRUNF]; out5[3] = (double)a->brSteps;
  out5[4] = (double)a->counters[A_BRCUSP];
  return SQDEM_OK;
}

sqdem_status sqdem_adj_report(sqdem_adj* a, double* out8) {
  if (!a || !out8) return SQDEM_ERR_ARG;
  out8[0] = (double)a->counters[A_MISMATCH]; out8[1] = (double)a->counters[A_EVALS];
  out8[2] = (double)a->counters[A_LMCALLS]; out8[3] = (double)a->counters[A_REPLAYED];
  out8[4] = a->msForward; out8[5] = a->msBackward; out8[6] = a->nsteps; out8[7] = a->every;
  return SQDEM_OK;
}

}  // extern "C"
