// SudoDEM3D superellipsoid per-timestep path — CPU ORACLE (test infrastructure only).
//
// This file is a C++17/FP64 restatement of the reference's hot path, written to
// check the GPU engine.  It is never shipped or called by the product path: only
// tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm load
// it.  Each function cites the reference file:line it follows (paths are relative
// to the SudoDEM repository root).
//
// Parity status: the reference itself cannot be compiled here (Boost.Python and a
// prebuilt third-party tree are required by SudoDEM3D/lib/base/Math.hpp:10,57-72 and
// SudoDEM3D/CMakeLists.txt:6,73), and the reference ships no test, golden vector or
// fixture for this path.  Parity of this restatement against the reference is
// therefore UNPINNED; it is anchored on (a) operation-for-operation restatement of
// the cited lines, (b) Eigen 3.3.5's evaluation order (vendored in
// SudoDEM3D/lib/Eigen: unrolled tree reductions, Core/Redux.h:91-122; coefficient
// products, Core/ProductEvaluators.h:550-553; Quaternion.h:475-485,536-568), and
// (c) known-answer tests built with the reference's own PositionPB construction
// (py/_superquadrics_utils.cpp:109-131).
//
// Build: -O2 -ffp-contract=off (the reference builds with -O2 and no FMA on x86-64,
// SudoDEM3D/CMakeLists.txt:64); -fopenmp for the multi-threaded baseline.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cfloat>
#include <vector>
#include <unordered_map>
#include <algorithm>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace sqo {

typedef double Real;
static const Real NaN = std::numeric_limits<Real>::quiet_NaN();
static const Real Inf = std::numeric_limits<Real>::infinity();

// ---------------------------------------------------------------------------
// Small linear algebra with Eigen 3.3.5 evaluation order.
// Reductions of length 3 unroll as a0 + (a1 + a2), length 4 as (a0+a1)+(a2+a3)
// (lib/Eigen/src/Core/Redux.h:91-105).
struct V3 {
  Real v[3];
  V3() { v[0] = v[1] = v[2] = 0; }
  V3(Real a, Real b, Real c) { v[0] = a; v[1] = b; v[2] = c; }
  Real& operator[](int i) { return v[i]; }
  Real operator[](int i) const { return v[i]; }
};
static inline V3 operator+(const V3& a, const V3& b) { return V3(a[0] + b[0], a[1] + b[1], a[2] + b[2]); }
static inline V3 operator-(const V3& a, const V3& b) { return V3(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
static inline V3 operator-(const V3& a) { return V3(-a[0], -a[1], -a[2]); }
static inline V3 operator*(Real s, const V3& a) { return V3(s * a[0], s * a[1], s * a[2]); }
static inline V3 operator*(const V3& a, Real s) { return V3(a[0] * s, a[1] * s, a[2] * s); }
static inline Real dot(const V3& a, const V3& b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }
static inline Real sqnorm(const V3& a) { return a[0] * a[0] + (a[1] * a[1] + a[2] * a[2]); }
static inline Real norm(const V3& a) { return std::sqrt(sqnorm(a)); }
// Geometry/OrthoMethods.h:34-48
static inline V3 cross(const V3& a, const V3& b) {
  return V3(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}
// Core/Dot.h:145-151 (normalize divides by sqrt of the squared norm when positive)
static inline void normalize(V3& a) {
  Real z = sqnorm(a);
  if (z > 0) { Real n = std::sqrt(z); a[0] /= n; a[1] /= n; a[2] /= n; }
}
struct M3 { Real m[9]; };
// Coefficient-based 3x3*3 product: row(i).col.sum() with the tree reduction.
static inline V3 mul(const M3& M, const V3& x) {
  return V3(M.m[0] * x[0] + (M.m[1] * x[1] + M.m[2] * x[2]),
            M.m[3] * x[0] + (M.m[4] * x[1] + M.m[5] * x[2]),
            M.m[6] * x[0] + (M.m[7] * x[1] + M.m[8] * x[2]));
}
// determinant by cofactor expansion along the first row
static inline Real det(const M3& A) {
  return A.m[0] * (A.m[4] * A.m[8] - A.m[5] * A.m[7]) - A.m[1] * (A.m[3] * A.m[8] - A.m[5] * A.m[6]) +
         A.m[2] * (A.m[3] * A.m[7] - A.m[4] * A.m[6]);
}
static inline M3 mmul(const M3& A, const M3& B) {
  M3 r;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      r.m[3 * i + j] = A.m[3 * i + 0] * B.m[0 + j] + (A.m[3 * i + 1] * B.m[3 + j] + A.m[3 * i + 2] * B.m[6 + j]);
  return r;
}
static inline bool m3zero(const M3& A) { for (int k = 0; k < 9; k++) if (A.m[k] != 0) return false; return true; }
struct Quat { Real w, x, y, z; };
// Geometry/Quaternion.h:536-568
static inline M3 toRot(const Quat& q) {
  const Real tx = 2.0 * q.x, ty = 2.0 * q.y, tz = 2.0 * q.z;
  const Real twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
  const Real txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
  const Real tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
  M3 r;
  r.m[0] = 1.0 - (tyy + tzz); r.m[1] = txy - twz;         r.m[2] = txz + twy;
  r.m[3] = txy + twz;         r.m[4] = 1.0 - (txx + tzz); r.m[5] = tyz - twx;
  r.m[6] = txz - twy;         r.m[7] = tyz + twx;         r.m[8] = 1.0 - (txx + tyy);
  return r;
}
static inline Quat conj(const Quat& q) { return Quat{q.w, -q.x, -q.y, -q.z}; }
// Quaternion coefficients are stored (x,y,z,w); squaredNorm = (x²+y²)+(z²+w²).
static inline void qnormalize(Quat& q) {
  Real z = (q.x * q.x + q.y * q.y) + (q.z * q.z + q.w * q.w);
  if (z > 0) { Real n = std::sqrt(z); q.x /= n; q.y /= n; q.z /= n; q.w /= n; }
}
// Geometry/Quaternion.h:475-485 (_transformVector)
static inline V3 qrotate(const Quat& q, const V3& v) {
  V3 qv(q.x, q.y, q.z);
  V3 uv = cross(qv, v);
  uv = uv + uv;
  V3 c = cross(qv, uv);
  return V3((v[0] + q.w * uv[0]) + c[0], (v[1] + q.w * uv[1]) + c[1], (v[2] + q.w * uv[2]) + c[2]);
}

// lib/base/Math.hpp:186 (Sign(0) == 0)
static inline Real Sign(Real f) { if (f < 0) return -1; if (f > 0) return 1; return 0; }

// lib/base/Math.hpp:192-212: Lanczos log-gamma (Numerical Recipes 3rd ed., Sect. 6.1)
// and Beta(z,w) = exp(lnG(z)+lnG(w)-lnG(z+w)).  The 14 coefficients are the published
// NR3 table, which the reference uses as-is; mass and inertia depend on them.
static double gammln(const double xx) {
  static const double cof[14] = {57.1562356658629235, -59.5979603554754912, 14.1360979747417471,
                                 -0.491913816097620199, .339946499848118887e-4, .465236289270485756e-4,
                                 -.983744753048795646e-4, .158088703224912494e-3, -.210264441724104883e-3,
                                 .217439618115212643e-3, -.164318106536763890e-3, .844182239838527433e-4,
                                 -.261908384015814087e-4, .368991826595316234e-5};
  double x, tmp, y, ser;
  y = x = xx;
  tmp = x + 5.24218750000000000;
  tmp = (x + 0.5) * std::log(tmp) - tmp;
  ser = 0.999999999999997092;
  for (int j = 0; j < 14; j++) ser += cof[j] / ++y;
  return tmp + std::log(2.5066282746310005 * ser / x);
}
static double betaf(const double z, const double w) { return std::exp(gammln(z) + gammln(w) - gammln(z + w)); }

// ---------------------------------------------------------------------------
// Superquadric shape (pkg/dem/Superquadrics.hpp:48-166, Superquadrics.cpp:29-120,269-307)
struct SQ {
  Real rx, ry, rz, eps1, eps2, r_max;
  bool isSphere;
  Real volume;
  V3 inertia;   // geometric (unit density)
  M3 loc, glob; // rot_mat2local / rot_mat2global cached on the shape
};

// Superquadrics.cpp:47-93 (Initial)
static void sqInitial(SQ& s) {
  s.r_max = (s.rx > s.ry) ? s.rx : s.ry;
  s.r_max = s.r_max > s.rz ? s.r_max : s.rz;
  if ((s.eps1 < 1.0) || (s.eps2 < 1.0)) s.r_max *= std::pow(2.0, 0.5);
  double a = s.rx * s.ry * s.rz * s.eps1 * s.eps2;
  double beta1 = betaf(1.5 * s.eps1, 0.5 * s.eps1) * betaf(0.5 * s.eps2, 2. * s.eps2 + 1);
  double beta2 = betaf(0.5 * s.eps1, 0.5 * s.eps1 + 1) * betaf(1.5 * s.eps2, s.eps2 + 1);
  s.volume = 2. * a * betaf(s.eps1 * 0.5, s.eps1 * 0.5) * betaf(s.eps2 * 0.5 + 1, s.eps2);
  s.inertia[0] = 0.5 * a * (std::pow(s.ry, 2.) * beta1 + 4. * std::pow(s.rz, 2.) * beta2);
  s.inertia[1] = 0.5 * a * (std::pow(s.rx, 2.) * beta1 + 4. * std::pow(s.rz, 2.) * beta2);
  s.inertia[2] = 0.5 * a * (std::pow(s.rx, 2.) + std::pow(s.ry, 2.)) * beta1;
}

// Last-bit noise on the transcendental calls of the narrowphase (a test instrument; off unless a
// seed is set).  With seed != 0 every pow/sin/cos/atan2 result of the Disfunction and of the
// Nelder-Mead geometry moves by -1, 0 or +1 unit, chosen by a hash of the value and the seed: one
// ulp when rel == 0, else rel * |value|.  This models another libm whose results differ from
// glibc's in the last bits (CUDA's do).  How far a pair's result moves over a few seeds is the
// reference's own conditioning at FP64: the part of its answer that its inputs and its
// arithmetic do not determine.
static uint64_t g_noiseSeed = 0;
static double g_noiseRel = 0;
static inline double NZ(double v) {
  if (!g_noiseSeed || !(v != 0) || !std::isfinite(v)) return v;
  uint64_t h;
  std::memcpy(&h, &v, 8);
  h ^= g_noiseSeed;
  h += 0x9e3779b97f4a7c15ULL;
  h = (h ^ (h >> 30)) * 0xbf58476d1ce4e5b9ULL;
  h = (h ^ (h >> 27)) * 0x94d049bb133111ebULL;
  h ^= h >> 31;
  const int s = (int)(h % 3) - 1;
  if (!s) return v;
  if (g_noiseRel > 0) return v + s * std::fabs(v) * g_noiseRel;
  return std::nextafter(v, s > 0 ? Inf : -Inf);
}
#define NPOW(a, b) NZ(std::pow(a, b))
#define NSIN(a) NZ(std::sin(a))
#define NCOS(a) NZ(std::cos(a))
#define NATAN2(a, b) NZ(std::atan2(a, b))

// Superquadrics.cpp:103-108
static bool sqIsInside(const SQ& s, V3 p) {
  p = mul(s.loc, p);
  return 1 > NPOW(NPOW(std::fabs(p[0] / s.rx), 2.0 / s.eps1) + NPOW(std::fabs(p[1] / s.ry), 2.0 / s.eps1),
                      s.eps1 / s.eps2) + NPOW(std::fabs(p[2] / s.rz), 2.0 / s.eps2);
}
// Superquadrics.cpp:110-120 (local surface point from the two surface angles)
static inline V3 sqSurface(const SQ& s, Real ph0, Real ph1) {
  V3 r;
  r[0] = Sign(NCOS(ph0)) * s.rx * NPOW(std::fabs(NCOS(ph0)), s.eps1) * NPOW(std::fabs(NCOS(ph1)), s.eps2);
  r[1] = Sign(NSIN(ph0)) * s.ry * NPOW(std::fabs(NSIN(ph0)), s.eps1) * NPOW(std::fabs(NCOS(ph1)), s.eps2);
  r[2] = Sign(NSIN(ph1)) * s.rz * NPOW(std::fabs(NSIN(ph1)), s.eps2);
  return r;
}
// Margins of the decisions one pair's narrowphase and law took this step (minimum over every
// evaluation / check of the pair):
//  [0] |c.(p2-p1)| (m) of every Disfunction evaluation (stop_flag: c.d > 0)
//  [1] ||cos| - 0.95| of every angle check (lmder2 stop 8)
//  [2] |‖Dp‖ - 1e-5| / 1e-5 of every damped step (lmder2 stop 2)
//  [3] |dF| (m) of every trial (accepted iff dF/dL > 0)
//  [4] |‖J^T f‖inf - 1e-15| / 1e-15 (lmder2 stop 1)
//  [5] |10 ‖p2-p1‖ - r_max| / r_max and [6] |isInside value - 1| of the restart rule
//  [7] |PenetrationDepth - 1e-18| (m) at the law's contact gate
//  [8] smallest |cos| of a surface angle next to an odd multiple of pi/2, or |sin| next to pi,
//      in any evaluation (FP64 rounds the angle to ~1e-16 there: the support point's own
//      rounding error grows as that value shrinks)
//  [9] number of Disfunction evaluations
static thread_local double* g_marg = nullptr;
static inline void margMin(int k, double v) {
  if (g_marg) { v = std::fabs(v); if (!(v >= g_marg[k])) g_marg[k] = v; }
}

// Superquadrics.cpp:269-307 (surface angles of the point whose outward normal is n, local frame)
static inline void sqNormal2Phi(const SQ& s, const V3& n, Real& ph0, Real& ph1) {
  ph0 = NATAN2(Sign(n[1]) * NPOW(std::fabs(s.ry * n[1]), 1 / (2. - s.eps1)),
                   Sign(n[0]) * NPOW(std::fabs(s.rx * n[0]), 1 / (2. - s.eps1)));
  ph1 = NATAN2(Sign(n[2]) * NPOW(std::fabs(s.rz * n[2] * NPOW(std::fabs(NCOS(ph0)), 2. - s.eps1)), 1 / (2. - s.eps2)),
                   NPOW(std::fabs(s.rx * n[0]), 1 / (2. - s.eps2)));
  if (g_marg) {
    margMin(8, std::cos(ph0)); margMin(8, std::cos(ph1));
    if (std::fabs(ph0) > 1.5707963267948966) margMin(8, std::sin(ph0));
  }
}
// Superquadrics.cpp:258-266 (local, unnormalised outward normal at angles phi)
static inline V3 sqNormal(const SQ& s, Real ph0, Real ph1) {
  V3 n;
  n[0] = Sign(NCOS(ph0)) / s.rx * NPOW(std::fabs(NCOS(ph0)), 2. - s.eps1) * NPOW(std::fabs(NCOS(ph1)), 2. - s.eps2);
  n[1] = Sign(NSIN(ph0)) / s.ry * NPOW(std::fabs(NSIN(ph0)), 2. - s.eps1) * NPOW(std::fabs(NCOS(ph1)), 2. - s.eps2);
  n[2] = Sign(NSIN(ph1)) / s.rz * NPOW(std::fabs(NSIN(ph1)), 2. - s.eps2);
  return n;
}

// ---------------------------------------------------------------------------
// Scene data
enum { KIND_SQ = 0, KIND_WALL = 1 };
static const unsigned DOF_ALL = 63u;

struct Mat { Real Kn, Ks, frictionAngle, betan, betas, density; Real G = 29e9, nu = 0.15; };   // G, nu: SuperquadricsMat2 (Superquadrics.hpp:266-277)

struct Body {
  int kind;
  int axis, sense;    // Wall (pkg/common/Wall.hpp:11-13)
  SQ sq;
  int mat;
  V3 pos; Quat ori; V3 vel, angVel, angMom; Real mass; V3 inertia;
  unsigned blockedDOFs; bool isDamped; bool aspherical;
  int groupMask;
  // Bound (core/Bound.hpp:24-31)
  bool hasBound; V3 bmin, bmax, refPos; Real sweepLength; long lastUpdateIter;
};

// SuperquadricsGeom (Superquadrics.hpp:175-208)
struct Geom {
  Real PenetrationDepth; Real contactAngle[2];
  V3 contactPoint, shearInc, relativeVn, relativeVs, normal, twist_axis, orthonormal_axis, point1, point2;
  bool isShearNew;
  // SuperquadricsGeom2 (Superquadrics.hpp:211-233), Hertz-Mindlin contact model
  Real curvatures1[2], curvatures2[2], curvatureAngle, alpha, K, E, curvatures_sum;
  bool isSphere;
};
// SuperquadricsPhys : FrictPhys (Superquadrics.hpp:303-321, FrictPhys.hpp:15-25)
struct Phys { Real kn, ks, tanphi, betan, betas; V3 normalForce, shearForce; };

struct Interaction {
  int id1, id2;
  bool hasGeom, hasPhys;
  bool geomFunctorSet;  // functorCache.geom (core/Interaction.hpp:35-43)
  bool geomExists;      // functorCache.geomExists
  Geom g; Phys p;
  long iterBorn; long linIx; int cellDist[3];
  bool sliding;         // the law capped the shear force at this step (Coulomb branch)
  // Distance of this step's decisions from their thresholds (test instrumentation: lets a
  // parity test tell contacts at a branch boundary, or evaluated where FP64 itself is
  // ill-conditioned, from the rest).  Filled by the narrowphase and the law; see Margins.
  double marg[10];
};


// InsertionSortCollider::Bounds (InsertionSortCollider.hpp:90-109)
struct Bounds {
  Real coord; int id; int period; bool hasBB; bool isMin;
  bool operator<(const Bounds& b) const { if (id == b.id && coord == b.coord) return isMin; return coord < b.coord; }
  bool operator>(const Bounds& b) const { if (id == b.id && coord == b.coord) return !isMin; return coord > b.coord; }
};

struct Stats { long lmCalls, lmIters, disCalls, restarts, nanNormals; long hist[16]; long nanForces; unsigned long long sig; };


struct Scene {
  std::vector<Body> bodies;
  std::vector<Mat> mats;
  std::vector<Interaction*> lin;                          // InteractionContainer::linIntrs
  std::unordered_map<uint64_t, Interaction*> byKey;       // Body::intrs maps
  Real dt = 1e-5; long iter = 0; Real time = 0;
  // NewtonIntegrator attributes (NewtonIntegrator.hpp:70-89)
  V3 gravity; Real damping = 0.2; int isSuperquadrics = 1; bool exactAsphericalRot = true;
  Real maxVelocitySq = NaN;
  // InsertionSortCollider attributes (InsertionSortCollider.hpp:212-222)
  Real verletDist = -0.5; int targetInterv = 50; Real minSweepDistFactor = 0.1; int sortAxis = 0;
  Real updatingDispFactor = -1; Real fastestBodyMaxDist = -1; int numReinit = 0; bool doSort = false;
  bool strideActive = false; bool newtonFound = false; bool interactionsDirty = false;
  std::vector<Bounds> BB[3];
  std::vector<Real> minima, maxima;
  long colliderRuns = 0; bool lastStepCollided = false;
  // forces (core/ForceContainer.hpp:44-162)
  int nThreads = 1;
  std::vector<std::vector<V3>> fbuf, tbuf;
  std::vector<V3> force, torque;
  Stats stats{};
  std::vector<Stats> tstats;
  // periodic cell (core/Cell.hpp, Cell.cpp:6-26)
  bool isPeriodic = false, colliderPeriodic = false, homoDeform = true, velGradChanged = false;
  M3 hSize{{1, 0, 0, 0, 1, 0, 0, 0, 1}}, trsf{{1, 0, 0, 0, 1, 0, 0, 0, 1}};
  M3 velGrad{{0, 0, 0, 0, 0, 0, 0, 0, 0}}, nextVelGrad{{0, 0, 0, 0, 0, 0, 0, 0, 0}};
  M3 prevVelGrad{{0, 0, 0, 0, 0, 0, 0, 0, 0}};   // NewtonIntegrator::prevVelGrad
  V3 cellSize = V3(1, 1, 1), prevCellSize = V3(NaN, NaN, NaN);
  long loIdx[3] = {0, 0, 0};
  // user hook between InteractionLoop and NewtonIntegrator (boundary controllers)
  void (*midHook)(void*) = nullptr; void* midHookArg = nullptr;
  // NewtonIntegrator::quiet_system_flag (NewtonIntegrator.hpp:73, .cpp:246-250,299)
  bool quietSystem = false;
  // Window with a frozen pair set (the adjoint's forward map): the collider does not run and
  // the law's bound-separation erase is skipped.  sig sums a hash of every branch taken
  // (contact state, force, Coulomb cap, Disfunction evaluations per pair; damping signs per body).
  bool frozenPairs = false;
  // Test-fixture option, off by default (the reference's behaviour): in a periodic cell, the
  // reference applies the torque of a contact across the boundary to body 2 at its unshifted
  // position (Superquadrics.cpp:1356, FIXME at :1550) and leaves the image's field velocity
  // velGrad*shift2 out of the relative velocity (:1042-1045); both make such contacts spin
  // particles up.  periodicFix applies both with shift2, so that a periodic packing generated by
  // the oracle has sound dynamics.
  bool periodicFix = false;
  unsigned long long sig = 0;
  // CompressionEngine (pkg/dem/Compression.hpp:39-252), run between InteractionLoop and Newton
  struct Servo* servo = nullptr;
  long stopAtIter = -1;   // Scene::stopAtIter as the engine requests it
  // contact model: 0 SuperquadricsGeom + SuperquadricsPhys + SuperquadricsLaw, 1 the Hertz-Mindlin
  // set Ig2_*_SuperquadricsGeom2 + Ip2_SuperquadricsMat2_SuperquadricsMat2_HertzMindlinPhys +
  // SuperquadricsLaw2
  int contactModel = 0;
};

static inline uint64_t pairKey(int a, int b) {
  if (a > b) std::swap(a, b);
  return (uint64_t(uint32_t(a)) << 32) | uint32_t(b);
}
static inline int threadNum() {
#ifdef _OPENMP
  return omp_get_thread_num();
#else
  return 0;
#endif
}

// InteractionContainer::insert (core/InteractionContainer.cpp:13-39)
static bool icInsert(Scene& S, int id1, int id2) {
  uint64_t k = pairKey(id1, id2);
  if (S.byKey.count(k)) return false;
  Interaction* I = new Interaction();
  std::memset(I, 0, sizeof(Interaction));
  I->id1 = id1; I->id2 = id2; I->geomExists = true;
  I->iterBorn = S.iter;
  I->linIx = (long)S.lin.size();
  S.lin.push_back(I);
  S.byKey[k] = I;
  return true;
}
// InteractionContainer::erase (core/InteractionContainer.cpp:54-93): move the last one into the hole
static void icEraseAt(Scene& S, long linIx) {
  Interaction* I = S.lin[linIx];
  S.byKey.erase(pairKey(I->id1, I->id2));
  long last = (long)S.lin.size() - 1;
  if (linIx < last) { S.lin[linIx] = S.lin[last]; S.lin[linIx]->linIx = linIx; }
  S.lin.pop_back();
  delete I;
}
// Interaction::reset (core/Interaction.cpp:19-29)
static inline void requestErase(Interaction* I) { I->hasGeom = false; I->hasPhys = false; I->geomExists = true; }

// Collider::mayCollide (pkg/common/Collider.cpp:14-27) for standalone bodies with
// avoidSelfInteractionMask == 0.
static inline bool mayCollide(const Body& a, const Body& b) { return (a.groupMask & b.groupMask) != 0; }

// ---------------------------------------------------------------------------
// Cell::integrateAndUpdate (core/Cell.cpp:6-26), the parts the hot path reads
static void cellIntegrate(Scene& S) {
  M3 inc;
  for (int k = 0; k < 9; k++) inc.m[k] = S.dt * S.velGrad.m[k];
  M3 t = mmul(inc, S.trsf);
  for (int k = 0; k < 9; k++) S.trsf.m[k] += t.m[k];
  M3 h = mmul(inc, S.hSize);
  for (int k = 0; k < 9; k++) S.hSize.m[k] += h.m[k];
  for (int i = 0; i < 3; i++) {
    V3 base(S.hSize.m[0 + i], S.hSize.m[3 + i], S.hSize.m[6 + i]);
    S.cellSize[i] = norm(base);
  }
}
static inline V3 cellShift(const Scene& S, const int cd[3]) {
  return mul(S.hSize, V3((Real)cd[0], (Real)cd[1], (Real)cd[2]));
}
// InsertionSortCollider::cellWrap / cellWrapRel (InsertionSortCollider.cpp:404-414)
static inline Real cellWrap(const Real x, const Real x0, const Real x1, int& period) {
  Real xNorm = (x - x0) / (x1 - x0);
  period = (int)std::floor(xNorm);
  return x0 + (xNorm - period) * (x1 - x0);
}
static inline Real cellWrapRel(const Real x, const Real x0, const Real x1) {
  Real xNorm = (x - x0) / (x1 - x0);
  return (xNorm - std::floor(xNorm)) * (x1 - x0);
}

// ---------------------------------------------------------------------------
// BoundDispatcher::processBody (pkg/common/Dispatching.cpp:30-62) with
// Bo1_Superquadrics_Aabb::go (Superquadrics.cpp:639-686) and Bo1_Wall_Aabb::go (Wall.cpp:13-21)
static void processBody(Scene& S, Body& b, Real sweepDist) {
  if (b.hasBound) {
    Real& sweepLength = b.sweepLength;
    if (S.targetInterv >= 0) {
      V3 disp = b.pos - b.refPos;
      Real dist = std::max(std::abs(disp[0]), std::max(std::abs(disp[1]), std::abs(disp[2])));
      if (dist) {
        Real newLength = dist * S.targetInterv / (S.iter - b.lastUpdateIter);
        newLength = std::max(0.9 * sweepLength, newLength);
        sweepLength = std::max(S.minSweepDistFactor * sweepDist, std::min(newLength, sweepDist));
      } else sweepLength = 0;
    } else sweepLength = sweepDist;
  }
  if (b.kind == KIND_SQ) {
    Real r = b.sq.r_max;
    b.bmin = b.pos + V3(-r, -r, -r);
    b.bmax = b.pos + V3(r, r, r);
  } else {
    b.bmin = V3(-Inf, -Inf, -Inf); b.bmin[b.axis] = b.pos[b.axis];
    b.bmax = V3(Inf, Inf, Inf);    b.bmax[b.axis] = b.pos[b.axis];
  }
  if (!b.hasBound) { b.hasBound = true; b.sweepLength = 0; }
  b.refPos = b.pos;
  b.lastUpdateIter = S.iter;
  const Real sl = b.sweepLength;
  if (sl > 0) {
    b.bmin = b.bmin - V3(sl, sl, sl);
    b.bmax = b.bmax + V3(sl, sl, sl);
  }
}

// InsertionSortCollider.hpp:166-171
static inline bool spatialOverlap(const Scene& S, int id1, int id2) {
  const Real* mn = S.minima.data(); const Real* mx = S.maxima.data();
  return (mn[3 * id1 + 0] <= mx[3 * id2 + 0]) && (mx[3 * id1 + 0] >= mn[3 * id2 + 0]) &&
         (mn[3 * id1 + 1] <= mx[3 * id2 + 1]) && (mx[3 * id1 + 1] >= mn[3 * id2 + 1]) &&
         (mn[3 * id1 + 2] <= mx[3 * id2 + 2]) && (mx[3 * id1 + 2] >= mn[3 * id2 + 2]);
}

// InsertionSortCollider::spatialOverlapPeri (InsertionSortCollider.cpp:491-543); bodies wider
// than half the cell are not supported (the reference throws unless allowBiggerThanPeriod).
static bool spatialOverlapPeri(const Scene& S, int id1, int id2, int periods[3]) {
  for (int axis = 0; axis < 3; axis++) {
    Real dim = S.cellSize[axis];
    Real m1 = S.minima[3 * id1 + axis], m2 = S.minima[3 * id2 + axis];
    Real wMn = (cellWrapRel(m1, m2, m2 + dim) < cellWrapRel(m2, m1, m1 + dim)) ? m2 : m1;
    int pmn1, pmx1, pmn2, pmx2;
    Real mn1 = cellWrap(m1, wMn, wMn + dim, pmn1), mx1 = cellWrap(S.maxima[3 * id1 + axis], wMn, wMn + dim, pmx1);
    Real mn2 = cellWrap(m2, wMn, wMn + dim, pmn2), mx2 = cellWrap(S.maxima[3 * id2 + axis], wMn, wMn + dim, pmx2);
    if ((pmn1 != pmx1) || (pmn2 != pmx2)) { periods[axis] = 0; return false; }
    periods[axis] = (int)(pmn1 - pmn2);
    if (!(mn1 <= mx2 && mx1 >= mn2)) return false;
  }
  return true;
}
// InsertionSortCollider::handleBoundInversionPeri (InsertionSortCollider.cpp:465-475)
static void handleBoundInversionPeri(Scene& S, int id1, int id2) {
  int periods[3];
  bool overlap = spatialOverlapPeri(S, id1, id2, periods);
  if (overlap && mayCollide(S.bodies[id1], S.bodies[id2]) && !S.byKey.count(pairKey(id1, id2))) {
    icInsert(S, id1, id2);
    Interaction* I = S.lin.back();
    for (int k = 0; k < 3; k++) I->cellDist[k] = periods[k];
  }
}
// InsertionSortCollider::insertionSortPeri (InsertionSortCollider.cpp:416-463)
static void insertionSortPeri(Scene& S, std::vector<Bounds>& v, int axis, bool doCollide) {
  long& loIdx = S.loIdx[axis];
  const long size = (long)v.size();
  const Real cellDim = S.cellSize[axis];
  auto norm_ = [size](long i) { if (i < 0) i += size; return i % size; };
  for (long _i = 0; _i < size; _i++) {
    const long i = norm_(_i);
    const long i_1 = norm_(i - 1);
    if (i == loIdx && v[i].coord < 0) { v[i].period -= 1; v[i].coord += cellDim; loIdx = norm_(loIdx + 1); }
    const Real iCmpCoord = v[i].coord + (i == loIdx ? cellDim : 0);
    if (v[i_1].coord <= iCmpCoord) continue;
    long j = i_1; Bounds vi = v[i]; const bool viHasBB = vi.hasBB;
    const bool isMin = v[i].isMin;
    while (v[j].coord > vi.coord + (norm_(j + 1) == loIdx ? cellDim : 0)) {
      long j1 = norm_(j + 1);
      Bounds& vNew = v[j1];
      vNew = v[j];
      if (j == loIdx && vi.coord < 0) { vi.period -= 1; vi.coord += cellDim; loIdx = norm_(loIdx + 1); }
      else if (j1 == loIdx) { vNew.period += 1; vNew.coord -= cellDim; loIdx = norm_(loIdx - 1); }
      if (isMin && !v[j].isMin && (doCollide && viHasBB && v[j].hasBB)) {
        if (vi.id != vNew.id) handleBoundInversionPeri(S, vi.id, vNew.id);
      }
      j = norm_(j - 1);
    }
    v[norm_(j + 1)] = vi;
  }
}

// InsertionSortCollider::handleBoundInversion (InsertionSortCollider.cpp:22-27)
static void handleBoundInversion(Scene& S, int id1, int id2) {
  if (spatialOverlap(S, id1, id2) && mayCollide(S.bodies[id1], S.bodies[id2]) && !S.byKey.count(pairKey(id1, id2)))
    icInsert(S, id1, id2);
}
// InsertionSortCollider::insertionSort (InsertionSortCollider.cpp:29-54), serial form
static void insertionSort(Scene& S, std::vector<Bounds>& v, bool doCollide) {
  long n = (long)v.size();
  for (long i = 1; i < n; i++) {
    const Bounds viInit = v[i]; long j = i - 1;
    const bool viInitBB = viInit.hasBB, isMin = viInit.isMin;
    while (j >= 0 && v[j] > viInit) {
      v[j + 1] = v[j];
      if (isMin && !v[j].isMin && doCollide && viInitBB && v[j].hasBB && (viInit.id != v[j].id))
        handleBoundInversion(S, viInit.id, v[j].id);
      j--;
    }
    v[j + 1] = viInit;
  }
}

// InsertionSortCollider::isActivated (InsertionSortCollider.cpp:177-189)
static bool colliderIsActivated(Scene& S) {
  if (!S.strideActive) return true;
  if (!S.newtonFound) return true;
  if (S.fastestBodyMaxDist < 0) { S.fastestBodyMaxDist = 0; return true; }
  S.fastestBodyMaxDist = S.maxVelocitySq;
  if (S.fastestBodyMaxDist >= 1 || S.fastestBodyMaxDist == 0) return true;
  if ((size_t)S.BB[0].size() != 2 * S.bodies.size()) return true;
  if (S.interactionsDirty) return true;
  if (S.doSort) { S.doSort = false; return true; }
  return false;
}

// InsertionSortCollider::action, non-periodic (InsertionSortCollider.cpp:191-400)
static void colliderAction(Scene& S) {
  long nBodies = (long)S.bodies.size();
  if (S.isPeriodic != S.colliderPeriodic) { for (int i = 0; i < 3; i++) S.BB[i].clear(); S.colliderPeriodic = S.isPeriodic; }
  const bool periodic = S.colliderPeriodic;
  bool doInitSort = false;
  if (S.doSort) { doInitSort = true; S.doSort = false; }
  if ((long)S.BB[0].size() != 2 * nBodies) {
    long BBsize = (long)S.BB[0].size();
    if (2 * nBodies < BBsize) { for (int i = 0; i < 3; i++) S.BB[i].clear(); BBsize = 0; }
    if (2 * nBodies - BBsize > 200 || BBsize == 0) doInitSort = true;
    for (int i = 0; i < 3; i++)
      for (long id = BBsize / 2; id < nBodies; id++) {
        S.BB[i].push_back(Bounds{0, (int)id, 0, false, true});
        S.BB[i].push_back(Bounds{0, (int)id, 0, false, false});
      }
  }
  if (S.minima.size() != (size_t)3 * nBodies) { S.minima.resize(3 * nBodies); S.maxima.resize(3 * nBodies); }
  if (S.verletDist < 0) S.verletDist = 0;  // no Sphere shapes in this path (:241-252)
  if (S.interactionsDirty) { doInitSort = true; S.interactionsDirty = false; }
  // boundDispatcher->action() (Dispatching.cpp:15-28)
  const Real sweepDist = S.verletDist;
#pragma omp parallel for num_threads(S.nThreads)
  for (long id = 0; id < nBodies; id++) processBody(S, S.bodies[id], sweepDist);
  if (S.verletDist > 0) S.newtonFound = true;
  if (!S.strideActive && S.verletDist > 0 && S.maxVelocitySq >= 0) S.strideActive = true;
  // copy bounds (:289-311)
  for (long i = 0; i < 2 * nBodies; i++)
    for (int j = 0; j < 3; j++) {
      Bounds& B = S.BB[j][i];
      const Body& b = S.bodies[B.id];
      const Real cellDim = S.cellSize[j];
      B.hasBB = b.hasBound;
      B.coord = (b.hasBound ? (B.isMin ? b.bmin[j] : b.bmax[j]) : b.pos[j]) - (periodic ? cellDim * B.period : 0.);
      if (doInitSort && periodic) B.coord = cellWrap(B.coord, 0, cellDim, B.period);
      if (B.isMin && j == 1 && b.hasBound) {
        for (int k = 0; k < 3; k++) { S.minima[3 * B.id + k] = b.bmin[k]; S.maxima[3 * B.id + k] = b.bmax[k]; }
      }
    }
  // conditionalyEraseNonReal (InteractionContainer.hpp:104-110; shouldBeErased = !spatialOverlap)
  for (long linPos = 0; linPos < (long)S.lin.size();) {
    Interaction* I = S.lin[linPos];
    bool real = I->hasGeom && I->hasPhys;
    int per[3];
    bool ov = periodic ? spatialOverlapPeri(S, I->id1, I->id2, per) : spatialOverlap(S, I->id1, I->id2);
    if (!real && !ov) icEraseAt(S, linPos);
    else linPos++;
  }
  if (!doInitSort) {
    if (!periodic) for (int i = 0; i < 3; i++) insertionSort(S, S.BB[i], true);
    else for (int i = 0; i < 3; i++) insertionSortPeri(S, S.BB[i], i, true);
  } else if (periodic) {
    for (int i = 0; i < 3; i++) { S.loIdx[i] = 0; std::sort(S.BB[i].begin(), S.BB[i].end()); }
    S.numReinit++;
    std::vector<Bounds>& V = S.BB[S.sortAxis];
    const long n2 = 2 * nBodies;
    for (long i = 0; i < n2; i++) {
      if (!(V[i].isMin && V[i].hasBB)) continue;
      const int iid = V[i].id;
      long cnt = 0;
      for (long j = (i + 1) % n2; V[j].id != iid; j = (j + 1) % n2) {
        const int jid = V[j].id;
        if (!(V[j].isMin && V[j].hasBB)) continue;
        handleBoundInversionPeri(S, iid, jid);
        if (cnt++ > 2 * nBodies) break;
      }
    }
  } else {
    for (int i = 0; i < 3; i++) std::sort(S.BB[i].begin(), S.BB[i].end());
    S.numReinit++;
    std::vector<Bounds>& V = S.BB[S.sortAxis];
    for (long i = 0; i < 2 * nBodies; i++) {
      if (!(V[i].isMin && V[i].hasBB)) continue;
      const int iid = V[i].id;
      for (long j = i + 1; j < 2 * nBodies && V[j].id != iid; j++) {
        const int jid = V[j].id;
        if (!(V[j].isMin && V[j].hasBB)) continue;
        if (spatialOverlap(S, iid, jid) && mayCollide(S.bodies[iid], S.bodies[jid]))
          if (!S.byKey.count(pairKey(iid, jid))) icInsert(S, iid, jid);
      }
    }
  }
  S.colliderRuns++;
}

// ---------------------------------------------------------------------------
// Narrowphase between two superellipsoids (pkg/dem/Superquadrics_Ig2.cpp)
struct PairCtx {
  const SQ* A; const SQ* B; V3 pos1, pos2;
  long* disCalls;
};
// Disfunction, 9-argument form (Superquadrics_Ig2.cpp:622-687)
static inline void disfunction(const PairCtx& c, Real pa0, Real pa1, V3& center, V3& p1, V3& p2, bool& stop_flag) {
  (*c.disCalls)++;
  V3 contact(NCOS(pa0) * NCOS(pa1), NSIN(pa0) * NCOS(pa1), NSIN(pa1));
  V3 contact1 = mul(c.A->loc, contact);
  Real ph0, ph1;
  sqNormal2Phi(*c.A, contact1, ph0, ph1);
  p1 = sqSurface(*c.A, ph0, ph1);
  p1 = mul(c.A->glob, p1) + c.pos1;
  V3 contact2 = mul(c.B->loc, contact);
  sqNormal2Phi(*c.B, (-1) * contact2, ph0, ph1);
  p2 = sqSurface(*c.B, ph0, ph1);
  p2 = mul(c.B->glob, p2) + c.pos2;
  V3 d = p2 - p1;
  center = 0.5 * (p1 + p2);
  if (dot(contact, d) > 0) stop_flag = true;
  if (g_marg) { margMin(0, dot(contact, d)); g_marg[9] += 1; }
}
// JacfunctionApp (Superquadrics_Ig2.cpp:1033-1054): forward differences with step paraDelta
static inline void jacApp(const PairCtx& c, Real pa0, Real pa1, const Real Dp[2], V3& center, V3& p1, V3& p2,
                          bool& stop_flag, Real J[3][2]) {
  disfunction(c, pa0, pa1, center, p1, p2, stop_flag);
  V3 f0 = p2 - p1;
  disfunction(c, pa0 + Dp[0], pa1, center, p1, p2, stop_flag);
  V3 f1 = p2 - p1;
  disfunction(c, pa0, pa1 + Dp[1], center, p1, p2, stop_flag);
  V3 f2 = p2 - p1;
  for (int i = 0; i < 3; i++) J[i][0] = (f1[i] - f0[i]) / Dp[0];
  for (int i = 0; i < 3; i++) J[i][1] = (f2[i] - f0[i]) / Dp[1];
}

struct LMInfo { int iters; int stop; };
// lmder2 (Superquadrics_Ig2.cpp:1057-1354) with opts {1.0, 1e-15, 1e-3, 1e-20}
static void lmder2(const PairCtx& c, Real p[2], int itmax, V3& p1, V3& p2, V3& center, bool& touching, V3& contact,
                   LMInfo& info) {
  const Real tau = 1.0, eps1 = 1e-15, eps2 = 1e-3, eps3 = 1e-20;
  const Real EPSILON = 1e-12, ONE_THIRD = 0.3333333333333334;
  touching = true;
  V3 p_f, pDp_f;
  Real jacTf[2], diag[2];
  Real jtj[2][2];
  Real Dp[2] = {1e-7, 1e-7};
  Real pDp[2];
  bool stop_flag = false;
  Real mu = 0, tmp;
  Real jacTf_inf = 0, p_L2, Dp_L2 = DBL_MAX, dF, dL;
  Real p_fL2, pDp_fL2;
  int nu = 2, nu2, stop = 0;
  int k;
  disfunction(c, p[0], p[1], center, p1, p2, stop_flag);
  p_f = p2 - p1;
  p_fL2 = norm(p_f);
  if (!std::isfinite(p_fL2)) stop = 7;
  for (k = 0; k < itmax && !stop; ++k) {
    if (p_fL2 <= eps3) { stop = 6; break; }
    if (stop_flag) { stop = 9; touching = false; break; }
    {
      contact[0] = NCOS(p[0]) * NCOS(p[1]);
      contact[1] = NSIN(p[0]) * NCOS(p[1]);
      contact[2] = NSIN(p[1]);
      Real angle = dot(p_f, contact) / (norm(p_f) * norm(contact));
      margMin(1, std::fabs(angle) - 0.95);
      if (std::fabs(angle) > 0.95) { stop = 8; break; }
    }
    Real J[3][2];
    jacApp(c, p[0], p[1], Dp, center, p1, p2, stop_flag, J);
    // J^T J and J^T (-f): coefficient products with the 3-term tree reduction
    jtj[0][0] = J[0][0] * J[0][0] + (J[1][0] * J[1][0] + J[2][0] * J[2][0]);
    jtj[0][1] = J[0][0] * J[0][1] + (J[1][0] * J[1][1] + J[2][0] * J[2][1]);
    jtj[1][0] = J[0][1] * J[0][0] + (J[1][1] * J[1][0] + J[2][1] * J[2][0]);
    jtj[1][1] = J[0][1] * J[0][1] + (J[1][1] * J[1][1] + J[2][1] * J[2][1]);
    jacTf[0] = J[0][0] * (-1.0 * p_f[0]) + (J[1][0] * (-1.0 * p_f[1]) + J[2][0] * (-1.0 * p_f[2]));
    jacTf[1] = J[0][1] * (-1.0 * p_f[0]) + (J[1][1] * (-1.0 * p_f[1]) + J[2][1] * (-1.0 * p_f[2]));
    jacTf_inf = (std::fabs(jacTf[0]) > std::fabs(jacTf[1]) ? std::fabs(jacTf[0]) : std::fabs(jacTf[1]));
    p_L2 = std::sqrt(p[0] * p[0] + p[1] * p[1]);
    margMin(4, (jacTf_inf - eps1) / eps1);
    if (jacTf_inf <= eps1) { Dp_L2 = 0.0; stop = 1; break; }
    if (k == 0) {
      tmp = (jtj[0][0] > jtj[1][1] ? jtj[0][0] : jtj[1][1]);
      mu = tau * tmp;
    }
    diag[0] = jtj[0][0]; diag[1] = jtj[1][1];
    while (1) {
      jtj[0][0] += mu;
      jtj[1][1] += mu;
      double n_a = jtj[0][0] * jtj[1][1] - jtj[0][1] * jtj[0][1];
      Dp[0] = (jacTf[0] * jtj[1][1] - jacTf[1] * jtj[0][1]) / n_a;
      Dp[1] = (jacTf[1] * jtj[0][0] - jacTf[0] * jtj[0][1]) / n_a;
      Dp_L2 = std::sqrt(Dp[0] * Dp[0] + Dp[1] * Dp[1]);
      margMin(2, (Dp_L2 - 1e-5) / 1e-5);
      if (Dp_L2 < 1e-5) { stop = 2; break; }
      pDp[0] = p[0] + Dp[0]; pDp[1] = p[1] + Dp[1];
      if (Dp_L2 >= (p_L2 + eps2) / (EPSILON * EPSILON)) { stop = 4; break; }
      disfunction(c, pDp[0], pDp[1], center, p1, p2, stop_flag);
      pDp_f = p2 - p1;
      pDp_fL2 = norm(pDp_f);
      if (!std::isfinite(pDp_fL2)) { stop = 7; break; }
      dL = Dp[0] * (mu * Dp[0] + jacTf[0]) + Dp[1] * (mu * Dp[1] + jacTf[1]);
      dF = p_fL2 - pDp_fL2;
      margMin(3, dF);
      tmp = dF / dL;
      if (tmp > 0.0) {
        tmp = 1.0 - NPOW(2 * tmp - 1., 3.);
        mu = mu * ((tmp >= ONE_THIRD) ? tmp : ONE_THIRD);
        nu = 2;
        p[0] = pDp[0]; p[1] = pDp[1];
        p_f = pDp_f;
        p_fL2 = pDp_fL2;
        break;
      }
      mu *= nu;
      nu2 = (int)((unsigned)nu << 1);  // wraps to a non-positive value after 2^30
      if (nu2 <= nu) { stop = 5; break; }
      nu = nu2;
      jtj[0][0] = diag[0]; jtj[1][1] = diag[1];
    }
  }
  if (k >= itmax) stop = 3;
  info.iters = k; info.stop = stop;
}

// Ig2_Superquadrics_Superquadrics_SuperquadricsGeom::precompute (Superquadrics.cpp:1030-1050)
static void precompute(Geom& g, const Body& b1, const Body& b2, Real dt, const V3& currentNormal, bool isNew, const V3& shift2,
                       const V3& shiftVel = V3()) {
  if (!isNew) {
    g.orthonormal_axis = cross(g.normal, currentNormal);
    Real angle = dt * 0.5 * dot(currentNormal, b1.angVel + b2.angVel);
    g.twist_axis = angle * currentNormal;
  } else g.twist_axis = g.orthonormal_axis = V3();
  g.normal = currentNormal;
  V3 c1x = g.contactPoint - b1.pos;
  V3 c2x = (g.contactPoint - b2.pos) - shift2;
  V3 relVel = ((b2.vel + shiftVel) + cross(b2.angVel, c2x)) - (b1.vel + cross(b1.angVel, c1x));
  g.relativeVn = dot(g.normal, relVel) * g.normal;
  g.relativeVs = relVel - g.relativeVn;
  g.shearInc = g.relativeVs * dt;
}

static inline void centerLine(const V3& pos1, const V3& pos2, Real para[2]) {
  V3 d0 = pos2 - pos1;
  para[0] = NATAN2(d0[1], d0[0]);
  para[1] = std::atan(d0[2] / std::sqrt(d0[0] * d0[0] + d0[1] * d0[1]));
  para[0] += 1e-5; para[1] += 1e-5;
}

// Ig2_Superquadrics_Superquadrics_SuperquadricsGeom::go (Superquadrics_Ig2.cpp:1880-2317)
static bool ig2SqSq(Scene& S, Interaction* I, const Body& b1, const Body& b2, const V3& shift2, Stats& st) {
  V3 position1 = b1.pos;
  V3 position2 = b2.pos + shift2;
  const SQ* A = &b1.sq; const SQ* B = &b2.sq;
  bool isNew = !I->hasGeom;
  Geom& g = I->g;
  Real para[2] = {1e-5, 1e-5};
  if (isNew) {
    std::memset(&g, 0, sizeof(Geom));
    g.isShearNew = true;
    I->hasGeom = true;
    centerLine(position1, position2, para);
  } else {
    g.isShearNew = g.PenetrationDepth <= 0;
    para[0] = g.contactAngle[0]; para[1] = g.contactAngle[1];
  }
  V3 contactNormal, center;
  double pDepth = 0.0;
  V3 p1, p2;
  if (A->isSphere && B->isSphere) {
    V3 dist = position2 - position1;
    double r_sum = A->r_max + B->r_max;
    double depth = r_sum - norm(dist);
    if (depth < 1E-18) { g.PenetrationDepth = 0; g.isShearNew = true; return true; }
    normalize(dist);
    p1 = position1 + A->r_max * dist;
    p2 = position2 - B->r_max * dist;
    contactNormal = p1 - p2;
    normalize(contactNormal);
    g.point1 = p1; g.point2 = p2;
    g.contactPoint = 0.5 * (p1 + p2);
    g.PenetrationDepth = depth;
  } else {
    double r_sum = A->r_max + B->r_max;
    if (norm(position1 - position2) > r_sum) { g.PenetrationDepth = 0; g.isShearNew = true; return true; }
    bool touching = true;
    PairCtx c{A, B, position1, position2, &st.disCalls};
    LMInfo info;
    long dc0 = st.disCalls;
    lmder2(c, para, 50, p1, p2, center, touching, contactNormal, info);
    st.lmCalls++; st.lmIters += info.iters;
    { long dc = st.disCalls - dc0; int b = 0; while ((1L << b) < dc && b < 15) b++; st.hist[b]++; }
    if (std::isnan(para[0]) || std::isnan(para[1]) || 7 == info.stop) {
      if (touching) {
        centerLine(position1, position2, para);
        lmder2(c, para, 50, p1, p2, center, touching, contactNormal, info);
        st.lmCalls++; st.lmIters += info.iters; st.restarts++;
      }
    }
    pDepth = dot(p1 - p2, contactNormal);
    if (touching && g_marg) {
      margMin(5, (10.0 * norm(p2 - p1) - A->r_max) / A->r_max);
      if (10.0 * norm(p2 - p1) > A->r_max) {
        V3 q = mul(A->loc, p2 - position1);
        margMin(6, NPOW(NPOW(std::fabs(q[0] / A->rx), 2.0 / A->eps1) + NPOW(std::fabs(q[1] / A->ry), 2.0 / A->eps1),
                            A->eps1 / A->eps2) + NPOW(std::fabs(q[2] / A->rz), 2.0 / A->eps2) - 1);
      }
    }
    if (touching) {
      if (10.0 * norm(p2 - p1) > A->r_max) {
        if (!(sqIsInside(*A, p2 - position1)) || !(sqIsInside(*B, p1 - position2))) {
          centerLine(position1, position2, para);
          lmder2(c, para, 50, p1, p2, center, touching, contactNormal, info);
          st.lmCalls++; st.lmIters += info.iters; st.restarts++;
          pDepth = dot(p1 - p2, contactNormal);
        }
      }
    }
    if (!touching) {
      g.contactAngle[0] = para[0]; g.contactAngle[1] = para[1];
      g.PenetrationDepth = 0; g.isShearNew = true;
      return true;
    }
    g.point1 = p1; g.point2 = p2;
    if (std::isnan(contactNormal[0])) st.nanNormals++;
    g.contactPoint = center;
    g.PenetrationDepth = pDepth;
    normalize(contactNormal);
  }
  precompute(g, b1, b2, S.dt, contactNormal, g.isShearNew, shift2, S.periodicFix ? mul(S.velGrad, shift2) : V3());
  g.normal = contactNormal;
  g.contactAngle[0] = para[0]; g.contactAngle[1] = para[1];
  return true;
}

// Ig2_Wall_Superquadrics_SuperquadricsGeom::go (Superquadrics_Ig2.cpp:2522-2611)
static bool ig2WallSq(Scene& S, Interaction* I, const Body& w, const Body& b, const V3& shift2) {
  const int PA = w.axis; const int sense = w.sense;
  const SQ* B = &b.sq;
  bool isNew = !I->hasGeom;
  Geom& g = I->g;
  if (isNew) {
    std::memset(&g, 0, sizeof(Geom));
    g.isShearNew = true;
    I->hasGeom = true;
  } else g.isShearNew = g.PenetrationDepth <= 0;
  V3 normal; normal[PA] = sense;
  V3 wall_pos = w.pos; V3 B_pos = b.pos;
  if (B->isSphere) {
    V3 p1 = B_pos; p1[PA] = wall_pos[PA];
    V3 point2 = B_pos - normal * B->r_max;
    double depth = B->r_max - norm(B_pos - p1);
    if (depth < 0.0) { g.PenetrationDepth = 0; g.isShearNew = true; return true; }
    g.point1 = p1; g.point2 = point2;
    g.contactPoint = 0.5 * (point2 + p1);
    g.PenetrationDepth = depth;
  } else {
    Real ph0, ph1;
    sqNormal2Phi(*B, -mul(B->loc, normal), ph0, ph1);
    V3 point2 = mul(B->glob, sqSurface(*B, ph0, ph1)) + B_pos;
    V3 p1 = point2; p1[PA] = wall_pos[PA];
    V3 d = point2 - p1;
    if (normal[PA] * d[PA] >= 0.0) { g.PenetrationDepth = 0; g.isShearNew = true; return true; }
    g.point1 = p1; g.point2 = point2;
    g.contactPoint = 0.5 * (point2 + p1);
    g.PenetrationDepth = norm(d);
  }
  precompute(g, w, b, S.dt, normal, g.isShearNew, shift2, S.periodicFix ? mul(S.velGrad, shift2) : V3());
  g.normal = normal;
  return true;
}

// Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys::go (Superquadrics.cpp:1086-1116)
static void ip2Coeffs(Scene& S, Interaction* I, Phys& p) {
  const Mat& m1 = S.mats[S.bodies[I->id1].mat];
  const Mat& m2 = S.mats[S.bodies[I->id2].mat];
  if (I->id1 > 5) {
    Real fa = std::min(m1.frictionAngle, m2.frictionAngle);
    p.tanphi = std::tan(fa);
    p.kn = 2.0 * m1.Kn * m2.Kn / (m1.Kn + m2.Kn);
    p.ks = 2.0 * m1.Ks * m2.Ks / (m1.Ks + m2.Ks);
  } else {
    p.tanphi = std::tan(m1.frictionAngle);
    p.kn = m1.Kn;
    p.ks = m1.Ks;
  }
  p.betan = std::max(m1.betan, m2.betan);
  p.betas = std::max(m1.betas, m2.betas);
}
static void ip2(Scene& S, Interaction* I) {
  if (I->hasPhys) return;
  Phys& p = I->p;
  std::memset(&p, 0, sizeof(Phys));
  I->hasPhys = true;
  ip2Coeffs(S, I, p);
}

// SuperquadricsGeom::rotate (Superquadrics.cpp:1053-1080)
static inline V3 rotateShear(const Geom& g, V3 sf) {
  sf = sf - cross(sf, g.orthonormal_axis);
  sf = sf - cross(sf, g.twist_axis);
  sf = sf - dot(g.normal, sf) * g.normal;
  return sf;
}

// SuperquadricsLaw::go (Superquadrics.cpp:1181-1363)
static bool law(Scene& S, Interaction* I, V3* F, V3* T) {
  if (!I->hasGeom) return true;
  const Body& A = S.bodies[I->id1];
  const Body& B = S.bodies[I->id2];
  Geom& g = I->g; Phys& ph = I->p;
  V3 ab_min = B.bmin, ab_max = B.bmax;
  if (S.isPeriodic) {
    V3 sh = cellShift(S, I->cellDist);
    ab_min = ab_min + sh;
    ab_max = ab_max + sh;
  }
  I->sliding = false;
  if (!S.frozenPairs && (A.bmin[0] >= ab_max[0] || ab_min[0] >= A.bmax[0] || A.bmin[1] >= ab_max[1] || ab_min[1] >= A.bmax[1] ||
      A.bmin[2] >= ab_max[2] || ab_min[2] >= A.bmax[2])) {
    ph.normalForce = V3(); ph.shearForce = V3();
    requestErase(I);
    return false;
  }
  margMin(7, g.PenetrationDepth - 1E-18);
  if (!(g.PenetrationDepth > 1E-18)) { ph.normalForce = V3(); ph.shearForce = V3(); return true; }
  V3 normalForce = g.normal * g.PenetrationDepth * ph.kn;
  V3 shearForce1;
  bool useDamping = (ph.betan > 1e-5 || ph.betas > 1e-5);
  Real cs = 0;
  V3 shearViscous;
  if (useDamping) {
    const bool Adyn = A.blockedDOFs != DOF_ALL, Bdyn = B.blockedDOFs != DOF_ALL;
    Real mbar = (!Adyn && Bdyn) ? B.mass : ((!Bdyn && Adyn) ? A.mass : (A.mass * B.mass / (A.mass + B.mass)));
    Real Cn_crit = 2. * std::sqrt(mbar * ph.kn);
    Real Cs_crit = 2. * std::sqrt(mbar * ph.ks);
    Real cn = Cn_crit * ph.betan;
    cs = Cs_crit * ph.betas;
    V3 normalViscous = cn * g.relativeVn;
    V3 normTemp = normalForce - normalViscous;
    if (dot(normTemp, g.normal) < 0.0) normalForce = V3();
    else normalForce = normalForce - normalViscous;
  }
  if (g.isShearNew) shearForce1 = V3();
  else shearForce1 = rotateShear(g, ph.shearForce);
  shearForce1 = shearForce1 - ph.ks * g.shearInc;
  Real maxFs = sqnorm(normalForce) * std::pow(ph.tanphi, 2);
  if (sqnorm(shearForce1) > maxFs) {
    I->sliding = true;
    Real ratio = std::sqrt(maxFs) / norm(shearForce1);
    shearForce1 = shearForce1 * ratio;
  } else if (useDamping) {
    shearViscous = cs * g.relativeVs;
  }
  if (std::isnan(shearForce1[0]) || std::isnan(normalForce[0])) { normalForce = V3(); shearForce1 = V3(); }
  V3 Fv = ((-normalForce) - shearForce1) + shearViscous;
  F[I->id1] = F[I->id1] + Fv;
  F[I->id2] = F[I->id2] + (-Fv);
  T[I->id1] = T[I->id1] + (-cross(A.pos - g.contactPoint, Fv));
  T[I->id2] = T[I->id2] + cross((S.periodicFix && S.isPeriodic ? B.pos + cellShift(S, I->cellDist) : B.pos) - g.contactPoint, Fv);
  ph.normalForce = normalForce;
  ph.shearForce = shearForce1;
  return true;
}

// ---------------------------------------------------------------------------
// Hertz-Mindlin contact model.
// CRotationMat (Superquadrics_Ig2.cpp:295-316): rotation taking x onto the direction from
// particle 1 to particle 2 (the frame of the Nelder-Mead angles).
static M3 cRotationMat(const V3& position1, const V3& position2) {
  const V3 x1(1., 0, 0);
  const V3 e1 = position2 - position1;
  const Real cos_phi = dot(x1, e1) / (norm(x1) * norm(e1));
  const Real cos_halfphi = std::sqrt(0.5 * (1 + cos_phi));
  const Real sin_halfphi = std::sqrt(0.5 * (1 - cos_phi));
  Quat q;
  if (std::fabs(cos_phi) > 1.0 - 1e-10) q = Quat{cos_halfphi, 0, 0, sin_halfphi};
  else {
    V3 n1 = cross(x1, e1);
    normalize(n1);
    n1 = n1 * sin_halfphi;
    q = Quat{cos_halfphi, n1[0], n1[1], n1[2]};
  }
  return toRot(q);
}
// Disfun (Superquadrics_Ig2.cpp:1624-1667): distance between the support points along the
// direction given by the angles in the CRotationMat frame
static Real disfun(const Real para[2], const SQ& A, const SQ& B, const V3& position1, const V3& position2, V3& p1,
                   V3& p2, const M3& gc, bool& touching, long* nev) {
  V3 contact(NCOS(para[0]) * NCOS(para[1]), NSIN(para[0]) * NCOS(para[1]), NSIN(para[1]));
  contact = mul(gc, contact);
  Real ph0, ph1;
  sqNormal2Phi(A, mul(A.loc, contact), ph0, ph1);
  p1 = mul(A.glob, sqSurface(A, ph0, ph1)) + position1;
  sqNormal2Phi(B, (-1.0) * mul(B.loc, contact), ph0, ph1);
  p2 = mul(B.glob, sqSurface(B, ph0, ph1)) + position2;
  const V3 d = p2 - p1;
  if (dot(contact, d) > 0) touching = false;
  if (nev) (*nev)++;
  return norm(d);
}
struct NMCtx { const SQ* A; const SQ* B; V3 pos1, pos2; M3 gc; long* nev; };
// amotry (:1668-1700)
static Real amotry(Real p[3][2], Real y[3], Real psum[2], int ihi, Real fac, const NMCtx& c, V3& pt1, V3& pt2,
                   bool& touching) {
  const Real fac1 = (1.0 - fac) / 2.0;
  const Real fac2 = fac1 - fac;
  Real ptry[2] = {psum[0] * fac1 - p[ihi][0] * fac2, psum[1] * fac1 - p[ihi][1] * fac2};
  const Real ytry = disfun(ptry, *c.A, *c.B, c.pos1, c.pos2, pt1, pt2, c.gc, touching, c.nev);
  if (ytry < y[ihi]) {
    y[ihi] = ytry;
    psum[0] += ptry[0] - p[ihi][0]; psum[1] += ptry[1] - p[ihi][1];
    p[ihi][0] = ptry[0]; p[ihi][1] = ptry[1];
  }
  return ytry;
}
// neldermead_simplex (:1701-1878).  The reference leaves its evaluation counter uninitialised
// (undefined behaviour in the NMAX test); it starts at 0 here.
static void neldermeadSimplex(const Real point[2], const Real dels[2], Real info[2], const NMCtx& c, V3& pt1, V3& pt2,
                              bool& touching, Real out[2]) {
  const Real ftol = 1e-3, TINY = 1.0e-10;
  const int NMAX = 5000;
  int nfunc = 0;
  Real fmin = 0;
  Real p[3][2], y[3], psum[2];
  for (int i = 0; i < 3; i++) { p[i][0] = point[0]; p[i][1] = point[1]; }
  p[1][0] += dels[0];
  p[2][1] += dels[1];
  auto ret = [&](const Real* v, Real dist) { info[0] = nfunc; info[1] = dist; out[0] = v[0]; out[1] = v[1]; };
  for (int i = 0; i < 3; i++) {
    y[i] = disfun(p[i], *c.A, *c.B, c.pos1, c.pos2, pt1, pt2, c.gc, touching, c.nev);
    nfunc++;
    if (!touching) { ret(p[0], y[0]); return; }
  }
  psum[0] = (p[0][0] + p[1][0]) + p[2][0]; psum[1] = (p[0][1] + p[1][1]) + p[2][1];
  for (;;) {
    int ilo = 0, ihi, inhi;
    if (!touching) { ret(p[0], fmin); return; }
    if (y[0] > y[1]) { inhi = 1; ihi = 0; } else { inhi = 0; ihi = 1; }
    for (int i = 0; i < 3; i++) {
      if (y[i] <= y[ilo]) ilo = i;
      if (y[i] > y[ihi]) { inhi = ihi; ihi = i; }
      else if (y[i] > y[inhi] && i != ihi) inhi = i;
    }
    const Real rtol = 2.0 * std::fabs(y[ihi] - y[ilo]) / (std::fabs(y[ihi]) + std::fabs(y[ilo]) + TINY);
    if (rtol < ftol) {
      std::swap(y[0], y[ilo]);
      std::swap(p[ilo][0], p[0][0]); std::swap(p[ilo][1], p[0][1]);
      fmin = y[0];
      ret(p[0], fmin);
      return;
    }
    if (nfunc >= NMAX) { ret(p[0], y[0]); return; }
    Real ytry = amotry(p, y, psum, ihi, -1.0, c, pt1, pt2, touching); nfunc++;
    if (!touching) { ret(p[0], y[0]); return; }
    if (ytry <= y[ilo]) {
      ytry = amotry(p, y, psum, ihi, 2.0, c, pt1, pt2, touching); nfunc++;
      if (!touching) { ret(p[0], y[0]); return; }
    } else if (ytry >= y[inhi]) {
      const Real ysave = y[ihi];
      ytry = amotry(p, y, psum, ihi, 0.5, c, pt1, pt2, touching); nfunc++;
      if (!touching) { ret(p[0], y[0]); return; }
      if (ytry >= ysave) {
        for (int i = 0; i < 3; i++) {
          if (i != ilo) {
            p[i][0] = psum[0] = 0.5 * (p[i][0] + p[ilo][0]);
            p[i][1] = psum[1] = 0.5 * (p[i][1] + p[ilo][1]);
            y[i] = disfun(psum, *c.A, *c.B, c.pos1, c.pos2, pt1, pt2, c.gc, touching, c.nev); nfunc++;
            if (!touching) { ret(p[0], y[0]); return; }
          }
        }
        psum[0] = (p[0][0] + p[1][0]) + p[2][0]; psum[1] = (p[0][1] + p[1][1]) + p[2][1];
      }
    }
  }
}
// Superquadrics::Curvatures (Superquadrics.cpp:128-224): principal curvatures from the first
// and second fundamental forms (the mixed term of the second form is left out, as in the
// reference) and the principal directions in the global frame.
static void sqCurvatures(const SQ& q, Real ph0, Real ph1, V3& dirMax, V3& dirMin, bool& maxFlag, Real k[2]) {
  maxFlag = true;
  if (std::fabs(ph0) < 1E-20) ph0 = 1E-20;
  if (std::fabs(ph1) < 1E-20) ph1 = 1E-20;
  const Real rx = q.rx, ry = q.ry, rz = q.rz, eps1 = q.eps1, eps2 = q.eps2;
  const Real s1 = NSIN(ph0), s2 = NSIN(ph1), c1 = NCOS(ph0), c2 = NCOS(ph1);
  const Real s_s1 = Sign(s1), s_s2 = Sign(s2), s_c1 = Sign(c1), s_c2 = Sign(c2);
  const Real abs_s1 = std::fabs(s1), abs_s2 = std::fabs(s2), abs_c1 = std::fabs(c1), abs_c2 = std::fabs(c2);
  const Real s10 = s_s1 * NPOW(abs_s1, eps1), s20 = s_s2 * NPOW(abs_s2, eps2);
  const Real c10 = s_c1 * NPOW(abs_c1, eps1), c20 = s_c2 * NPOW(abs_c2, eps2);
  const Real s12 = s_s1 * NPOW(abs_s1, eps1 - 2.0), s22 = s_s2 * NPOW(abs_s2, eps2 - 2.0);
  const Real c12 = s_c1 * NPOW(abs_c1, eps1 - 2.0), c22 = s_c2 * NPOW(abs_c2, eps2 - 2.0);
  const V3 R1(-rx * eps1 * c12 * c1 * c20 * s1, ry * eps1 * c1 * c20 * s12 * s1, 0);
  const V3 R2(-rx * eps2 * c10 * c22 * c2 * s2, -ry * eps2 * c22 * c2 * s10 * s2, rz * eps2 * c2 * s22 * s2);
  const V3 R11(rx * eps1 * c12 * s20 * s1 * s1 * (eps1 - 1.0) - rx * eps1 * c10 * c20,
               ry * eps1 * c1 * c1 * c20 * s12 * (eps1 - 1.0) - ry * eps1 * c20 * s10, 0);
  const V3 R22(rx * eps2 * c10 * c22 * s2 * s2 * (eps2 - 1.0) - rx * eps2 * c10 * c20,
               ry * eps2 * s10 * s1 * s1 * (eps2 - 1.0) - ry * eps2 * c20 * s10,
               rz * eps2 * c2 * c2 * s22 * (eps2 - 1.0) - rz * eps2 * s20);
  const V3 RR = cross(R1, R2);
  const Real rrn = norm(RR);
  const V3 n(RR[0] / rrn, RR[1] / rrn, RR[2] / rrn);
  const Real L = dot(R11, n), N = dot(R22, n), E = dot(R1, R1), F = dot(R1, R2), G = dot(R2, R2);
  const Real Kg = L * N / (E * G - F * F);
  const Real H = 0.5 * (E * N + G * L) / (E * G - F * F);
  const Real tmp0 = std::sqrt(std::fabs(H * H - Kg));
  const Real k1 = H + tmp0, k2 = H - tmp0;
  V3 d1 = R1 * (N - k1 * G) + R2 * k1 * F;
  if (norm(d1) == 0) maxFlag = false;
  else { normalize(d1); dirMax = mul(q.glob, d1); }
  V3 d2 = R1 * (N - k2 * G) + R2 * k2 * F;
  normalize(d2);
  dirMin = mul(q.glob, d2);
  k[0] = k1; k[1] = k2;
}
// SuperquadricsGeom2::HertzMindlin (Superquadrics.cpp:965-996): contact ellipse from the
// relative curvatures (semi-axis ratio alpha and the complete elliptic integrals K, E by the
// reference's polynomial fits)
static void hertzMindlin(Geom& g, const Real c1[2], const Real c2[2], Real theta) {
  Real rho11 = std::fabs(c1[0]), rho12 = std::fabs(c1[1]), rho21 = std::fabs(c2[0]), rho22 = std::fabs(c2[1]);
  if (rho11 * rho12 < 1E-18) rho11 = rho12 = 0.0;
  if (rho21 * rho22 < 1E-18) rho21 = rho22 = 0.0;
  const Real sum_rho = ((rho11 + rho12) + rho21) + rho22;
  const Real F_rho = -std::sqrt((std::pow(rho11 - rho12, 2) + std::pow(rho21 - rho22, 2)) +
                                2 * (std::fabs(rho11 - rho12)) * std::fabs(rho21 - rho22) * NCOS(2 * theta));
  const Real A = (sum_rho + F_rho) / 4., B = (sum_rho - F_rho) / 4.;
  g.curvatures_sum = A + B;
  const Real x_squ = std::pow(std::log10(B / A), 2);
  const Real gamma1 = 2 * (1 + x_squ * (0.40227436 + x_squ * (3.7491752e-2 + x_squ * (7.4855761e-4 + x_squ * 2.1667028e-6))));
  const Real gamma2 = 3 * (1 + x_squ * (0.42678878 + x_squ * (4.2605401e-2 + x_squ * (9.0786922e-4 + x_squ * 2.7868927e-6))));
  g.alpha = std::pow((B / A), gamma1 / gamma2);
  const Real m1 = 1 / std::pow(g.alpha, 2);
  g.K = (1.3862944 + m1 * (0.1119723 + 0.0725296 * m1)) - std::log(m1) * (0.5 + m1 * (0.1213478 + 0.0288729 * m1));
  g.E = (1 + m1 * (0.4630151 + 0.1077812 * m1)) - std::log(m1) * (0.2452727 + 0.0412496 * m1) * m1;
}
// Ig2_Superquadrics_Superquadrics_SuperquadricsGeom2::go (Superquadrics_Ig2.cpp:2322-2517).  The
// positions are used without the periodic shift, as in the reference.
static bool ig2SqSq2(Scene& S, Interaction* I, const Body& b1, const Body& b2, const V3& shift2, Stats& st) {
  const V3 position1 = b1.pos, position2 = b2.pos;
  const SQ* A = &b1.sq; const SQ* B = &b2.sq;
  const bool isNew = !I->hasGeom;
  Geom& g = I->g;
  Real dels[2] = {0.01, 0.01}, para[2] = {0.0, 0.0};
  if (isNew) {
    std::memset(&g, 0, sizeof(Geom));
    g.isShearNew = true;
    I->hasGeom = true;
    dels[0] = dels[1] = 0.1;
  } else {
    g.isShearNew = g.PenetrationDepth <= 0;
    dels[0] = dels[1] = 0.001;
  }
  V3 contactNormal, p1, p2;
  if (A->isSphere && B->isSphere) {
    V3 dist = position2 - position1;
    const Real r_sum = A->r_max + B->r_max;
    const Real depth = r_sum - norm(dist);
    if (depth < 1E-18) { g.PenetrationDepth = 0; g.isShearNew = true; return true; }
    normalize(dist);
    p1 = position1 + A->r_max * dist;
    p2 = position2 - B->r_max * dist;
    contactNormal = p1 - p2;
    normalize(contactNormal);
    g.point1 = p1; g.point2 = p2;
    g.contactPoint = 0.5 * (p1 + p2);
    g.PenetrationDepth = depth;
    g.curvatures_sum = r_sum / (A->r_max * B->r_max);
    g.isSphere = true;
  } else {
    const Real r_sum = A->r_max + B->r_max;
    if (norm(position1 - position2) > r_sum) { g.PenetrationDepth = 0; g.isShearNew = true; return true; }
    const M3 gc = cRotationMat(position1, position2);
    para[0] = g.contactAngle[0]; para[1] = g.contactAngle[1];
    bool touching = true;
    Real info[2];
    NMCtx c{A, B, position1, position2, gc, &st.disCalls};
    Real out[2];
    neldermeadSimplex(para, dels, info, c, p1, p2, touching, out);
    para[0] = out[0]; para[1] = out[1];
    st.lmCalls++; st.lmIters += (long)info[0];
    if (!touching) {
      g.contactAngle[0] = para[0]; g.contactAngle[1] = para[1];
      g.PenetrationDepth = 0; g.isShearNew = true;
      return true;
    }
    contactNormal = p1 - p2;
    normalize(contactNormal);
    g.point1 = p1; g.point2 = p2;
    g.contactPoint = 0.5 * (p1 + p2);
    g.PenetrationDepth = info[1];
    V3 contact(NCOS(para[0]) * NSIN(para[1]), NSIN(para[0]) * NSIN(para[1]), NCOS(para[1]));
    contact = mul(gc, contact);
    const V3 contact1 = mul(A->loc, contact), contact2 = mul(B->loc, contact);
    V3 dmax1, dmax2, dmin1, dmin2;
    bool f1, f2;
    Real c1[2], c2[2], ph0, ph1;
    sqNormal2Phi(*A, contact1, ph0, ph1);
    sqCurvatures(*A, ph0, ph1, dmax1, dmin1, f1, c1);
    sqNormal2Phi(*B, (-1) * contact2, ph0, ph1);
    sqCurvatures(*B, ph0, ph1, dmax2, dmin2, f2, c2);
    const V3 cd1 = (f1 && f2) ? dmax1 : dmin1, cd2 = (f1 && f2) ? dmax2 : dmin2;
    const V3 nd = contactNormal;
    const V3 dir1 = V3(cd1[0] * nd[0], cd1[1] * nd[1], cd1[2] * nd[2]) - cd1;
    const V3 dir2 = V3(cd2[0] * nd[0], cd2[1] * nd[1], cd2[2] * nd[2]) - cd2;
    Real angle = std::acos(dot(dir1, dir2) / (norm(dir1) * norm(dir2)));
    if (std::isnan(angle)) angle = 0.0;
    g.curvatures1[0] = c1[0]; g.curvatures1[1] = c1[1];
    g.curvatures2[0] = c2[0]; g.curvatures2[1] = c2[1];
    g.curvatureAngle = angle;
    hertzMindlin(g, c1, c2, angle);
  }
  precompute(g, b1, b2, S.dt, contactNormal, g.isShearNew, shift2, S.periodicFix ? mul(S.velGrad, shift2) : V3());
  g.normal = contactNormal;
  g.contactAngle[0] = para[0]; g.contactAngle[1] = para[1];
  return true;
}
// Ip2_SuperquadricsMat2_SuperquadricsMat2_HertzMindlinPhys::go (Superquadrics.cpp:1118-1160)
struct HMPhys { Real nuab, Gab, mu1, mu2; };
static HMPhys hmPhysOf(const Mat& m1, const Mat& m2) {
  HMPhys h;
  h.nuab = 0.5 * (m1.nu + m2.nu);
  h.Gab = 1.0 / ((1 - m1.nu) / m1.G + (1 - m2.nu) / m2.G);
  h.mu1 = 1. / m1.G + 1. / m2.G;
  h.mu2 = m1.nu / m1.G + m2.nu / m2.G;
  return h;
}
static void ip2HM(Scene& S, Interaction* I) {
  if (I->hasPhys) return;
  const Mat& m1 = S.mats[S.bodies[I->id1].mat];
  const Mat& m2 = S.mats[S.bodies[I->id2].mat];
  Phys& p = I->p;
  std::memset(&p, 0, sizeof(Phys));
  I->hasPhys = true;
  if (I->id1 > 5) p.tanphi = std::tan(std::min(m1.frictionAngle, m2.frictionAngle));
  else { p.tanphi = std::tan(m1.frictionAngle); p.kn = m1.Kn; p.ks = m1.Ks; }
  p.betan = std::max(m1.betan, m2.betan);
  p.betas = std::max(m1.betas, m2.betas);
}
// SuperquadricsLaw2::go (Superquadrics.cpp:1367-1557)
static bool law2(Scene& S, Interaction* I, V3* F, V3* T, Stats& st) {
  if (!I->hasGeom) return true;
  const int idA = I->id1, idB = I->id2;
  const Body& A = S.bodies[idA];
  const Body& B = S.bodies[idB];
  Geom& g = I->g; Phys& ph = I->p;
  if (A.bmin[0] >= B.bmax[0] || B.bmin[0] >= A.bmax[0] || A.bmin[1] >= B.bmax[1] || B.bmin[1] >= A.bmax[1] ||
      A.bmin[2] >= B.bmax[2] || B.bmin[2] >= A.bmax[2]) {
    ph.normalForce = V3(); ph.shearForce = V3();
    requestErase(I);
    return false;
  }
  if (!(g.PenetrationDepth > 1E-18)) { ph.normalForce = V3(); ph.shearForce = V3(); return true; }
  if (idA > 5) {
    const HMPhys h = hmPhysOf(S.mats[A.mat], S.mats[B.mat]);
    const Real depth = g.PenetrationDepth, cs_ = g.curvatures_sum;
    if (g.isSphere) {
      const Real tmp = std::sqrt(depth / cs_);
      ph.kn = 8. / 3. * h.Gab * tmp;
      ph.ks = 8. / (2.0 * h.mu1 - h.mu2) * tmp;
    } else {
      const Real E = g.E, K = g.K, alpha = g.alpha;
      const Real a = std::sqrt(depth * E / cs_ / K);
      ph.kn = (Real)((long double)(4. / 3.) * M_PIl * a * h.Gab * alpha / K);   // long double as the reference
      const Real e2 = 1 - 1 / std::pow(alpha, 2.0);
      const Real ksx = h.mu1 * K - h.mu2 * (K - E) / e2;
      const Real ksy = h.mu1 * K + h.mu2 * ((1 - e2) * K - E) / e2;
      ph.ks = (Real)(M_PIl * alpha * a * (1. / ksx + 1. / ksy));
    }
  }
  V3 normalForce = g.normal * g.PenetrationDepth * ph.kn;
  V3 shearForce1;
  const bool useDamping = (ph.betan > 0.00001 || ph.betas > 0.00001);
  Real cs = 0;
  if (useDamping) {
    const bool Adyn = A.blockedDOFs != DOF_ALL, Bdyn = B.blockedDOFs != DOF_ALL;
    const Real mbar = (!Adyn && Bdyn) ? B.mass : ((!Bdyn && Adyn) ? A.mass : (A.mass * B.mass / (A.mass + B.mass)));
    const Real Cn_crit = 2. * std::sqrt(mbar * ph.kn), Cs_crit = 2. * std::sqrt(mbar * ph.ks);
    const Real cn = Cn_crit * ph.betan;
    cs = Cs_crit * ph.betas;
    const V3 normalViscous = cn * g.relativeVn;
    const V3 normTemp = normalForce - normalViscous;
    if (dot(normTemp, g.normal) < 0.0) normalForce = V3();
    else normalForce = normalForce - normalViscous;
  }
  if (g.isShearNew) shearForce1 = V3();
  else shearForce1 = rotateShear(g, ph.shearForce);
  shearForce1 = shearForce1 - ph.ks * g.shearInc;
  const Real maxFs = sqnorm(normalForce) * std::pow(ph.tanphi, 2);
  if (sqnorm(shearForce1) > maxFs) {
    const Real ratio = std::sqrt(maxFs) / norm(shearForce1);
    shearForce1 = shearForce1 * ratio;
  } else if (useDamping) {
    shearForce1 = shearForce1 - cs * g.relativeVs;
  }
  if (std::isnan(shearForce1[0]) || std::isnan(normalForce[0])) {
    normalForce = V3(); shearForce1 = V3();
    st.nanForces++;   // the reference stops the run after this step (Scene::stopAtIter = iter + 1)
  }
  const V3 Fv = (-normalForce) - shearForce1;
  F[idA] = F[idA] + Fv;
  F[idB] = F[idB] + (-Fv);
  T[idA] = T[idA] + (-cross(A.pos - g.contactPoint, Fv));
  T[idB] = T[idB] + cross(B.pos - g.contactPoint, Fv);
  ph.normalForce = normalForce;
  ph.shearForce = shearForce1;
  return true;
}

// hash of one item's branches at one step (the signature of a frozen-pair window)
static inline unsigned long long branchHash(unsigned long long item, long step, unsigned long long bits) {
  unsigned long long z = ((item + 1) * 0x9E3779B97F4A7C15ull) ^ ((unsigned long long)(step + 1) << 40) ^ (bits * 0xC2B2AE3D27D4EB4Full);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// InteractionLoop::action (pkg/common/InteractionLoop.cpp:23-149)
static void interactionLoop(Scene& S) {
  const long size = (long)S.lin.size();
  const int nt = S.nThreads;
  if ((int)S.fbuf.size() != nt) { S.fbuf.assign(nt, {}); S.tbuf.assign(nt, {}); S.tstats.assign(nt, Stats{}); }
  for (int t = 0; t < nt; t++) {
    S.fbuf[t].assign(S.bodies.size(), V3());
    S.tbuf[t].assign(S.bodies.size(), V3());
  }
#pragma omp parallel for schedule(guided) num_threads(nt)
  for (long i = 0; i < size; i++) {
    Interaction* I = S.lin[i];
    const int tn = threadNum();
    if (!I->geomExists) continue;
    bool swap = false;
    const Body& ba = S.bodies[I->id1];
    const Body& bb = S.bodies[I->id2];
    if (!I->geomFunctorSet) {
      if (ba.kind == KIND_WALL && bb.kind == KIND_WALL) { I->geomExists = false; continue; }
      I->geomFunctorSet = true;
      if (ba.kind == KIND_SQ && bb.kind == KIND_WALL) swap = true;  // functor is (Wall, Superquadrics)
    } else if (ba.kind == KIND_WALL && bb.kind == KIND_WALL) { I->geomExists = false; continue; }
    if (swap) { std::swap(I->id1, I->id2); for (int k = 0; k < 3; k++) I->cellDist[k] *= -1; }
    const Body& b1 = S.bodies[I->id1];
    const Body& b2 = S.bodies[I->id2];
    V3 shift2;
    if (S.isPeriodic) shift2 = cellShift(S, I->cellDist);
    if (S.contactModel == 1) {
      if (b1.kind == KIND_WALL) ig2WallSq(S, I, b1, b2, shift2);   // Ig2_Wall_..._SuperquadricsGeom2: same geometry
      else ig2SqSq2(S, I, b1, b2, shift2, S.tstats[tn]);
      ip2HM(S, I);
      if (!law2(S, I, S.fbuf[tn].data(), S.tbuf[tn].data(), S.tstats[tn])) requestErase(I);
      continue;
    }
    const long dc0 = S.tstats[tn].disCalls;
    for (int k = 0; k < 9; k++) I->marg[k] = INFINITY;
    I->marg[9] = 0;
    g_marg = I->marg;
    if (b1.kind == KIND_WALL) ig2WallSq(S, I, b1, b2, shift2);
    else ig2SqSq(S, I, b1, b2, shift2, S.tstats[tn]);
    ip2(S, I);
    if (!law(S, I, S.fbuf[tn].data(), S.tbuf[tn].data())) requestErase(I);
    g_marg = nullptr;
    if (S.frozenPairs) {
      // the decisions at which the map jumps: the Levenberg-Marquardt path (Disfunction calls);
      // the contact gate and the Coulomb cap are continuous and not recorded
      S.tstats[tn].sig += branchHash(pairKey(I->id1, I->id2), S.iter, (unsigned long long)(S.tstats[tn].disCalls - dc0));
    }
  }
  for (int t = 0; t < nt; t++) {
    S.stats.lmCalls += S.tstats[t].lmCalls; S.stats.lmIters += S.tstats[t].lmIters;
    S.stats.disCalls += S.tstats[t].disCalls; S.stats.restarts += S.tstats[t].restarts;
    S.stats.nanNormals += S.tstats[t].nanNormals;
    S.sig += S.tstats[t].sig;
    if (S.tstats[t].nanForces) S.stopAtIter = S.iter + 1;
    S.stats.nanForces += S.tstats[t].nanForces;
    for (int k = 0; k < 16; k++) S.stats.hist[k] += S.tstats[t].hist[k];
    S.tstats[t] = Stats{};
  }
  // ForceContainer::sync (core/ForceContainer.hpp:134-162): sum thread buffers in thread order
  const long nb = (long)S.bodies.size();
  S.force.assign(nb, V3()); S.torque.assign(nb, V3());
  for (long id = 0; id < nb; id++) {
    V3 sf, st;
    for (int t = 0; t < nt; t++) { sf = sf + S.fbuf[t][id]; st = st + S.tbuf[t][id]; }
    S.force[id] = sf; S.torque[id] = st;
  }
}

// NewtonIntegrator (pkg/dem/NewtonIntegrator.cpp)
// DotQ (:470-477)
static inline Quat DotQ(const V3& a, const Quat& Q) {
  Quat d;
  d.w = (-Q.x * a[0] - Q.y * a[1] - Q.z * a[2]) / 2;
  d.x = (Q.w * a[0] - Q.z * a[1] + Q.y * a[2]) / 2;
  d.y = (Q.z * a[0] + Q.w * a[1] - Q.x * a[2]) / 2;
  d.z = (-Q.y * a[0] + Q.x * a[1] + Q.w * a[2]) / 2;
  return d;
}
// quaternion + and scalar*quaternion on coefficients (lib/base/Math.hpp:172-173)
static inline Quat qadd(const Quat& a, const Quat& b) { return Quat{a.w + b.w, a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline Quat qscale(Real f, const Quat& q) { return Quat{q.w * f, q.x * f, q.y * f, q.z * f}; }

// leapfrogAsphericalRotate with A = shape->rot_mat2local (:337-360, :391-429)
static void leapfrogSqRotate(Scene& S, Body& b, const V3& M) {
  const Real dt = S.dt;
  const M3& A = b.sq.loc;
  const V3 l_n = b.angMom + dt / 2. * M;
  const V3 l_b_n = mul(A, l_n);
  V3 w_b_n(l_b_n[0] / b.inertia[0], l_b_n[1] / b.inertia[1], l_b_n[2] / b.inertia[2]);
  const Quat dotQ_n = DotQ(w_b_n, b.ori);
  const Quat Q_half = qadd(b.ori, qscale(dt / 2., dotQ_n));
  b.angMom = b.angMom + dt * M;
  const V3 l_b_half = mul(A, b.angMom);
  V3 w_b_half(l_b_half[0] / b.inertia[0], l_b_half[1] / b.inertia[1], l_b_half[2] / b.inertia[2]);
  const Quat dotQ_half = DotQ(w_b_half, Q_half);
  b.ori = qadd(b.ori, qscale(dt, dotQ_half));
  b.angVel = qrotate(b.ori, w_b_half);
  qnormalize(b.ori);
  b.sq.loc = toRot(conj(b.ori));
  b.sq.glob = toRot(b.ori);
}
// leapfrogSphericalRotate without move/rot buffers (:319-335)
static void leapfrogSphericalRotate(Scene& S, Body& b) {
  Real angle2 = sqnorm(b.angVel);
  if (angle2 != 0) {
    Real angle = std::sqrt(angle2);
    V3 axis(b.angVel[0] / angle, b.angVel[1] / angle, b.angVel[2] / angle);
    // Quaternionr(AngleAxisr(angle*dt, axis)): w = cos(h), vec = sin(h)*axis
    Real h = 0.5 * (angle * S.dt);
    Real s = NSIN(h);
    Quat q{NCOS(h), s * axis[0], s * axis[1], s * axis[2]};
    // q * ori (Hamilton product, Eigen Quaternion.h quat_product)
    Quat o = b.ori;
    Quat r;
    r.w = q.w * o.w - q.x * o.x - q.y * o.y - q.z * o.z;
    r.x = q.w * o.x + q.x * o.w + q.y * o.z - q.z * o.y;
    r.y = q.w * o.y + q.y * o.w + q.z * o.x - q.x * o.z;
    r.z = q.w * o.z + q.z * o.w + q.x * o.y - q.y * o.x;
    b.ori = r;
  }
  qnormalize(b.ori);
}

// NewtonIntegrator::action for non-clump, non-periodic bodies (:99-304)
static void newtonAction(Scene& S) {
  const Real dt = S.dt;
  const long nb = (long)S.bodies.size();
  if (S.velGradChanged || !m3zero(S.nextVelGrad)) {
    S.velGrad = S.nextVelGrad;
    S.velGradChanged = false;
    for (int k = 0; k < 9; k++) S.nextVelGrad.m[k] = 0;
  }
  const bool periodic = S.isPeriodic, homoDeform = S.homoDeform;
  M3 dVelGrad, dtPrevVelGrad;
  for (int k = 0; k < 9; k++) { dVelGrad.m[k] = S.velGrad.m[k] - S.prevVelGrad.m[k]; dtPrevVelGrad.m[k] = dt * S.prevVelGrad.m[k]; }
  const M3 prevVelGrad = S.prevVelGrad;
  const bool sizeDiffers = S.prevCellSize[0] != S.cellSize[0] || S.prevCellSize[1] != S.cellSize[1] || S.prevCellSize[2] != S.cellSize[2];
  if (periodic && sizeDiffers && !std::isnan(S.prevCellSize[0]))
    S.maxVelocitySq = sqnorm(S.prevCellSize - S.cellSize) / std::pow(dt, 2);
  else S.maxVelocitySq = 0;
  std::vector<Real> thrMax(S.nThreads, 0.0);
  std::vector<unsigned long long> thrSig(S.nThreads, 0ull);
#pragma omp parallel for num_threads(S.nThreads)
  for (long id = 0; id < nb; id++) {
    Body& b = S.bodies[id];
    V3 f = S.force[id], m = S.torque[id];
    unsigned signBits = 0;
    const bool useAspherical = (S.exactAsphericalRot && b.aspherical && b.blockedDOFs != DOF_ALL);
    const bool isSphere = (b.kind == KIND_SQ) && b.sq.isSphere;
    const V3 fluctVel = periodic ? b.vel - mul(prevVelGrad, b.pos) : b.vel;
    if (b.blockedDOFs != DOF_ALL) {
      V3 linAccel;
      if (b.blockedDOFs == 0) linAccel = V3(f[0] / b.mass + S.gravity[0], f[1] / b.mass + S.gravity[1], f[2] / b.mass + S.gravity[2]);
      else for (int i = 0; i < 3; i++) if (!(b.blockedDOFs & (1u << i))) linAccel[i] += f[i] / b.mass + S.gravity[i];
      if (b.isDamped)  // cundallDamp2nd (:23-25)
        for (int i = 0; i < 3; i++) {
          const Real w = fluctVel[i] + 0.5 * dt * linAccel[i];
          const Real sg = Sign(linAccel[i] * w);
          if (linAccel[i] != 0) signBits |= (w > 0 ? 1u : (w < 0 ? 2u : 3u)) << (2 * i);
          linAccel[i] *= 1 - S.damping * sg;
        }
      if (periodic && homoDeform) linAccel = linAccel + mul(prevVelGrad, b.vel);
      b.vel = b.vel + dt * linAccel;
      if (!useAspherical) {
        V3 angAccel;
        if (b.blockedDOFs == 0) angAccel = V3(m[0] / b.inertia[0], m[1] / b.inertia[1], m[2] / b.inertia[2]);
        else for (int i = 0; i < 3; i++) if (!(b.blockedDOFs & (1u << (i + 3)))) angAccel[i] += m[i] / b.inertia[i];
        if (b.isDamped)
          for (int i = 0; i < 3; i++) angAccel[i] *= 1 - S.damping * Sign(angAccel[i] * (b.angVel[i] + 0.5 * dt * angAccel[i]));
        b.angVel = b.angVel + dt * angAccel;
      } else {
        for (int i = 0; i < 3; i++) if (b.blockedDOFs & (1u << (i + 3))) m[i] = 0;
        if (b.isDamped) {
          if (S.isSuperquadrics && isSphere) {
            V3 angAccel;
            if (b.blockedDOFs == 0) angAccel = V3(m[0] / b.inertia[0], m[1] / b.inertia[1], m[2] / b.inertia[2]);
            else for (int i = 0; i < 3; i++) if (!(b.blockedDOFs & (1u << (i + 3)))) angAccel[i] += m[i] / b.inertia[i];
            for (int i = 0; i < 3; i++) angAccel[i] *= 1 - S.damping * Sign(angAccel[i] * (b.angVel[i] + 0.5 * dt * angAccel[i]));
            b.angVel = b.angVel + dt * angAccel;
          } else {  // cundallDamp1st on the torque (:19-21)
            for (int i = 0; i < 3; i++) {
              const Real sg = Sign(m[i] * b.angVel[i]);
              if (m[i] != 0) signBits |= (b.angVel[i] > 0 ? 1u : (b.angVel[i] < 0 ? 2u : 3u)) << (2 * (i + 3));
              m[i] *= 1 - S.damping * sg;
            }
          }
        }
      }
    } else if (periodic && homoDeform) b.vel = b.vel + mul(dtPrevVelGrad, b.vel);
    if (S.quietSystem) {   // quiet_system_flag (:246-250): zero velocities, no move
      b.vel = V3(0, 0, 0);
      b.angVel = V3(0, 0, 0);
    } else {
      if (!useAspherical) leapfrogSphericalRotate(S, b);
      else if (S.isSuperquadrics) {
        if (!isSphere) leapfrogSqRotate(S, b, m);
        else leapfrogSphericalRotate(S, b);
      }
      if (periodic && homoDeform) b.vel = b.vel + mul(dVelGrad, b.pos);  // leapfrogTranslate (:306-317)
      b.pos = b.pos + b.vel * dt;
    }
    if (S.frozenPairs && b.kind == KIND_SQ) thrSig[threadNum()] += branchHash(id, S.iter, signBits | 4096u);
    // saveMaximaDisplacement (:72-85)
    if (b.hasBound) {
      V3 disp = b.pos - b.refPos;
      Real maxDisp = std::max(std::abs(disp[0]), std::max(std::abs(disp[1]), std::abs(disp[2])));
      if (!maxDisp || maxDisp < b.sweepLength) maxDisp = 0.5; else maxDisp = 2;
      Real& t = thrMax[threadNum()];
      t = std::max(t, maxDisp);
    }
  }
  if (S.quietSystem) S.quietSystem = false;
  for (Real t : thrMax) S.maxVelocitySq = std::max(S.maxVelocitySq, t);
  for (unsigned long long t : thrSig) S.sig += t;
  if (periodic) { S.prevCellSize = S.cellSize; S.prevVelGrad = S.velGrad; }
}

// ---------------------------------------------------------------------------
// Shop::unbalancedForce (pkg/dem/Shop_01.cpp:148-188): sum over dynamic bodies of |F + m g|
// (the reference returns the sum, not the mean), divided by twice the sum of |Fn + Fs| over
// real contacts with a non-zero normal force; with useMax, the largest body force divided by
// the summed contact forces on that body.
static Real unbalancedForce(const Scene& S, bool useMax) {
  Real sumF = 0, maxF = 0; long idMax = -1;
  for (size_t id = 0; id < S.bodies.size(); id++) {
    const Body& b = S.bodies[id];
    if (b.blockedDOFs == DOF_ALL) continue;   // !isDynamic()
    const Real currF = norm(S.force[id] + b.mass * S.gravity);
    if (currF > maxF) { maxF = currF; idMax = (long)id; }
    sumF += currF;
  }
  const Real meanF = sumF;
  sumF = 0; Real maxCF = 0;
  for (const Interaction* I : S.lin) {
    if (!(I->hasGeom && I->hasPhys)) continue;
    if (norm(I->p.normalForce) == 0) continue;
    const Real f = norm(I->p.normalForce + I->p.shearForce);
    sumF += f;
    if (I->id1 == idMax || I->id2 == idMax) maxCF += f;
  }
  sumF *= 2.0;
  return useMax ? maxF / maxCF : meanF / sumF;
}

// Shop::getStress (pkg/dem/Shop_02.cpp:350-376): sum over real contacts of
// (Fn + Fs) (pos1 - pos2 - hSize cellDist)^T, divided by the volume (the cell volume when 0).
static M3 shopGetStress(const Scene& S, Real volume) {
  if (volume == 0) volume = S.isPeriodic ? det(S.hSize) : 1;
  M3 st{{0, 0, 0, 0, 0, 0, 0, 0, 0}};
  for (const Interaction* I : S.lin) {
    if (!(I->hasGeom && I->hasPhys)) continue;
    V3 branch = S.bodies[I->id1].pos - S.bodies[I->id2].pos;
    if (S.isPeriodic) branch = branch - mul(S.hSize, V3(I->cellDist[0], I->cellDist[1], I->cellDist[2]));
    const V3 f = I->p.normalForce + I->p.shearForce;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) st.m[3 * i + j] += f[i] * branch[j];
  }
  for (int k = 0; k < 9; k++) st.m[k] /= volume;
  return st;
}

// CompressionEngine, cubic specimen, as compiled in the reference (SOLE_GAIN and NEW_SCHEME
// defined, Compression.hpp:24-31): walls are bodies 0-5 (left, right, front, back, bottom,
// top); each wall is moved directly by its own gain times (wall stress - goal), clamped to
// max_vel*dt.  recordData's file output is left out; its state side effects (box size,
// volume, strain) are kept.
struct Servo {
  // attributes (Compression.hpp:160-215)
  bool z_servo = true, continueFlag = false, hydroStrain = false;
  unsigned shearMode = 1;
  Real gain_alpha = 0.5, target_strain = 0.15;
  unsigned iterate_num_max = 100, solve_num_max = 2000, echo_interval = 1000, savedata_interval = 12;
  unsigned ramp_interval = 10000, ramp_chunks = 400;
  Real f_threshold = 0.01, fmin_threshold = 0.01, unbf_tol = 0.01, max_vel = 1.0, hydroStrainRate = 0;
  Real goalx = 0, goaly = 0, goalz = 0;
  bool activated[6] = {true, true, true, true, true, true};
  Real height0 = 0, width0 = 0, depth0 = 0;
  // state (constructor, Compression.hpp:217-240)
  bool firstRun = true, Flag_ForceTarget = false;
  Real width = 0, depth = 0, height = 0, x_area = 0, y_area = 0, z_area = 0;
  Real Init_boxVolume = 0, Current_boxVolume = 0, particlesVolume = 0, strain2 = 0;
  Real gain_x = 0, gain_y = 0, gain_z = 0, gain_x1 = 0, gain_y1 = 0, gain_z1 = 0;
  Real wsxx_left = 0, wsxx_right = 0, wsyy_front = 0, wsyy_back = 0, wszz_bottom = 0, wszz_top = 0;
  Real wsxx = 0, wsyy = 0, wszz = 0;
  unsigned iterate_num = 0, solve_num = 0, rampNum = 0;
  Real UnbalancedForce = 1;
};

static void svUpdateBoxSize(Scene& S, Servo& C) {   // Compression.cpp:99-114
  const Real left = S.bodies[0].pos[0], right = S.bodies[1].pos[0];
  const Real front = S.bodies[2].pos[1], back = S.bodies[3].pos[1];
  const Real top = S.bodies[5].pos[2], bottom = S.bodies[4].pos[2];
  C.width = right - left; C.depth = back - front; C.height = top - bottom;
  C.x_area = C.depth * C.height; C.y_area = C.width * C.height; C.z_area = C.depth * C.width;
}
static void svConsolSS(Scene& S, Servo& C) {        // Compression.cpp:1330-1362 (SOLE_GAIN)
  svUpdateBoxSize(S, C);
  C.wsxx_right = S.force[1][0] / C.x_area;
  C.wsxx_left = -S.force[0][0] / C.x_area;
  C.wsxx = 0.5 * (C.wsxx_left + C.wsxx_right);
  C.wsyy_back = S.force[3][1] / C.y_area;
  C.wsyy_front = -S.force[2][1] / C.y_area;
  C.wsyy = 0.5 * (C.wsyy_back + C.wsyy_front);
  C.wszz_top = S.force[5][2] / C.z_area;
  C.wszz_bottom = -S.force[4][2] / C.z_area;
  C.wszz = 0.5 * (C.wszz_top + C.wszz_bottom);
}
static void svGetGain(Scene& S, Servo& C) {          // Compression.cpp:1125-1220 (SOLE_GAIN)
  Real st[6] = {0, 0, 0, 0, 0, 0};
  for (const Interaction* I : S.lin) {
    if (!(I->hasGeom && I->hasPhys)) continue;
    const int id = I->id1 < I->id2 ? I->id1 : I->id2;
    if (id < 6) st[id] += I->p.kn;
  }
  C.gain_x = C.gain_alpha * C.x_area / st[0];
  C.gain_y = C.gain_alpha * C.y_area / st[2];
  C.gain_z = C.gain_alpha * C.z_area / st[4];
  C.gain_x1 = C.gain_alpha * C.x_area / st[1];
  C.gain_y1 = C.gain_alpha * C.y_area / st[3];
  C.gain_z1 = C.gain_alpha * C.z_area / st[5];
}
static inline Real svStep(Real gain, Real ws, Real goal, Real maxStep) {   // Sign(u) * min(|u|, max_vel dt)
  const Real u = gain * (ws - goal);
  const Real a = std::abs(u);
  return Sign(u) * ((maxStep < a) ? maxStep : a);
}
static void svServo(Scene& S, Servo& C, Real dt) {   // Compression.cpp:1252-1303 (SOLE_GAIN)
  svConsolSS(S, C);
  const Real ms = C.max_vel * dt;
  if (C.activated[0]) S.bodies[0].pos[0] += -svStep(C.gain_x, C.wsxx_left, C.goalx, ms);
  if (C.activated[1]) S.bodies[1].pos[0] += svStep(C.gain_x1, C.wsxx_right, C.goalx, ms);
  if (C.activated[2]) S.bodies[2].pos[1] += -svStep(C.gain_y, C.wsyy_front, C.goaly, ms);
  if (C.activated[3]) S.bodies[3].pos[1] += svStep(C.gain_y1, C.wsyy_back, C.goaly, ms);
  if (C.z_servo) {
    S.bodies[4].pos[2] += -svStep(C.gain_z, C.wszz_bottom, C.goalz, ms);
    S.bodies[5].pos[2] += svStep(C.gain_z1, C.wszz_top, C.goalz, ms);
  }
}
// getStressTensor (Compression.cpp:764-829) and getStress (:831-841): mean and deviatoric
// stress of the contact stress tensor in the box volume.
static void svGetStress(Scene& S, Servo& C, Real& mean, Real& dev) {
  svUpdateBoxSize(S, C);
  C.Current_boxVolume = C.height * C.z_area;
  Real sg[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};   // row-major Sigma(i,j)
  for (const Interaction* I : S.lin) {
    if (!(I->hasGeom && I->hasPhys)) continue;
    const V3 fn = I->p.normalForce, fs = I->p.shearForce;
    if (norm(fn) == 0) continue;
    if (I->id1 == I->id2) continue;
    const V3 l = S.bodies[I->id2].pos - S.bodies[I->id1].pos;
    const V3 f = fn + fs;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) sg[3 * i + j] += f[i] * l[j];
  }
  for (int k = 0; k < 9; k++) sg[k] /= C.Current_boxVolume;
  // Matrix3r::trace (diagonal sum, a0 + (a1 + a2)) and norm (column-major squaredNorm, Eigen's
  // unrolled halving reduction over 9 coefficients)
  mean = (sg[0] + (sg[4] + sg[8])) / 3.0;
  sg[0] -= mean; sg[4] -= mean; sg[8] -= mean;
  Real c[9];
  for (int k = 0; k < 9; k++) c[k] = sg[3 * (k % 3) + k / 3];
  const Real sq = ((c[0] * c[0] + c[1] * c[1]) + (c[2] * c[2] + c[3] * c[3])) +
                  ((c[4] * c[4] + c[5] * c[5]) + (c[6] * c[6] + (c[7] * c[7] + c[8] * c[8])));
  dev = std::sqrt(sq) * std::sqrt(1.5);
}
static void svRecordData(Scene& S, Servo& C) {       // Compression.cpp:843-925, state only
  Real mean, dev;
  svGetStress(S, C, mean, dev);
  C.strain2 = std::log(C.height0 / C.height);
}
static void svAction(Scene& S, Servo& C) {            // action_cubic, Compression.cpp:395-604
  if (C.firstRun) {
    const Real left = S.bodies[0].pos[0], right = S.bodies[1].pos[0];
    const Real front = S.bodies[2].pos[1], back = S.bodies[3].pos[1];
    const Real top = S.bodies[5].pos[2], bottom = S.bodies[4].pos[2];
    if (C.continueFlag) { C.width = right - left; C.depth = back - front; C.height = top - bottom; }
    else {
      C.width = C.width0 = right - left; C.depth = C.depth0 = back - front; C.height = C.height0 = top - bottom;
    }
    C.x_area = C.depth * C.height; C.y_area = C.width * C.height; C.z_area = C.depth * C.width;
    C.Init_boxVolume = C.height0 * C.width0 * C.depth0;
    C.particlesVolume = 0;
    for (const Body& b : S.bodies) if (b.kind == KIND_SQ) C.particlesVolume += b.sq.volume;
    C.rampNum = 0; C.firstRun = false;
    C.iterate_num = 0; C.solve_num = 0;
    svGetGain(S, C);
    C.Flag_ForceTarget = false;
  }
  const Real dt = S.dt;
  if (C.z_servo) {
    if (C.hydroStrain) {   // hydroConsolidation, Compression.cpp:264-322
      svUpdateBoxSize(S, C);
      const Real ls = S.force[0][0] / C.x_area, rs = S.force[1][0] / C.x_area;
      const Real fs = S.force[2][1] / C.y_area, bs = S.force[3][1] / C.y_area;
      const Real bos = S.force[4][2] / C.z_area, ts = S.force[5][2] / C.z_area;
      const Real dl = C.goalx - std::abs(ls), dr = C.goalx - std::abs(rs);
      const Real df = C.goaly - std::abs(fs), dbk = C.goaly - std::abs(bs);
      const Real dbo = C.goalz - std::abs(bos), dtp = C.goalz - std::abs(ts);
      auto mn = [](Real a, Real b) { return (b < a) ? b : a; };
      if (dl > 0) S.bodies[0].pos[0] += mn(0.1 * C.gain_x * dl, C.hydroStrainRate * C.width * dt);
      if (dr > 0) S.bodies[1].pos[0] -= mn(0.1 * C.gain_x1 * dr, C.hydroStrainRate * C.width * dt);
      if (df > 0) S.bodies[2].pos[1] += mn(0.1 * C.gain_y * df, C.hydroStrainRate * C.depth * dt);
      if (dbk > 0) S.bodies[3].pos[1] -= mn(0.1 * C.gain_y1 * dbk, C.hydroStrainRate * C.depth * dt);
      if (dbo > 0) S.bodies[4].pos[2] += mn(0.1 * C.gain_z * dbo, C.hydroStrainRate * C.height * dt);
      if (dtp > 0) S.bodies[5].pos[2] -= mn(0.1 * C.gain_z1 * dtp, C.hydroStrainRate * C.height * dt);
      C.iterate_num += 1;
      if (C.iterate_num >= C.iterate_num_max) { C.iterate_num = 1; svGetGain(S, C); }
      C.solve_num += 1;
      if (C.solve_num >= C.solve_num_max) {
        C.solve_num = 1;
        Real mean, dev;
        svGetStress(S, C, mean, dev);
        if ((std::abs(mean - C.goalx) / C.goalx < C.f_threshold) && (dev / mean < C.fmin_threshold))
          if (C.UnbalancedForce < C.unbf_tol) S.stopAtIter = S.iter + 1;
      }
    } else {               // generalConsolidation, NEW_SCHEME, Compression.cpp:324-358
      C.iterate_num += 1;
      C.solve_num += 1;
      svServo(S, C, dt);
      if (C.iterate_num >= C.iterate_num_max) { C.iterate_num = 0; svGetGain(S, C); }
      if (C.solve_num >= C.solve_num_max) {
        C.solve_num = 0;
        Real mean, dev;
        svGetStress(S, C, mean, dev);
        if ((std::abs(mean - C.goalx) < C.goalx * C.f_threshold) && (dev / mean < C.fmin_threshold)) {
          C.UnbalancedForce = unbalancedForce(S, false);
          if (C.UnbalancedForce < C.unbf_tol) { S.stopAtIter = S.iter + 1; S.quietSystem = true; }
        }
      }
    }
    if (S.iter % C.savedata_interval == 0) svRecordData(S, C);
    if (S.iter % C.echo_interval == 0) { C.UnbalancedForce = unbalancedForce(S, false); svConsolSS(S, C); }
  } else {                 // shear
    if (!C.continueFlag && C.rampNum < C.ramp_interval) {
      if (C.rampNum < 1 && C.Flag_ForceTarget) {
        svUpdateBoxSize(S, C);
        C.width0 = C.width; C.height0 = C.height; C.depth0 = C.depth;
      }
      C.rampNum++;
      const double ramp_inter = 0.5 * C.ramp_interval;
      double vel;
      if (C.rampNum < ramp_inter)
        vel = (double)(float(C.rampNum / (ramp_inter / C.ramp_chunks) + 1) / float(C.ramp_chunks)) * C.goalz * 2.0;
      else
        vel = ((double)(float((C.ramp_interval - C.rampNum) / (ramp_inter / C.ramp_chunks) + 1) / float(C.ramp_chunks)) + 1.0) * C.goalz;
      S.bodies[4].pos[2] += vel * dt * C.height;
      S.bodies[5].pos[2] += -vel * dt * C.height;
    } else {
      if (C.shearMode & 1) {
        C.iterate_num += 1;
        if (C.iterate_num >= C.iterate_num_max) { C.iterate_num = 1; svGetGain(S, C); }
      }
      S.bodies[4].pos[2] += C.goalz * dt * C.height;
      S.bodies[5].pos[2] += -C.goalz * dt * C.height;
    }
    if (C.shearMode & 1) svServo(S, C, dt);
    else {                 // constant volume (undrained)
      const Real left = S.bodies[0].pos[0], right = S.bodies[1].pos[0];
      const Real front = S.bodies[2].pos[1], back = S.bodies[3].pos[1];
      const Real top = S.bodies[5].pos[2], bottom = S.bodies[4].pos[2];
      C.width = right - left; C.depth = back - front; C.height = top - bottom;
      const double Sa = C.Init_boxVolume / C.height;
      const double dd = 0.5 * (Sa / C.width - C.depth);
      const double dw = Sa / (C.depth + dd) - C.width;
      S.bodies[0].pos[0] += -0.5 * dw; S.bodies[1].pos[0] += 0.5 * dw;
      S.bodies[2].pos[1] += -0.5 * dd; S.bodies[3].pos[1] += 0.5 * dd;
    }
    if (std::log(C.height0 / C.height) > C.target_strain) S.stopAtIter = S.iter + 1;
    if (S.iter % C.savedata_interval == 0) svRecordData(S, C);
    if (S.iter % C.echo_interval == 0) {
      C.UnbalancedForce = unbalancedForce(S, false);
      if (C.shearMode & 2) svConsolSS(S, C);
    }
  }
}

// Scene::moveToNextTimeStep (core/Scene.cpp:70-138) for
// O.engines = [ForceResetter, InsertionSortCollider, InteractionLoop, (hook), NewtonIntegrator]
static void step(Scene& S) {
  S.lastStepCollided = false;
  if (S.isPeriodic) cellIntegrate(S);
  if (!S.frozenPairs && colliderIsActivated(S)) { colliderAction(S); S.lastStepCollided = true; }
  interactionLoop(S);
  if (S.midHook) S.midHook(S.midHookArg);
  if (S.servo) svAction(S, *S.servo);
  newtonAction(S);
  S.iter++;
  S.time += S.dt;
}

}  // namespace sqo

// ===========================================================================
// C ABI used by tests and the CPU baseline (ctypes)
using namespace sqo;
extern "C" {

void* sqo_create(void) { return new Scene(); }
void sqo_destroy(void* h) {
  delete ((Scene*)h)->servo;
  Scene* S = (Scene*)h;
  for (Interaction* I : S->lin) delete I;
  delete S;
}
void sqo_set_threads(void* h, int n) { ((Scene*)h)->nThreads = n > 0 ? n : 1; }

// Frozen-pair window (the forward map the adjoint differentiates): on = no collider pass and
// no bound-separation erase from now on; the branch signature restarts at 0.
void sqo_set_frozen(void* h, int on) { Scene* S = (Scene*)h; S->frozenPairs = on != 0; S->sig = 0; }
unsigned long long sqo_signature(void* h) { return ((Scene*)h)->sig; }
// Recompute the Ip2 coefficients (kn, ks, tan(phi), betas) of every interaction that has a
// phys from the current materials, keeping its force history (the start of an adjoint window).
void sqo_reset_phys(void* h) {
  Scene* S = (Scene*)h;
  for (Interaction* I : S->lin)
    if (I->hasPhys) ip2Coeffs(*S, I, I->p);
}
void sqo_set_material(void* h, int m, double Kn, double Ks, double frictionAngle) {
  Mat& M = ((Scene*)h)->mats[m];
  M.Kn = Kn; M.Ks = Ks; M.frictionAngle = frictionAngle;
}
// Exponents of one body's shape (mass, inertia and r_max keep their values).
void sqo_set_eps(void* h, int body, double e1, double e2) {
  SQ& q = ((Scene*)h)->bodies[body].sq;
  q.eps1 = e1; q.eps2 = e2;
}

int sqo_add_material(void* h, double Kn, double Ks, double frictionAngle, double betan, double betas, double density) {
  Scene* S = (Scene*)h;
  S->mats.push_back(Mat{Kn, Ks, frictionAngle, betan, betas, density});
  return (int)S->mats.size() - 1;
}

// utils.wall (py/utils.py:311-327): fixed, aspherical=False, no bound until the first collider run
int sqo_add_wall(void* h, const double* pos, int axis, int sense, int mat) {
  Scene* S = (Scene*)h;
  Body b; std::memset(&b, 0, sizeof(Body));
  b.kind = KIND_WALL; b.axis = axis; b.sense = sense; b.mat = mat;
  b.pos = V3(pos[0], pos[1], pos[2]); b.ori = Quat{1, 0, 0, 0};
  b.mass = 0; b.blockedDOFs = DOF_ALL; b.isDamped = true; b.aspherical = false; b.groupMask = 1;
  b.hasBound = false; b.refPos = V3(NaN, NaN, NaN);
  S->bodies.push_back(b);
  return (int)S->bodies.size() - 1;
}

// NewSuperquadrics_rot2 (py/_superquadrics_utils.cpp:354-380) followed by body.state.pos = pos
int sqo_add_sq(void* h, double rx, double ry, double rz, double e1, double e2, int mat, const double* q_wxyz,
               int isSphere, const double* pos) {
  Scene* S = (Scene*)h;
  Body b; std::memset(&b, 0, sizeof(Body));
  b.kind = KIND_SQ; b.mat = mat;
  b.sq.rx = rx; b.sq.ry = ry; b.sq.rz = rz; b.sq.eps1 = e1; b.sq.eps2 = e2; b.sq.isSphere = isSphere != 0;
  sqInitial(b.sq);
  const Mat& m = S->mats[mat];
  b.mass = m.density * b.sq.volume;
  b.inertia = b.sq.inertia * m.density;
  Quat o{q_wxyz[0], q_wxyz[1], q_wxyz[2], q_wxyz[3]};
  qnormalize(o);  // Superquadrics::setOrientation (Superquadrics.hpp:86-91)
  b.ori = o;
  b.sq.loc = toRot(conj(o)); b.sq.glob = toRot(o);
  b.pos = V3(pos[0], pos[1], pos[2]);
  b.blockedDOFs = 0; b.isDamped = true; b.aspherical = true; b.groupMask = 1;
  b.hasBound = true; b.refPos = V3(NaN, NaN, NaN); b.sweepLength = 0; b.lastUpdateIter = 0;
  S->bodies.push_back(b);
  return (int)S->bodies.size() - 1;
}

// One Disfunction evaluation (Superquadrics_Ig2.cpp:622-687) between two free superellipsoids
// given by shape (rx, ry, rz, eps1, eps2), orientation (w, x, y, z; normalised as
// Superquadrics::setOrientation does) and centre; out = p1 (3), p2 (3), stop flag.  Also the
// margins of Margins [0] and [8] when margOut is non-null (10 values).
void sqo_disfunction(const double* shapeA5, const double* qA, const double* posA, const double* shapeB5,
                     const double* qB, const double* posB, double pa0, double pa1, double* out, double* margOut) {
  SQ sq[2];
  const double* sh[2] = {shapeA5, shapeB5};
  const double* qq[2] = {qA, qB};
  for (int k = 0; k < 2; k++) {
    std::memset(&sq[k], 0, sizeof(SQ));
    sq[k].rx = sh[k][0]; sq[k].ry = sh[k][1]; sq[k].rz = sh[k][2]; sq[k].eps1 = sh[k][3]; sq[k].eps2 = sh[k][4];
    sqInitial(sq[k]);
    Quat o{qq[k][0], qq[k][1], qq[k][2], qq[k][3]};
    qnormalize(o);
    sq[k].loc = toRot(conj(o)); sq[k].glob = toRot(o);
  }
  long calls = 0;
  PairCtx c{&sq[0], &sq[1], V3(posA[0], posA[1], posA[2]), V3(posB[0], posB[1], posB[2]), &calls};
  double marg[10];
  for (int k = 0; k < 9; k++) marg[k] = INFINITY;
  marg[9] = 0;
  if (margOut) g_marg = marg;
  V3 center, p1, p2;
  bool stop = false;
  disfunction(c, pa0, pa1, center, p1, p2, stop);
  g_marg = nullptr;
  for (int k = 0; k < 3; k++) { out[k] = p1[k]; out[3 + k] = p2[k]; }
  out[6] = stop ? 1 : 0;
  if (margOut) for (int k = 0; k < 10; k++) margOut[k] = marg[k];
}

// One lmder2 call (Superquadrics_Ig2.cpp:1057-1354, itmax 50) between two free superellipsoids
// (as sqo_disfunction) from the angles p0 (2).  out: angles (2), p1 (3), p2 (3), contact (3),
// touching, iterations, stop code, Disfunction evaluations.
void sqo_lmder2(const double* shapeA5, const double* qA, const double* posA, const double* shapeB5, const double* qB,
                const double* posB, const double* p0, double* out) {
  SQ sq[2];
  const double* sh[2] = {shapeA5, shapeB5};
  const double* qq[2] = {qA, qB};
  for (int k = 0; k < 2; k++) {
    std::memset(&sq[k], 0, sizeof(SQ));
    sq[k].rx = sh[k][0]; sq[k].ry = sh[k][1]; sq[k].rz = sh[k][2]; sq[k].eps1 = sh[k][3]; sq[k].eps2 = sh[k][4];
    sqInitial(sq[k]);
    Quat o{qq[k][0], qq[k][1], qq[k][2], qq[k][3]};
    qnormalize(o);
    sq[k].loc = toRot(conj(o)); sq[k].glob = toRot(o);
  }
  long calls = 0;
  PairCtx c{&sq[0], &sq[1], V3(posA[0], posA[1], posA[2]), V3(posB[0], posB[1], posB[2]), &calls};
  Real p[2] = {p0[0], p0[1]};
  V3 p1, p2, center, contact;
  bool touching = true;
  LMInfo info;
  lmder2(c, p, 50, p1, p2, center, touching, contact, info);
  out[0] = p[0]; out[1] = p[1];
  for (int k = 0; k < 3; k++) { out[2 + k] = p1[k]; out[5 + k] = p2[k]; out[8 + k] = contact[k]; }
  out[11] = touching ? 1 : 0; out[12] = info.iters; out[13] = info.stop; out[14] = (double)calls;
}

void sqo_set_periodic_fix(void* h, int on) { ((Scene*)h)->periodicFix = on != 0; }

// Test instrument: last-bit noise on the narrowphase's transcendental calls (NZ above); seed 0
// turns it off.  Process-wide: set it between steps, not while one runs.
void sqo_set_math_noise(unsigned long long seed, double rel) { g_noiseSeed = seed; g_noiseRel = rel; }

void sqo_set_params(void* h, double dt, const double* gravity, double damping, double verletDist, int targetInterv,
                    double minSweepDistFactor, int sortAxis) {
  Scene* S = (Scene*)h;
  S->dt = dt; S->gravity = V3(gravity[0], gravity[1], gravity[2]); S->damping = damping;
  S->verletDist = verletDist; S->targetInterv = targetInterv; S->minSweepDistFactor = minSweepDistFactor;
  S->sortAxis = sortAxis;
}

// Periodic cell (Cell::setHSize + Cell::setVelGrad semantics): hSize columns are the cell
// base vectors, velGrad takes effect at the next NewtonIntegrator pass.
void sqo_set_periodic(void* h, const double* hSize9, const double* velGrad9) {
  Scene* S = (Scene*)h;
  S->isPeriodic = true;
  for (int k = 0; k < 9; k++) S->hSize.m[k] = hSize9[k];
  S->trsf = M3{{1, 0, 0, 0, 1, 0, 0, 0, 1}};
  for (int i = 0; i < 3; i++) S->cellSize[i] = norm(V3(S->hSize.m[0 + i], S->hSize.m[3 + i], S->hSize.m[6 + i]));
  if (velGrad9) { for (int k = 0; k < 9; k++) S->nextVelGrad.m[k] = velGrad9[k]; S->velGradChanged = true; }
}
void sqo_set_velgrad(void* h, const double* velGrad9) {
  Scene* S = (Scene*)h;
  for (int k = 0; k < 9; k++) S->nextVelGrad.m[k] = velGrad9[k];
  S->velGradChanged = true;
}
// hSize9 velGrad9 prevVelGrad9 size3 prevCellSize3 -> 33 doubles
void sqo_get_cell(void* h, double* o) {
  Scene* S = (Scene*)h;
  for (int k = 0; k < 9; k++) { o[k] = S->hSize.m[k]; o[9 + k] = S->velGrad.m[k]; o[18 + k] = S->prevVelGrad.m[k]; }
  for (int k = 0; k < 3; k++) { o[27 + k] = S->cellSize[k]; o[30 + k] = S->prevCellSize[k]; }
}
void sqo_set_cell(void* h, const double* o) {
  Scene* S = (Scene*)h;
  for (int k = 0; k < 9; k++) { S->hSize.m[k] = o[k]; S->velGrad.m[k] = o[9 + k]; S->prevVelGrad.m[k] = o[18 + k]; }
  for (int k = 0; k < 3; k++) { S->cellSize[k] = o[27 + k]; S->prevCellSize[k] = o[30 + k]; }
  S->velGradChanged = false;
  for (int k = 0; k < 9; k++) S->nextVelGrad.m[k] = 0;
}

// O.run(n): stops at Scene::stopAtIter when an engine has set it
void sqo_step(void* h, int n) {
  Scene* S = (Scene*)h;
  for (int i = 0; i < n; i++) {
    if (S->stopAtIter >= 0 && S->iter >= S->stopAtIter) break;
    step(*S);
  }
}
// Run only the collider (if activated) and return whether it ran; for pair-set checks.
int sqo_collide(void* h) {
  Scene* S = (Scene*)h;
  if (colliderIsActivated(*S)) { colliderAction(*S); return 1; }
  return 0;
}
int sqo_last_step_collided(void* h) { return ((Scene*)h)->lastStepCollided ? 1 : 0; }
long sqo_iter(void* h) { return ((Scene*)h)->iter; }
int sqo_num_bodies(void* h) { return (int)((Scene*)h)->bodies.size(); }
long sqo_num_interactions(void* h) { return (long)((Scene*)h)->lin.size(); }
void sqo_stats(void* h, long* out5) {
  Stats& s = ((Scene*)h)->stats;
  out5[0] = s.lmCalls; out5[1] = s.lmIters; out5[2] = s.disCalls; out5[3] = s.restarts; out5[4] = s.nanNormals;
}
// histogram of Disfunction evaluations per LM solve, bucket b = ceil(log2(count))
void sqo_eval_hist(void* h, long* out16) { for (int k = 0; k < 16; k++) out16[k] = ((Scene*)h)->stats.hist[k]; }
double sqo_max_velocity_sq(void* h) { return ((Scene*)h)->maxVelocitySq; }

// Body state, 37 doubles per body:
// pos3 ori4(wxyz) vel3 angVel3 angMom3 force3 torque3 bmin3 bmax3 refPos3 sweepLength lastUpdateIter mass inertia3
enum { BODY_STRIDE = 37 };
void sqo_get_bodies(void* h, double* out) {
  Scene* S = (Scene*)h;
  for (size_t i = 0; i < S->bodies.size(); i++) {
    const Body& b = S->bodies[i]; double* o = out + i * BODY_STRIDE;
    for (int k = 0; k < 3; k++) o[k] = b.pos[k];
    o[3] = b.ori.w; o[4] = b.ori.x; o[5] = b.ori.y; o[6] = b.ori.z;
    for (int k = 0; k < 3; k++) { o[7 + k] = b.vel[k]; o[10 + k] = b.angVel[k]; o[13 + k] = b.angMom[k]; }
    V3 f = i < S->force.size() ? S->force[i] : V3(), t = i < S->torque.size() ? S->torque[i] : V3();
    for (int k = 0; k < 3; k++) { o[16 + k] = f[k]; o[19 + k] = t[k]; }
    for (int k = 0; k < 3; k++) { o[22 + k] = b.bmin[k]; o[25 + k] = b.bmax[k]; o[28 + k] = b.refPos[k]; }
    o[31] = b.sweepLength; o[32] = (double)b.lastUpdateIter; o[33] = b.mass;
    for (int k = 0; k < 3; k++) o[34 + k] = b.inertia[k];
  }
}
// Overwrite dynamic state (pos, ori, vel, angVel, angMom) and bound state of all bodies
// from the same 37-double layout; forces/mass/inertia columns are ignored.
void sqo_set_bodies(void* h, const double* in) {
  Scene* S = (Scene*)h;
  for (size_t i = 0; i < S->bodies.size(); i++) {
    Body& b = S->bodies[i]; const double* o = in + i * BODY_STRIDE;
    b.pos = V3(o[0], o[1], o[2]);
    b.ori = Quat{o[3], o[4], o[5], o[6]};
    b.vel = V3(o[7], o[8], o[9]); b.angVel = V3(o[10], o[11], o[12]); b.angMom = V3(o[13], o[14], o[15]);
    b.bmin = V3(o[22], o[23], o[24]); b.bmax = V3(o[25], o[26], o[27]); b.refPos = V3(o[28], o[29], o[30]);
    b.sweepLength = o[31]; b.lastUpdateIter = (long)o[32];
    if (b.kind == KIND_SQ) { b.sq.loc = toRot(conj(b.ori)); b.sq.glob = toRot(b.ori); }
  }
}

// Interaction records, 57 doubles each:
// id1 id2 real hasGeom depth angle2 contactPoint3 normal3 shearInc3 point1_3 point2_3 isShearNew
// kn ks tanphi normalForce3 shearForce3 twist3 ortho3 relVn3 relVs3 cellDist3
// curvatures1_2 curvatures2_2 curvatureAngle alpha K E curvatures_sum isSphere (SuperquadricsGeom2)
enum { INTR_STRIDE = 57 };
void sqo_get_interactions(void* h, double* out) {
  Scene* S = (Scene*)h;
  for (size_t i = 0; i < S->lin.size(); i++) {
    const Interaction* I = S->lin[i]; double* o = out + i * INTR_STRIDE;
    const Geom& g = I->g; const Phys& p = I->p;
    o[0] = I->id1; o[1] = I->id2; o[2] = (I->hasGeom && I->hasPhys) ? 1 : 0; o[3] = I->hasGeom ? 1 : 0;
    o[4] = g.PenetrationDepth; o[5] = g.contactAngle[0]; o[6] = g.contactAngle[1];
    for (int k = 0; k < 3; k++) {
      o[7 + k] = g.contactPoint[k]; o[10 + k] = g.normal[k]; o[13 + k] = g.shearInc[k];
      o[16 + k] = g.point1[k]; o[19 + k] = g.point2[k];
    }
    o[22] = g.isShearNew ? 1 : 0;
    o[23] = p.kn; o[24] = p.ks; o[25] = p.tanphi;
    for (int k = 0; k < 3; k++) {
      o[26 + k] = p.normalForce[k]; o[29 + k] = p.shearForce[k]; o[32 + k] = g.twist_axis[k];
      o[35 + k] = g.orthonormal_axis[k]; o[38 + k] = g.relativeVn[k]; o[41 + k] = g.relativeVs[k];
    }
    for (int k = 0; k < 3; k++) o[44 + k] = I->cellDist[k];
    o[47] = g.curvatures1[0]; o[48] = g.curvatures1[1]; o[49] = g.curvatures2[0]; o[50] = g.curvatures2[1];
    o[51] = g.curvatureAngle; o[52] = g.alpha; o[53] = g.K; o[54] = g.E; o[55] = g.curvatures_sum; o[56] = g.isSphere ? 1 : 0;
  }
}
// Decision margins of the last step (Margins above), one row of 10 per interaction in the
// order of sqo_get_interactions.
void sqo_get_margins(void* h, double* out) {
  Scene* S = (Scene*)h;
  for (size_t i = 0; i < S->lin.size(); i++)
    for (int k = 0; k < 10; k++) out[i * 10 + k] = S->lin[i]->marg[k];
}
// Replace the whole interaction container by the given records (same layout); the
// functor cache is rebuilt as the InteractionLoop would have left it.
void sqo_set_interactions(void* h, long n, const double* in) {
  Scene* S = (Scene*)h;
  for (Interaction* I : S->lin) delete I;
  S->lin.clear(); S->byKey.clear();
  for (long i = 0; i < n; i++) {
    const double* o = in + i * INTR_STRIDE;
    int id1 = (int)o[0], id2 = (int)o[1];
    icInsert(*S, id1, id2);
    Interaction* I = S->lin.back();
    I->iterBorn = 0;
    const Body& a = S->bodies[id1]; const Body& b = S->bodies[id2];
    I->geomFunctorSet = !(a.kind == KIND_WALL && b.kind == KIND_WALL) && (o[3] != 0 || o[2] != 0);
    I->geomExists = !(a.kind == KIND_WALL && b.kind == KIND_WALL && I->geomFunctorSet);
    I->hasGeom = o[3] != 0; I->hasPhys = o[2] != 0;
    Geom& g = I->g; Phys& p = I->p;
    g.PenetrationDepth = o[4]; g.contactAngle[0] = o[5]; g.contactAngle[1] = o[6];
    for (int k = 0; k < 3; k++) {
      g.contactPoint[k] = o[7 + k]; g.normal[k] = o[10 + k]; g.shearInc[k] = o[13 + k];
      g.point1[k] = o[16 + k]; g.point2[k] = o[19 + k];
    }
    g.isShearNew = o[22] != 0;
    p.kn = o[23]; p.ks = o[24]; p.tanphi = o[25];
    for (int k = 0; k < 3; k++) {
      p.normalForce[k] = o[26 + k]; p.shearForce[k] = o[29 + k]; g.twist_axis[k] = o[32 + k];
      g.orthonormal_axis[k] = o[35 + k]; g.relativeVn[k] = o[38 + k]; g.relativeVs[k] = o[41 + k];
    }
    for (int k = 0; k < 3; k++) I->cellDist[k] = (int)o[44 + k];
    g.curvatures1[0] = o[47]; g.curvatures1[1] = o[48]; g.curvatures2[0] = o[49]; g.curvatures2[1] = o[50];
    g.curvatureAngle = o[51]; g.alpha = o[52]; g.K = o[53]; g.E = o[54]; g.curvatures_sum = o[55]; g.isSphere = o[56] != 0;
  }
}

// Collider/integrator scalar state: iter, maxVelocitySq, fastestBodyMaxDist, strideActive,
// newtonFound, verletDist(current), numReinit, colliderRuns
void sqo_get_scalars(void* h, double* o) {
  Scene* S = (Scene*)h;
  o[0] = (double)S->iter; o[1] = S->maxVelocitySq; o[2] = S->fastestBodyMaxDist; o[3] = S->strideActive;
  o[4] = S->newtonFound; o[5] = S->verletDist; o[6] = S->numReinit; o[7] = (double)S->colliderRuns;
  o[8] = S->BB[0].empty() ? 0 : 1;
}
void sqo_set_scalars(void* h, const double* o) {
  Scene* S = (Scene*)h;
  S->iter = (long)o[0]; S->maxVelocitySq = o[1]; S->fastestBodyMaxDist = o[2]; S->strideActive = o[3] != 0;
  S->newtonFound = o[4] != 0; S->verletDist = o[5];
  if (o[8] == 0) for (int j = 0; j < 3; j++) S->BB[j].clear();
}
// Rebuild the collider's sorted bound lists from the current body bounds, as the
// previous collider run would have left them (insertion-sorted, hence sorted by
// coordinate; equal coordinates keep id order).
void sqo_rebuild_sorted_bounds(void* h) {
  Scene* S = (Scene*)h;
  long nb = (long)S->bodies.size();
  S->minima.assign(3 * nb, 0); S->maxima.assign(3 * nb, 0);
  for (int j = 0; j < 3; j++) {
    S->BB[j].clear();
    for (long id = 0; id < nb; id++) {
      const Body& b = S->bodies[id];
      Bounds lo{b.hasBound ? b.bmin[j] : b.pos[j], (int)id, 0, b.hasBound, true};
      Bounds hi{b.hasBound ? b.bmax[j] : b.pos[j], (int)id, 0, b.hasBound, false};
      S->BB[j].push_back(lo); S->BB[j].push_back(hi);
    }
    std::stable_sort(S->BB[j].begin(), S->BB[j].end());
  }
  for (long id = 0; id < nb; id++)
    for (int k = 0; k < 3; k++) { S->minima[3 * id + k] = S->bodies[id].bmin[k]; S->maxima[3 * id + k] = S->bodies[id].bmax[k]; }
}

// Stand-alone narrowphase for known-answer tests: bodies a, b of the scene, optional
// prior geometry (contactAngle, depth, normal) when isNew == 0.  Writes
// depth, normal3, contactPoint3, point1_3, point2_3, angle2, touching -> 15 doubles; returns LM stop code.
int sqo_pair_geom(void* h, int ia, int ib, int isNew, const double* prior4, double* out) {
  Scene* S = (Scene*)h;
  Interaction I; std::memset(&I, 0, sizeof(I));
  I.id1 = ia; I.id2 = ib;
  if (!isNew) {
    I.hasGeom = true; I.g.contactAngle[0] = prior4[0]; I.g.contactAngle[1] = prior4[1]; I.g.PenetrationDepth = prior4[2];
  }
  Stats st{};
  const Body& a = S->bodies[ia]; const Body& b = S->bodies[ib];
  if (a.kind == KIND_WALL) ig2WallSq(*S, &I, a, b, V3());
  else ig2SqSq(*S, &I, a, b, V3(), st);
  const Geom& g = I.g;
  out[0] = g.PenetrationDepth;
  for (int k = 0; k < 3; k++) { out[1 + k] = g.normal[k]; out[4 + k] = g.contactPoint[k]; out[7 + k] = g.point1[k]; out[10 + k] = g.point2[k]; }
  out[13] = g.contactAngle[0]; out[14] = g.contactAngle[1];
  return (int)st.lmIters;
}

// Stand-alone Hertz-Mindlin geometry (Ig2_Superquadrics_Superquadrics_SuperquadricsGeom2) of
// bodies a, b, with the prior (contactAngle, depth) when isNew == 0.  Writes depth, normal3,
// contactPoint3, point1_3, point2_3, angle2, curvatures1_2, curvatures2_2, curvatureAngle,
// alpha, K, E, curvatures_sum, isSphere -> 25 doubles; returns the Nelder-Mead evaluations.
int sqo_pair_geom2(void* h, int ia, int ib, int isNew, const double* prior4, double* out) {
  Scene* S = (Scene*)h;
  Interaction I; std::memset(&I, 0, sizeof(I));
  I.id1 = ia; I.id2 = ib;
  if (!isNew) {
    I.hasGeom = true; I.g.contactAngle[0] = prior4[0]; I.g.contactAngle[1] = prior4[1]; I.g.PenetrationDepth = prior4[2];
  }
  Stats st{};
  const Body& a = S->bodies[ia]; const Body& b = S->bodies[ib];
  ig2SqSq2(*S, &I, a, b, V3(), st);
  const Geom& g = I.g;
  out[0] = g.PenetrationDepth;
  for (int k = 0; k < 3; k++) { out[1 + k] = g.normal[k]; out[4 + k] = g.contactPoint[k]; out[7 + k] = g.point1[k]; out[10 + k] = g.point2[k]; }
  out[13] = g.contactAngle[0]; out[14] = g.contactAngle[1];
  out[15] = g.curvatures1[0]; out[16] = g.curvatures1[1]; out[17] = g.curvatures2[0]; out[18] = g.curvatures2[1];
  out[19] = g.curvatureAngle; out[20] = g.alpha; out[21] = g.K; out[22] = g.E; out[23] = g.curvatures_sum; out[24] = g.isSphere ? 1 : 0;
  return (int)st.lmIters;
}
// Superquadrics::Curvatures at surface angles (ph0, ph1) of a shape with identity orientation:
// k1, k2, dirMax3, dirMin3, maxFlag -> 9 doubles
void sqo_curvatures(double rx, double ry, double rz, double e1, double e2, double ph0, double ph1, double* out) {
  SQ q; std::memset(&q, 0, sizeof(q));
  q.rx = rx; q.ry = ry; q.rz = rz; q.eps1 = e1; q.eps2 = e2;
  sqInitial(q);
  q.loc = toRot(Quat{1, 0, 0, 0}); q.glob = q.loc;
  V3 dmax, dmin; bool f; Real k[2];
  sqCurvatures(q, ph0, ph1, dmax, dmin, f, k);
  out[0] = k[0]; out[1] = k[1];
  for (int j = 0; j < 3; j++) { out[2 + j] = dmax[j]; out[5 + j] = dmin[j]; }
  out[8] = f ? 1 : 0;
}
// SuperquadricsGeom2::HertzMindlin: curvature_sum, alpha, K, E
void sqo_hertz_mindlin(const double* c1, const double* c2, double theta, double* out4) {
  Geom g; std::memset(&g, 0, sizeof(g));
  hertzMindlin(g, c1, c2, theta);
  out4[0] = g.curvatures_sum; out4[1] = g.alpha; out4[2] = g.K; out4[3] = g.E;
}

// Shape properties (Superquadrics::Initial): volume, inertia3 (geometric), r_max
void sqo_shape_props(double rx, double ry, double rz, double e1, double e2, double* out5) {
  SQ s; std::memset(&s, 0, sizeof(s));
  s.rx = rx; s.ry = ry; s.rz = rz; s.eps1 = e1; s.eps2 = e2;
  sqInitial(s);
  out5[0] = s.volume; out5[1] = s.inertia[0]; out5[2] = s.inertia[1]; out5[3] = s.inertia[2]; out5[4] = s.r_max;
}
// Local surface point / normal / Normal2Phi for known-answer construction
void sqo_surface(double rx, double ry, double rz, double e1, double e2, double ph0, double ph1, double* out3) {
  SQ s; std::memset(&s, 0, sizeof(s)); s.rx = rx; s.ry = ry; s.rz = rz; s.eps1 = e1; s.eps2 = e2;
  V3 p = sqSurface(s, ph0, ph1); out3[0] = p[0]; out3[1] = p[1]; out3[2] = p[2];
}
void sqo_normal(double rx, double ry, double rz, double e1, double e2, double ph0, double ph1, double* out3) {
  SQ s; std::memset(&s, 0, sizeof(s)); s.rx = rx; s.ry = ry; s.rz = rz; s.eps1 = e1; s.eps2 = e2;
  V3 p = sqNormal(s, ph0, ph1); out3[0] = p[0]; out3[1] = p[1]; out3[2] = p[2];
}
void sqo_normal2phi(double rx, double ry, double rz, double e1, double e2, const double* n3, double* out2) {
  SQ s; std::memset(&s, 0, sizeof(s)); s.rx = rx; s.ry = ry; s.rz = rz; s.eps1 = e1; s.eps2 = e2;
  sqNormal2Phi(s, V3(n3[0], n3[1], n3[2]), out2[0], out2[1]);
}


// CompressionEngine configuration, 30 doubles: enabled, z_servo, continueFlag, hydroStrain,
// shearMode, activated[6] (left,right,front,back,bottom,top), iterate_num_max, solve_num_max,
// echo_interval, savedata_interval, ramp_interval, ramp_chunks, goalx, goaly, goalz,
// gain_alpha, target_strain, f_threshold, fmin_threshold, unbf_tol, max_vel, hydroStrainRate,
// width0, height0, depth0.
void sqo_set_servo(void* h, const double* c) {
  Scene& S = *(Scene*)h;
  delete S.servo; S.servo = nullptr;
  if (!(c[0] != 0)) return;
  Servo* C = new Servo();
  C->z_servo = c[1] != 0; C->continueFlag = c[2] != 0; C->hydroStrain = c[3] != 0; C->shearMode = (unsigned)c[4];
  for (int k = 0; k < 6; k++) C->activated[k] = c[5 + k] != 0;
  C->iterate_num_max = (unsigned)c[11]; C->solve_num_max = (unsigned)c[12]; C->echo_interval = (unsigned)c[13];
  C->savedata_interval = (unsigned)c[14]; C->ramp_interval = (unsigned)c[15]; C->ramp_chunks = (unsigned)c[16];
  C->goalx = c[17]; C->goaly = c[18]; C->goalz = c[19];
  C->gain_alpha = c[20]; C->target_strain = c[21]; C->f_threshold = c[22]; C->fmin_threshold = c[23];
  C->unbf_tol = c[24]; C->max_vel = c[25]; C->hydroStrainRate = c[26];
  C->width0 = c[27]; C->height0 = c[28]; C->depth0 = c[29];
  S.servo = C;
}
// CompressionEngine state, 36 doubles: width, depth, height, x_area, y_area, z_area, wsxx, wsyy,
// wszz, wsxx_left, wsxx_right, wsyy_front, wsyy_back, wszz_bottom, wszz_top, gain_x, gain_x1,
// gain_y, gain_y1, gain_z, gain_z1, UnbalancedForce, particlesVolume, Init_boxVolume,
// Current_boxVolume, strain2, iterate_num, solve_num, rampNum, Flag_ForceTarget, firstRun,
// width0, height0, depth0, stopAtIter, quiet_system_flag.
void sqo_get_servo(void* h, double* o) {
  Scene& S = *(Scene*)h;
  for (int k = 0; k < 36; k++) o[k] = 0;
  o[34] = (double)S.stopAtIter; o[35] = S.quietSystem ? 1 : 0;
  if (!S.servo) return;
  const Servo& C = *S.servo;
  const double v[34] = {C.width, C.depth, C.height, C.x_area, C.y_area, C.z_area, C.wsxx, C.wsyy, C.wszz,
                        C.wsxx_left, C.wsxx_right, C.wsyy_front, C.wsyy_back, C.wszz_bottom, C.wszz_top,
                        C.gain_x, C.gain_x1, C.gain_y, C.gain_y1, C.gain_z, C.gain_z1, C.UnbalancedForce,
                        C.particlesVolume, C.Init_boxVolume, C.Current_boxVolume, C.strain2,
                        (double)C.iterate_num, (double)C.solve_num, (double)C.rampNum, C.Flag_ForceTarget ? 1.0 : 0.0,
                        C.firstRun ? 1.0 : 0.0, C.width0, C.height0, C.depth0};
  for (int k = 0; k < 34; k++) o[k] = v[k];
}
void sqo_put_servo(void* h, const double* o) {
  Scene& S = *(Scene*)h;
  S.stopAtIter = (long)o[34]; S.quietSystem = o[35] != 0;
  if (!S.servo) return;
  Servo& C = *S.servo;
  C.width = o[0]; C.depth = o[1]; C.height = o[2]; C.x_area = o[3]; C.y_area = o[4]; C.z_area = o[5];
  C.wsxx = o[6]; C.wsyy = o[7]; C.wszz = o[8]; C.wsxx_left = o[9]; C.wsxx_right = o[10]; C.wsyy_front = o[11];
  C.wsyy_back = o[12]; C.wszz_bottom = o[13]; C.wszz_top = o[14];
  C.gain_x = o[15]; C.gain_x1 = o[16]; C.gain_y = o[17]; C.gain_y1 = o[18]; C.gain_z = o[19]; C.gain_z1 = o[20];
  C.UnbalancedForce = o[21]; C.particlesVolume = o[22]; C.Init_boxVolume = o[23]; C.Current_boxVolume = o[24];
  C.strain2 = o[25]; C.iterate_num = (unsigned)o[26]; C.solve_num = (unsigned)o[27]; C.rampNum = (unsigned)o[28];
  C.Flag_ForceTarget = o[29] != 0; C.firstRun = o[30] != 0; C.width0 = o[31]; C.height0 = o[32]; C.depth0 = o[33];
}
// Contact model: 0 SuperquadricsGeom/Phys/Law, 1 SuperquadricsGeom2 + HertzMindlinPhys + Law2
void sqo_set_contact_model(void* h, int model) { ((Scene*)h)->contactModel = model; }
// SuperquadricsMat2 {G, nu} of material m
void sqo_set_moduli(void* h, int m, double G, double nu) { ((Scene*)h)->mats[m].G = G; ((Scene*)h)->mats[m].nu = nu; }
void sqo_stats_nan_forces(void* h, long* out) { *out = ((Scene*)h)->stats.nanForces; }
void sqo_set_quiet(void* h, int on) { ((Scene*)h)->quietSystem = on != 0; }
double sqo_unbalanced_force(void* h, int useMax) { return unbalancedForce(*(Scene*)h, useMax != 0); }
void sqo_get_stress(void* h, double volume, double* out9) {
  const M3 st = shopGetStress(*(Scene*)h, volume);
  for (int k = 0; k < 9; k++) out9[k] = st.m[k];
}
}  // extern "C"
