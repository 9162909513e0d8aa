// Device arithmetic of the Hertz-Mindlin contact model for superellipsoids: the geometry
// functor Ig2_Superquadrics_Superquadrics_SuperquadricsGeom2 (a Nelder-Mead search for the
// closest support points, pkg/dem/Superquadrics_Ig2.cpp:1624-1878, 2322-2517), principal
// curvatures (Superquadrics::Curvatures, pkg/dem/Superquadrics.cpp:131-231) and the contact
// ellipse fits (SuperquadricsGeom2::HertzMindlin, Superquadrics.cpp:974-1013).
//
// Same conventions as sq_device.cuh: the reference's operand order, no FMA contraction.
#pragma once
#include "sq_device.cuh"

namespace sqdem {

// CRotationMat (Superquadrics_Ig2.cpp:295-316): rotation taking the x axis onto the direction
// from particle 1 to particle 2; the frame of the Nelder-Mead angles.  abs() there is the
// floating-point overload.
__device__ __forceinline__ Rot cRotationMat(D3 position1, D3 position2) {
  const D3 x1 = d3(1., 0, 0);
  const D3 e1 = position2 - position1;
  const double cos_phi = dot(x1, e1) / (nrm(x1) * nrm(e1));
  const double cos_halfphi = sqrt(0.5 * (1 + cos_phi));
  const double sin_halfphi = sqrt(0.5 * (1 - cos_phi));
  if (fabs(cos_phi) > 1.0 - 1e-10) return quatToRot(cos_halfphi, 0, 0, sin_halfphi);
  D3 n1 = cross(x1, e1);
  normalize(n1);
  n1 = n1 * sin_halfphi;
  return quatToRot(cos_halfphi, n1.x, n1.y, n1.z);
}

// Disfun (Superquadrics_Ig2.cpp:1624-1667): support point p1 of particle 1 along the direction
// of angles (q0, q1) in the frame gc, support point p2 of particle 2 along the opposite
// direction; returns |p2 - p1|.  apart is set when the points are separated along the
// direction (the particles do not touch).
__device__ __forceinline__ double disfunNM(const SqShape& A, const SqShape& B, const Rot& gc, double q0, double q1,
                                           D3& p1, D3& p2, bool& apart) {
  double s0, c0, s1, c1;
  sincos(q0, &s0, &c0);
  sincos(q1, &s1, &c1);
  const D3 contact = mulG(gc, d3(c0 * c1, s0 * c1, s1));
  p1 = mulG(A.R, supportLocal(A, mulL(A.R, contact))) + A.pos;
  p2 = mulG(B.R, supportLocal(B, (-1.0) * mulL(B.R, contact))) + B.pos;
  const D3 d = p2 - p1;
  apart = dot(contact, d) > 0;
  return nrm(d);
}

// Superquadrics::Normal2Phi (Superquadrics.cpp:269-307): the surface angles of the point whose
// outward normal is n (local frame); the first half of supportLocal.
__device__ __forceinline__ void normal2Phi(const SqShape& s, D3 n, double& ph0, double& ph1) {
  const double Y = pow(fabs(s.ry * n.y), s.i1), X = pow(fabs(s.rx * n.x), s.i1), W = pow(fabs(s.rx * n.x), s.i2);
  ph0 = atan2(sgn(n.y) * Y, sgn(n.x) * X);
  const double t = pow(fabs(cos(ph0)), s.a1);
  const double Z = pow(fabs(s.rz * n.z * t), s.i2);
  ph1 = atan2(sgn(n.z) * Z, W);
}

// Superquadrics::Curvatures (Superquadrics.cpp:131-231): principal curvatures k[0] >= k[1]
// at the surface angles (ph0, ph1) from the first and second fundamental forms (the mixed
// term of the second form is left out, as in the reference), and the principal directions
// in the global frame.  maxFlag is false when the direction of k[0] is degenerate.
__device__ __forceinline__ void curvatures(const SqShape& q, double ph0, double ph1, D3& dirMax, D3& dirMin,
                                           bool& maxFlag, double k[2]) {
  maxFlag = true;
  if (fabs(ph0) < 1E-20) ph0 = 1E-20;
  if (fabs(ph1) < 1E-20) ph1 = 1E-20;
  const double rx = q.rx, ry = q.ry, rz = q.rz, eps1 = q.e1, eps2 = q.e2;
  double s1, c1, s2, c2;
  sincos(ph0, &s1, &c1);
  sincos(ph1, &s2, &c2);
  const double s_s1 = sgn(s1), s_s2 = sgn(s2), s_c1 = sgn(c1), s_c2 = sgn(c2);
  const double abs_s1 = fabs(s1), abs_s2 = fabs(s2), abs_c1 = fabs(c1), abs_c2 = fabs(c2);
  const double s10 = s_s1 * pow(abs_s1, eps1), s20 = s_s2 * pow(abs_s2, eps2);
  const double c10 = s_c1 * pow(abs_c1, eps1), c20 = s_c2 * pow(abs_c2, eps2);
  const double s12 = s_s1 * pow(abs_s1, eps1 - 2.0), s22 = s_s2 * pow(abs_s2, eps2 - 2.0);
  const double c12 = s_c1 * pow(abs_c1, eps1 - 2.0), c22 = s_c2 * pow(abs_c2, eps2 - 2.0);
  const D3 R1 = d3(-rx * eps1 * c12 * c1 * c20 * s1, ry * eps1 * c1 * c20 * s12 * s1, 0);
  const D3 R2 = d3(-rx * eps2 * c10 * c22 * c2 * s2, -ry * eps2 * c22 * c2 * s10 * s2, rz * eps2 * c2 * s22 * s2);
  const D3 R11 = d3(rx * eps1 * c12 * s20 * s1 * s1 * (eps1 - 1.0) - rx * eps1 * c10 * c20,
                    ry * eps1 * c1 * c1 * c20 * s12 * (eps1 - 1.0) - ry * eps1 * c20 * s10, 0);
  const D3 R22 = d3(rx * eps2 * c10 * c22 * s2 * s2 * (eps2 - 1.0) - rx * eps2 * c10 * c20,
                    ry * eps2 * s10 * s1 * s1 * (eps2 - 1.0) - ry * eps2 * c20 * s10,
                    rz * eps2 * c2 * c2 * s22 * (eps2 - 1.0) - rz * eps2 * s20);
  const D3 RR = cross(R1, R2);
  const double rrn = nrm(RR);
  const D3 n = d3(RR.x / rrn, RR.y / rrn, RR.z / rrn);
  const double L = dot(R11, n), N = dot(R22, n), E = dot(R1, R1), F = dot(R1, R2), G = dot(R2, R2);
  const double Kg = L * N / (E * G - F * F);
  const double H = 0.5 * (E * N + G * L) / (E * G - F * F);
  const double tmp0 = sqrt(fabs(H * H - Kg));
  const double k1 = H + tmp0, k2 = H - tmp0;
  D3 d1 = R1 * (N - k1 * G) + R2 * k1 * F;
  if (nrm(d1) == 0) maxFlag = false;
  else { normalize(d1); dirMax = mulG(q.R, d1); }
  D3 d2 = R1 * (N - k2 * G) + R2 * k2 * F;
  normalize(d2);
  dirMin = mulG(q.R, d2);
  k[0] = k1; k[1] = k2;
}

// Contact ellipse of SuperquadricsGeom2 (the fields its HertzMindlin method sets).
struct HMEllipse { double sum, alpha, K, E; };

// SuperquadricsGeom2::HertzMindlin (Superquadrics.cpp:974-1013): relative curvatures A, B of
// the two surfaces at angle theta between their principal directions; semi-axis ratio alpha
// and the complete elliptic integrals K, E by the reference's polynomial fits.
__device__ __forceinline__ HMEllipse hertzMindlin(const double c1[2], const double c2[2], double theta) {
  double rho11 = fabs(c1[0]), rho12 = fabs(c1[1]), rho21 = fabs(c2[0]), rho22 = fabs(c2[1]);
  if (rho11 * rho12 < 1E-18) rho11 = rho12 = 0.0;
  if (rho21 * rho22 < 1E-18) rho21 = rho22 = 0.0;
  const double sum_rho = ((rho11 + rho12) + rho21) + rho22;
  // std::pow(x, 2) is x*x correctly rounded: written as the product
  const double d1 = rho11 - rho12, d2 = rho21 - rho22;
  const double F_rho = -sqrt((d1 * d1 + d2 * d2) +
                             2 * (fabs(rho11 - rho12)) * fabs(rho21 - rho22) * cos(2 * theta));
  const double A = (sum_rho + F_rho) / 4., B = (sum_rho - F_rho) / 4.;
  HMEllipse h;
  h.sum = A + B;
  const double lg = log10(B / A);
  const double x_squ = lg * lg;
  const double gamma1 = 2 * (1 + x_squ * (0.40227436 + x_squ * (3.7491752e-2 + x_squ * (7.4855761e-4 + x_squ * 2.1667028e-6))));
  const double gamma2 = 3 * (1 + x_squ * (0.42678878 + x_squ * (4.2605401e-2 + x_squ * (9.0786922e-4 + x_squ * 2.7868927e-6))));
  h.alpha = pow((B / A), gamma1 / gamma2);
  const double m1 = 1 / (h.alpha * h.alpha);
  h.K = (1.3862944 + m1 * (0.1119723 + 0.0725296 * m1)) - log(m1) * (0.5 + m1 * (0.1213478 + 0.0288729 * m1));
  h.E = (1 + m1 * (0.4630151 + 0.1077812 * m1)) - log(m1) * (0.2452727 + 0.0412496 * m1) * m1;
  return h;
}

// neldermead_simplex (Superquadrics_Ig2.cpp:1701-1878) restated as a state machine that asks
// for exactly one Disfun evaluation per step: the three vertices of the first simplex, then
// per iteration a reflection, an expansion or contraction, and the shrink evaluations.  The
// decisions and the arithmetic are the reference's (amotry, :1668-1700); the evaluation
// counter starts at 0 (the reference leaves it uninitialised).
enum { NM_V0 = 0, NM_V1 = 1, NM_V2 = 2, NM_REFLECT, NM_EXPAND, NM_CONTRACT, NM_SHRINK };
static const double NM_FTOL = 1e-3, NM_TINY = 1.0e-10;
static const int NM_NMAX = 5000;

struct NMState {
  int st, nfunc, ilo, ihi, inhi, si;
  bool touching;
  double p[3][2], y[3], psum[2], ptry[2], ysave;
  double q0, q1;       // the point asked for
  double r0, r1, dist; // result: returned vertex and its distance
};

__device__ __forceinline__ void nmStart(NMState& M, double a0, double a1, double del) {
  for (int i = 0; i < 3; i++) { M.p[i][0] = a0; M.p[i][1] = a1; }
  M.p[1][0] += del;
  M.p[2][1] += del;
  M.nfunc = 0; M.touching = true; M.st = NM_V0;
  M.ilo = 0; M.ihi = 0; M.inhi = 0; M.si = 0;   // set by the ranking after the first simplex
  M.q0 = M.p[0][0]; M.q1 = M.p[0][1];
}
__device__ __forceinline__ bool nmReturn(NMState& M) {
  M.r0 = M.p[0][0]; M.r1 = M.p[0][1]; M.dist = M.y[0];
  return false;
}
// amotry's trial point for the factor fac through the face opposite the high vertex
__device__ __forceinline__ void nmTry(NMState& M, double fac, int st) {
  const double fac1 = (1.0 - fac) / 2.0;
  const double fac2 = fac1 - fac;
  M.ptry[0] = M.psum[0] * fac1 - M.p[M.ihi][0] * fac2;
  M.ptry[1] = M.psum[1] * fac1 - M.p[M.ihi][1] * fac2;
  M.q0 = M.ptry[0]; M.q1 = M.ptry[1]; M.st = st;
}
// amotry's replacement of the high vertex by a better trial point
__device__ __forceinline__ void nmAccept(NMState& M, double ytry) {
  if (ytry < M.y[M.ihi]) {
    M.y[M.ihi] = ytry;
    M.psum[0] += M.ptry[0] - M.p[M.ihi][0];
    M.psum[1] += M.ptry[1] - M.p[M.ihi][1];
    M.p[M.ihi][0] = M.ptry[0]; M.p[M.ihi][1] = M.ptry[1];
  }
}
// top of the iteration: order the vertices, test convergence, ask for the reflection
__device__ __forceinline__ bool nmTop(NMState& M) {
  M.ilo = 0;
  if (M.y[0] > M.y[1]) { M.inhi = 1; M.ihi = 0; } else { M.inhi = 0; M.ihi = 1; }
  for (int i = 0; i < 3; i++) {
    if (M.y[i] <= M.y[M.ilo]) M.ilo = i;
    if (M.y[i] > M.y[M.ihi]) { M.inhi = M.ihi; M.ihi = i; }
    else if (M.y[i] > M.y[M.inhi] && i != M.ihi) M.inhi = i;
  }
  const double rtol = 2.0 * fabs(M.y[M.ihi] - M.y[M.ilo]) / (fabs(M.y[M.ihi]) + fabs(M.y[M.ilo]) + NM_TINY);
  if (rtol < NM_FTOL) {
    const int l = M.ilo;
    const double t = M.y[0]; M.y[0] = M.y[l]; M.y[l] = t;
    const double a = M.p[l][0], b = M.p[l][1];
    M.p[l][0] = M.p[0][0]; M.p[l][1] = M.p[0][1];
    M.p[0][0] = a; M.p[0][1] = b;
    return nmReturn(M);
  }
  if (M.nfunc >= NM_NMAX) return nmReturn(M);
  nmTry(M, -1.0, NM_REFLECT);
  return true;
}
// next vertex of the shrink towards the low vertex, or the top of the next iteration
__device__ __forceinline__ bool nmShrinkNext(NMState& M) {
  for (int i = M.si + 1; i < 3; i++) {
    if (i != M.ilo) {
      M.p[i][0] = M.psum[0] = 0.5 * (M.p[i][0] + M.p[M.ilo][0]);
      M.p[i][1] = M.psum[1] = 0.5 * (M.p[i][1] + M.p[M.ilo][1]);
      M.si = i; M.q0 = M.psum[0]; M.q1 = M.psum[1]; M.st = NM_SHRINK;
      return true;
    }
  }
  M.psum[0] = (M.p[0][0] + M.p[1][0]) + M.p[2][0];
  M.psum[1] = (M.p[0][1] + M.p[1][1]) + M.p[2][1];
  return nmTop(M);
}
// consume the evaluation f at the point asked for; returns true while the search continues
__device__ __forceinline__ bool nmConsume(NMState& M, double f, bool apart) {
  if (apart) M.touching = false;
  M.nfunc++;
  switch (M.st) {
    case NM_V0: case NM_V1: case NM_V2: {
      const int i = M.st;
      M.y[i] = f;
      if (!M.touching) return nmReturn(M);
      if (i < 2) { M.st = i + 1; M.q0 = M.p[i + 1][0]; M.q1 = M.p[i + 1][1]; return true; }
      M.psum[0] = (M.p[0][0] + M.p[1][0]) + M.p[2][0];
      M.psum[1] = (M.p[0][1] + M.p[1][1]) + M.p[2][1];
      return nmTop(M);
    }
    case NM_REFLECT:
      nmAccept(M, f);
      if (!M.touching) return nmReturn(M);
      if (f <= M.y[M.ilo]) { nmTry(M, 2.0, NM_EXPAND); return true; }
      if (f >= M.y[M.inhi]) { M.ysave = M.y[M.ihi]; nmTry(M, 0.5, NM_CONTRACT); return true; }
      return nmTop(M);
    case NM_EXPAND:
      nmAccept(M, f);
      if (!M.touching) return nmReturn(M);
      return nmTop(M);
    case NM_CONTRACT:
      nmAccept(M, f);
      if (!M.touching) return nmReturn(M);
      if (f >= M.ysave) { M.si = -1; return nmShrinkNext(M); }
      return nmTop(M);
    default:  // NM_SHRINK
      M.y[M.si] = f;
      if (!M.touching) return nmReturn(M);
      return nmShrinkNext(M);
  }
}

// amotry's trial point for the factor fac from the vertex sum ps and the high vertex ph
__device__ __forceinline__ double2 nmTryPoint(const double ps[2], const double ph[2], double fac) {
  const double fac1 = (1.0 - fac) / 2.0;
  const double fac2 = fac1 - fac;
  return make_double2(ps[0] * fac1 - ph[0] * fac2, ps[1] * fac1 - ph[1] * fac2);
}

// Points the search asks for after the one it asks for now, under the outcomes of that
// evaluation (written to q[1..], at most S - 1 of them; returns how many points, q[0] being
// the current one).  Every point is computed with the operations the state machine uses, so
// one that the search later asks for matches bit for bit.  The vertex order after an
// evaluation follows from the comparison that selects the branch (all values distinct).
__device__ __forceinline__ int nmPlan(const NMState& M, double2* q, int S) {
  int n = 0;
  q[n++] = make_double2(M.q0, M.q1);
  if (M.st == NM_V0 || M.st == NM_V1 || M.st == NM_V2) {
    // vertices of the first simplex still to be evaluated; after the third the next point
    // depends on the ranking, which is not known yet
    for (int v = M.st + 1; v < 3 && n < S; v++) q[n++] = make_double2(M.p[v][0], M.p[v][1]);
    return n;
  }
  const double* ph = M.p[M.ihi];
  double psA[2];   // vertex sum once the trial point replaces the high vertex
  psA[0] = M.psum[0] + (M.ptry[0] - ph[0]);
  psA[1] = M.psum[1] + (M.ptry[1] - ph[1]);
  if (M.st == NM_REFLECT) {
    // better than the best: expansion; worse than the second highest: contraction (from the
    // simplex with or without the trial point); in between: the next reflection, through the
    // old second-highest vertex, now the highest
    if (n < S) q[n++] = nmTryPoint(psA, M.ptry, 2.0);
    if (n < S) q[n++] = nmTryPoint(psA, M.ptry, 0.5);
    if (n < S) q[n++] = nmTryPoint(M.psum, ph, 0.5);
    if (n < S) q[n++] = nmTryPoint(psA, M.p[M.inhi], -1.0);
  } else if (M.st == NM_EXPAND) {
    // the expanded vertex stays the lowest; the next reflection goes through the old
    // second-highest vertex, with or without the expansion point in the sum
    if (n < S) q[n++] = nmTryPoint(psA, M.p[M.inhi], -1.0);
    if (n < S) q[n++] = nmTryPoint(M.psum, M.p[M.inhi], -1.0);
  } else {
    // a rejected contraction (or a shrink step) continues with the shrink towards the low vertex
    const int from = M.st == NM_SHRINK ? M.si + 1 : 0;
    for (int i = from; i < 3 && n < S; i++)
      if (i != M.ilo) {
        q[n++] = make_double2(0.5 * (M.p[i][0] + M.p[M.ilo][0]), 0.5 * (M.p[i][1] + M.p[M.ilo][1]));
        break;
      }
  }
  return n;
}

}  // namespace sqdem
