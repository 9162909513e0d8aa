// The search of lmder2 (pkg/dem/Superquadrics_Ig2.cpp:1057-1354) in double-float arithmetic:
// the state machine of the mixed form's lanes, with every decision guarded by its rounding band
// (LMF_DEFER: the caller hands the search to the FP64 path).  __host__ __device__, so that the
// CPU tests run whole searches with it against the oracle's lmder2.
#pragma once
#include "sq_ff.cuh"

namespace sqdem {

enum { LMF_ST_INIT = 1, LMF_ST_PROBE0 = 2, LMF_ST_PROBE1 = 3, LMF_ST_TRIAL = 4 };

struct LMF {
  int e, st, phase, k, stop, nu;
  bool stopFlag, touching, isNew, fromCenter;
  ff p0, p1, q0, q1, mu, Dp0, Dp1, pfL2;
  ff j00, j01, j11, diag0, diag1, jt0, jt1;
  ff pf[3], f1[3], c[3], P1[3], P2[3];
  float E;
  unsigned calls, iters, maxit, rounds;
  float pad;   // 73 words: an odd stride, so the lanes' states in shared memory fall in distinct banks
};
enum { LMF_MORE = 0, LMF_END = 1, LMF_DEFER = 2 };

FFH ff ffInitStep() { return ffFromD(1e-7); }

FFH void lmfStartSolve(LMF& L) {
  L.touching = true; L.stopFlag = false; L.stop = 0;
  L.q0 = L.p0; L.q1 = L.p1; L.st = LMF_ST_INIT;
}

// top of lmder2's for-loop: loop condition, then the checks before the Jacobian (a called
// function, as lmfInner and the damped solve: inlined, their copies at every call site overflow
// the instruction cache)
FFN int lmfOuter(LMF& L) {
  // A search that reaches itmax (stop 3) is still moving after 50 iterations: along such a
  // path the difference between double-float and FP64 rounding, amplified by the 1e-7
  // finite-difference steps, compounds, so it is deferred to the FP64 path.
  if (L.k >= 50) return LMF_DEFER;
  if (L.stop) return LMF_END;
  if (L.pfL2.hi < L.E) return LMF_DEFER;   // p_fL2 <= 1e-20 (stop 6) within the band
  if (L.stopFlag) { L.stop = 9; L.touching = false; return LMF_END; }
  // |cos(f, c)| > 0.95  <=>  (f.c)^2 > 0.95^2 |f|^2 |c|^2
  const ff fc = ffDot3(L.pf[0], L.pf[1], L.pf[2], L.c[0], L.c[1], L.c[2]);
  const ff f2 = ffDot3(L.pf[0], L.pf[1], L.pf[2], L.pf[0], L.pf[1], L.pf[2]);
  const ff c2 = ffDot3(L.c[0], L.c[1], L.c[2], L.c[0], L.c[1], L.c[2]);
  const ff th = ffFromD(0.95);
  const ff diff = ffSub(ffMul(fc, fc), ffMul(ffMul(th, th), ffMul(f2, c2)));
  const float band = 1.9f * (1e-12f * f2.hi + 4.f * L.E * sqrtf(f2.hi)) * c2.hi;
  if (!(fabsf(diff.hi) >= band)) return LMF_DEFER;
  if (diff.hi > 0.f) { L.stop = 8; return LMF_END; }
  L.q0 = ffAdd(L.p0, L.Dp0); L.q1 = L.p1; L.st = LMF_ST_PROBE0;
  return LMF_MORE;
}
// the damped step (jtj + mu I) Dp = jt
struct LMFStep { ff Dp0, Dp1, dp2; };
FFN LMFStep lmfSolveV(ff j00, ff j01, ff j11, ff jt0, ff jt1) {
  LMFStep r;
  const ff inv = ffDiv(mkff(1.f, 0.f), ffSub(ffMul(j00, j11), ffMul(j01, j01)));
  r.Dp0 = ffMul(ffSub(ffMul(jt0, j11), ffMul(jt1, j01)), inv);
  r.Dp1 = ffMul(ffSub(ffMul(jt1, j00), ffMul(jt0, j01)), inv);
  r.dp2 = ffAdd(ffMul(r.Dp0, r.Dp0), ffMul(r.Dp1, r.Dp1));
  return r;
}
FFH void lmfSolve(ff j00, ff j01, ff j11, ff jt0, ff jt1, ff& Dp0, ff& Dp1, ff& dp2) {
  const LMFStep r = lmfSolveV(j00, j01, j11, jt0, jt1);
  Dp0 = r.Dp0; Dp1 = r.Dp1; dp2 = r.dp2;
}
// top of the damping while-loop
FFN int lmfInner(LMF& L) {
  L.j00 = ffAdd(L.j00, L.mu);
  L.j11 = ffAdd(L.j11, L.mu);
  ff dp2;
  lmfSolve(L.j00, L.j01, L.j11, L.jt0, L.jt1, L.Dp0, L.Dp1, dp2);
  // ||Dp|| < 1e-5  <=>  ||Dp||^2 < 1e-10
  if (!(fabsf(dp2.hi * 1e10f - 1.f) >= 2e-5f)) return LMF_DEFER;
  if (dp2.hi < 1e-10f) { L.stop = 2; L.k++; return lmfOuter(L); }
  L.q0 = ffAdd(L.p0, L.Dp0); L.q1 = ffAdd(L.p1, L.Dp1);
  const float pL2 = sqrtf(L.p0.hi * L.p0.hi + L.p1.hi * L.p1.hi);
  if (sqrtf(dp2.hi) >= (pL2 + 1e-3f) * 1e24f) { L.stop = 4; L.k++; return lmfOuter(L); }
  L.st = LMF_ST_TRIAL;
  return LMF_MORE;
}
// consume the evaluation the lane asked for
FFH int lmfConsume(LMF& L, const FFEval& v) {
  if (v.ill) return LMF_DEFER;
  if (!(fabsf(v.sep.hi) >= L.E)) return LMF_DEFER;
  if (v.sep.hi > 0.f) L.stopFlag = true;
  for (int i = 0; i < 3; i++) { L.P1[i] = v.p1[i]; L.P2[i] = v.p2[i]; }
  switch (L.st) {
    case LMF_ST_INIT:
      for (int i = 0; i < 3; i++) { L.pf[i] = v.d[i]; L.c[i] = v.c[i]; }
      L.pfL2 = ffSqrt(ffDot3(L.pf[0], L.pf[1], L.pf[2], L.pf[0], L.pf[1], L.pf[2]));
      L.k = 0; L.mu = mkff(0.f, 0.f); L.nu = 2; L.Dp0 = ffInitStep(); L.Dp1 = ffInitStep();
      return lmfOuter(L);
    case LMF_ST_PROBE0:
      for (int i = 0; i < 3; i++) L.f1[i] = v.d[i];
      L.q0 = L.p0; L.q1 = ffAdd(L.p1, L.Dp1); L.st = LMF_ST_PROBE1;
      return LMF_MORE;
    case LMF_ST_PROBE1: {
      const ff i0 = ffDiv(mkff(1.f, 0.f), L.Dp0), i1 = ffDiv(mkff(1.f, 0.f), L.Dp1);
      ff J0[3], J1[3];
      for (int i = 0; i < 3; i++) { J0[i] = ffMul(ffSub(L.f1[i], L.pf[i]), i0); J1[i] = ffMul(ffSub(v.d[i], L.pf[i]), i1); }
      L.j00 = ffDot3(J0[0], J0[1], J0[2], J0[0], J0[1], J0[2]);
      L.j01 = ffDot3(J0[0], J0[1], J0[2], J1[0], J1[1], J1[2]);
      L.j11 = ffDot3(J1[0], J1[1], J1[2], J1[0], J1[1], J1[2]);
      L.jt0 = ffNeg(ffDot3(J0[0], J0[1], J0[2], L.pf[0], L.pf[1], L.pf[2]));
      L.jt1 = ffNeg(ffDot3(J1[0], J1[1], J1[2], L.pf[0], L.pf[1], L.pf[2]));
      const float jinf = fmaxf(fabsf(L.jt0.hi), fabsf(L.jt1.hi));
      if (!(fabsf(jinf * 1e15f - 1.f) >= 1e-5f)) return LMF_DEFER;
      if (jinf <= 1e-15f) { L.stop = 1; return LMF_END; }
      if (L.k == 0) L.mu = ffGt(L.j00, L.j11) ? L.j00 : L.j11;
      L.diag0 = L.j00; L.diag1 = L.j11;
      return lmfInner(L);
    }
    default: {  // LMF_ST_TRIAL
      const ff pdL2 = ffSqrt(ffDot3(v.d[0], v.d[1], v.d[2], v.d[0], v.d[1], v.d[2]));
      const ff dF = ffSub(L.pfL2, pdL2);
      if (!(fabsf(dF.hi) >= L.E)) return LMF_DEFER;
      if (dF.hi > 0.f) {   // dF / dL > 0: dL = 2 mu |Dp|^2 + |J Dp|^2 > 0
        const ff dL = ffAdd(ffMul(L.Dp0, ffAdd(ffMul(L.mu, L.Dp0), L.jt0)), ffMul(L.Dp1, ffAdd(ffMul(L.mu, L.Dp1), L.jt1)));
        const ff t = ffAddF(ffMulF(ffDiv(dF, dL), 2.f), -1.f);
        const ff tmp = ffAddF(ffNeg(ffMul(ffMul(t, t), t)), 1.f);
        const ff third = ffFromD(0.3333333333333334);
        L.mu = ffMul(L.mu, ffGt(third, tmp) ? third : tmp);
        L.nu = 2;
        L.p0 = L.q0; L.p1 = L.q1;
        for (int i = 0; i < 3; i++) { L.pf[i] = v.d[i]; L.c[i] = v.c[i]; }
        L.pfL2 = pdL2;
        L.k++;
        return lmfOuter(L);
      }
      L.mu = ffMulF(L.mu, (float)L.nu);
      const int nu2 = (int)((unsigned)L.nu << 1);
      if (nu2 <= L.nu) { L.stop = 5; L.k++; return lmfOuter(L); }
      L.nu = nu2;
      L.j00 = L.diag0; L.j11 = L.diag1;
      return lmfInner(L);
    }
  }
}

// Points the search evaluates next (as lmPlan does for the FP64 kernel), computed with the
// state machine's own double-float operations so that a planned point equals bit for bit the
// one the search later asks for.
FFH void lmfPlan(const LMF& L, float4* q, int* own, int S, int lane) {
  int n = 0;
  q[n] = make_float4(L.q0.hi, L.q0.lo, L.q1.hi, L.q1.lo); own[n++] = lane;
  if (L.st == LMF_ST_INIT) {
    const ff a = ffAdd(L.p0, ffInitStep()), b = ffAdd(L.p1, ffInitStep());
    if (n < S) { q[n] = make_float4(a.hi, a.lo, L.p1.hi, L.p1.lo); own[n++] = lane; }
    if (n < S) { q[n] = make_float4(L.p0.hi, L.p0.lo, b.hi, b.lo); own[n++] = lane; }
  } else if (L.st == LMF_ST_PROBE0) {
    const ff b = ffAdd(L.p1, L.Dp1);
    if (n < S) { q[n] = make_float4(L.p0.hi, L.p0.lo, b.hi, b.lo); own[n++] = lane; }
  } else if (L.st == LMF_ST_TRIAL) {
    ff mu = L.mu, t0 = L.q0, t1 = L.q1, d0 = L.Dp0, d1 = L.Dp1;
    int nu = L.nu;
    while (n < S) {
      const ff a = ffAdd(t0, d0), b = ffAdd(t1, d1);
      q[n] = make_float4(a.hi, a.lo, t1.hi, t1.lo); own[n++] = lane;
      if (n >= S) break;
      q[n] = make_float4(t0.hi, t0.lo, b.hi, b.lo); own[n++] = lane;
      if (n >= S) break;
      mu = ffMulF(mu, (float)nu);
      const int nu2 = (int)((unsigned)nu << 1);
      if (nu2 <= nu) break;
      nu = nu2;
      ff dp2;
      lmfSolve(ffAdd(L.diag0, mu), L.j01, ffAdd(L.diag1, mu), L.jt0, L.jt1, d0, d1, dp2);
      if (dp2.hi < 1e-10f) break;
      t0 = ffAdd(L.p0, d0); t1 = ffAdd(L.p1, d1);
      q[n] = make_float4(t0.hi, t0.lo, t1.hi, t1.lo); own[n++] = lane;
    }
  }
}
FFH bool sameFF(float4 a, ff q0, ff q1) {
  return ffBits(a.x) == ffBits(q0.hi) && ffBits(a.y) == ffBits(q0.lo) &&
         ffBits(a.z) == ffBits(q1.hi) && ffBits(a.w) == ffBits(q1.lo);
}


}  // namespace sqdem
