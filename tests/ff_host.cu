// Host build of the mixed form's double-float Disfunction (test infrastructure only).
//
// sq_ff.cuh's routines are __host__ __device__ and use only IEEE float operations and fmaf, so
// this host build computes what the kernels compute, bit for bit; the CPU tests compare it with
// the oracle's FP64 Disfunction.  Nothing here is loaded by the package.
#include "../sudodem_gb300/csrc/sq_lmff.cuh"
#include <cmath>

using namespace sqdem;

// renorm: normalise the quaternion as Superquadrics::setOrientation does (a body being created);
// 0: use it as stored (a body's current orientation, as the engines do)
static void hostShape(SqShape& s, const double* shape5, const double* q, const double* pos, int renorm = 1) {
  double w = q[0], x = q[1], y = q[2], z = q[3];
  if (renorm) {
    // Eigen's normalize: squaredNorm = (x^2 + y^2) + (z^2 + w^2)
    const double n = std::sqrt((x * x + y * y) + (z * z + w * w));
    w /= n; x /= n; y /= n; z /= n;
  }
  // r_max of Superquadrics::Initial (Superquadrics.cpp:47-93)
  double rmax = shape5[0] > shape5[1] ? shape5[0] : shape5[1];
  rmax = rmax > shape5[2] ? rmax : shape5[2];
  if (shape5[3] < 1.0 || shape5[4] < 1.0) rmax *= std::pow(2.0, 0.5);
  shapeInit(s, shape5[0], shape5[1], shape5[2], shape5[3], shape5[4], rmax);
  s.R = quatToRot(w, x, y, z);
  s.pos = d3(pos[0], pos[1], pos[2]);
}

// out: p1 (3), p2 (3) relative to A's centre, d = p2 - p1 (3), sep, ill, contact (3), as doubles
extern "C" void ffh_disfunction(const double* shapeA5, const double* qA, const double* posA, const double* shapeB5,
                                const double* qB, const double* posB, double pa0, double pa1, double* out) {
  SqShape A, B;
  hostShape(A, shapeA5, qA, posA);
  hostShape(B, shapeB5, qB, posB);
  FFPair P;
  ffPairInit(P, A, B);
  FFEval r;
  ffDisfunction(P, pa0, pa1, r);
  for (int i = 0; i < 3; i++) {
    out[i] = ffToD(r.p1[i]); out[3 + i] = ffToD(r.p2[i]); out[6 + i] = ffToD(r.d[i]); out[11 + i] = ffToD(r.c[i]);
  }
  out[9] = ffToD(r.sep);
  out[10] = r.ill ? 1 : 0;
}

// elementary functions, for their own tests: op 0 log2, 1 exp2 (x as double -> ff), 2 sin, 3 cos
extern "C" void ffh_elem(int op, const double* x, long n, double* out) {
  for (long i = 0; i < n; i++) {
    ff s, c;
    switch (op) {
      case 0: out[i] = ffToD(ffLog2(ffFromD(x[i]))); break;
      case 1: out[i] = ffToD(ffExp2(ffFromD(x[i]))); break;
      case 2: ffSinCos(x[i], s, c); out[i] = ffToD(s); break;
      default: ffSinCos(x[i], s, c); out[i] = ffToD(c); break;
    }
  }
}

// One lmder2 call with the double-float state machine of the mixed form, from angles p0 (2).
// out: angles (2), p1 (3), p2 (3) relative to A's centre, contact (3), touching, iterations,
// stop code, evaluations, outcome (1 ended, 2 deferred to FP64).
extern "C" void ffh_lmder2(const double* shapeA5, const double* qA, const double* posA, const double* shapeB5,
                           const double* qB, const double* posB, const double* p0, double* out, int renorm) {
  SqShape A, B;
  hostShape(A, shapeA5, qA, posA, renorm);
  hostShape(B, shapeB5, qB, posB, renorm);
  FFPair P;
  ffPairInit(P, A, B);
  LMF L;
  L.p0 = ffFromD(p0[0]); L.p1 = ffFromD(p0[1]);
  L.E = 4e-13f * (P.A.rmax + P.B.rmax);
  L.touching = true;
  for (int i = 0; i < 3; i++) L.c[i] = L.P1[i] = L.P2[i] = mkff(0.f, 0.f);
  lmfStartSolve(L);
  int r = LMF_MORE, evals = 0;
  while (r == LMF_MORE && evals < 100000) {
    FFEval v;
    ffDisfunction(P.A, P.B, P.pB, L.q0, L.q1, v);
    evals++;
    r = lmfConsume(L, v);
  }
  out[0] = ffToD(L.p0); out[1] = ffToD(L.p1);
  for (int i = 0; i < 3; i++) { out[2 + i] = ffToD(L.P1[i]); out[5 + i] = ffToD(L.P2[i]); out[8 + i] = ffToD(L.c[i]); }
  out[11] = L.touching ? 1 : 0; out[12] = L.k; out[13] = L.stop; out[14] = evals; out[15] = r;
}

// The same evaluation as tests/ff_device_probe.cu's kernel, on the host: in 26 doubles per case
// (shapeA5, qA4 used as given, posA3, shapeB5, qB4, posB3, pa0, pa1), out 14 doubles.
extern "C" void ffh_disfunction_raw(const double* in, long n, double* out) {
  for (long i = 0; i < n; i++) {
    const double* v = in + 26 * i;
    SqShape A, B;
    double ra = v[0] > v[1] ? v[0] : v[1]; ra = ra > v[2] ? ra : v[2];
    double rb = v[12] > v[13] ? v[12] : v[13]; rb = rb > v[14] ? rb : v[14];
    shapeInit(A, v[0], v[1], v[2], v[3], v[4], ra);
    A.R = quatToRot(v[5], v[6], v[7], v[8]);
    A.pos = d3(v[9], v[10], v[11]);
    shapeInit(B, v[12], v[13], v[14], v[15], v[16], rb);
    B.R = quatToRot(v[17], v[18], v[19], v[20]);
    B.pos = d3(v[21], v[22], v[23]);
    FFPair P;
    ffPairInit(P, A, B);
    FFEval r;
    ffDisfunction(P, v[24], v[25], r);
    double* o = out + 14 * i;
    for (int k = 0; k < 3; k++) { o[k] = ffToD(r.p1[k]); o[3 + k] = ffToD(r.p2[k]); o[6 + k] = ffToD(r.d[k]); o[11 + k] = ffToD(r.c[k]); }
    o[9] = ffToD(r.sep);
    o[10] = r.ill ? 1 : 0;
  }
}
