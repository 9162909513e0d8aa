// Host build of the mixed form's double-float Disfunction (test infrastructure only).
//
// sq_ff.cuh's routines are __host__ __device__ and use only IEEE float operations and fmaf, so
// this host build computes what the kernels compute, bit for bit; the CPU tests compare it with
// the oracle's FP64 Disfunction.  Nothing here is loaded by the package.
#include "../sudodem_gb300/csrc/sq_ff.cuh"
#include <cmath>

using namespace sqdem;

static void hostShape(SqShape& s, const double* shape5, const double* q, const double* pos) {
  double w = q[0], x = q[1], y = q[2], z = q[3];
  // Eigen's normalize (Superquadrics::setOrientation): squaredNorm = (x^2 + y^2) + (z^2 + w^2)
  const double n = std::sqrt((x * x + y * y) + (z * z + w * w));
  w /= n; x /= n; y /= n; z /= n;
  double rmax = shape5[0] > shape5[1] ? shape5[0] : shape5[1];
  rmax = rmax > shape5[2] ? rmax : shape5[2];
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
