// Device side of the double-float routines for the CPU/GPU equality test (test infrastructure
// only): the same sq_ff.cuh functions as tests/ff_host.cu, evaluated by a kernel, so that a GPU
// test can compare the device's results with the host build's bit for bit.
#include "../sudodem_gb300/csrc/sq_lmff.cuh"
#include <cuda_runtime.h>

using namespace sqdem;

__global__ void k_probe_elem(int op, const double* x, long n, double* out) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  ff s, c;
  switch (op) {
    case 0: out[i] = ffToD(ffLog2(ffFromD(x[i]))); break;
    case 1: out[i] = ffToD(ffExp2(ffFromD(x[i]))); break;
    case 2: ffSinCos(x[i], s, c); out[i] = ffToD(s); break;
    default: ffSinCos(x[i], s, c); out[i] = ffToD(c); break;
  }
}

// in: per case shapeA5, qA4, posA3, shapeB5, qB4, posB3, pa0, pa1 (26 doubles; quaternions used
// as given); out: p1 (3), p2 (3), d (3), sep, ill, contact (3) relative to A's centre (14)
__global__ void k_probe_disf(const double* in, long n, double* out) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
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

static int run(const double* hin, size_t nin, double* hout, size_t nout, int which, int op, long n) {
  double *din = nullptr, *dout = nullptr;
  if (cudaMalloc(&din, nin * 8) != cudaSuccess || cudaMalloc(&dout, nout * 8) != cudaSuccess) return 1;
  cudaMemcpy(din, hin, nin * 8, cudaMemcpyHostToDevice);
  const int bs = 128;
  const int nb = (int)((n + bs - 1) / bs);
  if (which == 0) k_probe_elem<<<nb, bs>>>(op, din, n, dout);
  else k_probe_disf<<<nb, bs>>>(din, n, dout);
  cudaError_t e = cudaMemcpy(hout, dout, nout * 8, cudaMemcpyDeviceToHost);
  cudaFree(din);
  cudaFree(dout);
  return e == cudaSuccess && cudaGetLastError() == cudaSuccess ? 0 : 2;
}

extern "C" int ffd_elem(int op, const double* x, long n, double* out) { return run(x, n, out, n, 0, op, n); }
extern "C" int ffd_disfunction(const double* in26, long n, double* out14) { return run(in26, 26 * n, out14, 14 * n, 1, 0, n); }
