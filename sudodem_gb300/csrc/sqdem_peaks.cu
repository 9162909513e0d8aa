// Pipe peaks of the GPU the library runs on: the denominators of the contact stage's roofline.
//
// The contact stage is bound by instruction issue, not by HBM bytes: its Levenberg-Marquardt
// searches spend their time in Disfunction evaluations (pkg/dem/Superquadrics_Ig2.cpp:622-687),
// each ~18 pow + 4 atan2 + 6 sincos.  These kernels measure, on the device itself:
//   * the FP64 and FP32 fused multiply-add rates (independent FMA chains, 2 flops each);
//   * the rate of FP64 Disfunction evaluations when every lane of a full grid evaluates
//     independent points (the evaluation-mix peak that bounds k_contacts_lm).
// No counterpart in the reference.  Compiled with --fmad=false like the engine; the FMA loops
// use explicit fma() / fmaf() so they still issue fused multiply-adds.
#include <cuda_runtime.h>
#include <cstdint>
#include "sq_device.cuh"
#include "sq_ff.cuh"
#include "../../include/sqdem.h"

namespace sqpeak {
using namespace sqdem;

static const int PK_BS = 256;

__global__ void __launch_bounds__(PK_BS) k_peak_dfma(double* out, int iters) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double a0 = 1.0 + 1e-9 * t, a1 = a0 + 1e-3, a2 = a0 + 2e-3, a3 = a0 + 3e-3;
  double a4 = a0 + 4e-3, a5 = a0 + 5e-3, a6 = a0 + 6e-3, a7 = a0 + 7e-3;
  const double b = 0.999999999, c = 1e-10;
  for (int i = 0; i < iters; i++) {
    a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
  }
  const double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == 12345.678) out[0] = s;   // keeps the chains live; never true
}

__global__ void __launch_bounds__(PK_BS) k_peak_ffma(float* out, int iters) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  float a[16];
  for (int k = 0; k < 16; k++) a[k] = 1.0f + 1e-6f * (t & 1023) + 1e-3f * k;
  const float b = 0.9999999f, c = 1e-7f;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 16; k++) a[k] = fmaf(a[k], b, c);
  }
  float s = 0;
  for (int k = 0; k < 16; k++) s += a[k];
  if (s == 12345.678f) out[0] = s;
}

// A deterministic pseudo-random shape pair per thread (half-axes 0.8-1.2 mm, exponents
// 0.3-1.8, unit quaternions), centres 1.9 mm apart: the inputs of a typical contact.
__device__ __forceinline__ double hrand(uint32_t& s) {
  s = s * 1664525u + 1013904223u;
  return (s >> 8) * (1.0 / 16777216.0);
}
__device__ __forceinline__ void randomPair(int t, SqShape& A, SqShape& B) {
  uint32_t s = 0x9e3779b9u ^ (uint32_t)t * 2654435761u;
  for (int body = 0; body < 2; body++) {
    SqShape& S = body ? B : A;
    const double rx = 0.8e-3 + 0.4e-3 * hrand(s), ry = 0.8e-3 + 0.4e-3 * hrand(s), rz = 0.8e-3 + 0.4e-3 * hrand(s);
    const double e1 = 0.3 + 1.5 * hrand(s), e2 = 0.3 + 1.5 * hrand(s);
    shapeInit(S, rx, ry, rz, e1, e2, 1.2e-3 * 1.4142135623730951);
    double w = hrand(s) - 0.5, x = hrand(s) - 0.5, y = hrand(s) - 0.5, z = hrand(s) - 0.5;
    const double n = sqrt(w * w + x * x + y * y + z * z);
    S.R = quatToRot(w / n, x / n, y / n, z / n);
    S.pos = d3(body ? 1.9e-3 : 0.0, 0.0, 0.0);
  }
}

__global__ void __launch_bounds__(PK_BS) k_peak_disf64(double* out, int evals) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  SqShape A, B;
  randomPair(t, A, B);
  double acc = 0, p0 = 1e-5 + 1e-4 * (t & 255), p1 = 1e-5;
  for (int i = 0; i < evals; i++) {
    D3 C, P1, P2;
    bool f = false;
    disfunction(A, B, p0, p1, C, P1, P2, f);
    acc += P2.x - P1.x;
    p0 += 1e-3; p1 -= 7e-4;
  }
  if (acc == 12345.678) out[0] = acc;
}

__global__ void __launch_bounds__(PK_BS) k_peak_disff(double* out, int evals) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  SqShape A, B;
  randomPair(t, A, B);
  FFPair P;
  ffPairInit(P, A, B);
  double acc = 0, p0 = 1e-5 + 1e-4 * (t & 255), p1 = 1e-5;
  for (int i = 0; i < evals; i++) {
    FFEval r;
    ffDisfunction(P, p0, p1, r);
    acc += r.d[0].hi;
    p0 += 1e-3; p1 -= 7e-4;
  }
  if (acc == 12345.678) out[0] = acc;
}

}  // namespace sqpeak

using namespace sqpeak;

extern "C" sqdem_status sqdem_pipe_peaks(int device, double* out) {
  if (!out) return SQDEM_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return SQDEM_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return SQDEM_ERR_CUDA;
  double* d = nullptr;
  if (cudaMalloc(&d, 64) != cudaSuccess) return SQDEM_ERR_CUDA;
  cudaStream_t s;
  cudaEvent_t e0, e1;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto timeIt = [&](auto launch) {
    launch();   // warm-up
    cudaEventRecord(e0, s);
    launch();
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    return (double)ms;
  };
  const int fmaBlocks = sms * 8, fmaIters = 1 << 14;
  const double fmaThreads = (double)fmaBlocks * PK_BS;
  double ms = timeIt([&] { k_peak_dfma<<<fmaBlocks, PK_BS, 0, s>>>(d, fmaIters / 4); });
  out[0] = fmaThreads * (fmaIters / 4) * 8 * 2 / (ms * 1e-3) / 1e12;
  ms = timeIt([&] { k_peak_ffma<<<fmaBlocks, PK_BS, 0, s>>>((float*)d, fmaIters); });
  out[1] = fmaThreads * fmaIters * 16 * 2 / (ms * 1e-3) / 1e12;
  const int evBlocks = sms * 4, ev64 = 8, evff = 64;
  const double evThreads = (double)evBlocks * PK_BS;
  ms = timeIt([&] { k_peak_disf64<<<evBlocks, PK_BS, 0, s>>>(d, ev64); });
  out[2] = evThreads * ev64 / (ms * 1e-3) / 1e9;
  ms = timeIt([&] { k_peak_disff<<<evBlocks, PK_BS, 0, s>>>(d, evff); });
  out[3] = evThreads * evff / (ms * 1e-3) / 1e9;
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  cudaFree(d);
  return err == cudaSuccess ? SQDEM_OK : SQDEM_ERR_CUDA;
}
