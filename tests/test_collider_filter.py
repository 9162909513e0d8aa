"""The collider's FP32 decision of the periodic overlap test (overlapPeriFast) agrees with the
exact FP64 restatement of InsertionSortCollider::spatialOverlapPeri
(InsertionSortCollider.cpp:491-543, overlapPeri) on every pair it decides.

Both functions are taken from the CUDA source and compiled as host code; random and
adversarial bound pairs (touching bounds, equal lower bounds, offsets near half the cell,
bodies many periods apart, bodies longer than a quarter cell) are checked.  CPU only.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "sudodem_gb300", "csrc", "sqdem_engine.cu")

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
using std::floor; using std::fabs;
struct double4 { double x, y, z, w; };
struct float4 { float x, y, z, w; };
struct SceneState { double cellSize[3]; };
static inline double comp(double4 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
static inline float4 mk4(float a, float b, float c) { float4 r; r.x = a; r.y = b; r.z = c; r.w = 0; return r; }
@FUNCS@
int main(int argc, char** argv) {
  std::mt19937_64 rng(atoll(argv[1]));
  const long long npairs = atoll(argv[2]);
  std::uniform_real_distribution<double> U(0, 1);
  long long decided = 0, wrong = 0;
  for (long long it = 0; it < npairs; it++) {
    SceneState S;
    double L[3], c1[3], h1[3], c2[3], h2[3];
    const int mode = (int)(it % 6);
    for (int k = 0; k < 3; k++) {
      const double D = 0.01 + 0.2 * U(rng);
      L[k] = D; S.cellSize[k] = D;
      h1[k] = D * (mode == 5 ? 0.3 * U(rng) : 0.03 * U(rng));
      h2[k] = D * (mode == 5 ? 0.3 * U(rng) : 0.03 * U(rng));
      c1[k] = (U(rng) - 0.5) * D * (mode == 4 ? 40 : 3);
      double off;
      switch (mode) {
        case 0: off = (U(rng) - 0.5) * 4 * (h1[k] + h2[k]); break;
        case 1: off = (h1[k] + h2[k]) * (1 + (U(rng) - 0.5) * 1e-6); break;
        case 2: off = (h1[k] - h2[k]) + (U(rng) - 0.5) * 1e-9 * D; break;
        case 3: off = 0.5 * D + (U(rng) - 0.5) * 1e-6 * D; break;
        default: off = (U(rng) - 0.5) * D; break;
      }
      c2[k] = c1[k] + off + (int)((U(rng) - 0.5) * (mode == 4 ? 20 : 4)) * D;
    }
    double4 mn1 = {c1[0] - h1[0], c1[1] - h1[1], c1[2] - h1[2], 0}, mx1 = {c1[0] + h1[0], c1[1] + h1[1], c1[2] + h1[2], 0};
    double4 mn2 = {c2[0] - h2[0], c2[1] - h2[1], c2[2] - h2[2], 0}, mx2 = {c2[0] + h2[0], c2[1] + h2[1], c2[2] + h2[2], 0};
    int per[3];
    const bool exact = overlapPeri(S, mn1, mx1, mn2, mx2, per);
    // FP32 centres and half extents as the cell binning forms them
    float4 fc1 = mk4((float)(0.5 * (mn1.x + mx1.x)), (float)(0.5 * (mn1.y + mx1.y)), (float)(0.5 * (mn1.z + mx1.z)));
    float4 fh1 = mk4((float)(0.5 * (mx1.x - mn1.x)), (float)(0.5 * (mx1.y - mn1.y)), (float)(0.5 * (mx1.z - mn1.z)));
    float4 fc2 = mk4((float)(0.5 * (mn2.x + mx2.x)), (float)(0.5 * (mn2.y + mx2.y)), (float)(0.5 * (mn2.z + mx2.z)));
    float4 fh2 = mk4((float)(0.5 * (mx2.x - mn2.x)), (float)(0.5 * (mx2.y - mn2.y)), (float)(0.5 * (mx2.z - mn2.z)));
    float Lf[3], iL[3];
    for (int k = 0; k < 3; k++) { Lf[k] = (float)L[k]; iL[k] = 1.f / Lf[k]; }
    const int f = overlapPeriFast(fc1, fh1, fc2, fh2, Lf, iL);
    if (f != 0) { decided++; if ((f > 0) != exact) wrong++; }
  }
  printf("%lld %lld\n", decided, wrong);
  return 0;
}
"""


def _grab(src, sig):
    a = src.index(sig)
    b = src.index("\n}\n", a) + 3
    return src[a:b].replace("__device__ __forceinline__", "static inline")


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_periodic_overlap_fast_decision_matches_exact():
    src = open(SRC).read()
    funcs = "\n".join(_grab(src, s) for s in (
        "__device__ __forceinline__ double cellWrapD(", "__device__ __forceinline__ double cellWrapRelD(",
        "__device__ __forceinline__ bool overlapPeri(", "__device__ __forceinline__ int overlapPeriFast("))
    with tempfile.TemporaryDirectory() as tmp:
        cpp, exe = os.path.join(tmp, "h.cpp"), os.path.join(tmp, "h")
        with open(cpp, "w") as f:
            f.write(HARNESS.replace("@FUNCS@", funcs))
        subprocess.run(["g++", "-O2", "-ffp-contract=off", "-o", exe, cpp], check=True)
        total = 0
        for seed in (11, 12):
            out = subprocess.run([exe, str(seed), "1500000"], check=True, capture_output=True, text=True).stdout
            decided, wrong = map(int, out.split())
            assert wrong == 0
            total += decided
        assert total > 2_000_000   # most pairs are decided without the exact test
