// libsqdem_gpu.so — GB300 (sm_103a) engine for SudoDEM3D's superellipsoid timestep.
//
// One timestep is this kernel sequence on the context stream (captured once in a CUDA
// graph and replayed):
//
//   k_gate          InsertionSortCollider::isActivated   (InsertionSortCollider.cpp:177-189)
//   collider pass   InsertionSortCollider::action        (InsertionSortCollider.cpp:191-400)
//     k_bounds        BoundDispatcher::processBody + Bo1_* (Dispatching.cpp:30-62,
//                     Superquadrics.cpp:639-686, Wall.cpp:13-21)
//     k_grid_setup / k_cell_count / scan / k_cell_scatter   counting-sort binning on a
//                     uniform grid whose cell is at least the largest bound extent
//     k_candidates    overlap tests against the 27 neighbour cells and the walls, then a
//                     sorted per-body candidate row merged with the body's previous row
//                     (conditionalyEraseNonReal + insert, InteractionContainer.cpp:13-39)
//     k_merge         writes the new contact table (rows ordered by partner id), keeping
//                     contact history for pairs that survive
//     k_pcount / k_pscatter / k_psort / k_wall_*   incidence lists for the force gather
//   k_contacts      InteractionLoop body: Ig2_* + Ip2_* + SuperquadricsLaw
//                   (InteractionLoop.cpp:56-141; Superquadrics_Ig2.cpp:1880-2317,2522-2611;
//                   Superquadrics.cpp:1030-1116,1181-1363)
//   k_wall_forces   ForceContainer sum for walls (ForceContainer.hpp:134-162)
//   k_integrate     ForceContainer sum for particles + NewtonIntegrator::action
//                   (NewtonIntegrator.cpp:99-304)
//   k_end           Scene::moveToNextTimeStep epilogue (Scene.cpp:114-115)
//
// Collider kernels return at once when k_gate decided the collider does not run this step.
// Compiled with --fmad=false: FP64 results keep the reference's rounding sequence up to the
// last-ulp differences between CUDA's and glibc's pow/atan2/sin/cos.
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <cmath>
#include <vector>
#include <string>
#include <algorithm>
#include <limits>
#include <mutex>
#include "sq_device.cuh"
#include "sq_hm.cuh"
#include "sq_ff.cuh"
#include "sq_lmff.cuh"
#include "../../include/sqdem.h"

// Work queue of the contact stage for sqdem_contacts_static_queue: a fixed device array so
// that entry point needs no allocation.  Every GPU that loads the library holds it (4 MiB)
// until the process exits; all calls share it.  SQDEM_STATIC_QUEUE_MAX comes from sqdem.h.
static __device__ __align__(256) int g_static_lm_queue[SQDEM_STATIC_QUEUE_MAX];

namespace sqdem {

// ---------------------------------------------------------------------------
// Device-side state
enum : unsigned {
  F_GEOM = 1u,        // Interaction::geom present
  F_PHYS = 2u,        // Interaction::phys present
  F_SHEARNEW = 4u,    // SuperquadricsGeom::isShearNew
  F_OWNER_ID1 = 8u,   // the row owner is Interaction::id1 (else the partner is)
  F_FORCE = 16u,      // the law applied a force this step
};
// Bits 20-23 of an entry's flags: bit length of the Levenberg-Marquardt iterations its search
// took at the last step (0 when no search ran).  The pre-pass queues new contacts and searches
// that took at least 4 iterations first, so that the longest searches start first.
static const unsigned F_ITERS_SHIFT = 20, F_ITERS_MASK = 15u << 20;
static const unsigned LONG_ITERS_BUCKET = 3;   // iterations >= 4
static const unsigned VLONG_ITERS_BUCKET = 6;  // iterations >= 32: the searches that bound the kernel
__device__ __forceinline__ unsigned itersBucket(int iters) { return iters > 0 ? min(15u, 32u - __clz((unsigned)iters)) : 0u; }
enum { KIND_SQ = 0, KIND_WALL = 1 };
static const unsigned DOF_ALL = 63u;

struct Params {
  double dt, g[3], damping, verletDist, minSweepDistFactor, h0;
  int targetInterv, sortAxis, isSuperquadrics, exactAsphericalRot, recordFull;
  int lmSpread;   // idle lanes evaluate the points running searches ask for next
  int contactModel;   // SQDEM_CONTACT_LINEAR or SQDEM_CONTACT_HERTZ_MINDLIN
  int periodicFix;    // sqdem_set_periodic_fix: torque arm and relative velocity of image contacts
  int vlongBucket;    // iteration bucket from which a search goes to the long-search queue
};

enum { E_NAN_NORMAL = 0, E_NAN_FORCE, E_LM_CALLS, E_LM_ITERS, E_LM_MAX, E_OVERFLOW, E_COLLIDER_RUNS, E_STEPS, E_EVAL32, E_EVAL64, E_ROUNDS_MAX,
       E_FALLBACK, E_ROUNDS_MAX_FF, E_LONG_QUEUE, E_NUM };

// CompressionEngine (pkg/dem/Compression.hpp:39-252), cubic specimen: configuration and state.
struct ServoDev {
  int enabled, z_servo, continueFlag, hydroStrain, shearMode, activated[6];
  unsigned iterate_num_max, solve_num_max, echo_interval, savedata_interval, ramp_interval, ramp_chunks;
  double goalx, goaly, goalz, gain_alpha, target_strain, f_threshold, fmin_threshold, unbf_tol, max_vel, hydroStrainRate;
  double height0, width0, depth0;
  int firstRun, Flag_ForceTarget;
  double width, depth, height, x_area, y_area, z_area, Init_boxVolume, Current_boxVolume, particlesVolume, strain2;
  double gain_x, gain_y, gain_z, gain_x1, gain_y1, gain_z1;
  double wsxx_left, wsxx_right, wsyy_front, wsyy_back, wszz_bottom, wszz_top, wsxx, wsyy, wszz;
  unsigned iterate_num, solve_num, rampNum;
  double UnbalancedForce;
  double pvol;   // summed particle volumes in body order (host), particlesVolume at the first run
  int need;      // reductions this step: 1 contact stress tensor, 2 unbalanced force
};

struct SceneState {
  long long iter; double time;
  long long haltAt;   // Scene::stopAtIter as an engine requested it (-1: none); steps from there on do nothing
  int skip, quiet;    // this step does nothing; NewtonIntegrator::quiet_system_flag
  ServoDev sv;
  double maxVelocitySq, fastestBodyMaxDist, verletDistCur;
  int strideActive, newtonFound, doSort, dirty, bbInit;
  int runCollider, initSort, newtonRan, maxDispCode;
  int P, Pnew, nWW, overflowRun;
  int lmCount, lmHead;
  int vlCount, vlHead;   // long-search queue: fbQueue[0, vlCount), filled by pass 1
  int fbCount, fbHead;   // searches the mixed form deferred to FP64: fbQueue[vlCount, vlCount + fbCount)
  int nmFin;   // Hertz-Mindlin searches that ended touching, for the finish pass
  int nmShort; // searches queued from the back of the queue (expected short)
  int numReinit; long long colliderRuns;
  unsigned long long bbLo[3], bbHi[3];   // order-preserving encodings of the bbox of particle bound centres
  double org[3]; double h; int dim[3]; int nCells;
  // periodic cell (core/Cell.hpp): hSize and velocity gradients row-major
  int periodic, homoDeform, velGradChanged;
  double hSize[9], trsf[9], velGrad[9], nextVelGrad[9], prevVelGrad[9], dVelGrad[9], dtPrevVelGrad[9];
  double cellSize[3], prevCellSize[3], prevRunCellSize[3], cellTerm;
  unsigned long long err[E_NUM];
};

// Contact table, structure of arrays (one set per buffer).
struct Table {
  int* owner; int* partner; unsigned* flags;
  double2* angle; double* depth; double4* normal; double4* shear; double4* nforce;
  double4* phys;          // kn, ks, tanphi, -
  double4* F; double4* cp;
  int4* cd;               // Interaction::cellDist in (id1, id2) order: shift2 = hSize*cd moves id2
  // full geometry record (written only when Params::recordFull)
  double4* p1; double4* p2; double4* shearInc; double4* twist; double4* ortho; double4* relVn; double4* relVs;
  // SuperquadricsGeom2 fields (Hertz-Mindlin model, full record only): curvatures1 (2),
  // curvatures2 (2) | curvatureAngle, alpha, K, E | curvatures_sum, isSphere
  double4* hmCurv; double4* hmEll; double2* hmSum;
};

struct Dev {
  int N, W, Pcap, Gmax, MAXC, NP;   // NP = particles
  Params* prm; SceneState* S;
  // bodies
  double4 *pos, *ori, *vel, *angVel, *angMom, *inertia, *shpA, *shpB;   // shpA (rx,ry,rz,rmax) shpB (e1,e2,-,-)
  double* mass; int4* info;  // info: kind, mat, isSphere, wall axis | (sense+1)<<4
  unsigned* blocked; int* damped; int* aspherical;
  double4 *bmin, *bmax, *ref, *pmin, *pmax;    // bmin.w sweepLength, bmax.w lastUpdateIter, ref.w hasBound
  double4 *force, *torque;
  int* walls;                 // ids of walls
  double4* mats;              // Kn, Ks, frictionAngle, density
  double2* matsB;             // betan, betas
  double2* matsE;             // SuperquadricsMat2 G, nu
  // tables
  Table A, B;
  int* rowStart; int* rowStartNew; int* rowCount;
  int* cand; int* candCount;
  int* pCount; int* pStart; int* pFill; int* pList;
  int* wCount; int* wList; int* wBlk;
  int2* ww;
  int* lmQueue; int qCap;   // work queue of the contact searches and its capacity
  int* fbQueue;             // mixed form: searches deferred to the FP64 kernel (capacity Pcap)
  FFShape* bodyFF;          // mixed form: double-float shape and rotation of each body, this step
  // grid
  int* bodyCell; int* cellCount; int* cellStart; int* cellFill; int* cellBodies;
  float4* cellBox;   // per cell slot: bound centre (xyz) and, in the next entry, half extents (xyz)
  int* scanTmp;
  unsigned long long* bbPart;
  // boundary controller: per-wall kn sums of real contacts, per-block partial sums
  double* wallKn; double* svPart; int svBlocks;
  int wallChunks, lmBlocks;   // grids sized to the scene
};

__device__ __forceinline__ unsigned long long encOrd(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double decOrd(unsigned long long u) {
  unsigned long long b = (u >> 63) ? (u & 0x7fffffffffffffffull) : ~u;
  return __longlong_as_double((long long)b);
}
__device__ __forceinline__ D3 xyz(double4 v) { return d3(v.x, v.y, v.z); }
__device__ __forceinline__ double4 dd4(D3 a, double w) { return make_double4(a.x, a.y, a.z, w); }
__device__ __forceinline__ double comp(double4 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// 3x3 row-major matrix times vector with the coefficient-product order of Eigen
__device__ __forceinline__ D3 m3v(const double* M, D3 v) {
  return d3(M[0] * v.x + (M[1] * v.y + M[2] * v.z), M[3] * v.x + (M[4] * v.y + M[5] * v.z),
            M[6] * v.x + (M[7] * v.y + M[8] * v.z));
}
// shift2 = hSize * cellDist (InteractionLoop.cpp:100-106)
__device__ __forceinline__ D3 cellShift(const SceneState& S, int4 cd) {
  if (!S.periodic) return d3(0, 0, 0);
  return m3v(S.hSize, d3((double)cd.x, (double)cd.y, (double)cd.z));
}
// The image's field velocity velGrad * shift2 that the reference leaves out of the relative
// velocity of a contact across the periodic boundary (Superquadrics.cpp:1042-1045); added only
// with the periodic-boundary correction on (sqdem_set_periodic_fix), zero otherwise.
__device__ __forceinline__ D3 shiftVelOf(const SceneState& S, const Params& P, D3 shift2) {
  if (!P.periodicFix || !S.periodic) return d3(0, 0, 0);
  const double* v = S.velGrad;
  return d3(v[0] * shift2.x + (v[1] * shift2.y + v[2] * shift2.z), v[3] * shift2.x + (v[4] * shift2.y + v[5] * shift2.z),
            v[6] * shift2.x + (v[7] * shift2.y + v[8] * shift2.z));
}
// InsertionSortCollider::cellWrap / cellWrapRel (InsertionSortCollider.cpp:404-414)
__device__ __forceinline__ double cellWrapD(double x, double x0, double x1, int& period) {
  double xNorm = (x - x0) / (x1 - x0);
  period = (int)floor(xNorm);
  return x0 + (xNorm - period) * (x1 - x0);
}
__device__ __forceinline__ double cellWrapRelD(double x, double x0, double x1) {
  double xNorm = (x - x0) / (x1 - x0);
  return (xNorm - floor(xNorm)) * (x1 - x0);
}
// InsertionSortCollider::spatialOverlapPeri (InsertionSortCollider.cpp:491-543) on the bounds
// of bodies 1 and 2; periods = image of body 2 relative to body 1.
__device__ __forceinline__ bool overlapPeri(const SceneState& S, double4 mn1v, double4 mx1v, double4 mn2v, double4 mx2v,
                                            int per[3]) {
#pragma unroll
  for (int axis = 0; axis < 3; axis++) {
    const double dim = S.cellSize[axis];
    const double m1 = comp(mn1v, axis), m2 = comp(mn2v, axis);
    const double wMn = (cellWrapRelD(m1, m2, m2 + dim) < cellWrapRelD(m2, m1, m1 + dim)) ? m2 : m1;
    int pmn1, pmx1, pmn2, pmx2;
    const double mn1 = cellWrapD(m1, wMn, wMn + dim, pmn1), mx1 = cellWrapD(comp(mx1v, axis), wMn, wMn + dim, pmx1);
    const double mn2 = cellWrapD(m2, wMn, wMn + dim, pmn2), mx2 = cellWrapD(comp(mx2v, axis), wMn, wMn + dim, pmx2);
    if ((pmn1 != pmx1) || (pmn2 != pmx2)) { per[axis] = 0; return false; }
    per[axis] = pmn1 - pmn2;
    if (!(mn1 <= mx2 && mx1 >= mn2)) return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// Exclusive scan over n+1 ints (in[n] treated as 0), three launches, gated.
static const int SCAN_BS = 1024, SCAN_IPT = 4, SCAN_TILE = SCAN_BS * SCAN_IPT;

__device__ __forceinline__ int blockExclusiveScan(int v, int* sh, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) { int y = __shfl_up_sync(0xffffffffu, x, o); if (lane >= o) x += y; }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int s = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) { int y = __shfl_up_sync(0xffffffffu, s, o); if (lane >= o) s += y; }
    sh[lane] = s;
  }
  __syncthreads();
  total = sh[(blockDim.x >> 5) - 1];
  int res = x - v + (wid > 0 ? sh[wid - 1] : 0);
  __syncthreads();
  return res;
}

__global__ void k_scan_reduce(const int* __restrict__ in, int n, int* __restrict__ blockSums, const int* gate) {
  if (gate && !*gate) return;
  __shared__ int sh[32];
  int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_IPT;
  int s = 0;
  for (int k = 0; k < SCAN_IPT; k++) { int i = base + k; if (i < n) s += in[i]; }
  int total;
  blockExclusiveScan(s, sh, total);
  if (threadIdx.x == 0) blockSums[blockIdx.x] = total;
}
__global__ void k_scan_blocks(int* blockSums, int nb, const int* gate) {
  if (gate && !*gate) return;
  __shared__ int sh[32];
  int carry = 0;
  for (int b0 = 0; b0 < nb; b0 += blockDim.x) {
    int i = b0 + threadIdx.x;
    int v = i < nb ? blockSums[i] : 0;
    int total;
    int ex = blockExclusiveScan(v, sh, total);
    if (i < nb) blockSums[i] = ex + carry;
    carry += total;
    __syncthreads();
  }
}
// out[i] = sum(in[0..i)) for i in [0, n]; out[n] = total
__global__ void k_scan_apply(const int* __restrict__ in, int n, const int* __restrict__ blockSums, int* __restrict__ out,
                             const int* gate) {
  if (gate && !*gate) return;
  __shared__ int sh[32];
  int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_IPT;
  int v[SCAN_IPT]; int s = 0;
  for (int k = 0; k < SCAN_IPT; k++) { int i = base + k; v[k] = (i < n) ? in[i] : 0; s += v[k]; }
  int total;
  int ex = blockExclusiveScan(s, sh, total) + blockSums[blockIdx.x];
  for (int k = 0; k < SCAN_IPT; k++) { int i = base + k; if (i <= n) out[i] = ex; ex += v[k]; }
}

// ---------------------------------------------------------------------------
// Collider gate: InsertionSortCollider::isActivated (InsertionSortCollider.cpp:177-189)
// plus the start of action() (:205-252) and the NewtonIntegrator maxVelocitySq readout.
__global__ void k_gate(Dev d) {
  SceneState& S = *d.S;
  S.skip = (S.haltAt >= 0 && S.iter >= S.haltAt) ? 1 : 0;
  if (S.skip) { S.runCollider = 0; S.lmCount = 0; S.lmHead = 0; S.fbCount = 0; S.fbHead = 0; S.vlCount = 0; S.vlHead = 0; S.nmFin = 0; S.nmShort = 0; return; }
  if (S.newtonRan) {
    const double code = S.maxDispCode == 2 ? 2.0 : (S.maxDispCode == 1 ? 0.5 : 0.0);
    S.maxVelocitySq = fmax_ref(S.cellTerm, code);
    S.maxDispCode = 0; S.newtonRan = 0;
  }
  if (S.periodic) {  // Cell::integrateAndUpdate (core/Cell.cpp:6-26), step prologue
    double inc[9], t[9], h[9];
    for (int k = 0; k < 9; k++) inc[k] = d.prm->dt * S.velGrad[k];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        t[3 * i + j] = inc[3 * i] * S.trsf[j] + (inc[3 * i + 1] * S.trsf[3 + j] + inc[3 * i + 2] * S.trsf[6 + j]);
        h[3 * i + j] = inc[3 * i] * S.hSize[j] + (inc[3 * i + 1] * S.hSize[3 + j] + inc[3 * i + 2] * S.hSize[6 + j]);
      }
    for (int k = 0; k < 9; k++) { S.trsf[k] += t[k]; S.hSize[k] += h[k]; }
    for (int i = 0; i < 3; i++) S.cellSize[i] = nrm(d3(S.hSize[i], S.hSize[3 + i], S.hSize[6 + i]));
  }
  int run;
  if (!S.strideActive) run = 1;
  else if (!S.newtonFound) run = 1;
  else if (S.fastestBodyMaxDist < 0) { S.fastestBodyMaxDist = 0; run = 1; }
  else {
    S.fastestBodyMaxDist = S.maxVelocitySq;
    if (S.fastestBodyMaxDist >= 1 || S.fastestBodyMaxDist == 0) run = 1;
    else if (!S.bbInit) run = 1;
    else if (S.dirty) run = 1;
    else run = 0;
  }
  S.runCollider = run;
  S.lmCount = 0; S.lmHead = 0; S.fbCount = 0; S.fbHead = 0; S.vlCount = 0; S.vlHead = 0; S.nmFin = 0; S.nmShort = 0;
  if (run) {
    int init = 0;
    if (S.doSort) { init = 1; S.doSort = 0; }
    if (!S.bbInit) init = 1;
    if (S.verletDistCur < 0) S.verletDistCur = 0;
    if (S.dirty) { init = 1; S.dirty = 0; }
    S.initSort = init;
    S.overflowRun = 0;
    for (int k = 0; k < 3; k++) { S.bbLo[k] = ~0ull; S.bbHi[k] = 0ull; }
  }
}

// BoundDispatcher::processBody (Dispatching.cpp:30-62), Bo1_Superquadrics_Aabb::go
// (Superquadrics.cpp:639-686), Bo1_Wall_Aabb::go (Wall.cpp:13-21).
__global__ void k_bounds(Dev d) {
  const SceneState& S = *d.S;
  if (!S.runCollider) return;
  const Params& P = *d.prm;
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  double cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
  if (b < d.N) {
    const double sweepDist = S.verletDistCur;
    double4 pos = d.pos[b];
    double4 mn = d.bmin[b], mx = d.bmax[b], rf = d.ref[b];
    int4 inf = d.info[b];
    bool hasBound = rf.w != 0;
    double sweepLength = mn.w;
    double lastUpd = mx.w;
    if (hasBound) {
      if (P.targetInterv >= 0) {
        D3 disp = xyz(pos) - xyz(rf);
        double dist = fmax_ref(fabs(disp.x), fmax_ref(fabs(disp.y), fabs(disp.z)));
        if (dist != 0) {  // NaN (never bounded) also takes this branch
          double newLength = dist * P.targetInterv / (double)(S.iter - (long long)lastUpd);
          newLength = fmax_ref(0.9 * sweepLength, newLength);
          sweepLength = fmax_ref(P.minSweepDistFactor * sweepDist, fmin_ref(newLength, sweepDist));
        } else sweepLength = 0;
      } else sweepLength = sweepDist;
    }
    d.pmin[b] = mn; d.pmax[b] = mx;
    D3 lo, hi;
    if (inf.x == KIND_SQ) {
      double r = d.shpA[b].w;
      lo = xyz(pos) + d3(-r, -r, -r);
      hi = xyz(pos) + d3(r, r, r);
    } else {
      int ax = inf.w & 15;
      lo = d3(-INFINITY, -INFINITY, -INFINITY); hi = d3(INFINITY, INFINITY, INFINITY);
      if (ax == 0) { lo.x = hi.x = pos.x; } else if (ax == 1) { lo.y = hi.y = pos.y; } else { lo.z = hi.z = pos.z; }
    }
    if (!hasBound) sweepLength = 0;
    if (sweepLength > 0) {
      lo = lo - d3(sweepLength, sweepLength, sweepLength);
      hi = hi + d3(sweepLength, sweepLength, sweepLength);
    }
    d.bmin[b] = dd4(lo, sweepLength);
    d.bmax[b] = dd4(hi, (double)S.iter);
    d.ref[b] = make_double4(pos.x, pos.y, pos.z, 1.0);
    if (inf.x == KIND_SQ) {
      D3 c = 0.5 * (lo + hi);
      cmin[0] = cmax[0] = c.x; cmin[1] = cmax[1] = c.y; cmin[2] = cmax[2] = c.z;
    }
  }
  // block bbox of particle bound centres -> global atomics on ordered encodings
#pragma unroll
  for (int k = 0; k < 3; k++) {
    double a = cmin[k], z = cmax[k];
    for (int o = 16; o > 0; o >>= 1) {
      a = fmin(a, __shfl_down_sync(0xffffffffu, a, o));
      z = fmax(z, __shfl_down_sync(0xffffffffu, z, o));
    }
    if ((threadIdx.x & 31) == 0 && a <= z) {
      atomicMin(&d.S->bbLo[k], encOrd(a));
      atomicMax(&d.S->bbHi[k], encOrd(z));
    }
  }
}

__global__ void k_grid_setup(Dev d) {
  SceneState& S = *d.S;
  if (!S.runCollider) return;
  const Params& P = *d.prm;
  // post-dispatch stride bookkeeping (InsertionSortCollider.cpp:263-284)
  if (S.verletDistCur > 0) S.newtonFound = 1;
  if (!S.strideActive && S.verletDistCur > 0 && S.maxVelocitySq >= 0) S.strideActive = 1;
  double lo[3], hi[3];
  bool any = true;
  for (int k = 0; k < 3; k++) {
    if (S.bbLo[k] == ~0ull) { any = false; lo[k] = 0; hi[k] = 0; }
    else { lo[k] = decOrd(S.bbLo[k]); hi[k] = decOrd(S.bbHi[k]); }
  }
  if (!any) for (int k = 0; k < 3; k++) { lo[k] = 0; hi[k] = 0; }
  if (S.periodic) { for (int k = 0; k < 3; k++) { lo[k] = 0; hi[k] = S.cellSize[k]; } }
  for (int k = 0; k < 3; k++)
    if (!isfinite(lo[k]) || !isfinite(hi[k]) || !(hi[k] >= lo[k])) { lo[k] = 0; hi[k] = 0; }
  double h = P.h0;
  if (!(h > 0) || !isfinite(h)) h = 1.0;
  long long cells = 1;
  int dim[3] = {1, 1, 1};
  for (int it = 0; it < 4096; it++) {
    cells = 1;
    for (int k = 0; k < 3; k++) {
      double q = floor((hi[k] - lo[k]) / h);
      long long n = (q >= 0 && q < (double)(1 << 20)) ? (long long)q + 3 : (1ll << 20);
      dim[k] = (int)n; cells *= n;
    }
    if (cells <= d.Gmax) break;
    h *= 1.25;
  }
  if (cells > d.Gmax) { dim[0] = dim[1] = dim[2] = 1; cells = 1; }
  if (S.periodic) {
    // cells tile the periodic box exactly: cell edge = size/dim >= h
    cells = 1;
    for (int k = 0; k < 3; k++) {
      double q = floor(S.cellSize[k] / h);
      int n = (q >= 1 && q < (double)(1 << 20)) ? (int)q : 1;
      dim[k] = n; cells *= n;
    }
    while (cells > d.Gmax) { for (int k = 0; k < 3; k++) dim[k] = max(1, dim[k] / 2); cells = (long long)dim[0] * dim[1] * dim[2]; }
    for (int k = 0; k < 3; k++) { S.org[k] = 0; S.dim[k] = dim[k]; }
    S.h = h;
    S.nCells = (int)cells;
    return;
  }
  for (int k = 0; k < 3; k++) { S.org[k] = lo[k] - h; S.dim[k] = dim[k]; }
  S.h = h;
  S.nCells = (int)cells;
}

__global__ void k_zero_cells(Dev d) {
  if (!d.S->runCollider) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= d.Gmax; i += gridDim.x * blockDim.x) {
    d.cellCount[i] = 0; d.cellFill[i] = 0;
  }
}

// clamped cell coordinate; NaN maps to 0 so that no index leaves [0, dim)
__device__ __forceinline__ int cellCoord(double c, double org, double h, int dim) {
  double f = floor((c - org) / h);
  if (!(f >= 0)) return 0;
  if (f > (double)(dim - 1)) return dim - 1;
  return (int)f;
}

// periodic: wrapped coordinate (Cell::wrapNum) mapped onto dim cells of the box
__device__ __forceinline__ int cellCoordPeri(double c, double L, int dim) {
  double norm = c / L;
  double w = norm - floor(norm);
  double f = floor(w * dim);
  if (!(f >= 0)) return 0;
  if (f > (double)(dim - 1)) return dim - 1;
  return (int)f;
}
__device__ __forceinline__ void bodyCellCoords(const SceneState& S, double4 mn, double4 mx, int& cx, int& cy, int& cz) {
  if (S.periodic) {
    cx = cellCoordPeri(0.5 * (mn.x + mx.x), S.cellSize[0], S.dim[0]);
    cy = cellCoordPeri(0.5 * (mn.y + mx.y), S.cellSize[1], S.dim[1]);
    cz = cellCoordPeri(0.5 * (mn.z + mx.z), S.cellSize[2], S.dim[2]);
  } else {
    cx = cellCoord(0.5 * (mn.x + mx.x), S.org[0], S.h, S.dim[0]);
    cy = cellCoord(0.5 * (mn.y + mx.y), S.org[1], S.h, S.dim[1]);
    cz = cellCoord(0.5 * (mn.z + mx.z), S.org[2], S.h, S.dim[2]);
  }
}

__global__ void k_cell_count(Dev d) {
  const SceneState& S = *d.S;
  if (!S.runCollider) return;
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= d.N) return;
  if (d.info[b].x != KIND_SQ) { d.bodyCell[b] = -1; return; }
  double4 mn = d.bmin[b], mx = d.bmax[b];
  int cx, cy, cz;
  bodyCellCoords(S, mn, mx, cx, cy, cz);
  int cell = (cz * S.dim[1] + cy) * S.dim[0] + cx;
  d.bodyCell[b] = cell;
  atomicAdd(&d.cellCount[cell], 1);
}
__global__ void k_cell_scatter(Dev d) {
  if (!d.S->runCollider) return;
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= d.N) return;
  int cell = d.bodyCell[b];
  if (cell < 0) return;
  int slot = d.cellStart[cell] + atomicAdd(&d.cellFill[cell], 1);
  d.cellBodies[slot] = b;
  const double4 mn = d.bmin[b], mx = d.bmax[b];
  d.cellBox[2 * slot] = make_float4((float)(0.5 * (mn.x + mx.x)), (float)(0.5 * (mn.y + mx.y)), (float)(0.5 * (mn.z + mx.z)), 0.f);
  d.cellBox[2 * slot + 1] = make_float4((float)(0.5 * (mx.x - mn.x)), (float)(0.5 * (mx.y - mn.y)), (float)(0.5 * (mx.z - mn.z)), 0.f);
}

// FP32 pre-filter of the candidate search: true when the two bounds cannot overlap, in any
// periodic image (minimum-image distance of the centres above the summed half extents on
// some axis).  The margin (1e-6 of the coordinates' scale, ~20 FP32 ulps) keeps it
// conservative, so the exact FP64 tests below decide every pair it lets through and the
// pair set is unchanged; it spares most candidates the 18 FP64 divisions of overlapPeri.
__device__ __forceinline__ bool boxesApart(float4 ca, float4 ha, float4 cb, float4 hb, bool periodic, const float* L,
                                           const float* invL) {
  const float c1[3] = {ca.x, ca.y, ca.z}, h1[3] = {ha.x, ha.y, ha.z};
  const float c2[3] = {cb.x, cb.y, cb.z}, h2[3] = {hb.x, hb.y, hb.z};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float dc = c2[k] - c1[k];
    float scale = fabsf(c1[k]) + fabsf(c2[k]) + h1[k] + h2[k];
    if (periodic) { dc -= L[k] * rintf(dc * invL[k]); scale += L[k]; }
    if (fabsf(dc) > h1[k] + h2[k] + 1e-6f * scale) return true;
  }
  return false;
}

// InsertionSortCollider::spatialOverlapPeri (the exact test, overlapPeri) decided from FP32
// bound centres and half extents wherever its outcome does not hang on rounding: returns 1
// (overlap), -1 (no overlap) or 0 (undecided: run overlapPeri).  Per axis, with d the offset
// of body 1's lower bound after body 2's modulo the cell size L: for d < L/2 the exact test's
// window starts at body 2's lower bound, no bound straddles it, and the axis overlaps iff
// d <= len2; for d > L/2 the window starts at body 1's lower bound and the axis overlaps iff
// L - d <= len1.  Within a margin (1e-5 of the coordinates' scale, ~40x the FP32 error) of
// d = 0, L/2 or L, of d = len2 (L - d = len1), or for a body longer than L/2, the exact test
// decides.  Any axis that is clearly apart makes the pair apart, as in the exact test.
__device__ __forceinline__ int overlapPeriFast(float4 c1, float4 h1, float4 c2, float4 h2, const float* L,
                                               const float* invL) {
  const float a1[3] = {c1.x, c1.y, c1.z}, b1[3] = {h1.x, h1.y, h1.z};
  const float a2[3] = {c2.x, c2.y, c2.z}, b2[3] = {h2.x, h2.y, h2.z};
  int res = 1;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float D = L[k];
    const float len1 = 2.f * b1[k], len2 = 2.f * b2[k];
    const float eps = 1e-5f * (fabsf(a1[k]) + fabsf(a2[k]) + b1[k] + b2[k] + D);
    float dd = (a1[k] - b1[k]) - (a2[k] - b2[k]);
    dd -= D * floorf(dd * invL[k]);
    if (!(len1 < 0.5f * D - eps && len2 < 0.5f * D - eps && dd > eps && dd < D - eps && fabsf(dd - 0.5f * D) > eps)) {
      res = 0;
      continue;
    }
    const float gap = dd < 0.5f * D ? dd - len2 : (D - dd) - len1;
    if (gap > eps) return -1;
    if (gap > -eps) res = 0;
  }
  return res;
}

// closed overlap test, InsertionSortCollider::spatialOverlap (InsertionSortCollider.hpp:166-171)
__device__ __forceinline__ bool overlapClosed(double4 amn, double4 amx, double4 bmn, double4 bmx) {
  return (amn.x <= bmx.x) && (amx.x >= bmn.x) && (amn.y <= bmx.y) && (amx.y >= bmn.y) && (amn.z <= bmx.z) &&
         (amx.z >= bmn.z);
}

// Orientation of a pair that enters the container at this collider pass.
// Returns 1: (i, j) with i = id1; 0: (j, i); -1: the reference's sort would not insert it.
//  * full sort (first pass, doSort, dirty): the body whose lower bound comes first on
//    sortAxis is id1 (InsertionSortCollider.cpp:357-376; equal coordinates: lower id);
//  * incremental insertion sort: axes 0,1,2 in turn; on the first axis where the lower
//    bound of one body moved below the upper bound of the other since the previous pass,
//    the body whose lower bound moved is id1 (InsertionSortCollider.cpp:29-54).
__device__ __forceinline__ int orientNew(const Dev& d, int i, int j, int initSort, int sortAxis) {
  const SceneState& S = *d.S;
  double4 imn = d.bmin[i], jmn = d.bmin[j];
  double4 imx = d.bmax[i], jmx = d.bmax[j];
  // periodic: compare i with the image of j that overlaps it (shift of j by per * size)
  double shNow[3] = {0, 0, 0}, shPrev[3] = {0, 0, 0};
  if (S.periodic) {
    int per[3];
    overlapPeri(S, imn, imx, jmn, jmx, per);
    for (int k = 0; k < 3; k++) {
      shNow[k] = per[k] * S.cellSize[k];
      shPrev[k] = per[k] * S.prevRunCellSize[k];
    }
  }
  if (initSort) {
    double a = comp(imn, sortAxis), b = comp(jmn, sortAxis) + shNow[sortAxis];
    if (a < b) return 1;
    if (b < a) return 0;
    return i < j ? 1 : 0;
  }
  double4 ipn = d.pmin[i], ipx = d.pmax[i], jpn = d.pmin[j], jpx = d.pmax[j];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double jpxk = comp(jpx, k) + shPrev[k], jpnk = comp(jpn, k) + shPrev[k];
    const double jmxk = comp(jmx, k) + shNow[k], jmnk = comp(jmn, k) + shNow[k];
    if (jpxk < comp(ipn, k) && jmxk > comp(imn, k)) return 1;
    if (comp(ipx, k) < jpnk && comp(imx, k) > jmnk) return 0;
  }
  // No crossing seen.  Without periodicity this needs exactly equal coordinates, and the
  // reference's sort would not insert the pair either.  In a periodic cell the image shifts
  // above only approximate the circular sort order, so an overlapping pair is inserted with
  // the full-sort orientation rather than missed.
  if (S.periodic) {
    double a = comp(imn, sortAxis), b = comp(jmn, sortAxis) + shNow[sortAxis];
    if (a < b) return 1;
    if (b < a) return 0;
    return i < j ? 1 : 0;
  }
  return -1;
}

// Candidate row of particle i: partners j>i (particles) and all walls whose bounds overlap
// i's, sorted by partner id, each tagged with its orientation bit (bit 31).  The union with
// i's previous row gives the new row length: old entries survive if real or overlapping
// (conditionalyEraseNonReal), new overlapping pairs are inserted when the sort would insert
// them.
static const int UNDECIDED = 0x40000000;   // candidate tag: overlap left to the exact test

// Threads take the particles in cell order (cellBodies), so that a warp scans neighbouring
// cells and its loads of cellBodies/cellBox overlap; bodies outside the grid (walls) get an
// empty row from the thread of their own index.
__global__ void k_candidates(Dev d) {
  const SceneState& S = *d.S;
  if (!S.runCollider) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.N) return;
  if (d.bodyCell[t] < 0) { d.rowCount[t] = 0; d.candCount[t] = 0; }
  if (t >= d.cellStart[S.nCells]) return;
  const int i = d.cellBodies[t];
  const double4 imn = d.bmin[i], imx = d.bmax[i];
  int* cand = d.cand + (size_t)i * d.MAXC;
  int n = 0; bool over = false;
  int cx, cy, cz;
  bodyCellCoords(S, imn, imx, cx, cy, cz);
  int seen[27];
  int nseen = 0;
  const float4 ci = make_float4((float)(0.5 * (imn.x + imx.x)), (float)(0.5 * (imn.y + imx.y)), (float)(0.5 * (imn.z + imx.z)), 0.f);
  const float4 hi = make_float4((float)(0.5 * (imx.x - imn.x)), (float)(0.5 * (imx.y - imn.y)), (float)(0.5 * (imx.z - imn.z)), 0.f);
  float Lf[3] = {1.f, 1.f, 1.f}, invLf[3] = {1.f, 1.f, 1.f};
  if (S.periodic)
    for (int k = 0; k < 3; k++) { Lf[k] = (float)S.cellSize[k]; invLf[k] = 1.f / Lf[k]; }
  for (int dz = -1; dz <= 1; dz++) {
    int z = cz + dz;
    if (S.periodic) z = (z + S.dim[2]) % S.dim[2]; else if (z < 0 || z >= S.dim[2]) continue;
    for (int dy = -1; dy <= 1; dy++) {
      int y = cy + dy;
      if (S.periodic) y = (y + S.dim[1]) % S.dim[1]; else if (y < 0 || y >= S.dim[1]) continue;
      for (int dx = -1; dx <= 1; dx++) {
        int x = cx + dx;
        if (S.periodic) x = (x + S.dim[0]) % S.dim[0]; else if (x < 0 || x >= S.dim[0]) continue;
        int cell = (z * S.dim[1] + y) * S.dim[0] + x;
        bool dup = false;
        for (int q = 0; q < nseen; q++) dup |= (seen[q] == cell);
        if (dup) continue;
        seen[nseen++] = cell;
        int s0 = d.cellStart[cell], e0 = d.cellStart[cell + 1];
        for (int k = s0; k < e0; k++) {
          int j = d.cellBodies[k];
          if (j <= i) continue;
          const float4 cj = d.cellBox[2 * k], hj = d.cellBox[2 * k + 1];
          int v;   // 1 overlap, 0 undecided (exact test below), -1 apart
          if (S.periodic) v = overlapPeriFast(ci, hi, cj, hj, Lf, invLf);
          else v = boxesApart(ci, hi, cj, hj, false, Lf, invLf) ? -1 : 0;
          if (v < 0) continue;
          if (n < d.MAXC) cand[n++] = v > 0 ? j : (j | UNDECIDED); else over = true;
        }
      }
    }
  }
  // exact tests of the undecided candidates, in a loop of their own so that the lanes of a
  // warp run the FP64 work of spatialOverlapPeri together
  {
    int m = 0;
    for (int a = 0; a < n; a++) {
      int j = cand[a];
      if (j & UNDECIDED) {
        j &= ~UNDECIDED;
        bool ov;
        if (S.periodic) { int per[3]; ov = overlapPeri(S, imn, imx, d.bmin[j], d.bmax[j], per); }
        else ov = overlapClosed(imn, imx, d.bmin[j], d.bmax[j]);
        if (!ov) continue;
      }
      cand[m++] = j;
    }
    n = m;
  }
  for (int w = 0; w < d.W; w++) {
    int j = d.walls[w];
    if (overlapClosed(imn, imx, d.bmin[j], d.bmax[j])) {
      if (n < d.MAXC) cand[n++] = j; else over = true;
    }
  }
  if (over) atomicAdd(&d.S->err[E_OVERFLOW], 1ull);
  // insertion sort by partner id
  for (int a = 1; a < n; a++) {
    int v = cand[a]; int b = a - 1;
    while (b >= 0 && cand[b] > v) { cand[b + 1] = cand[b]; b--; }
    cand[b + 1] = v;
  }
  // union with the previous row
  const int os = d.rowStart[i], oe = d.rowStart[i + 1];
  int o = os, c = 0, cnt = 0, m = 0;
  while (o < oe || c < n) {
    int po = o < oe ? d.A.partner[o] : 0x7fffffff;
    int pc = c < n ? cand[c] : 0x7fffffff;
    if (po == pc) { cnt++; cand[m++] = pc; o++; c++; }     // survives, history kept
    else if (po < pc) {                                     // not overlapping any more
      if ((d.A.flags[o] & (F_GEOM | F_PHYS)) == (F_GEOM | F_PHYS)) cnt++;
      o++;
    } else {                                                // new pair
      int orient;
      if (d.info[pc].x == KIND_WALL) {
        orient = S.initSort ? 1 : orientNew(d, i, pc, 0, 0);
        if (orient >= 0) orient = 0;  // the geometry functor is (Wall, Superquadrics): wall is id1
      } else orient = orientNew(d, i, pc, S.initSort, d.prm->sortAxis);
      if (orient >= 0) { cnt++; cand[m++] = pc | (orient ? (int)0x80000000 : 0); }
      c++;
    }
  }
  d.candCount[i] = m;
  d.rowCount[i] = cnt;
}

__global__ void k_check_capacity(Dev d) {
  SceneState& S = *d.S;
  if (!S.runCollider) return;
  int Pn = d.rowStartNew[d.N];
  S.Pnew = Pn;
  if (Pn > d.Pcap) { S.overflowRun = 1; atomicAdd(&S.err[E_OVERFLOW], 1ull); }
}

__device__ __forceinline__ void copyEntry(const Table& s, int a, const Table& t, int b, bool full) {
  t.owner[b] = s.owner[a]; t.partner[b] = s.partner[a]; t.flags[b] = s.flags[a];
  t.angle[b] = s.angle[a]; t.depth[b] = s.depth[a]; t.normal[b] = s.normal[a]; t.shear[b] = s.shear[a];
  t.nforce[b] = s.nforce[a]; t.phys[b] = s.phys[a]; t.F[b] = s.F[a]; t.cp[b] = s.cp[a]; t.cd[b] = s.cd[a];
  if (full) {
    t.p1[b] = s.p1[a]; t.p2[b] = s.p2[a]; t.shearInc[b] = s.shearInc[a]; t.twist[b] = s.twist[a];
    t.ortho[b] = s.ortho[a]; t.relVn[b] = s.relVn[a]; t.relVs[b] = s.relVs[a];
    t.hmCurv[b] = s.hmCurv[a]; t.hmEll[b] = s.hmEll[a]; t.hmSum[b] = s.hmSum[a];
  }
}
__device__ __forceinline__ void initEntry(const Table& t, int b, int owner, int partner, bool ownerIsId1, bool full) {
  const double4 z = make_double4(0, 0, 0, 0);
  t.owner[b] = owner; t.partner[b] = partner; t.flags[b] = F_SHEARNEW | (ownerIsId1 ? F_OWNER_ID1 : 0u);
  t.angle[b] = make_double2(0, 0); t.depth[b] = 0; t.normal[b] = z; t.shear[b] = z; t.nforce[b] = z;
  t.phys[b] = z; t.F[b] = z; t.cp[b] = z; t.cd[b] = make_int4(0, 0, 0, 0);
  if (full) {
    t.p1[b] = z; t.p2[b] = z; t.shearInc[b] = z; t.twist[b] = z; t.ortho[b] = z; t.relVn[b] = z; t.relVs[b] = z;
    t.hmCurv[b] = z; t.hmEll[b] = z; t.hmSum[b] = make_double2(0, 0);
  }
}

__global__ void k_merge(Dev d) {
  const SceneState& S = *d.S;
  if (!S.runCollider || S.overflowRun) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.N) return;
  if (d.info[i].x != KIND_SQ) return;
  const bool full = d.prm->recordFull != 0;
  const int* cand = d.cand + (size_t)i * d.MAXC;
  const int n = d.candCount[i];
  const int os = d.rowStart[i], oe = d.rowStart[i + 1];
  int out = d.rowStartNew[i];
  int o = os, c = 0;
  while (o < oe || c < n) {
    int po = o < oe ? d.A.partner[o] : 0x7fffffff;
    int raw = c < n ? cand[c] : 0x7fffffff;
    int pc = raw & 0x7fffffff;
    if (po == pc) { copyEntry(d.A, o, d.B, out++, full); o++; c++; }
    else if (po < pc) {
      if ((d.A.flags[o] & (F_GEOM | F_PHYS)) == (F_GEOM | F_PHYS)) copyEntry(d.A, o, d.B, out++, full);
      o++;
    } else {
      const bool ownerIsId1 = (raw & 0x80000000) != 0;
      initEntry(d.B, out, i, pc, ownerIsId1, full);
      if (S.periodic) {
        const int a = ownerIsId1 ? i : pc, b = ownerIsId1 ? pc : i;
        int per[3];
        overlapPeri(S, d.bmin[a], d.bmax[a], d.bmin[b], d.bmax[b], per);
        d.B.cd[out] = make_int4(per[0], per[1], per[2], 0);
      }
      out++; c++;
    }
  }
}

__global__ void k_copy_back(Dev d) {
  const SceneState& S = *d.S;
  if (!S.runCollider || S.overflowRun) return;
  const bool full = d.prm->recordFull != 0;
  const int Pn = S.Pnew;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < Pn; e += gridDim.x * blockDim.x) copyEntry(d.B, e, d.A, e, full);
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b <= d.N; b += gridDim.x * blockDim.x) {
    d.rowStart[b] = d.rowStartNew[b];
    if (b < d.N) { d.pCount[b] = 0; d.pFill[b] = 0; }
  }
}

__global__ void k_commit(Dev d) {
  SceneState& S = *d.S;
  if (!S.runCollider) return;
  if (!S.overflowRun) S.P = S.Pnew;
  S.bbInit = 1;
  for (int k = 0; k < 3; k++) S.prevRunCellSize[k] = S.cellSize[k];
  if (S.initSort) S.numReinit++;
  S.colliderRuns++;
  S.err[E_COLLIDER_RUNS]++;
  // wall-wall pairs (never real: no geometry functor for (Wall, Wall)), reported only
  int n = 0;
  for (int a = 0; a < d.W; a++)
    for (int b = a + 1; b < d.W; b++) {
      int ia = d.walls[a], ib = d.walls[b];
      if (overlapClosed(d.bmin[ia], d.bmax[ia], d.bmin[ib], d.bmax[ib])) d.ww[n++] = make_int2(min(ia, ib), max(ia, ib));
    }
  S.nWW = n;
}

// incidence lists: entries in which a particle is the partner (not the row owner)
__global__ void k_pcount(Dev d) {
  const SceneState& S = *d.S;
  if (!S.runCollider || S.overflowRun) return;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < S.P; e += gridDim.x * blockDim.x) {
    int p = d.A.partner[e];
    if (d.info[p].x == KIND_SQ) atomicAdd(&d.pCount[p], 1);
  }
}
__global__ void k_pscatter(Dev d) {
  const SceneState& S = *d.S;
  if (!S.runCollider || S.overflowRun) return;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < S.P; e += gridDim.x * blockDim.x) {
    int p = d.A.partner[e];
    if (d.info[p].x == KIND_SQ) d.pList[d.pStart[p] + atomicAdd(&d.pFill[p], 1)] = e;
  }
}
// make each partner list ascending in entry index (deterministic summation order)
__global__ void k_psort(Dev d) {
  const SceneState& S = *d.S;
  if (!S.runCollider || S.overflowRun) return;
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= d.N) return;
  int s = d.pStart[b], e = d.pStart[b + 1];
  for (int a = s + 1; a < e; a++) {
    int v = d.pList[a]; int c = a - 1;
    while (c >= s && d.pList[c] > v) { d.pList[c + 1] = d.pList[c]; c--; }
    d.pList[c + 1] = v;
  }
}
// Per-wall lists of table entries in table order (the order the wall force sums follow).
// The table is cut into WALL_CHUNKS contiguous chunks, one block each: k_wall_count counts
// each wall's entries per chunk; k_wall_lists places chunk b's entries of wall w after
// those of the walls before w and of the chunks before b, in table order within the chunk
// (one block scan per wall and tile).
static const int WALL_CHUNKS = 256, MAX_WALLS = 64;   // WALL_CHUNKS: most chunks of a table
__device__ __forceinline__ int wallSlot(const Dev& d, int p) {
  if (d.info[p].x != KIND_WALL) return -1;
  for (int w = 0; w < d.W; w++) if (d.walls[w] == p) return w;
  return -1;
}
__device__ __forceinline__ void wallChunk(int P, int chunks, int b, int& lo, int& hi) {
  const int len = (P + chunks - 1) / chunks;
  lo = min(P, b * len); hi = min(P, lo + len);
}
__global__ void k_wall_count(Dev d) {
  const SceneState& S = *d.S;
  if (!S.runCollider || S.overflowRun) return;
  __shared__ int cnt[MAX_WALLS];
  for (int w = threadIdx.x; w < d.W; w += blockDim.x) cnt[w] = 0;
  __syncthreads();
  int lo, hi;
  wallChunk(S.P, d.wallChunks, blockIdx.x, lo, hi);
  for (int e = lo + threadIdx.x; e < hi; e += blockDim.x) {
    const int w = wallSlot(d, d.A.partner[e]);
    if (w >= 0) atomicAdd(&cnt[w], 1);
  }
  __syncthreads();
  for (int w = threadIdx.x; w < d.W; w += blockDim.x) d.wBlk[blockIdx.x * d.W + w] = cnt[w];
}
__global__ void k_wall_lists(Dev d) {
  const SceneState& S = *d.S;
  if (!S.runCollider || S.overflowRun) return;
  __shared__ int sh[32];
  __shared__ int tot[MAX_WALLS], off[MAX_WALLS];
  for (int w = threadIdx.x; w < d.W; w += blockDim.x) {
    int before = 0, all = 0;
    for (int b = 0; b < d.wallChunks; b++) {
      const int c = d.wBlk[b * d.W + w];
      all += c;
      if (b < blockIdx.x) before += c;
    }
    tot[w] = all; off[w] = before;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int start = 0;
    for (int w = 0; w < d.W; w++) {
      off[w] += start;
      if (blockIdx.x == 0) { d.wCount[w] = tot[w]; d.wCount[d.W + w] = start; }
      start += tot[w];
    }
  }
  __syncthreads();
  int lo, hi;
  wallChunk(S.P, d.wallChunks, blockIdx.x, lo, hi);
  for (int e0 = lo; e0 < hi; e0 += blockDim.x) {
    const int e = e0 + threadIdx.x;
    const int ws = e < hi ? wallSlot(d, d.A.partner[e]) : -1;
    for (int w = 0; w < d.W; w++) {
      const int f = ws == w ? 1 : 0;
      int tt;
      const int ex = blockExclusiveScan(f, sh, tt);
      if (f) d.wList[off[w] + ex] = e;
      __syncthreads();
      if (threadIdx.x == 0) off[w] += tt;
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// Narrowphase + contact physics + law for one table entry.
struct BodyView {
  D3 pos, vel, angVel; double4 ori; double4 shpA, shpB; int4 info; double mass; unsigned blocked;
};
__device__ __forceinline__ BodyView loadBody(const Dev& d, int b) {
  BodyView v;
  v.pos = xyz(d.pos[b]); v.vel = xyz(d.vel[b]); v.angVel = xyz(d.angVel[b]); v.ori = d.ori[b];
  v.shpA = d.shpA[b]; v.shpB = d.shpB[b]; v.info = d.info[b]; v.mass = d.mass[b]; v.blocked = d.blocked[b];
  return v;
}

struct GeomOut {
  bool precomputed;   // contact branch taken (precompute ran, normal/contactPoint updated)
  double depth; double ang0, ang1; bool angSet;
  D3 normal, cp, p1, p2, shearInc, twist, ortho, relVn, relVs;
  bool isShearNew;
  int lmIters, lmStop, lmCalls; bool nanNormal;
  // SuperquadricsGeom2 fields set this step: 0 none, 1 sphere pair (curvatures_sum, isSphere),
  // 2 curvatures, curvature angle and contact ellipse
  int hm; double hc[4], hAng; HMEllipse hEll;
};

// SuperquadricsGeom::precompute (Superquadrics.cpp:1030-1050)
__device__ __forceinline__ void precomputeD(GeomOut& g, const D3& oldNormal, const BodyView& b1, const BodyView& b2,
                                            double dt, D3 currentNormal, bool isNew, D3 shift2, D3 shiftVel) {
  if (!isNew) {
    g.ortho = cross(oldNormal, currentNormal);
    double angle = dt * 0.5 * dot(currentNormal, b1.angVel + b2.angVel);
    g.twist = angle * currentNormal;
  } else { g.twist = d3(0, 0, 0); g.ortho = d3(0, 0, 0); }
  g.normal = currentNormal;
  D3 c1x = g.cp - b1.pos;
  D3 c2x = (g.cp - b2.pos) - shift2;
  // shiftVel is zero unless the periodic-boundary correction is on (sqdem_set_periodic_fix)
  D3 relVel = ((b2.vel + shiftVel) + cross(b2.angVel, c2x)) - (b1.vel + cross(b1.angVel, c1x));
  g.relVn = dot(g.normal, relVel) * g.normal;
  g.relVs = relVel - g.relVn;
  g.shearInc = g.relVs * dt;
}

__device__ __forceinline__ void makeShape(SqShape& s, const BodyView& b) {
  shapeInit(s, b.shpA.x, b.shpA.y, b.shpA.z, b.shpB.x, b.shpB.y, b.shpA.w);
  s.R = quatToRot(b.ori.x, b.ori.y, b.ori.z, b.ori.w);
  s.pos = b.pos;
}

// Ig2_Superquadrics_Superquadrics_SuperquadricsGeom::go for the two cases that need no
// Levenberg-Marquardt search: both bodies flagged as spheres (Superquadrics_Ig2.cpp:1950-1970)
// and centres farther apart than the bounding radii (:1973-1979).
__device__ void geomSqSqSimple(GeomOut& g, bool isNew, double prevDepth, D3 oldNormal, D3 oldCp,
                               const BodyView& b1, const BodyView& b2, double dt, D3 shift2, D3 shiftVel) {
  g.precomputed = false; g.angSet = false; g.lmIters = 0; g.lmStop = 0; g.lmCalls = 0; g.nanNormal = false; g.hm = 0;
  g.cp = oldCp;
  const D3 position1 = b1.pos, position2 = b2.pos + shift2;
  double para[2];
  if (isNew) { g.isShearNew = true; centerLine(position1, position2, para); }
  else { g.isShearNew = prevDepth <= 0; para[0] = 0; para[1] = 0; }
  const double rmaxA = b1.shpA.w, rmaxB = b2.shpA.w;
  if (!(b1.info.z != 0 && b2.info.z != 0)) { g.depth = 0; g.isShearNew = true; return; }
  D3 dist = position2 - position1;
  double depth = (rmaxA + rmaxB) - nrm(dist);
  if (depth < 1E-18) { g.depth = 0; g.isShearNew = true; return; }
  normalize(dist);
  const D3 p1 = position1 + rmaxA * dist;
  const D3 p2 = position2 - rmaxB * dist;
  D3 contactNormal = p1 - p2;
  normalize(contactNormal);
  g.p1 = p1; g.p2 = p2;
  g.cp = 0.5 * (p1 + p2);
  g.depth = depth;
  g.precomputed = true;
  precomputeD(g, oldNormal, b1, b2, dt, contactNormal, g.isShearNew, shift2, shiftVel);
  g.normal = contactNormal;
  if (isNew) { g.ang0 = para[0]; g.ang1 = para[1]; g.angSet = true; }
}

// Ig2_Wall_Superquadrics_SuperquadricsGeom::go (Superquadrics_Ig2.cpp:2522-2611)
__device__ void geomWallSq(GeomOut& g, bool isNew, double prevDepth, D3 oldNormal, D3 oldCp, const BodyView& w,
                           const BodyView& b, double dt) {
  g.precomputed = false; g.angSet = false; g.lmIters = 0; g.lmStop = 0; g.lmCalls = 0; g.nanNormal = false; g.hm = 0;
  g.cp = oldCp;
  const int PA = w.info.w & 15;
  const double sense = (double)((w.info.w >> 4) - 1);
  g.isShearNew = isNew ? true : (prevDepth <= 0);
  D3 normal = d3(0, 0, 0);
  if (PA == 0) normal.x = sense; else if (PA == 1) normal.y = sense; else normal.z = sense;
  const double wallc = PA == 0 ? w.pos.x : (PA == 1 ? w.pos.y : w.pos.z);
  if (b.info.z != 0) {
    D3 p1 = b.pos;
    if (PA == 0) p1.x = wallc; else if (PA == 1) p1.y = wallc; else p1.z = wallc;
    D3 point2 = b.pos - normal * b.shpA.w;
    double depth = b.shpA.w - nrm(b.pos - p1);
    if (depth < 0.0) { g.depth = 0; g.isShearNew = true; return; }
    g.p1 = p1; g.p2 = point2;
    g.cp = 0.5 * (point2 + p1);
    g.depth = depth;
  } else {
    SqShape B;
    makeShape(B, b);
    D3 point2 = mulG(B.R, supportLocal(B, -mulL(B.R, normal))) + b.pos;
    D3 p1 = point2;
    if (PA == 0) p1.x = wallc; else if (PA == 1) p1.y = wallc; else p1.z = wallc;
    D3 dd = point2 - p1;
    double nd = PA == 0 ? normal.x * dd.x : (PA == 1 ? normal.y * dd.y : normal.z * dd.z);
    if (nd >= 0.0) { g.depth = 0; g.isShearNew = true; return; }
    g.p1 = p1; g.p2 = point2;
    g.cp = 0.5 * (point2 + p1);
    g.depth = nrm(dd);
  }
  g.precomputed = true;
  precomputeD(g, oldNormal, w, b, dt, normal, g.isShearNew, d3(0, 0, 0), d3(0, 0, 0));
  g.normal = normal;
}

// Ig2_Superquadrics_Superquadrics_SuperquadricsGeom2::go for the cases without a Nelder-Mead
// search (Superquadrics_Ig2.cpp:2348-2390): both bodies spheres, or centres farther apart than
// the bounding radii.  The reference uses the unshifted positions here (only precompute
// sees shift2).
__device__ void geomSqSq2Simple(GeomOut& g, bool isNew, double prevDepth, D3 oldNormal, D3 oldCp,
                                const BodyView& b1, const BodyView& b2, double dt, D3 shift2, D3 shiftVel) {
  g.precomputed = false; g.angSet = false; g.lmIters = 0; g.lmStop = 0; g.lmCalls = 0; g.nanNormal = false; g.hm = 0;
  g.cp = oldCp;
  g.isShearNew = isNew ? true : (prevDepth <= 0);
  const D3 position1 = b1.pos, position2 = b2.pos;
  const double rmaxA = b1.shpA.w, rmaxB = b2.shpA.w;
  const double r_sum = rmaxA + rmaxB;
  if (!(b1.info.z != 0 && b2.info.z != 0)) { g.depth = 0; g.isShearNew = true; return; }
  D3 dist = position2 - position1;
  const double depth = r_sum - nrm(dist);
  if (depth < 1E-18) { g.depth = 0; g.isShearNew = true; return; }
  normalize(dist);
  const D3 p1 = position1 + rmaxA * dist;
  const D3 p2 = position2 - rmaxB * dist;
  D3 contactNormal = p1 - p2;
  normalize(contactNormal);
  g.p1 = p1; g.p2 = p2;
  g.cp = 0.5 * (p1 + p2);
  g.depth = depth;
  g.hm = 1; g.hEll.sum = r_sum / (rmaxA * rmaxB);
  g.precomputed = true;
  precomputeD(g, oldNormal, b1, b2, dt, contactNormal, g.isShearNew, shift2, shiftVel);
  g.normal = contactNormal;
  g.ang0 = 0; g.ang1 = 0; g.angSet = true;
}

// SuperquadricsGeom::rotate (Superquadrics.cpp:1053-1080)
__device__ __forceinline__ D3 rotateShear(const GeomOut& g, D3 sf) {
  sf = sf - cross(sf, g.ortho);
  sf = sf - cross(sf, g.twist);
  sf = sf - dot(g.normal, sf) * g.normal;
  return sf;
}

struct Counters { unsigned long long lmCalls, lmIters, lmMax, nanN, nanF; };

__device__ __forceinline__ void flushCounters(const Dev& d, Counters c) {
  for (int o = 16; o > 0; o >>= 1) {
    c.lmCalls += __shfl_down_sync(0xffffffffu, c.lmCalls, o); c.lmIters += __shfl_down_sync(0xffffffffu, c.lmIters, o);
    c.lmMax += __shfl_down_sync(0xffffffffu, c.lmMax, o); c.nanN += __shfl_down_sync(0xffffffffu, c.nanN, o);
    c.nanF += __shfl_down_sync(0xffffffffu, c.nanF, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (c.lmCalls) atomicAdd(&d.S->err[E_LM_CALLS], c.lmCalls);
    if (c.lmIters) atomicAdd(&d.S->err[E_LM_ITERS], c.lmIters);
    if (c.lmMax) atomicAdd(&d.S->err[E_LM_MAX], c.lmMax);
    if (c.nanN) atomicAdd(&d.S->err[E_NAN_NORMAL], c.nanN);
    if (c.nanF) atomicAdd(&d.S->err[E_NAN_FORCE], c.nanF);
  }
}

// Ip2_SuperquadricsMat2_SuperquadricsMat2_HertzMindlinPhys::go (Superquadrics.cpp:1118-1160) and
// SuperquadricsLaw2::go (Superquadrics.cpp:1367-1557) for one entry whose geometry g was just
// computed.  phys = (kn, ks, tanphi, -); particle pairs (id1 > 5) get kn and ks from the contact
// ellipse every step they touch, walls (ids 0-5) keep their material's Kn, Ks.  kn and ks are
// computed in double where the reference uses long double for pi and the products (a relative
// difference of a few 1e-16).  A NaN force stops the run after this step (Scene::stopAtIter).
__device__ void finishHM(const Dev& d, int e, unsigned fl, int id1, const BodyView& b1, const BodyView& b2,
                         const GeomOut& g, Counters& cnt) {
  const double4 m1 = d.mats[b1.info.y], m2 = d.mats[b2.info.y];
  const double2 mb1 = d.matsB[b1.info.y], mb2 = d.matsB[b2.info.y];
  double4 ph;
  if (!(fl & F_PHYS)) {
    if (id1 > 5) {
      ph.x = 0; ph.y = 0; ph.z = tan(fmin_ref(m1.z, m2.z));
    } else {
      ph.z = tan(m1.z); ph.x = m1.x; ph.y = m1.y;
    }
    ph.w = 0;
    fl |= F_PHYS;
  } else ph = d.A.phys[e];
  const double2 beta = make_double2(fmax_ref(mb1.x, mb2.x), fmax_ref(mb1.y, mb2.y));
  if (!(g.depth > 1E-18)) {
    d.A.phys[e] = ph;
    d.A.nforce[e] = make_double4(0, 0, 0, 0);
    d.A.shear[e] = make_double4(0, 0, 0, 0);
    d.A.flags[e] = fl & ~F_FORCE;
    return;
  }
  if (id1 > 5) {
    const double2 E1 = d.matsE[b1.info.y], E2 = d.matsE[b2.info.y];   // (G, nu)
    const double Gab = 1.0 / ((1 - E1.y) / E1.x + (1 - E2.y) / E2.x);
    const double mu1 = 1. / E1.x + 1. / E2.x;
    const double mu2 = E1.y / E1.x + E2.y / E2.x;
    const double depth = g.depth;
    const double csum = g.hEll.sum;
    if (g.hm == 1) {
      const double tmp = sqrt(depth / csum);
      ph.x = 8. / 3. * Gab * tmp;
      ph.y = 8. / (2.0 * mu1 - mu2) * tmp;
    } else {
      const double E = g.hEll.E, K = g.hEll.K, alpha = g.hEll.alpha;
      const double a = sqrt(depth * E / csum / K);
      ph.x = 4. / 3. * M_PI * a * Gab * alpha / K;
      const double e2 = 1 - 1 / (alpha * alpha);
      const double ksx = mu1 * K - mu2 * (K - E) / e2;
      const double ksy = mu1 * K + mu2 * ((1 - e2) * K - E) / e2;
      ph.y = M_PI * alpha * a * (1. / ksx + 1. / ksy);
    }
  }
  d.A.phys[e] = ph;
  D3 normalForce = g.normal * g.depth * ph.x;
  const bool useDamping = (beta.x > 0.00001 || beta.y > 0.00001);
  double cs = 0;
  if (useDamping) {
    const bool Adyn = b1.blocked != DOF_ALL, Bdyn = b2.blocked != DOF_ALL;
    const double mbar = (!Adyn && Bdyn) ? b2.mass : ((!Bdyn && Adyn) ? b1.mass : (b1.mass * b2.mass / (b1.mass + b2.mass)));
    const double Cn_crit = 2. * sqrt(mbar * ph.x), Cs_crit = 2. * sqrt(mbar * ph.y);
    const double cn = Cn_crit * beta.x;
    cs = Cs_crit * beta.y;
    const D3 normalViscous = cn * g.relVn;
    const D3 normTemp = normalForce - normalViscous;
    if (dot(normTemp, g.normal) < 0.0) normalForce = d3(0, 0, 0);
    else normalForce = normalForce - normalViscous;
  }
  D3 shearForce1;
  if (g.isShearNew) shearForce1 = d3(0, 0, 0);
  else shearForce1 = rotateShear(g, xyz(d.A.shear[e]));
  shearForce1 = shearForce1 - ph.y * g.shearInc;
  const double maxFs = sqn(normalForce) * (ph.z * ph.z);   // std::pow(x, 2) is x*x correctly rounded
  if (sqn(shearForce1) > maxFs) {
    const double ratio = sqrt(maxFs) / nrm(shearForce1);
    shearForce1 = shearForce1 * ratio;
  } else if (useDamping) {
    shearForce1 = shearForce1 - cs * g.relVs;
  }
  if (isnan(shearForce1.x) || isnan(normalForce.x)) {
    normalForce = d3(0, 0, 0); shearForce1 = d3(0, 0, 0); cnt.nanF++;
    d.S->haltAt = d.S->iter + 1;
  }
  d.A.F[e] = dd4((-normalForce) - shearForce1, 0);
  d.A.nforce[e] = dd4(normalForce, 0);
  d.A.shear[e] = dd4(shearForce1, 0);
  d.A.flags[e] = fl | F_FORCE;
}

// Geometry history writes, Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys::go
// (Superquadrics.cpp:1086-1116) and SuperquadricsLaw::go (Superquadrics.cpp:1209-1361) for
// one entry whose geometry g was just computed.
__device__ void finishEntry(const Dev& d, int e, unsigned fl, bool isNew, int id1, const BodyView& b1,
                            const BodyView& b2, const GeomOut& g, Counters& cnt) {
  const bool full = d.prm->recordFull != 0;
  cnt.nanN += g.nanNormal;
  fl |= F_GEOM;
  fl = g.isShearNew ? (fl | F_SHEARNEW) : (fl & ~F_SHEARNEW);
  d.A.depth[e] = g.depth;
  if (g.angSet) d.A.angle[e] = make_double2(g.ang0, g.ang1);
  else if (isNew) d.A.angle[e] = make_double2(0, 0);
  if (g.precomputed) { d.A.normal[e] = dd4(g.normal, 0); d.A.cp[e] = dd4(g.cp, 0); }
  else if (isNew) { d.A.normal[e] = make_double4(0, 0, 0, 0); d.A.cp[e] = make_double4(0, 0, 0, 0); }
  if (full && g.precomputed) {
    d.A.p1[e] = dd4(g.p1, 0); d.A.p2[e] = dd4(g.p2, 0); d.A.shearInc[e] = dd4(g.shearInc, 0);
    d.A.twist[e] = dd4(g.twist, 0); d.A.ortho[e] = dd4(g.ortho, 0);
    d.A.relVn[e] = dd4(g.relVn, 0); d.A.relVs[e] = dd4(g.relVs, 0);
  } else if (full && isNew) {
    const double4 z = make_double4(0, 0, 0, 0);
    d.A.p1[e] = z; d.A.p2[e] = z; d.A.shearInc[e] = z; d.A.twist[e] = z; d.A.ortho[e] = z; d.A.relVn[e] = z; d.A.relVs[e] = z;
  }
  if (full && isNew) { d.A.hmCurv[e] = make_double4(0, 0, 0, 0); d.A.hmEll[e] = make_double4(0, 0, 0, 0); d.A.hmSum[e] = make_double2(0, 0); }
  if (full && g.hm == 1) d.A.hmSum[e] = make_double2(g.hEll.sum, 1.0);
  if (full && g.hm == 2) {
    d.A.hmCurv[e] = make_double4(g.hc[0], g.hc[1], g.hc[2], g.hc[3]);
    d.A.hmEll[e] = make_double4(g.hAng, g.hEll.alpha, g.hEll.K, g.hEll.E);
    d.A.hmSum[e] = make_double2(g.hEll.sum, d.A.hmSum[e].y);
  }
  if (d.prm->contactModel == SQDEM_CONTACT_HERTZ_MINDLIN) { finishHM(d, e, fl, id1, b1, b2, g, cnt); return; }
  double4 ph;
  double2 beta;
  const double2 mb1 = d.matsB[b1.info.y], mb2 = d.matsB[b2.info.y];
  beta.x = fmax_ref(mb1.x, mb2.x); beta.y = fmax_ref(mb1.y, mb2.y);
  if (!(fl & F_PHYS)) {
    const double4 m1 = d.mats[b1.info.y], m2 = d.mats[b2.info.y];
    if (id1 > 5) {
      double fa = fmin_ref(m1.z, m2.z);
      ph.z = tan(fa);
      ph.x = 2.0 * m1.x * m2.x / (m1.x + m2.x);
      ph.y = 2.0 * m1.y * m2.y / (m1.y + m2.y);
    } else {
      ph.z = tan(m1.z); ph.x = m1.x; ph.y = m1.y;
    }
    ph.w = 0;
    d.A.phys[e] = ph;
    fl |= F_PHYS;
  } else ph = d.A.phys[e];
  if (!(g.depth > 1E-18)) {
    d.A.nforce[e] = make_double4(0, 0, 0, 0);
    d.A.shear[e] = make_double4(0, 0, 0, 0);
    fl &= ~F_FORCE;
  } else {
    D3 normalForce = g.normal * g.depth * ph.x;
    const bool useDamping = (beta.x > 1e-5 || beta.y > 1e-5);
    double cs = 0;
    D3 shearViscous = d3(0, 0, 0);
    if (useDamping) {
      const bool Adyn = b1.blocked != DOF_ALL, Bdyn = b2.blocked != DOF_ALL;
      double mbar = (!Adyn && Bdyn) ? b2.mass : ((!Bdyn && Adyn) ? b1.mass : (b1.mass * b2.mass / (b1.mass + b2.mass)));
      double Cn_crit = 2. * sqrt(mbar * ph.x);
      double Cs_crit = 2. * sqrt(mbar * ph.y);
      double cn = Cn_crit * beta.x;
      cs = Cs_crit * beta.y;
      D3 normalViscous = cn * g.relVn;
      D3 normTemp = normalForce - normalViscous;
      if (dot(normTemp, g.normal) < 0.0) normalForce = d3(0, 0, 0);
      else normalForce = normalForce - normalViscous;
    }
    D3 shearForce1;
    if (g.isShearNew) shearForce1 = d3(0, 0, 0);
    else shearForce1 = rotateShear(g, xyz(d.A.shear[e]));
    shearForce1 = shearForce1 - ph.y * g.shearInc;
    double maxFs = sqn(normalForce) * (ph.z * ph.z);
    if (sqn(shearForce1) > maxFs) {
      double ratio = sqrt(maxFs) / nrm(shearForce1);
      shearForce1 = shearForce1 * ratio;
    } else if (useDamping) {
      shearViscous = cs * g.relVs;
    }
    if (isnan(shearForce1.x) || isnan(normalForce.x)) { normalForce = d3(0, 0, 0); shearForce1 = d3(0, 0, 0); cnt.nanF++; }
    D3 Fv = ((-normalForce) - shearForce1) + shearViscous;
    d.A.F[e] = dd4(Fv, 0);
    d.A.nforce[e] = dd4(normalForce, 0);
    d.A.shear[e] = dd4(shearForce1, 0);
    fl |= F_FORCE;
  }
  fl = (fl & ~F_ITERS_MASK) | (itersBucket(g.lmCalls > 0 ? g.lmIters : 0) << F_ITERS_SHIFT);
  d.A.flags[e] = fl;
}

__device__ __forceinline__ void entryIds(const Dev& d, int e, unsigned fl, int& id1, int& id2) {
  const int owner = d.A.owner[e], partner = d.A.partner[e];
  id1 = (fl & F_OWNER_ID1) ? owner : partner;
  id2 = (fl & F_OWNER_ID1) ? partner : owner;
}

// FP32 shape of a body for the separation screens (all in FP32)
__device__ __forceinline__ void shapeInitF32(SqShapeF& s, const BodyView& b, F3 relPos) {
  s.rx = (float)b.shpA.x; s.ry = (float)b.shpA.y; s.rz = (float)b.shpA.z;
  s.e1 = (float)b.shpB.x; s.e2 = (float)b.shpB.y;
  s.a1 = 2.f - s.e1; s.i1 = 1.f / (2.f - s.e1); s.i2 = 1.f / (2.f - s.e2);
  const float w = (float)b.ori.x, x = (float)b.ori.y, y = (float)b.ori.z, z = (float)b.ori.w;
  const float tx = 2.f * x, ty = 2.f * y, tz = 2.f * z;
  const float twx = tx * w, twy = ty * w, twz = tz * w, txx = tx * x, txy = ty * x, txz = tz * x;
  const float tyy = ty * y, tyz = tz * y, tzz = tz * z;
  s.R[0] = 1.f - (tyy + tzz); s.R[1] = txy - twz; s.R[2] = txz + twy;
  s.R[3] = txy + twz; s.R[4] = 1.f - (txx + tzz); s.R[5] = tyz - twx;
  s.R[6] = txz - twy; s.R[7] = tyz + twx; s.R[8] = 1.f - (txx + tyy);
  s.px = relPos.x; s.py = relPos.y; s.pz = relPos.z;
}

// Separation screen of a superquadric pair at the point where lmder2 would start.  If one FP32
// Disfunction evaluation there shows a support gap c.(p2 - p1) larger than SCREEN_MARGIN times
// the summed bounding radii (FP32 error is ~1e-7 of the size), the FP64 evaluation at the same
// point has a positive gap too, so lmder2 stops at its first check with stop_flag set
// (Superquadrics_Ig2.cpp:1138-1143): not touching, contactAngle unchanged, depth 0.
static const float SCREEN_MARGIN = 1e-4f;
__device__ bool screenSeparated(const BodyView& b1, const BodyView& b2, double pa0, double pa1, D3 shift2) {
  if (!isfinite(pa0) || !isfinite(pa1)) return false;
  SqShapeF A, B;
  const D3 rel = (b2.pos + shift2) - b1.pos;
  shapeInitF32(A, b1, f3(0, 0, 0));
  shapeInitF32(B, b2, f3((float)rel.x, (float)rel.y, (float)rel.z));
  F3 p1, p2;
  float sep;
  disfunctionF(A, B, (float)pa0, (float)pa1, p1, p2, sep);
  return sep > SCREEN_MARGIN * (float)(b1.shpA.w + b2.shpA.w);
}

// The same screen for the Nelder-Mead search of the Hertz-Mindlin geometry over the three
// vertices of its first simplex, in the order the search evaluates them
// (Superquadrics_Ig2.cpp:1724-1739).  Along the direction of each vertex (angles in the
// CRotationMat frame) the FP32 gap c.(p2 - p1) is compared with +-SCREEN_MARGIN of the summed
// bounding radii: when the vertices before vertex k are clearly not separating and vertex k
// clearly is, the FP64 search ends at its k-th evaluation with the particles apart and returns
// the first vertex.  Returns that evaluation count (1-3), or 0 when the FP64 search must run.
// The frame and the support points are computed in FP32 (the frame's branch on the FP64 cosine).
__device__ int screenSeparatedNM(const BodyView& b1, const BodyView& b2, double pa0, double pa1, double del) {
  if (!isfinite(pa0) || !isfinite(pa1)) return 0;
  const D3 rel = b2.pos - b1.pos;   // unshifted positions, as the Hertz-Mindlin geometry
  const F3 e = f3((float)rel.x, (float)rel.y, (float)rel.z);
  SqShapeF A, B;
  shapeInitF32(A, b1, f3(0, 0, 0));
  shapeInitF32(B, b2, e);
  // CRotationMat in FP32 (x onto e: a rotation about x cross e), with the branch for e along
  // x taken on the FP64 cosine, as the FP64 frame takes it
  const double cphi64 = dot(d3(1., 0, 0), rel) / (nrm(d3(1., 0, 0)) * nrm(rel));
  const float cphi = (float)cphi64;
  const float ch = sqrtf(0.5f * (1 + cphi)), sh = sqrtf(0.5f * (1 - cphi));
  float qw = ch, qx = 0, qy = 0, qz = sh;
  if (!(fabs(cphi64) > 1.0 - 1e-10)) {
    const float ny = -e.z, nz = e.y, nn = sqrtf(ny * ny + nz * nz);
    qy = ny / nn * sh; qz = nz / nn * sh;
  }
  const float tx = 2.f * qx, ty = 2.f * qy, tz = 2.f * qz;
  const float twx = tx * qw, twy = ty * qw, twz = tz * qw, txx = tx * qx, txy = ty * qx, txz = tz * qx;
  const float tyy = ty * qy, tyz = tz * qy, tzz = tz * qz;
  const float g[9] = {1.f - (tyy + tzz), txy - twz, txz + twy, txy + twz, 1.f - (txx + tzz), tyz - twx,
                      txz - twy, tyz + twx, 1.f - (txx + tyy)};
  const float margin = SCREEN_MARGIN * (float)(b1.shpA.w + b2.shpA.w);
  for (int k = 0; k < 3; k++) {
    const double q0 = k == 1 ? pa0 + del : pa0, q1 = k == 2 ? pa1 + del : pa1;
    float s0, c0, s1, c1;
    sincosf((float)q0, &s0, &c0);
    sincosf((float)q1, &s1, &c1);
    const F3 l = f3(c0 * c1, s0 * c1, s1);
    const F3 c = f3(g[0] * l.x + (g[1] * l.y + g[2] * l.z), g[3] * l.x + (g[4] * l.y + g[5] * l.z),
                    g[6] * l.x + (g[7] * l.y + g[8] * l.z));
    const F3 p1 = supportF(A, c);
    const F3 p2 = supportF(B, f3(-c.x, -c.y, -c.z));
    const float sep = dotf(c, f3(p2.x - p1.x, p2.y - p1.y, p2.z - p1.z));
    if (sep > margin) return k + 1;
    if (!(sep < -margin)) return 0;
  }
  return 0;
}

// Pass 1 over the table: every entry that needs no Levenberg-Marquardt iteration is finished
// here (bound-separated pairs, wall contacts, sphere pairs, bounding-sphere rejections, pairs the
// FP32 screen proves separated at the LM start point); the rest is queued for k_contacts_lm.
__global__ void __launch_bounds__(128, 3) k_contacts_pre(Dev d) {
  const SceneState& S = *d.S;
  if (S.skip) return;
  const int Pn = S.P;
  const double dt = d.prm->dt;
  Counters cnt = {0, 0, 0, 0, 0};
  const int stride = gridDim.x * blockDim.x;
  for (int e0 = blockIdx.x * blockDim.x; e0 < Pn; e0 += stride) {
    const int e = e0 + threadIdx.x;
    bool queue = false, shortq = false;
    if (e < Pn) {
      unsigned fl = d.A.flags[e];
      int id1, id2;
      entryIds(d, e, fl, id1, id2);
      const D3 shift2 = cellShift(S, d.A.cd[e]);
      // SuperquadricsLaw's bound-separation erase (Superquadrics.cpp:1194-1207) discards what
      // the geometry functor computed, so it is tested first (B's bounds shifted by shift2).
      const double4 amn = d.bmin[id1], amx = d.bmax[id1];
      double4 bmn = d.bmin[id2], bmx = d.bmax[id2];
      if (S.periodic) {
        bmn.x += shift2.x; bmn.y += shift2.y; bmn.z += shift2.z;
        bmx.x += shift2.x; bmx.y += shift2.y; bmx.z += shift2.z;
      }
      if (amn.x >= bmx.x || bmn.x >= amx.x || amn.y >= bmx.y || bmn.y >= amx.y || amn.z >= bmx.z || bmn.z >= amx.z) {
        d.A.flags[e] = (fl & ~(F_GEOM | F_PHYS | F_FORCE)) | F_SHEARNEW;
        d.A.nforce[e] = make_double4(0, 0, 0, 0);
        d.A.shear[e] = make_double4(0, 0, 0, 0);
      } else {
        const BodyView b1 = loadBody(d, id1), b2 = loadBody(d, id2);
        const bool isNew = !(fl & F_GEOM);
        const double prevDepth = isNew ? 0.0 : d.A.depth[e];
        const D3 oldNormal = isNew ? d3(0, 0, 0) : xyz(d.A.normal[e]);
        const D3 oldCp = isNew ? d3(0, 0, 0) : xyz(d.A.cp[e]);
        GeomOut g;
        bool done = true;
        if (b1.info.x == KIND_WALL) geomWallSq(g, isNew, prevDepth, oldNormal, oldCp, b1, b2, dt);
        else if (d.prm->contactModel == SQDEM_CONTACT_HERTZ_MINDLIN) {
          const bool sph = (b1.info.z != 0) && (b2.info.z != 0);
          if (sph || nrm(b1.pos - b2.pos) > b1.shpA.w + b2.shpA.w) {
            geomSqSq2Simple(g, isNew, prevDepth, oldNormal, oldCp, b1, b2, dt, shift2, shiftVelOf(S, *d.prm, shift2));
          } else {
            const double2 an = isNew ? make_double2(0, 0) : d.A.angle[e];
            const int nev = screenSeparatedNM(b1, b2, an.x, an.y, isNew ? 0.1 : 0.001);
            if (nev) {
              g.precomputed = false; g.nanNormal = false; g.lmIters = nev; g.lmStop = 0; g.lmCalls = 1; g.hm = 0;
              g.cp = oldCp; g.depth = 0; g.isShearNew = true;
              g.ang0 = an.x; g.ang1 = an.y; g.angSet = true;
              cnt.lmCalls++; cnt.lmIters += nev;
            } else done = false;
          }
        } else {
          const bool sph = (b1.info.z != 0) && (b2.info.z != 0);
          if (!sph && !(nrm(b1.pos - (b2.pos + shift2)) > b1.shpA.w + b2.shpA.w)) {
            double para[2];
            if (isNew) centerLine(b1.pos, b2.pos + shift2, para);
            else { const double2 an = d.A.angle[e]; para[0] = an.x; para[1] = an.y; }
            if (screenSeparated(b1, b2, para[0], para[1], shift2)) {
              g.precomputed = false; g.nanNormal = false; g.lmIters = 0; g.lmStop = 0; g.lmCalls = 1;
              g.cp = oldCp; g.depth = 0; g.isShearNew = true;
              g.ang0 = para[0]; g.ang1 = para[1]; g.angSet = true;
              cnt.lmCalls++;
            } else done = false;
          } else geomSqSqSimple(g, isNew, prevDepth, oldNormal, oldCp, b1, b2, dt, shift2, shiftVelOf(S, *d.prm, shift2));
        }
        if (done) finishEntry(d, e, fl, isNew, id1, b1, b2, g, cnt);
        else {
          queue = true;
          // searches expected short go to the back of the queue, so that the long ones start
          // first: Nelder-Mead searches of a contact touching at the previous step (the warm start
          // usually converges on its first simplex), Levenberg-Marquardt searches of an existing
          // contact that took fewer than 4 iterations at the last step
          shortq = d.prm->contactModel == SQDEM_CONTACT_HERTZ_MINDLIN
                       ? (!isNew && prevDepth > 0)
                       : (!isNew && ((fl & F_ITERS_MASK) >> F_ITERS_SHIFT) < LONG_ITERS_BUCKET);
          // Levenberg-Marquardt searches that took 32 or more iterations at the last step go to
          // the long-search queue (fbQueue): the FP64 kernel spreads them over its warps, at
          // most LONG_PER_WARP per warp, and gives them the spare evaluation slots, so that the
          // chains of dependent evaluations that bound the stage advance an iteration per round;
          // the mixed form runs them in FP64 (a double-float search that long would be deferred)
          if (d.prm->contactModel != SQDEM_CONTACT_HERTZ_MINDLIN && !isNew &&
              (int)((fl & F_ITERS_MASK) >> F_ITERS_SHIFT) >= d.prm->vlongBucket) {
            queue = false;
            const int k = atomicAdd(&d.S->vlCount, 1);
            d.fbQueue[k] = e;
            atomicAdd(&d.S->err[E_LONG_QUEUE], 1ull);
          }
        }
      }
    }
    // warp-aggregated appends to the queue: front (lmCount) and back (nmShort)
    const int lane = threadIdx.x & 31;
    const unsigned m = __ballot_sync(0xffffffffu, queue && !shortq);
    if (m) {
      const int leader = __ffs(m) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(&d.S->lmCount, __popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (queue && !shortq) d.lmQueue[base + __popc(m & ((1u << lane) - 1))] = e;
    }
    const unsigned ms = __ballot_sync(0xffffffffu, shortq);
    if (ms) {
      const int leader = __ffs(ms) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(&d.S->nmShort, __popc(ms));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (shortq) d.lmQueue[d.qCap - 1 - (base + __popc(ms & ((1u << lane) - 1)))] = e;
    }
  }
  flushCounters(d, cnt);
}

// Pass 2: the Levenberg-Marquardt searches of lmder2 (Superquadrics_Ig2.cpp:1057-1354),
// restated as a per-lane state machine.  Every round each lane of a warp evaluates exactly
// one Disfunction (Superquadrics_Ig2.cpp:622-687) at the point its state asks for, so the
// warp stays converged on the expensive evaluation while lanes sit at different iterations
// of different contacts; a lane that finishes a contact takes the next one from the queue.
// The sequence of evaluations, decisions and results per contact is that of the reference:
// only JacfunctionApp's re-evaluation at the current point is skipped, whose outputs equal
// the stored ones bit for bit and are overwritten by the two probes that follow.
enum { ST_INIT = 1, ST_PROBE0 = 2, ST_PROBE1 = 3, ST_TRIAL = 4 };

struct LMLane {
  int e, st, phase, k, stop, nu;
  bool stopFlag, touching, isNew, fromCenter;
  double p0, p1, q0, q1, mu, Dp0, Dp1, pfL2, pL2;
  double j00, j01, j11, diag0, diag1, jt0, jt1;
  D3 pf, f1, contact, P1, P2, C;
  unsigned calls, iters, maxit, rounds;
  bool isLong;   // taken from the long-search queue: first claim on the spare slots
};

static const int LM_BS = 128;

// x^3 for the damping update of lmder2 (pow(2*tmp - 1., 3.), Superquadrics_Ig2.cpp:1299): x^2
// split exactly into h + l with a fused multiply-add, then h x + l x with one rounding — the
// correctly rounded cube except in cases of measure ~2^-50, where it is off by one ulp, as a
// general-purpose pow may be.  Four FMA-class operations instead of a general FP64 pow.
__device__ __forceinline__ double cube(double x) {
  const double h = x * x;
  const double l = fma(x, x, -h);
  return fma(h, x, l * x);
}

__device__ __forceinline__ void lmStartSolve(LMLane& L) {
  L.touching = true; L.stopFlag = false; L.stop = 0;
  L.q0 = L.p0; L.q1 = L.p1; L.st = ST_INIT;
}

// top of lmder2's for-loop: loop condition, then the checks before the Jacobian
__device__ __forceinline__ bool lmOuter(LMLane& L) {
  if (!(L.k < 50 && !L.stop)) { if (L.k >= 50) L.stop = 3; return false; }
  if (L.pfL2 <= 1e-20) { L.stop = 6; return false; }
  if (L.stopFlag) { L.stop = 9; L.touching = false; return false; }
  double s0, c0, s1, c1;
  sincos(L.p0, &s0, &c0);
  sincos(L.p1, &s1, &c1);
  L.contact = d3(c0 * c1, s0 * c1, s1);
  double angle = dot(L.pf, L.contact) / (nrm(L.pf) * nrm(L.contact));
  if (fabs(angle) > 0.95) { L.stop = 8; return false; }
  L.q0 = L.p0 + L.Dp0; L.q1 = L.p1; L.st = ST_PROBE0;
  return true;
}
// top of the damping while-loop
__device__ __forceinline__ bool lmInner(LMLane& L) {
  L.j00 += L.mu;
  L.j11 += L.mu;
  const double n_a = L.j00 * L.j11 - L.j01 * L.j01;
  L.Dp0 = (L.jt0 * L.j11 - L.jt1 * L.j01) / n_a;
  L.Dp1 = (L.jt1 * L.j00 - L.jt0 * L.j01) / n_a;
  const double Dp_L2 = sqrt(L.Dp0 * L.Dp0 + L.Dp1 * L.Dp1);
  if (Dp_L2 < 1e-5) { L.stop = 2; L.k++; return lmOuter(L); }
  L.q0 = L.p0 + L.Dp0; L.q1 = L.p1 + L.Dp1;
  if (Dp_L2 >= (L.pL2 + 1e-3) / (1e-12 * 1e-12)) { L.stop = 4; L.k++; return lmOuter(L); }
  L.st = ST_TRIAL;
  return true;
}
// consume the evaluation the lane asked for; returns true while the solve continues
__device__ __forceinline__ bool lmConsume(LMLane& L) {
  switch (L.st) {
    case ST_INIT:
      L.pf = L.P2 - L.P1;
      L.pfL2 = nrm(L.pf);
      L.stop = isfinite(L.pfL2) ? 0 : 7;
      L.k = 0; L.mu = 0; L.nu = 2; L.Dp0 = 1e-7; L.Dp1 = 1e-7;
      return lmOuter(L);
    case ST_PROBE0:
      L.f1 = L.P2 - L.P1;
      L.q0 = L.p0; L.q1 = L.p1 + L.Dp1; L.st = ST_PROBE1;
      return true;
    case ST_PROBE1: {
      const D3 f2 = L.P2 - L.P1, f0 = L.pf;
      const double J00 = (L.f1.x - f0.x) / L.Dp0, J10 = (L.f1.y - f0.y) / L.Dp0, J20 = (L.f1.z - f0.z) / L.Dp0;
      const double J01 = (f2.x - f0.x) / L.Dp1, J11 = (f2.y - f0.y) / L.Dp1, J21 = (f2.z - f0.z) / L.Dp1;
      L.j00 = J00 * J00 + (J10 * J10 + J20 * J20);
      L.j01 = J00 * J01 + (J10 * J11 + J20 * J21);
      L.j11 = J01 * J01 + (J11 * J11 + J21 * J21);
      L.jt0 = J00 * (-1.0 * f0.x) + (J10 * (-1.0 * f0.y) + J20 * (-1.0 * f0.z));
      L.jt1 = J01 * (-1.0 * f0.x) + (J11 * (-1.0 * f0.y) + J21 * (-1.0 * f0.z));
      const double jinf = (fabs(L.jt0) > fabs(L.jt1) ? fabs(L.jt0) : fabs(L.jt1));
      L.pL2 = sqrt(L.p0 * L.p0 + L.p1 * L.p1);
      if (jinf <= 1e-15) { L.stop = 1; return false; }
      if (L.k == 0) L.mu = 1.0 * (L.j00 > L.j11 ? L.j00 : L.j11);
      L.diag0 = L.j00; L.diag1 = L.j11;
      return lmInner(L);
    }
    default: {  // ST_TRIAL
      const D3 pDp_f = L.P2 - L.P1;
      const double pDp_fL2 = nrm(pDp_f);
      if (!isfinite(pDp_fL2)) { L.stop = 7; L.k++; return lmOuter(L); }
      const double dL = L.Dp0 * (L.mu * L.Dp0 + L.jt0) + L.Dp1 * (L.mu * L.Dp1 + L.jt1);
      const double dF = L.pfL2 - pDp_fL2;
      double tmp = dF / dL;
      if (tmp > 0.0) {
        tmp = 1.0 - cube(2 * tmp - 1.);
        L.mu = L.mu * ((tmp >= 0.3333333333333334) ? tmp : 0.3333333333333334);
        L.nu = 2;
        L.p0 = L.q0; L.p1 = L.q1;
        L.pf = pDp_f; L.pfL2 = pDp_fL2;
        L.k++;
        return lmOuter(L);
      }
      L.mu *= L.nu;
      const int nu2 = (int)((unsigned)L.nu << 1);
      if (nu2 <= L.nu) { L.stop = 5; L.k++; return lmOuter(L); }
      L.nu = nu2;
      L.j00 = L.diag0; L.j11 = L.diag1;
      return lmInner(L);
    }
  }
}

// Points lmder2 evaluates next: the requested one in slot 0, then the points that follow it
// under each outcome of the requested evaluation: after INIT the two probes at the start
// point; after PROBE0 the second probe; after a TRIAL the two probes at the trial point
// (accepted), then the next trial with mu*nu (rejected) and its probes, and so on.  Along
// every outcome the points asked for appear in increasing slot order (the order of the
// consume pass).  Every point is computed with the operations the state machine itself
// uses, so a point it later asks for matches bit for bit.  (Ordering the trials first when
// the last iteration had rejections was measured slower.)  Writes q[i] and own[i] = lane
// for each planned slot i < S.
__device__ __forceinline__ void lmPlan(const LMLane& L, double2* q, int* own, int S, int lane) {
  int n = 0;
  q[n] = make_double2(L.q0, L.q1); own[n++] = lane;
  if (L.st == ST_INIT) {
    if (n < S) { q[n] = make_double2(L.p0 + 1e-7, L.p1); own[n++] = lane; }
    if (n < S) { q[n] = make_double2(L.p0, L.p1 + 1e-7); own[n++] = lane; }
  } else if (L.st == ST_PROBE0) {
    if (n < S) { q[n] = make_double2(L.p0, L.p1 + L.Dp1); own[n++] = lane; }
  } else if (L.st == ST_TRIAL) {
    double mu = L.mu, t0 = L.q0, t1 = L.q1, d0 = L.Dp0, d1 = L.Dp1;
    int nu = L.nu;
    while (n < S) {
      q[n] = make_double2(t0 + d0, t1); own[n++] = lane;
      if (n >= S) break;
      q[n] = make_double2(t0, t1 + d1); own[n++] = lane;
      if (n >= S) break;
      // the trial after a rejection of this one (lmConsume's rejection branch, then lmInner)
      mu *= nu;
      const int nu2 = (int)((unsigned)nu << 1);
      if (nu2 <= nu) break;
      nu = nu2;
      const double j00 = L.diag0 + mu, j11 = L.diag1 + mu;
      const double n_a = j00 * j11 - L.j01 * L.j01;
      d0 = (L.jt0 * j11 - L.jt1 * L.j01) / n_a;
      d1 = (L.jt1 * j00 - L.jt0 * L.j01) / n_a;
      const double Dp_L2 = sqrt(d0 * d0 + d1 * d1);
      if (Dp_L2 < 1e-5) break;
      t0 = L.p0 + d0; t1 = L.p1 + d1;
      if (Dp_L2 >= (L.pL2 + 1e-3) / (1e-12 * 1e-12)) break;
      q[n] = make_double2(t0, t1); own[n++] = lane;
    }
  }
}

__device__ __forceinline__ bool sameBits(double2 a, double q0, double q1) {
  return __double_as_longlong(a.x) == __double_as_longlong(q0) && __double_as_longlong(a.y) == __double_as_longlong(q1);
}

// One lmder2 call finished: the restart rules of Superquadrics_Ig2.cpp:2013-2053, and when no
// restart follows, the end of Ig2_Superquadrics_Superquadrics_SuperquadricsGeom::go, Ip2 and
// the law.  Returns true when the contact is finished.
__device__ __forceinline__ bool lmCallEnd(const Dev& d, LMLane& L, const SqShape& A, const SqShape& B, Counters& cnt) {
  const SceneState& S = *d.S;
  for (;;) {
    L.calls++; L.iters += L.k; L.maxit += (L.stop == 3);
    bool restart = false;
    if (L.phase == 0) {
      L.phase = 1;
      if ((isnan(L.p0) || isnan(L.p1) || 7 == L.stop) && L.touching) restart = true;
    } else if (L.phase == 1) {
      L.phase = 3;
      if (L.touching && 10.0 * nrm(L.P2 - L.P1) > A.rmax && (!isInside(A, L.P2 - A.pos) || !isInside(B, L.P1 - B.pos))) {
        L.phase = 2; restart = true;
      }
    } else L.phase = 3;
    if (!restart && L.phase == 1) {  // no NaN restart: continue with the local-minimum check
      L.phase = 3;
      if (L.touching && 10.0 * nrm(L.P2 - L.P1) > A.rmax && (!isInside(A, L.P2 - A.pos) || !isInside(B, L.P1 - B.pos))) {
        L.phase = 2; restart = true;
      }
    }
    if (!restart) break;
    if (!L.fromCenter) {
      double para[2];
      centerLine(A.pos, B.pos, para);
      L.p0 = para[0]; L.p1 = para[1];
      L.fromCenter = true;
      lmStartSolve(L);
      return false;
    }
    // The restarted call would start where the call that just ended started (the centre
    // line), from the state lmStartSolve sets: it is the same computation, and its outcome
    // is the one at hand.  It is counted as run, and the restart rules go on from there.
  }
  // end of Ig2_Superquadrics_Superquadrics_SuperquadricsGeom::go, then Ip2 + law
  const int e = L.e;
  const unsigned fl = d.A.flags[e];
  int id1, id2;
  entryIds(d, e, fl, id1, id2);
  const BodyView b1 = loadBody(d, id1), b2 = loadBody(d, id2);
  GeomOut g;
  g.lmCalls = L.calls; g.lmIters = L.iters; g.lmStop = 0; g.nanNormal = false;
  g.isShearNew = L.isNew ? true : (d.A.depth[e] <= 0);
  g.cp = L.isNew ? d3(0, 0, 0) : xyz(d.A.cp[e]);
  g.ang0 = L.p0; g.ang1 = L.p1; g.angSet = true;
  if (!L.touching) {
    g.precomputed = false; g.depth = 0; g.isShearNew = true;
  } else {
    const double pDepth = dot(L.P1 - L.P2, L.contact);
    g.p1 = L.P1; g.p2 = L.P2;
    if (isnan(L.contact.x)) g.nanNormal = true;
    g.cp = L.C;
    g.depth = pDepth;
    D3 cn = L.contact;
    normalize(cn);
    const D3 oldNormal = L.isNew ? d3(0, 0, 0) : xyz(d.A.normal[e]);
    g.precomputed = true;
    precomputeD(g, oldNormal, b1, b2, d.prm->dt, cn, g.isShearNew, cellShift(S, d.A.cd[e]),
                shiftVelOf(S, *d.prm, cellShift(S, d.A.cd[e])));
    g.normal = cn;
  }
  cnt.lmCalls += L.calls; cnt.lmIters += L.iters; cnt.lmMax += L.maxit;
  finishEntry(d, e, fl, L.isNew, id1, b1, b2, g, cnt);
  return true;
}

// One Disfunction evaluation (Superquadrics_Ig2.cpp:622-687) by a group of six lanes:
// lanes 0-2 of the group compute body A's support point, lanes 3-5 body B's, and the
// independent pow calls of each level of supportLocal run on separate lanes (Y,X,W |
// t,u,v | Z | pc1,w), so that the dependency chain is 4 pow + 2 atan2 + 3 sincos instead of
// 18 pow + 4 atan2 + 6 sincos.  Every value is computed with the operations of
// disfunction/supportLocal (bitwise the same results).  Lane 0 of the group ends with p1,
// p2 and the stop predicate.  All 32 lanes call it (full-warp shuffles); g0 is the group's
// first lane, sub the lane's place in it.  (Four-lane groups, eight points per round, were
// measured slower: one more pow on the chain.)
static const int COOP_LANES = 6, COOP_POINTS = 5;
// FP64 search kernel: searches a warp holds while its queues have work, long-queue searches
// per warp, and the spare slots one search may take in a round (trial, two probes, the next
// trials after rejections)
static const int LONG_PER_WARP = 2, MAX_EXTRA = 4;
__device__ __forceinline__ void coopEval(const SqShape& A, const SqShape& B, double q0, double q1, int g0, int sub,
                                         D3& p1, D3& p2, bool& flag, const Rot* G = nullptr, double* dist = nullptr) {
  const unsigned FULL = 0xffffffffu;
  const int body = sub >= 3 ? 1 : 0;
  const int k = sub - 3 * body;
  const int gb = g0 + 3 * body;
  const SqShape& s = body ? B : A;
  double sv, cv;
  sincos(sub == 1 ? q1 : q0, &sv, &cv);
  const double sa0 = __shfl_sync(FULL, sv, g0), ca0 = __shfl_sync(FULL, cv, g0);
  const double sa1 = __shfl_sync(FULL, sv, g0 + 1), ca1 = __shfl_sync(FULL, cv, g0 + 1);
  const D3 contact = G ? mulG(*G, d3(ca0 * ca1, sa0 * ca1, sa1)) : d3(ca0 * ca1, sa0 * ca1, sa1);
  D3 n = mulL(s.R, contact);
  if (body) n = (-1.0) * n;
  const double v1 = pow(k == 0 ? fabs(s.ry * n.y) : fabs(s.rx * n.x), k == 2 ? s.i2 : s.i1);
  const double Y = __shfl_sync(FULL, v1, gb), X = __shfl_sync(FULL, v1, gb + 1), W = __shfl_sync(FULL, v1, gb + 2);
  const double ph0 = atan2(sgn(n.y) * Y, sgn(n.x) * X);
  double s0, c0;
  sincos(ph0, &s0, &c0);
  const double v2 = pow(k == 2 ? fabs(s0) : fabs(c0), k == 0 ? s.a1 : s.e1);
  const double t = __shfl_sync(FULL, v2, gb), u = __shfl_sync(FULL, v2, gb + 1), v = __shfl_sync(FULL, v2, gb + 2);
  const double Z = pow(fabs(s.rz * n.z * t), s.i2);
  const double ph1 = atan2(sgn(n.z) * Z, W);
  double s1, c1;
  sincos(ph1, &s1, &c1);
  const double v3 = pow(k == 1 ? fabs(s1) : fabs(c1), s.e2);
  const double pc1 = __shfl_sync(FULL, v3, gb), w = __shfl_sync(FULL, v3, gb + 1);
  D3 r;
  r.x = sgn(c0) * s.rx * u * pc1;
  r.y = sgn(s0) * s.ry * v * pc1;
  r.z = sgn(s1) * s.rz * w;
  const D3 p = mulG(s.R, r) + s.pos;
  const double x2 = __shfl_sync(FULL, p.x, g0 + 3), y2 = __shfl_sync(FULL, p.y, g0 + 3), z2 = __shfl_sync(FULL, p.z, g0 + 3);
  p1 = p;
  p2 = d3(x2, y2, z2);
  const D3 dd = p2 - p1;
  flag = dot(contact, dd) > 0;
  if (dist) *dist = nrm(dd);
}

// Slot allocation of one evaluation round: every searching lane (in) gets one slot, the rest
// of the budget goes evenly to all, the remainder to the searches of highest priority (prio:
// the long-search flag above the rounds run so far, the likeliest to bound the kernel), at
// most maxExtra more each.  Returns the lane's slot count (spc) and first slot (base), and the
// round's largest slot count (jmax) for the uniform consume pass.
__device__ __forceinline__ void allocSlots(bool in, unsigned prio, int budget, int maxExtra, int& spc, int& base,
                                           int& jmax) {
  const int lane = threadIdx.x & 31;
  const unsigned act = __ballot_sync(0xffffffffu, in);
  const int nA = __popc(act);
  const int share = budget / nA, extra = budget - share * nA;
  if (!in) prio = 0u;
  int before = 0;
  for (int o = 0; o < 32; o++) {
    const unsigned po = __shfl_sync(0xffffffffu, prio, o);
    if ((act >> o) & 1u) before += (po > prio || (po == prio && o < lane)) ? 1 : 0;
  }
  spc = in ? share + max(0, min(maxExtra, extra - before * maxExtra)) : 0;
  base = spc;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, base, o);
    if (lane >= o) base += y;
  }
  base -= spc;
  jmax = share + min(maxExtra, extra);
}

// Pass 2, FP64.  Rounds of one Disfunction evaluation per lane.  While the queue has work,
// every lane evaluates the point its own search asks for.  Once the queue is drained, the
// lanes left without a contact evaluate, for the searches still running in their warp, the
// points those searches will ask for next (lmPlan); each search then consumes, in its own
// order, every evaluation whose point is the one it asks for.  A search with 31 idle lanes
// beside it thus advances one whole iteration (trial + two probes, or a run of rejected
// trials) per round instead of one evaluation, which shortens the dependency chain of the
// longest searches that bound the kernel.  While at most COOP_POINTS searches run in the
// warp, each point is evaluated by a group of six lanes (coopEval), which shortens each
// round as well.  Results are those of the one-point rounds: an evaluation depends only on
// its point and the two shapes.
// Two builds: MINB = 1 keeps every lane's state in registers (222, two blocks per SM); MINB =
// 3 caps registers at 168 for three blocks per SM (more warps to hide FP64 latency, at the cost
// of a few hundred bytes of spills per thread).  The launch shape (search blocks per SM)
// selects one; the autotuner times both.
// mode: LM_FP64 the FP64 form (main queue and long-search queue); LM_DEFERRED the mixed form's
// FP64 pass: its long-search queue and the searches the double-float kernels deferred.  (Running
// the long-search queue on a second stream beside the double-float kernel was measured slower:
// its blocks take the SM resources the double-float kernel's warps need.)
enum { LM_FP64 = 0, LM_DEFERRED = 2 };
template <int MINB>
__global__ void __launch_bounds__(LM_BS, MINB) k_contacts_lm(Dev d, int mode) {
  __shared__ SqShape shA[LM_BS], shB[LM_BS];
  __shared__ double2 slotQ[LM_BS];
  __shared__ int slotOwner[LM_BS];
  const SceneState& S = *d.S;
  // the main queue (lmQueue: long searches first, then the short ones from its back) and the
  // long-search queue in fbQueue: the searches of 32+ iterations at the last step
  // ([0, vlCount)), in the mixed form's FP64 pass followed by the deferred searches
  // ([vlCount, vlCount + fbCount))
  const int fallback = mode != LM_FP64;   // no main queue: the long-search queue alone
  const int nFront = S.lmCount, count = S.lmCount + S.nmShort;
  const int longBase = 0;
  const int nLongQ = mode == LM_DEFERRED ? S.vlCount + S.fbCount : S.vlCount;
  int* longHead = mode == LM_DEFERRED ? &d.S->fbHead : &d.S->vlHead;
  const int lane = threadIdx.x & 31;
  const int wbase = threadIdx.x & ~31;
  const bool spread = d.prm->lmSpread != 0;
  // searches a warp holds: in the main pass at most LONG_PER_WARP from the long queue, and in
  // all 32 less MAX_EXTRA per long search held while the main queue has work (those slots go
  // to the long searches); in the second pass of the mixed form as many as spread the queue
  // over all warps, at most COOP_POINTS
  const int warps = gridDim.x * (LM_BS / 32);
  const int cap = !spread ? 32 : fallback ? min(COOP_POINTS, max(1, (nLongQ + warps - 1) / warps)) : 32;
  Counters cnt = {0, 0, 0, 0, 0};
  unsigned long long ev64 = 0;
  unsigned roundsMax = 0;
  LMLane L;
  L.isLong = false;
  bool active = false;
  bool mainDone = fallback != 0, longDone = false;   // warp-uniform: the queues this warp found empty
  auto start = [&](int e) {
    // start a contact: Ig2_Superquadrics_Superquadrics_SuperquadricsGeom::go up to lmder2
    SqShape& A = shA[threadIdx.x];
    SqShape& B = shB[threadIdx.x];
    L.e = e;
    const unsigned fl = d.A.flags[L.e];
    int id1, id2;
    entryIds(d, L.e, fl, id1, id2);
    const double4 o1 = d.ori[id1], o2 = d.ori[id2];
    const double4 a1 = d.shpA[id1], a2 = d.shpA[id2], e1 = d.shpB[id1], e2 = d.shpB[id2];
    shapeInit(A, a1.x, a1.y, a1.z, e1.x, e1.y, a1.w); A.R = quatToRot(o1.x, o1.y, o1.z, o1.w); A.pos = xyz(d.pos[id1]);
    shapeInit(B, a2.x, a2.y, a2.z, e2.x, e2.y, a2.w); B.R = quatToRot(o2.x, o2.y, o2.z, o2.w);
    B.pos = xyz(d.pos[id2]) + cellShift(S, d.A.cd[L.e]);
    L.isNew = !(fl & F_GEOM);
    if (L.isNew) { double para[2]; centerLine(A.pos, B.pos, para); L.p0 = para[0]; L.p1 = para[1]; }
    else { const double2 an = d.A.angle[L.e]; L.p0 = an.x; L.p1 = an.y; }
    L.fromCenter = L.isNew;
    L.contact = d3(0, 0, 0); L.P1 = d3(0, 0, 0); L.P2 = d3(0, 0, 0); L.C = d3(0, 0, 0);
    L.phase = 0; L.calls = 0; L.iters = 0; L.maxit = 0; L.rounds = 0;
    lmStartSolve(L);
    active = true;
  };
  while (true) {
    // take work: idle lanes claim entries with one atomic per warp and queue, up to the caps
    const unsigned below = (1u << lane) - 1;
    if (!longDone) {
      const unsigned idle = __ballot_sync(0xffffffffu, !active);
      const int nAct = 32 - __popc(idle);
      const int held = __popc(__ballot_sync(0xffffffffu, active && L.isLong));
      const int perWarp = (fallback || !spread) ? cap : LONG_PER_WARP;
      const int want = min(__popc(idle), min(perWarp - held, cap - nAct));
      if (want > 0) {
        int base = 0;
        if (lane == 0) base = atomicAdd(longHead, want);
        base = __shfl_sync(0xffffffffu, base, 0);
        const int r = __popc(idle & below);
        if (!active && r < want && base + r < nLongQ) { start(d.fbQueue[longBase + base + r]); L.isLong = true; }
        if (base + want >= nLongQ) longDone = true;
      }
    }
    if (!mainDone) {
      const unsigned idle = __ballot_sync(0xffffffffu, !active);
      const int held = spread ? __popc(__ballot_sync(0xffffffffu, active && L.isLong)) : 0;
      const int room = cap - MAX_EXTRA * held - (32 - __popc(idle));
      const int want = min(__popc(idle), room);
      if (want > 0) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&d.S->lmHead, want);
        base = __shfl_sync(0xffffffffu, base, 0);
        const int r = __popc(idle & below);
        if (!active && r < want) {
          const int idx = base + r;
          if (idx < count) { start(idx < nFront ? d.lmQueue[idx] : d.lmQueue[d.qCap - 1 - (idx - nFront)]); L.isLong = false; }
        }
        if (base + want >= count) mainDone = true;
      }
    }
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!act && mainDone && longDone) break;
    if (!act) continue;
    // Points per running search: 1 while the queues have work and the warp holds 32 searches.
    // Otherwise the warp's evaluation slots (five groups of six lanes, coopEval, while at most
    // COOP_POINTS searches run, else 32 single lanes) are shared out: one each, the rest to the
    // long searches first, then to those that have run the most rounds.
    const int nA = __popc(act);
    const bool drained = spread && mainDone && longDone;
    const bool capped = spread && !drained && (cap < 32 || __any_sync(0xffffffffu, active && L.isLong));
    const bool coop = (drained || capped) && nA <= COOP_POINTS;
    const unsigned prio = (L.isLong ? 0x80000000u : 0u) | min(L.rounds, 0x7fffffffu);
    int spc, base, jmax;
    allocSlots(active, prio, (drained || capped) ? (coop ? COOP_POINTS : 32) : nA, drained ? 1 : MAX_EXTRA, spc, base,
               jmax);
    slotOwner[threadIdx.x] = -1;
    __syncwarp();
    if (active) lmPlan(L, &slotQ[wbase + base], &slotOwner[wbase + base], spc, lane);
    __syncwarp();
    D3 P1 = d3(0, 0, 0), P2 = d3(0, 0, 0);
    bool flag = false;
    if (coop) {
      // group g of six lanes evaluates slot g; lanes 30-31 and groups without a point mirror
      // slot 0 (its owner always exists) so that every lane computes on valid inputs
      const int graw = lane / COOP_LANES;
      const int grp = graw < COOP_POINTS ? graw : 0;
      const int sub = graw < COOP_POINTS ? lane - grp * COOP_LANES : lane - COOP_POINTS * COOP_LANES;
      const int o = slotOwner[wbase + grp];
      const bool has = graw < COOP_POINTS && o >= 0;
      const int slot = has ? grp : 0;
      const int src = wbase + slotOwner[wbase + slot];
      const double2 q = slotQ[wbase + slot];
      coopEval(shA[src], shB[src], q.x, q.y, grp * COOP_LANES, sub, P1, P2, flag);
      if (has && sub == 0) ev64++;
    } else {
      const int own = slotOwner[threadIdx.x];
      if (own >= 0) {
        const double2 q = slotQ[threadIdx.x];
        D3 C;
        disfunction(shA[wbase + own], shB[wbase + own], q.x, q.y, C, P1, P2, flag);
        ev64++;
      }
    }
    if (active) L.rounds++;
    for (int j = 0; j < jmax; j++) {
      const int si = base + j;
      const bool mine = j < spc;
      const int src = mine ? (coop ? si * COOP_LANES : si) : lane;
      const double x1 = __shfl_sync(0xffffffffu, P1.x, src), y1 = __shfl_sync(0xffffffffu, P1.y, src),
                   z1 = __shfl_sync(0xffffffffu, P1.z, src);
      const double x2 = __shfl_sync(0xffffffffu, P2.x, src), y2 = __shfl_sync(0xffffffffu, P2.y, src),
                   z2 = __shfl_sync(0xffffffffu, P2.z, src);
      const bool f = __shfl_sync(0xffffffffu, (int)flag, src) != 0;
      if (mine && active && slotOwner[wbase + si] == lane && sameBits(slotQ[wbase + si], L.q0, L.q1)) {
        L.P1 = d3(x1, y1, z1);
        L.P2 = d3(x2, y2, z2);
        L.C = 0.5 * (L.P1 + L.P2);
        if (f) L.stopFlag = true;
        if (!lmConsume(L) && lmCallEnd(d, L, shA[threadIdx.x], shB[threadIdx.x], cnt)) {
          active = false;
          roundsMax = max(roundsMax, L.rounds);
        }
      }
    }
    __syncwarp();
  }
  flushCounters(d, cnt);
  for (int o = 16; o > 0; o >>= 1) {
    ev64 += __shfl_down_sync(0xffffffffu, ev64, o);
    roundsMax = max(roundsMax, __shfl_down_sync(0xffffffffu, roundsMax, o));
  }
  if (lane == 0) { atomicAdd(&d.S->err[E_EVAL64], ev64); atomicMax(&d.S->err[E_ROUNDS_MAX], (unsigned long long)roundsMax); }
}

// ---------------------------------------------------------------------------
// Pass 2 of the Hertz-Mindlin model: the Nelder-Mead searches of
// Ig2_Superquadrics_Superquadrics_SuperquadricsGeom2::go (Superquadrics_Ig2.cpp:2391-2430),
// one per lane, each round one Disfun evaluation per lane (NMState asks for one point per
// step), a lane that finishes a contact taking the next one from the queue.  The search
// starts at the stored contactAngle with the simplex size 0.1 rad for a new geometry and
// 0.001 rad for an existing one.
struct NMLane {
  int e;
  bool isNew;
  NMState M;
  D3 P1, P2;   // support points of the last evaluation (the reference keeps those)
  unsigned rounds;
};

// End of Ig2_Superquadrics_Superquadrics_SuperquadricsGeom2::go after a search that found the
// particles apart (Superquadrics_Ig2.cpp:2392-2397): contactAngle = the returned vertex, no
// contact; then Ip2 + Law2.
__device__ void nmFinishApart(const Dev& d, int e, double r0, double r1, int nfunc, Counters& cnt) {
  const unsigned fl = d.A.flags[e];
  int id1, id2;
  entryIds(d, e, fl, id1, id2);
  const BodyView b1 = loadBody(d, id1), b2 = loadBody(d, id2);
  const bool isNew = !(fl & F_GEOM);
  GeomOut g;
  g.lmCalls = 1; g.lmIters = nfunc; g.lmStop = 0; g.nanNormal = false; g.hm = 0;
  g.cp = isNew ? d3(0, 0, 0) : xyz(d.A.cp[e]);
  g.ang0 = r0; g.ang1 = r1; g.angSet = true;
  g.precomputed = false; g.depth = 0; g.isShearNew = true;
  cnt.lmCalls += 1; cnt.lmIters += nfunc;
  finishEntry(d, e, fl, isNew, id1, b1, b2, g, cnt);
}

// Pass 3 of the Hertz-Mindlin model: the end of
// Ig2_Superquadrics_Superquadrics_SuperquadricsGeom2::go for every search that ended touching
// (Superquadrics_Ig2.cpp:2398-2516): normal and depth from the last evaluation's support
// points, principal curvatures of both surfaces at the returned direction, the contact
// ellipse; then Ip2 + Law2.  One thread per contact.  The searches leave their results in the
// merge buffer of the collider (free until the next collider pass): owner = entry,
// flags = evaluations, angle = returned vertex, depth = distance, p1/p2 = support points.
__global__ void __launch_bounds__(128) k_contacts_nm_finish(Dev d) {
  const SceneState& S = *d.S;
  if (S.skip) return;
  const int n = S.nmFin;
  Counters cnt = {0, 0, 0, 0, 0};
  for (int i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
    const int i = i0 + threadIdx.x;
    if (i < n) {
      const int e = d.B.owner[i];
      const int nfunc = (int)d.B.flags[i];
      const double2 r = d.B.angle[i];
      const double dist = d.B.depth[i];
      const D3 P1 = xyz(d.B.p1[i]), P2 = xyz(d.B.p2[i]);
      const unsigned fl = d.A.flags[e];
      int id1, id2;
      entryIds(d, e, fl, id1, id2);
      const BodyView b1 = loadBody(d, id1), b2 = loadBody(d, id2);
      const bool isNew = !(fl & F_GEOM);
      SqShape A, B;
      makeShape(A, b1);
      makeShape(B, b2);
      const Rot gc = cRotationMat(b1.pos, b2.pos);
      GeomOut g;
      g.lmCalls = 1; g.lmIters = nfunc; g.lmStop = 0; g.nanNormal = false;
      g.isShearNew = isNew ? true : (d.A.depth[e] <= 0);
      g.ang0 = r.x; g.ang1 = r.y; g.angSet = true;
      D3 contactNormal = P1 - P2;
      normalize(contactNormal);
      g.p1 = P1; g.p2 = P2;
      g.cp = 0.5 * (P1 + P2);
      g.depth = dist;
      double sa0, ca0, sa1, ca1;
      sincos(r.x, &sa0, &ca0);
      sincos(r.y, &sa1, &ca1);
      const D3 contact = mulG(gc, d3(ca0 * sa1, sa0 * sa1, ca1));
      const D3 contact1 = mulL(A.R, contact), contact2 = mulL(B.R, contact);
      D3 dmax1 = d3(0, 0, 0), dmin1, dmax2 = d3(0, 0, 0), dmin2;
      bool f1, f2;
      double c1[2], c2[2], ph0, ph1;
      normal2Phi(A, contact1, ph0, ph1);
      curvatures(A, ph0, ph1, dmax1, dmin1, f1, c1);
      normal2Phi(B, (-1.0) * contact2, ph0, ph1);
      curvatures(B, ph0, ph1, dmax2, dmin2, f2, c2);
      const D3 cd1 = (f1 && f2) ? dmax1 : dmin1, cd2 = (f1 && f2) ? dmax2 : dmin2;
      const D3 nd = contactNormal;
      const D3 dir1 = d3(cd1.x * nd.x, cd1.y * nd.y, cd1.z * nd.z) - cd1;
      const D3 dir2 = d3(cd2.x * nd.x, cd2.y * nd.y, cd2.z * nd.z) - cd2;
      double angle = acos(dot(dir1, dir2) / (nrm(dir1) * nrm(dir2)));
      if (isnan(angle)) angle = 0.0;
      g.hm = 2;
      g.hc[0] = c1[0]; g.hc[1] = c1[1]; g.hc[2] = c2[0]; g.hc[3] = c2[1]; g.hAng = angle;
      g.hEll = hertzMindlin(c1, c2, angle);
      const D3 oldNormal = isNew ? d3(0, 0, 0) : xyz(d.A.normal[e]);
      g.precomputed = true;
      precomputeD(g, oldNormal, b1, b2, d.prm->dt, contactNormal, g.isShearNew, cellShift(S, d.A.cd[e]),
                  shiftVelOf(S, *d.prm, cellShift(S, d.A.cd[e])));
      g.normal = contactNormal;
      cnt.lmCalls += 1; cnt.lmIters += nfunc; cnt.lmMax += (nfunc >= NM_NMAX);
      finishEntry(d, e, fl, isNew, id1, b1, b2, g, cnt);
    }
  }
  flushCounters(d, cnt);
}

__global__ void __launch_bounds__(LM_BS) k_contacts_nm(Dev d) {
  __shared__ SqShape shA[LM_BS], shB[LM_BS];
  __shared__ Rot shG[LM_BS];
  __shared__ double2 slotQ[LM_BS];
  __shared__ int slotOwner[LM_BS];
  const SceneState& S = *d.S;
  const int nFront = S.lmCount, count = S.lmCount + S.nmShort;
  const int lane = threadIdx.x & 31;
  const int wbase = threadIdx.x & ~31;
  const bool spread = d.prm->lmSpread != 0;
  Counters cnt = {0, 0, 0, 0, 0};
  unsigned long long ev64 = 0;
  unsigned roundsMax = 0;
  NMLane L;
  bool active = false, exhausted = false;
  while (true) {
    const unsigned idle = __ballot_sync(0xffffffffu, !active && !exhausted);
    if (idle) {
      const int leader = __ffs(idle) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(&d.S->lmHead, __popc(idle));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!active && !exhausted) {
        const int idx = base + __popc(idle & ((1u << lane) - 1));
        if (idx < count) {
          SqShape& A = shA[threadIdx.x];
          SqShape& B = shB[threadIdx.x];
          L.e = idx < nFront ? d.lmQueue[idx] : d.lmQueue[d.qCap - 1 - (idx - nFront)];
          const unsigned fl = d.A.flags[L.e];
          int id1, id2;
          entryIds(d, L.e, fl, id1, id2);
          const double4 o1 = d.ori[id1], o2 = d.ori[id2];
          const double4 a1 = d.shpA[id1], a2 = d.shpA[id2], e1 = d.shpB[id1], e2 = d.shpB[id2];
          shapeInit(A, a1.x, a1.y, a1.z, e1.x, e1.y, a1.w); A.R = quatToRot(o1.x, o1.y, o1.z, o1.w); A.pos = xyz(d.pos[id1]);
          shapeInit(B, a2.x, a2.y, a2.z, e2.x, e2.y, a2.w); B.R = quatToRot(o2.x, o2.y, o2.z, o2.w); B.pos = xyz(d.pos[id2]);
          shG[threadIdx.x] = cRotationMat(A.pos, B.pos);
          L.isNew = !(fl & F_GEOM);
          const double2 an = L.isNew ? make_double2(0, 0) : d.A.angle[L.e];
          nmStart(L.M, an.x, an.y, L.isNew ? 0.1 : 0.001);
          L.P1 = d3(0, 0, 0); L.P2 = d3(0, 0, 0); L.rounds = 0;
          active = true;
        } else exhausted = true;
      }
    }
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!act) break;
    // One point per search while the queue has work.  Once it is drained the warp's slots
    // (five groups of six lanes, coopEval, while at most COOP_POINTS searches run, else 32
    // lanes) are shared out, and each search fills its share with the points nmPlan says it
    // may ask for next.
    const int nA = __popc(act);
    const bool drained = spread && __any_sync(0xffffffffu, exhausted);
    const bool coop = drained && nA <= COOP_POINTS;
    int spc, base, jmax;
    allocSlots(active, L.rounds, drained ? (coop ? COOP_POINTS : 32) : nA, 1, spc, base, jmax);
    slotOwner[threadIdx.x] = -1;
    __syncwarp();
    if (active) {
      const int n = nmPlan(L.M, &slotQ[wbase + base], spc);
      for (int i = 0; i < n; i++) slotOwner[wbase + base + i] = lane;
    }
    __syncwarp();
    D3 P1 = d3(0, 0, 0), P2 = d3(0, 0, 0);
    bool flag = false;
    double f = 0;
    if (coop) {
      const int graw = lane / COOP_LANES;
      const int grp = graw < COOP_POINTS ? graw : 0;
      const int sub = graw < COOP_POINTS ? lane - grp * COOP_LANES : lane - COOP_POINTS * COOP_LANES;
      const int o = slotOwner[wbase + grp];
      const bool has = graw < COOP_POINTS && o >= 0;
      const int slot = has ? grp : 0;
      const int src = wbase + slotOwner[wbase + slot];
      const double2 q = slotQ[wbase + slot];
      coopEval(shA[src], shB[src], q.x, q.y, grp * COOP_LANES, sub, P1, P2, flag, &shG[src], &f);
      if (has && sub == 0) ev64++;
    } else {
      const int own = slotOwner[threadIdx.x];
      if (own >= 0) {
        const double2 q = slotQ[threadIdx.x];
        f = disfunNM(shA[wbase + own], shB[wbase + own], shG[wbase + own], q.x, q.y, P1, P2, flag);
        ev64++;
      }
    }
    if (active) L.rounds++;
    for (int j = 0; j < jmax; j++) {
      const int si = base + j;
      const bool mine = j < spc;
      const int src = mine ? (coop ? si * COOP_LANES : si) : lane;
      const double x1 = __shfl_sync(0xffffffffu, P1.x, src), y1 = __shfl_sync(0xffffffffu, P1.y, src),
                   z1 = __shfl_sync(0xffffffffu, P1.z, src);
      const double x2 = __shfl_sync(0xffffffffu, P2.x, src), y2 = __shfl_sync(0xffffffffu, P2.y, src),
                   z2 = __shfl_sync(0xffffffffu, P2.z, src);
      const double fs = __shfl_sync(0xffffffffu, f, src);
      const bool apart = __shfl_sync(0xffffffffu, (int)flag, src) != 0;
      bool done = false;
      if (mine && active && slotOwner[wbase + si] == lane && sameBits(slotQ[wbase + si], L.M.q0, L.M.q1)) {
        L.P1 = d3(x1, y1, z1); L.P2 = d3(x2, y2, z2);
        done = !nmConsume(L.M, fs, apart);
      }
      // searches that ended touching go to the finish pass (warp-aggregated append)
      const bool fin = done && L.M.touching;
      const unsigned m = __ballot_sync(0xffffffffu, fin);
      if (m) {
        const int leader = __ffs(m) - 1;
        int b0 = 0;
        if (lane == leader) b0 = atomicAdd(&d.S->nmFin, __popc(m));
        b0 = __shfl_sync(0xffffffffu, b0, leader);
        if (fin) {
          const int i = b0 + __popc(m & ((1u << lane) - 1));
          d.B.owner[i] = L.e; d.B.flags[i] = (unsigned)L.M.nfunc;
          d.B.angle[i] = make_double2(L.M.r0, L.M.r1); d.B.depth[i] = L.M.dist;
          d.B.p1[i] = dd4(L.P1, 0); d.B.p2[i] = dd4(L.P2, 0);
        }
      }
      if (done && !L.M.touching) nmFinishApart(d, L.e, L.M.r0, L.M.r1, L.M.nfunc, cnt);
      if (done) { active = false; roundsMax = max(roundsMax, L.rounds); }
    }
    __syncwarp();
  }
  flushCounters(d, cnt);
  for (int o = 16; o > 0; o >>= 1) {
    ev64 += __shfl_down_sync(0xffffffffu, ev64, o);
    roundsMax = max(roundsMax, __shfl_down_sync(0xffffffffu, roundsMax, o));
  }
  if (lane == 0) { atomicAdd(&d.S->err[E_EVAL64], ev64); atomicMax(&d.S->err[E_ROUNDS_MAX], (unsigned long long)roundsMax); }
}

// ---------------------------------------------------------------------------
// Mixed form of pass 2: the searches of lmder2 (Superquadrics_Ig2.cpp:1057-1354) in
// double-float arithmetic on the FP32 pipes (sq_ff.cuh), Disfunction included, with the same
// lockstep lanes, work queue and spare-lane evaluation as the FP64 kernel.  GB300 issues FP64 at
// 1/64 of its FP32 rate: a double-float evaluation costs ~1/12 of the FP64 one, and the search's
// own arithmetic (Jacobian, normal equations, damping, step control) in double-float costs a
// few percent of its evaluations instead of more than they do.
//
// Every decision of lmder2 and of the geometry functor is taken on double-float values only
// when its margin exceeds the difference double-float and FP64 rounding can make: the stop flag
// c.(p2-p1) > 0 and the trial acceptance dF > 0 outside E = 4e-13 of the summed bounding radii
// (~1e-15 m; both arithmetics round these to ~1e-17 m), the 0.95 cosine test outside
// 1e-12 + 4E/|f|, the |Dp| < 1e-5 and |J^T f|inf <= 1e-15 tests outside 1e-5 relative, the
// restart rule's distance and isInside tests outside 1e-9, the law's contact gate outside E.
// A search that meets a decision inside its band, or an evaluation the double-float routines
// do not reproduce (ill: exactly axis-aligned normals, non-finite values), is deferred whole:
// the lane drops it without writing anything and appends it to the fallback queue, which the
// FP64 kernel (k_contacts_lm on that queue) then runs from the same inputs.  The starting
// angles (table or centre line, FP64), the contact points, depth, normal, precompute, Ip2 and
// the law stay FP64.

// Double-float shape of each body for this step (the mixed form's searches load it instead of
// converting per contact).
__global__ void k_body_ff(Dev d) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= d.N) return;
  FFShape f;
  const int4 info = d.info[b];
  if (info.x == KIND_SQ) {
    SqShape s;
    const double4 a = d.shpA[b], e = d.shpB[b], o = d.ori[b];
    shapeInit(s, a.x, a.y, a.z, e.x, e.y, a.w);
    s.R = quatToRot(o.x, o.y, o.z, o.w);
    ffShapeInit(f, s);
  } else {
    memset(&f, 0, sizeof(f));
  }
  d.bodyFF[b] = f;
}

// Superquadrics::isInside value (Superquadrics.cpp:103-108) of point p relative to the centre
__device__ __forceinline__ double insideValue(const SqShape& s, D3 p) {
  p = mulL(s.R, p);
  return pow(pow(fabs(p.x / s.rx), 2.0 / s.e1) + pow(fabs(p.y / s.ry), 2.0 / s.e1), s.e1 / s.e2) +
         pow(fabs(p.z / s.rz), 2.0 / s.e2);
}
__device__ __forceinline__ void shapeFromGlobal(SqShape& s, const Dev& d, int b) {
  const double4 a = d.shpA[b], e = d.shpB[b], o = d.ori[b];
  shapeInit(s, a.x, a.y, a.z, e.x, e.y, a.w);
  s.R = quatToRot(o.x, o.y, o.z, o.w);
}

// One lmder2 call ended: the restart rules of Superquadrics_Ig2.cpp:2013-2053 (as lmCallEnd).
// Returns LMF_MORE when a restarted call begins, LMF_END when the contact's geometry is final,
// LMF_DEFER when a restart decision falls inside its band.
__device__ __noinline__ int lmfCallEnd(const Dev& d, LMF& L, int id1, int id2, D3 pB) {
  for (;;) {
    L.calls++; L.iters += L.k; L.maxit += (L.stop == 3);
    bool restart = false;
    if (L.phase == 0) L.phase = 1;   // no NaN/stop-7 restart: non-finite evaluations were deferred
    if (L.phase == 1) {
      L.phase = 3;
      if (L.touching) {
        ff dd[3];
        for (int i = 0; i < 3; i++) dd[i] = ffSub(L.P2[i], L.P1[i]);
        const float dist = sqrtf(ffDot3(dd[0], dd[1], dd[2], dd[0], dd[1], dd[2]).hi);
        const float rmaxA = d.bodyFF[id1].rmax;
        const float x = 10.f * dist / rmaxA - 1.f;
        if (!(fabsf(x) >= 1e-6f)) return LMF_DEFER;
        if (x > 0.f) {
          SqShape A, B;
          shapeFromGlobal(A, d, id1);
          shapeFromGlobal(B, d, id2);
          const D3 p2a = d3(ffToD(L.P2[0]), ffToD(L.P2[1]), ffToD(L.P2[2]));
          const D3 p1b = d3(ffToD(L.P1[0]), ffToD(L.P1[1]), ffToD(L.P1[2])) - pB;
          const double va = insideValue(A, p2a), vb = insideValue(B, p1b);
          if (!(fabs(va - 1.0) >= 1e-9) || !(fabs(vb - 1.0) >= 1e-9)) return LMF_DEFER;
          if (!(1 > va) || !(1 > vb)) { L.phase = 2; restart = true; }
        }
      }
    } else L.phase = 3;
    if (!restart) return LMF_END;
    if (!L.fromCenter) {
      double para[2];
      centerLine(xyz(d.pos[id1]), xyz(d.pos[id2]) + cellShift(*d.S, d.A.cd[L.e]), para);
      L.p0 = ffFromD(para[0]); L.p1 = ffFromD(para[1]);
      L.fromCenter = true;
      lmfStartSolve(L);
      return LMF_MORE;
    }
    // the restarted call would repeat the one that just ended (same start, same state): its
    // outcome is the one at hand; counted as run
  }
}

// Pass 2, mixed form (see the section comment).  Rounds of one double-float evaluation per
// lane; once the queue is drained, the lanes without a contact evaluate the points the running
// searches of their warp ask for next (lmfPlan), as in k_contacts_lm.  Each lane's search state
// and each round's evaluation results live in shared memory and the bodies' double-float shapes
// are read from bodyFF, so that the registers serve the evaluation (more resident warps hide
// the latency of its dependent FP32 chains).  A finished search's geometry goes to a compact
// list in the merge buffer (table B); k_contacts_lm_ff_finish completes it in FP64.
static const int FFEV_WORDS = 27;   // c, p1, p2, d (ff, 3 each), sep (ff), ill
__global__ void __launch_bounds__(LM_BS) k_contacts_lm_ff(Dev d) {
  __shared__ LMF sL[LM_BS];
  __shared__ float sEv[FFEV_WORDS][LM_BS];
  __shared__ int sId[2][LM_BS];
  __shared__ float sPB[6][LM_BS];
  __shared__ float4 slotQ[LM_BS];
  __shared__ int slotOwner[LM_BS];
  const SceneState& S = *d.S;
  const int nFront = S.lmCount, count = S.lmCount + S.nmShort;   // long searches first
  const int t = threadIdx.x;
  const int lane = t & 31;
  const int wbase = t & ~31;
  const bool spread = d.prm->lmSpread != 0;
  unsigned long long ev32 = 0, deferred = 0;
  unsigned roundsMax = 0;
  LMF& L = sL[t];
  // a warp holds 32 searches while the queue has work (capping it to leave spare slots for the
  // longest searches, as the FP64 kernel does for its long-search queue, was measured slower
  // here: the double-float rounds are short and the bulk throughput dominates)
  const int cap = 32;
  bool active = false, done = false;   // done: warp-uniform, the queue is empty
  while (true) {
    const unsigned idleAll = __ballot_sync(0xffffffffu, !active);
    const int want = done ? 0 : min(__popc(idleAll), cap - (32 - __popc(idleAll)));
    if (want > 0) {
      int base = 0;
      if (lane == 0) base = atomicAdd(&d.S->lmHead, want);
      base = __shfl_sync(0xffffffffu, base, 0);
      const int r = __popc(idleAll & ((1u << lane) - 1));
      if (base + want >= count) done = true;
      if (!active && r < want) {
        const int idx = base + r;
        if (idx < count) {
          const int e = idx < nFront ? d.lmQueue[idx] : d.lmQueue[d.qCap - 1 - (idx - nFront)];
          const unsigned fl = d.A.flags[e];
          int id1, id2;
          entryIds(d, e, fl, id1, id2);
          const D3 shift2 = cellShift(S, d.A.cd[e]);
          const D3 pa = xyz(d.pos[id1]), pb = xyz(d.pos[id2]) + shift2;
          sId[0][t] = id1; sId[1][t] = id2;
          const ff px = ffFromD(pb.x - pa.x), py = ffFromD(pb.y - pa.y), pz = ffFromD(pb.z - pa.z);
          sPB[0][t] = px.hi; sPB[1][t] = px.lo; sPB[2][t] = py.hi; sPB[3][t] = py.lo; sPB[4][t] = pz.hi; sPB[5][t] = pz.lo;
          L.e = e;
          L.E = 4e-13f * (d.bodyFF[id1].rmax + d.bodyFF[id2].rmax);
          L.isNew = !(fl & F_GEOM);
          if (L.isNew) { double para[2]; centerLine(pa, pb, para); L.p0 = ffFromD(para[0]); L.p1 = ffFromD(para[1]); }
          else { const double2 an = d.A.angle[e]; L.p0 = ffFromD(an.x); L.p1 = ffFromD(an.y); }
          L.fromCenter = L.isNew;
          L.phase = 0; L.calls = 0; L.iters = 0; L.maxit = 0; L.rounds = 0;
          lmfStartSolve(L);
          active = true;
        }
      }
    }
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!act) {
      if (done) break;
      continue;
    }
    const int nA = __popc(act);
    const bool drained = spread && done;
    int spc, base, jmax;
    allocSlots(active, active ? L.rounds : 0u, drained ? 32 : nA, 1, spc, base, jmax);
    slotOwner[t] = -1;
    __syncwarp();
    if (active) lmfPlan(L, &slotQ[wbase + base], &slotOwner[wbase + base], spc, lane);
    __syncwarp();
    {
      // lanes without a slot evaluate the warp's first slot (whose owner always exists) so that
      // every lane computes on valid inputs
      const int own = slotOwner[t];
      const int slot = own >= 0 ? t : wbase;
      const int src = wbase + slotOwner[slot];
      const float4 q = slotQ[slot];
      const ff pB[3] = {mkff(sPB[0][src], sPB[1][src]), mkff(sPB[2][src], sPB[3][src]), mkff(sPB[4][src], sPB[5][src])};
      FFEval v;
      ffDisfunction(d.bodyFF[sId[0][src]], d.bodyFF[sId[1][src]], pB, mkff(q.x, q.y), mkff(q.z, q.w), v);
      for (int i = 0; i < 3; i++) {
        sEv[2 * i][t] = v.c[i].hi; sEv[2 * i + 1][t] = v.c[i].lo;
        sEv[6 + 2 * i][t] = v.p1[i].hi; sEv[7 + 2 * i][t] = v.p1[i].lo;
        sEv[12 + 2 * i][t] = v.p2[i].hi; sEv[13 + 2 * i][t] = v.p2[i].lo;
        sEv[18 + 2 * i][t] = v.d[i].hi; sEv[19 + 2 * i][t] = v.d[i].lo;
      }
      sEv[24][t] = v.sep.hi; sEv[25][t] = v.sep.lo; sEv[26][t] = v.ill ? 1.f : 0.f;
      if (own >= 0) ev32++;
    }
    __syncwarp();
    if (active) {
      L.rounds++;
      for (int j = 0; j < spc; j++) {
        const int si = wbase + base + j;
        if (!(slotOwner[si] == lane && sameFF(slotQ[si], L.q0, L.q1))) continue;
        FFEval w;
        for (int i = 0; i < 3; i++) {
          w.c[i] = mkff(sEv[2 * i][si], sEv[2 * i + 1][si]);
          w.p1[i] = mkff(sEv[6 + 2 * i][si], sEv[7 + 2 * i][si]);
          w.p2[i] = mkff(sEv[12 + 2 * i][si], sEv[13 + 2 * i][si]);
          w.d[i] = mkff(sEv[18 + 2 * i][si], sEv[19 + 2 * i][si]);
        }
        w.sep = mkff(sEv[24][si], sEv[25][si]);
        w.ill = sEv[26][si] != 0.f;
        int r = lmfConsume(L, w);
        if (r == LMF_END) r = lmfCallEnd(d, L, sId[0][t], sId[1][t],
                                         d3(ffToD(mkff(sPB[0][t], sPB[1][t])), ffToD(mkff(sPB[2][t], sPB[3][t])),
                                            ffToD(mkff(sPB[4][t], sPB[5][t]))));
        if (r == LMF_END) {
          // the search's geometry to the finish list (merge buffer), completed in FP64 by
          // k_contacts_lm_ff_finish
          const int i = atomicAdd(&d.S->nmFin, 1);
          d.B.owner[i] = L.e;
          d.B.angle[i] = make_double2(ffToD(L.p0), ffToD(L.p1));
          d.B.p1[i] = make_double4(ffToD(L.P1[0]), ffToD(L.P1[1]), ffToD(L.P1[2]), 0);
          d.B.p2[i] = make_double4(ffToD(L.P2[0]), ffToD(L.P2[1]), ffToD(L.P2[2]), 0);
          d.B.normal[i] = make_double4(ffToD(L.c[0]), ffToD(L.c[1]), ffToD(L.c[2]), 0);
          d.B.cd[i] = make_int4((int)L.calls, (int)L.iters, (int)L.maxit, L.touching ? 1 : 0);
        } else if (r == LMF_DEFER) {
          const int k = atomicAdd(&d.S->fbCount, 1);
          d.fbQueue[d.S->vlCount + k] = L.e;
          deferred++;
        }
        if (r != LMF_MORE) {
          active = false;
          roundsMax = max(roundsMax, L.rounds);
          break;   // the rest of this round's slots were planned for the call that ended
        }
      }
    }
    __syncwarp();
  }
  for (int o = 16; o > 0; o >>= 1) {
    ev32 += __shfl_down_sync(0xffffffffu, ev32, o);
    deferred += __shfl_down_sync(0xffffffffu, deferred, o);
    roundsMax = max(roundsMax, __shfl_down_sync(0xffffffffu, roundsMax, o));
  }
  if (lane == 0) {
    atomicAdd(&d.S->err[E_EVAL32], ev32);
    atomicAdd(&d.S->err[E_FALLBACK], deferred);
    atomicMax(&d.S->err[E_ROUNDS_MAX_FF], (unsigned long long)roundsMax);
  }
}

// The end of Ig2_Superquadrics_Superquadrics_SuperquadricsGeom::go (Superquadrics_Ig2.cpp:
// 2054-2095) in FP64 for the searches k_contacts_lm_ff finished, one thread per search: the
// contact points in the global frame, the depth (deferred to the FP64 kernel when inside the
// band of the law's contact gate), normal, precompute, then Ip2 and the law.
__global__ void __launch_bounds__(128) k_contacts_lm_ff_finish(Dev d) {
  const SceneState& S = *d.S;
  if (S.skip) return;
  const int n = S.nmFin;
  const double dt = d.prm->dt;
  Counters cnt = {0, 0, 0, 0, 0};
  unsigned long long deferred = 0;
  for (int i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
    const int i = i0 + threadIdx.x;
    if (i >= n) continue;
    const int e = d.B.owner[i];
    const int4 info = d.B.cd[i];
    const unsigned fl = d.A.flags[e];
    int id1, id2;
    entryIds(d, e, fl, id1, id2);
    const BodyView b1 = loadBody(d, id1), b2 = loadBody(d, id2);
    const bool isNew = !(fl & F_GEOM);
    GeomOut g;
    g.lmCalls = info.x; g.lmIters = info.y; g.lmStop = 0; g.nanNormal = false;
    g.isShearNew = isNew ? true : (d.A.depth[e] <= 0);
    g.cp = isNew ? d3(0, 0, 0) : xyz(d.A.cp[e]);
    const double2 an = d.B.angle[i];
    g.ang0 = an.x; g.ang1 = an.y; g.angSet = true;
    bool ok = true;
    if (!info.w) {
      g.precomputed = false; g.depth = 0; g.isShearNew = true;
    } else {
      const D3 P1 = b1.pos + xyz(d.B.p1[i]), P2 = b1.pos + xyz(d.B.p2[i]);
      const D3 contact = xyz(d.B.normal[i]);
      const double pDepth = dot(P1 - P2, contact);
      const double E = 4e-13 * (b1.shpA.w + b2.shpA.w);
      if (!(fabs(pDepth - 1e-18) >= E)) ok = false;   // the law's contact gate inside its band
      g.p1 = P1; g.p2 = P2;
      g.cp = 0.5 * (P1 + P2);
      g.depth = pDepth;
      D3 cn = contact;
      normalize(cn);
      const D3 oldNormal = isNew ? d3(0, 0, 0) : xyz(d.A.normal[e]);
      g.precomputed = true;
      precomputeD(g, oldNormal, b1, b2, dt, cn, g.isShearNew, cellShift(S, d.A.cd[e]),
                  shiftVelOf(S, *d.prm, cellShift(S, d.A.cd[e])));
      g.normal = cn;
    }
    if (ok) {
      cnt.lmCalls += info.x; cnt.lmIters += info.y; cnt.lmMax += info.z;
      finishEntry(d, e, fl, isNew, id1, b1, b2, g, cnt);
    } else {
      const int k = atomicAdd(&d.S->fbCount, 1);
      d.fbQueue[d.S->vlCount + k] = e;
      deferred++;
    }
  }
  flushCounters(d, cnt);
  if (deferred) atomicAdd(&d.S->err[E_FALLBACK], deferred);
}

// contribution of table entry e to body b (b is id1 when asId1)
__device__ __forceinline__ void addContribution(const Dev& d, int e, bool asId1, D3 pos, D3& f, D3& t) {
  const D3 F = xyz(d.A.F[e]);
  const D3 cp = xyz(d.A.cp[e]);
  // the reference takes body 2's torque arm from its unshifted position (Superquadrics.cpp:1356,
  // FIXME at :1550); the periodic-boundary correction takes it from the image body 2 touches
  if (!asId1 && d.prm->periodicFix && d.S->periodic) pos = pos + cellShift(*d.S, d.A.cd[e]);
  if (asId1) { f = f + F; t = t + (-cross(pos - cp, F)); }
  else { f = f + (-F); t = t + cross(pos - cp, F); }
}

// ForceContainer sum for walls: one block per wall, fixed-order reduction; also the sum of
// kn over the wall's real contacts (CompressionEngine::get_gain, Compression.cpp:1125-1220).
__global__ void k_wall_forces(Dev d) {
  const SceneState& S = *d.S;
  if (S.skip) return;
  __shared__ double sh[7][128];
  const int w = blockIdx.x;
  const int wid = d.walls[w];
  const D3 pos = xyz(d.pos[wid]);
  const int s = d.wCount[d.W + w], n = d.wCount[w];
  D3 f = d3(0, 0, 0), t = d3(0, 0, 0);
  double kn = 0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    int e = d.wList[s + k];
    const unsigned fl = d.A.flags[e];
    if ((fl & (F_GEOM | F_PHYS)) == (F_GEOM | F_PHYS)) kn += d.A.phys[e].x;
    if (!(fl & F_FORCE)) continue;
    addContribution(d, e, !(fl & F_OWNER_ID1), pos, f, t);
  }
  sh[0][threadIdx.x] = f.x; sh[1][threadIdx.x] = f.y; sh[2][threadIdx.x] = f.z;
  sh[3][threadIdx.x] = t.x; sh[4][threadIdx.x] = t.y; sh[5][threadIdx.x] = t.z; sh[6][threadIdx.x] = kn;
  __syncthreads();
  for (int o = 64; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
      for (int c = 0; c < 7; c++) sh[c][threadIdx.x] = sh[c][threadIdx.x] + sh[c][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    d.force[wid] = make_double4(sh[0][0], sh[1][0], sh[2][0], 0);
    d.torque[wid] = make_double4(sh[3][0], sh[4][0], sh[5][0], 0);
    d.wallKn[w] = sh[6][0];
  }
}

// Per-body force sum as NewtonIntegrator sees it (rows owned, then the incidence list).
__device__ __forceinline__ void gatherBody(const Dev& d, int b, D3 pos, D3& f, D3& m) {
  f = d3(0, 0, 0); m = d3(0, 0, 0);
  for (int e = d.rowStart[b]; e < d.rowStart[b + 1]; e++) {
    unsigned fl = d.A.flags[e];
    if (fl & F_FORCE) addContribution(d, e, (fl & F_OWNER_ID1) != 0, pos, f, m);
  }
  for (int k = d.pStart[b]; k < d.pStart[b + 1]; k++) {
    int e = d.pList[k];
    unsigned fl = d.A.flags[e];
    if (fl & F_FORCE) addContribution(d, e, (fl & F_OWNER_ID1) == 0, pos, f, m);
  }
}

// Reductions of the boundary controller and of Shop::getStress / Shop::unbalancedForce, one
// block partial each (summed in block order by the reader: deterministic).  Partial layout:
// [0..8] sum over real contacts with |Fn| != 0 of (Fn+Fs)(pos_id2 - pos_id1)^T (row-major),
// [9] sum of |Fn+Fs| over the same contacts, [10] sum over dynamic bodies of |F + m g|,
// [11..19] sum over all real contacts of (Fn+Fs)(pos_id1 - pos_id2 - hSize cellDist)^T.
// need: 1 stress tensors, 2 force sums; midStep: body forces gathered from the table (the
// controller runs before NewtonIntegrator), else the forces of the last step.
static const int SV_PART = 20;
__device__ __forceinline__ void blockSum(double* sh, int nv, double* v, double* out) {
  // sh: nv x blockDim doubles
  for (int c = 0; c < nv; c++) sh[c * blockDim.x + threadIdx.x] = v[c];
  __syncthreads();
  for (int o = blockDim.x >> 1; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
      for (int c = 0; c < nv; c++) sh[c * blockDim.x + threadIdx.x] += sh[c * blockDim.x + threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) for (int c = 0; c < nv; c++) out[c] = sh[c * blockDim.x];
}
__global__ void __launch_bounds__(128) k_servo_sums(Dev d, int needArg, int midStep) {
  const SceneState& S = *d.S;
  const int need = needArg < 0 ? S.sv.need : needArg;
  if ((needArg < 0 && S.skip) || !need) return;
  __shared__ double sh[SV_PART * 128];
  double v[SV_PART];
  for (int c = 0; c < SV_PART; c++) v[c] = 0;
  const int stride = gridDim.x * blockDim.x;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < S.P; e += stride) {
    const unsigned fl = d.A.flags[e];
    if ((fl & (F_GEOM | F_PHYS)) != (F_GEOM | F_PHYS)) continue;
    int id1, id2;
    entryIds(d, e, fl, id1, id2);
    const D3 fn = xyz(d.A.nforce[e]), fs = xyz(d.A.shear[e]);
    const D3 f = fn + fs;
    const D3 p1 = xyz(d.pos[id1]), p2 = xyz(d.pos[id2]);
    if (need & 1) {
      D3 br = p1 - p2;
      if (S.periodic) br = br - cellShift(S, d.A.cd[e]);
      const double fa[3] = {f.x, f.y, f.z}, ba[3] = {br.x, br.y, br.z};
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) v[11 + 3 * i + j] += fa[i] * ba[j];
    }
    if (nrm(fn) == 0) continue;
    if (need & 1) {
      const D3 l = p2 - p1;
      const double fa[3] = {f.x, f.y, f.z}, la[3] = {l.x, l.y, l.z};
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) v[3 * i + j] += fa[i] * la[j];
    }
    if (need & 2) v[9] += nrm(f);
  }
  if (need & 2) {
    const Params& P = *d.prm;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < d.N; b += stride) {
      if (d.blocked[b] == DOF_ALL) continue;
      D3 F, M;
      if (midStep && d.info[b].x == KIND_SQ) gatherBody(d, b, xyz(d.pos[b]), F, M);
      else F = xyz(d.force[b]);
      const double m = d.mass[b];
      v[10] += nrm(d3(F.x + m * P.g[0], F.y + m * P.g[1], F.z + m * P.g[2]));
    }
  }
  blockSum(sh, SV_PART, v, d.svPart + (size_t)blockIdx.x * SV_PART);
}

// CompressionEngine::action for a cubic specimen as compiled in the reference (SOLE_GAIN and
// NEW_SCHEME, Compression.hpp:24-31; action_cubic, Compression.cpp:395-604), one thread,
// between the wall force sums and NewtonIntegrator.  Walls are bodies 0-5 (left, right, front,
// back, bottom, top), each moved directly by its own gain times (wall stress - goal), clamped
// to max_vel*dt.  recordData's file output is left out; its state side effects (box size,
// volume, strain) are kept.  Sums over contacts follow table order.
__device__ __forceinline__ void svBox(const Dev& d, ServoDev& C) {   // updateBoxSize (:99-114)
  const double left = d.pos[0].x, right = d.pos[1].x, front = d.pos[2].y, back = d.pos[3].y;
  const double top = d.pos[5].z, bottom = d.pos[4].z;
  C.width = right - left; C.depth = back - front; C.height = top - bottom;
  C.x_area = C.depth * C.height; C.y_area = C.width * C.height; C.z_area = C.depth * C.width;
}
__device__ __forceinline__ void svConsol(const Dev& d, ServoDev& C) {   // consol_ss (:1330-1362)
  svBox(d, C);
  C.wsxx_right = d.force[1].x / C.x_area;
  C.wsxx_left = -d.force[0].x / C.x_area;
  C.wsxx = 0.5 * (C.wsxx_left + C.wsxx_right);
  C.wsyy_back = d.force[3].y / C.y_area;
  C.wsyy_front = -d.force[2].y / C.y_area;
  C.wsyy = 0.5 * (C.wsyy_back + C.wsyy_front);
  C.wszz_top = d.force[5].z / C.z_area;
  C.wszz_bottom = -d.force[4].z / C.z_area;
  C.wszz = 0.5 * (C.wszz_top + C.wszz_bottom);
}
__device__ __forceinline__ void svGain(const Dev& d, ServoDev& C) {     // get_gain (:1125-1220)
  C.gain_x = C.gain_alpha * C.x_area / d.wallKn[0];
  C.gain_y = C.gain_alpha * C.y_area / d.wallKn[2];
  C.gain_z = C.gain_alpha * C.z_area / d.wallKn[4];
  C.gain_x1 = C.gain_alpha * C.x_area / d.wallKn[1];
  C.gain_y1 = C.gain_alpha * C.y_area / d.wallKn[3];
  C.gain_z1 = C.gain_alpha * C.z_area / d.wallKn[5];
}
__device__ __forceinline__ double svStep(double gain, double ws, double goal, double maxStep) {
  const double u = gain * (ws - goal);
  const double a = fabs(u);
  return sgn(u) * ((maxStep < a) ? maxStep : a);
}
__device__ __forceinline__ void svServo(const Dev& d, ServoDev& C, double dt) {   // servo (:1252-1303)
  svConsol(d, C);
  const double ms = C.max_vel * dt;
  if (C.activated[0]) d.pos[0].x += -svStep(C.gain_x, C.wsxx_left, C.goalx, ms);
  if (C.activated[1]) d.pos[1].x += svStep(C.gain_x1, C.wsxx_right, C.goalx, ms);
  if (C.activated[2]) d.pos[2].y += -svStep(C.gain_y, C.wsyy_front, C.goaly, ms);
  if (C.activated[3]) d.pos[3].y += svStep(C.gain_y1, C.wsyy_back, C.goaly, ms);
  if (C.z_servo) {
    d.pos[4].z += -svStep(C.gain_z, C.wszz_bottom, C.goalz, ms);
    d.pos[5].z += svStep(C.gain_z1, C.wszz_top, C.goalz, ms);
  }
}
__device__ __forceinline__ double svTotal(const Dev& d, int c) {
  double s = 0;
  for (int b = 0; b < d.svBlocks; b++) s += d.svPart[(size_t)b * SV_PART + c];
  return s;
}
// getStressTensor (:764-829) and getStress (:831-841)
__device__ __forceinline__ void svStress(const Dev& d, ServoDev& C, double& mean, double& dev) {
  svBox(d, C);
  C.Current_boxVolume = C.height * C.z_area;
  double sg[9];
  for (int k = 0; k < 9; k++) sg[k] = svTotal(d, k) / C.Current_boxVolume;
  mean = (sg[0] + (sg[4] + sg[8])) / 3.0;
  sg[0] -= mean; sg[4] -= mean; sg[8] -= mean;
  double c[9];
  for (int k = 0; k < 9; k++) c[k] = sg[3 * (k % 3) + k / 3];
  const double sq = ((c[0] * c[0] + c[1] * c[1]) + (c[2] * c[2] + c[3] * c[3])) +
                    ((c[4] * c[4] + c[5] * c[5]) + (c[6] * c[6] + (c[7] * c[7] + c[8] * c[8])));
  dev = sqrt(sq) * sqrt(1.5);
}
// recordData (:843-925) without its file: getStress's box update and the axial strain
__device__ __forceinline__ void svRecord(const Dev& d, ServoDev& C) {
  svBox(d, C);
  C.Current_boxVolume = C.height * C.z_area;
  C.strain2 = log(C.height0 / C.height);
}
__device__ __forceinline__ double svUnbalanced(const Dev& d) {   // Shop::unbalancedForce(false)
  return svTotal(d, 10) / (svTotal(d, 9) * 2.0);
}
// which reductions this step's action reads (the counters as the action will see them)
__global__ void k_servo_gate(Dev d) {
  SceneState& S = *d.S;
  ServoDev& C = S.sv;
  C.need = 0;
  if (S.skip || !C.enabled) return;
  const bool echo = C.echo_interval != 0 && S.iter % C.echo_interval == 0;
  if (C.z_servo) {
    const unsigned solve = (C.firstRun ? 0u : C.solve_num) + 1;
    if (solve >= C.solve_num_max) C.need |= C.hydroStrain ? 1 : 3;
    if (echo) C.need |= 2;
  } else if (echo) C.need |= 2;
}
__global__ void k_servo(Dev d) {
  SceneState& S = *d.S;
  ServoDev& C = S.sv;
  if (S.skip || !C.enabled) return;
  const double dt = d.prm->dt;
  if (C.firstRun) {
    const double left = d.pos[0].x, right = d.pos[1].x, front = d.pos[2].y, back = d.pos[3].y;
    const double top = d.pos[5].z, bottom = d.pos[4].z;
    if (C.continueFlag) { C.width = right - left; C.depth = back - front; C.height = top - bottom; }
    else {
      C.width = C.width0 = right - left; C.depth = C.depth0 = back - front; C.height = C.height0 = top - bottom;
    }
    C.x_area = C.depth * C.height; C.y_area = C.width * C.height; C.z_area = C.depth * C.width;
    C.Init_boxVolume = C.height0 * C.width0 * C.depth0;
    C.particlesVolume = C.pvol;
    C.rampNum = 0; C.firstRun = 0;
    C.iterate_num = 0; C.solve_num = 0;
    svGain(d, C);
    C.Flag_ForceTarget = 0;
  }
  const bool echo = C.echo_interval != 0 && S.iter % C.echo_interval == 0;
  const bool save = C.savedata_interval != 0 && S.iter % C.savedata_interval == 0;
  if (C.z_servo) {
    if (C.hydroStrain) {   // hydroConsolidation (:264-322)
      svBox(d, C);
      const double ls = d.force[0].x / C.x_area, rs = d.force[1].x / C.x_area;
      const double fs = d.force[2].y / C.y_area, bs = d.force[3].y / C.y_area;
      const double bos = d.force[4].z / C.z_area, ts = d.force[5].z / C.z_area;
      const double dl = C.goalx - fabs(ls), dr = C.goalx - fabs(rs);
      const double df = C.goaly - fabs(fs), dbk = C.goaly - fabs(bs);
      const double dbo = C.goalz - fabs(bos), dtp = C.goalz - fabs(ts);
      if (dl > 0) d.pos[0].x += fmin_ref(0.1 * C.gain_x * dl, C.hydroStrainRate * C.width * dt);
      if (dr > 0) d.pos[1].x -= fmin_ref(0.1 * C.gain_x1 * dr, C.hydroStrainRate * C.width * dt);
      if (df > 0) d.pos[2].y += fmin_ref(0.1 * C.gain_y * df, C.hydroStrainRate * C.depth * dt);
      if (dbk > 0) d.pos[3].y -= fmin_ref(0.1 * C.gain_y1 * dbk, C.hydroStrainRate * C.depth * dt);
      if (dbo > 0) d.pos[4].z += fmin_ref(0.1 * C.gain_z * dbo, C.hydroStrainRate * C.height * dt);
      if (dtp > 0) d.pos[5].z -= fmin_ref(0.1 * C.gain_z1 * dtp, C.hydroStrainRate * C.height * dt);
      C.iterate_num += 1;
      if (C.iterate_num >= C.iterate_num_max) { C.iterate_num = 1; svGain(d, C); }
      C.solve_num += 1;
      if (C.solve_num >= C.solve_num_max) {
        C.solve_num = 1;
        double mean, dev;
        svStress(d, C, mean, dev);
        if ((fabs(mean - C.goalx) / C.goalx < C.f_threshold) && (dev / mean < C.fmin_threshold))
          if (C.UnbalancedForce < C.unbf_tol && S.haltAt < 0) S.haltAt = S.iter + 1;
      }
    } else {               // generalConsolidation, NEW_SCHEME (:324-358)
      C.iterate_num += 1;
      C.solve_num += 1;
      svServo(d, C, dt);
      if (C.iterate_num >= C.iterate_num_max) { C.iterate_num = 0; svGain(d, C); }
      if (C.solve_num >= C.solve_num_max) {
        C.solve_num = 0;
        double mean, dev;
        svStress(d, C, mean, dev);
        if ((fabs(mean - C.goalx) < C.goalx * C.f_threshold) && (dev / mean < C.fmin_threshold)) {
          C.UnbalancedForce = svUnbalanced(d);
          if (C.UnbalancedForce < C.unbf_tol) { if (S.haltAt < 0) S.haltAt = S.iter + 1; S.quiet = 1; }
        }
      }
    }
    if (save) svRecord(d, C);
    if (echo) { C.UnbalancedForce = svUnbalanced(d); svConsol(d, C); }
  } else {                 // shear
    if (!C.continueFlag && C.rampNum < C.ramp_interval) {
      if (C.rampNum < 1 && C.Flag_ForceTarget) {
        svBox(d, C);
        C.width0 = C.width; C.height0 = C.height; C.depth0 = C.depth;
      }
      C.rampNum++;
      const double ramp_inter = 0.5 * C.ramp_interval;
      double vel;
      if (C.rampNum < ramp_inter)
        vel = (double)((float)(C.rampNum / (ramp_inter / C.ramp_chunks) + 1) / (float)C.ramp_chunks) * C.goalz * 2.0;
      else
        vel = ((double)((float)((C.ramp_interval - C.rampNum) / (ramp_inter / C.ramp_chunks) + 1) / (float)C.ramp_chunks) + 1.0) * C.goalz;
      d.pos[4].z += vel * dt * C.height;
      d.pos[5].z += -vel * dt * C.height;
    } else {
      if (C.shearMode & 1) {
        C.iterate_num += 1;
        if (C.iterate_num >= C.iterate_num_max) { C.iterate_num = 1; svGain(d, C); }
      }
      d.pos[4].z += C.goalz * dt * C.height;
      d.pos[5].z += -C.goalz * dt * C.height;
    }
    if (C.shearMode & 1) svServo(d, C, dt);
    else {                 // constant volume (undrained)
      const double left = d.pos[0].x, right = d.pos[1].x, front = d.pos[2].y, back = d.pos[3].y;
      const double top = d.pos[5].z, bottom = d.pos[4].z;
      C.width = right - left; C.depth = back - front; C.height = top - bottom;
      const double Sa = C.Init_boxVolume / C.height;
      const double dd = 0.5 * (Sa / C.width - C.depth);
      const double dw = Sa / (C.depth + dd) - C.width;
      d.pos[0].x += -0.5 * dw; d.pos[1].x += 0.5 * dw;
      d.pos[2].y += -0.5 * dd; d.pos[3].y += 0.5 * dd;
    }
    if (log(C.height0 / C.height) > C.target_strain && S.haltAt < 0) S.haltAt = S.iter + 1;
    if (save) svRecord(d, C);
    if (echo) { C.UnbalancedForce = svUnbalanced(d); if (C.shearMode & 2) svConsol(d, C); }
  }
}

// NewtonIntegrator (NewtonIntegrator.cpp): DotQ (:470-477)
struct Q4 { double w, x, y, z; };
__device__ __forceinline__ Q4 DotQ(D3 a, Q4 Q) {
  Q4 r;
  r.w = (-Q.x * a.x - Q.y * a.y - Q.z * a.z) / 2;
  r.x = (Q.w * a.x - Q.z * a.y + Q.y * a.z) / 2;
  r.y = (Q.z * a.x + Q.w * a.y - Q.x * a.z) / 2;
  r.z = (-Q.y * a.x + Q.x * a.y + Q.w * a.z) / 2;
  return r;
}
__device__ __forceinline__ void qnormalize(Q4& q) {
  double z = (q.x * q.x + q.y * q.y) + (q.z * q.z + q.w * q.w);
  if (z > 0) { double n = sqrt(z); q.x /= n; q.y /= n; q.z /= n; q.w /= n; }
}
__device__ __forceinline__ D3 qrotate(Q4 q, D3 v) {
  D3 qv = d3(q.x, q.y, q.z);
  D3 uv = cross(qv, v);
  uv = uv + uv;
  D3 c = cross(qv, uv);
  return d3((v.x + q.w * uv.x) + c.x, (v.y + q.w * uv.y) + c.y, (v.z + q.w * uv.z) + c.z);
}
// leapfrogSphericalRotate without move/rot buffers (:319-335)
__device__ __forceinline__ void sphericalRotate(Q4& o, D3 w, double dt) {
  double angle2 = sqn(w);
  if (angle2 != 0) {
    double angle = sqrt(angle2);
    D3 axis = d3(w.x / angle, w.y / angle, w.z / angle);
    double h = 0.5 * (angle * dt);
    double sh, ch; sincos(h, &sh, &ch);
    Q4 q; q.w = ch; q.x = sh * axis.x; q.y = sh * axis.y; q.z = sh * axis.z;
    Q4 r;
    r.w = q.w * o.w - q.x * o.x - q.y * o.y - q.z * o.z;
    r.x = q.w * o.x + q.x * o.w + q.y * o.z - q.z * o.y;
    r.y = q.w * o.y + q.y * o.w + q.z * o.x - q.x * o.z;
    r.z = q.w * o.z + q.z * o.w + q.x * o.y - q.y * o.x;
    o = r;
  }
  qnormalize(o);
}

__global__ void __launch_bounds__(256) k_integrate(Dev d) {
  const SceneState& S = *d.S;
  if (S.skip) return;
  const Params& P = *d.prm;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  int code = 0;
  if (b < d.N) {
    const int4 inf = d.info[b];
    const double dt = P.dt;
    D3 pos = xyz(d.pos[b]);
    double4 o4 = d.ori[b];
    Q4 ori; ori.w = o4.x; ori.x = o4.y; ori.y = o4.z; ori.z = o4.w;
    D3 vel = xyz(d.vel[b]), angVel = xyz(d.angVel[b]), angMom = xyz(d.angMom[b]);
    const unsigned blocked = d.blocked[b];
    const bool damped = d.damped[b] != 0;
    const bool aspherical = d.aspherical[b] != 0;
    D3 f = d3(0, 0, 0), m = d3(0, 0, 0);
    if (inf.x == KIND_SQ) {
      for (int e = d.rowStart[b]; e < d.rowStart[b + 1]; e++) {
        unsigned fl = d.A.flags[e];
        if (fl & F_FORCE) addContribution(d, e, (fl & F_OWNER_ID1) != 0, pos, f, m);
      }
      for (int k = d.pStart[b]; k < d.pStart[b + 1]; k++) {
        int e = d.pList[k];
        unsigned fl = d.A.flags[e];
        if (fl & F_FORCE) addContribution(d, e, (fl & F_OWNER_ID1) == 0, pos, f, m);
      }
      d.force[b] = dd4(f, 0); d.torque[b] = dd4(m, 0);
    } else {
      f = xyz(d.force[b]); m = xyz(d.torque[b]);
    }
    const double mass = d.mass[b];
    const double4 I4 = d.inertia[b];
    const D3 inertia = xyz(I4);
    const bool useAspherical = (P.exactAsphericalRot && aspherical && blocked != DOF_ALL);
    const bool isSphere = (inf.x == KIND_SQ) && inf.z != 0;
    const double damping = P.damping;
    const bool peri = S.periodic != 0, homo = peri && S.homoDeform;
    const D3 fluctVel = peri ? vel - m3v(S.prevVelGrad, pos) : vel;   // Cell::bodyFluctuationVel
    if (blocked != DOF_ALL) {
      D3 a;
      if (blocked == 0) a = d3(f.x / mass + P.g[0], f.y / mass + P.g[1], f.z / mass + P.g[2]);
      else {
        a = d3(0, 0, 0);
        if (!(blocked & 1u)) a.x += f.x / mass + P.g[0];
        if (!(blocked & 2u)) a.y += f.y / mass + P.g[1];
        if (!(blocked & 4u)) a.z += f.z / mass + P.g[2];
      }
      if (damped) {
        a.x *= 1 - damping * sgn(a.x * (fluctVel.x + 0.5 * dt * a.x));
        a.y *= 1 - damping * sgn(a.y * (fluctVel.y + 0.5 * dt * a.y));
        a.z *= 1 - damping * sgn(a.z * (fluctVel.z + 0.5 * dt * a.z));
      }
      if (homo) a = a + m3v(S.prevVelGrad, vel);
      vel = vel + dt * a;
      if (!useAspherical || (P.isSuperquadrics && isSphere && damped)) {
        D3 aa;
        if (blocked == 0) aa = d3(m.x / inertia.x, m.y / inertia.y, m.z / inertia.z);
        else {
          aa = d3(0, 0, 0);
          if (!(blocked & 8u)) aa.x += m.x / inertia.x;
          if (!(blocked & 16u)) aa.y += m.y / inertia.y;
          if (!(blocked & 32u)) aa.z += m.z / inertia.z;
        }
        if (damped) {
          aa.x *= 1 - damping * sgn(aa.x * (angVel.x + 0.5 * dt * aa.x));
          aa.y *= 1 - damping * sgn(aa.y * (angVel.y + 0.5 * dt * aa.y));
          aa.z *= 1 - damping * sgn(aa.z * (angVel.z + 0.5 * dt * aa.z));
        }
        angVel = angVel + dt * aa;
      } else {
        if (blocked & 8u) m.x = 0;
        if (blocked & 16u) m.y = 0;
        if (blocked & 32u) m.z = 0;
        if (damped) {  // cundallDamp1st on the torque (:19-21)
          m.x *= 1 - damping * sgn(m.x * angVel.x);
          m.y *= 1 - damping * sgn(m.y * angVel.y);
          m.z *= 1 - damping * sgn(m.z * angVel.z);
        }
      }
    } else if (homo) vel = vel + m3v(S.dtPrevVelGrad, vel);
    if (S.quiet) {   // quiet_system_flag (NewtonIntegrator.cpp:246-250): zero velocities, no move
      vel = d3(0, 0, 0);
      angVel = d3(0, 0, 0);
    } else if (!useAspherical || (P.isSuperquadrics && isSphere)) {
      sphericalRotate(ori, angVel, dt);
    } else if (P.isSuperquadrics) {
      // leapfrogAsphericalRotate with A = rot_mat2local (:337-360, :391-429)
      const Rot R = quatToRot(ori.w, ori.x, ori.y, ori.z);
      const D3 l_n = angMom + dt / 2. * m;
      const D3 l_b_n = mulL(R, l_n);
      const D3 w_b_n = d3(l_b_n.x / inertia.x, l_b_n.y / inertia.y, l_b_n.z / inertia.z);
      const Q4 dq = DotQ(w_b_n, ori);
      const double hdt = dt / 2.;
      Q4 Qh; Qh.w = ori.w + dq.w * hdt; Qh.x = ori.x + dq.x * hdt; Qh.y = ori.y + dq.y * hdt; Qh.z = ori.z + dq.z * hdt;
      angMom = angMom + dt * m;
      const D3 l_b_h = mulL(R, angMom);
      const D3 w_b_h = d3(l_b_h.x / inertia.x, l_b_h.y / inertia.y, l_b_h.z / inertia.z);
      const Q4 dqh = DotQ(w_b_h, Qh);
      ori.w = ori.w + dqh.w * dt; ori.x = ori.x + dqh.x * dt; ori.y = ori.y + dqh.y * dt; ori.z = ori.z + dqh.z * dt;
      angVel = qrotate(ori, w_b_h);
      qnormalize(ori);
    }
    if (!S.quiet) {
      if (homo) vel = vel + m3v(S.dVelGrad, pos);   // leapfrogTranslate (:306-317)
      pos = pos + vel * dt;
    }
    d.pos[b] = dd4(pos, 0);
    d.ori[b] = make_double4(ori.w, ori.x, ori.y, ori.z);
    d.vel[b] = dd4(vel, 0); d.angVel[b] = dd4(angVel, 0); d.angMom[b] = dd4(angMom, 0);
    // saveMaximaDisplacement (:72-85)
    const double4 rf = d.ref[b];
    if (rf.w != 0) {
      D3 disp = pos - xyz(rf);
      double maxDisp = fmax_ref(fabs(disp.x), fmax_ref(fabs(disp.y), fabs(disp.z)));
      double sl = d.bmin[b].w;
      code = (maxDisp == 0 || maxDisp < sl) ? 1 : 2;
    }
  }
  for (int o = 16; o > 0; o >>= 1) code = max(code, __shfl_down_sync(0xffffffffu, code, o));
  if ((threadIdx.x & 31) == 0 && code) atomicMax(&d.S->maxDispCode, code);
  if (b == 0) d.S->newtonRan = 1;
  (void)S;
}

__global__ void k_reset_queue(Dev d) {
  d.S->lmCount = 0; d.S->lmHead = 0; d.S->fbCount = 0; d.S->fbHead = 0; d.S->vlCount = 0; d.S->vlHead = 0;
  d.S->nmFin = 0; d.S->nmShort = 0;
}

// Start of NewtonIntegrator::action (NewtonIntegrator.cpp:107-117): pending velGrad, the
// cell-size-change velocity that seeds maxVelocitySq, and the gradients the body update uses.
__global__ void k_newton_begin(Dev d) {
  SceneState& S = *d.S;
  if (S.skip) return;
  if (!S.periodic) { S.cellTerm = 0; return; }
  bool nz = false;
  for (int k = 0; k < 9; k++) nz |= (S.nextVelGrad[k] != 0);
  if (S.velGradChanged || nz) {
    for (int k = 0; k < 9; k++) { S.velGrad[k] = S.nextVelGrad[k]; S.nextVelGrad[k] = 0; }
    S.velGradChanged = 0;
  }
  const double dt = d.prm->dt;
  for (int k = 0; k < 9; k++) { S.dVelGrad[k] = S.velGrad[k] - S.prevVelGrad[k]; S.dtPrevVelGrad[k] = dt * S.prevVelGrad[k]; }
  const bool differs = S.prevCellSize[0] != S.cellSize[0] || S.prevCellSize[1] != S.cellSize[1] || S.prevCellSize[2] != S.cellSize[2];
  if (differs && !isnan(S.prevCellSize[0])) {
    const D3 dd = d3(S.prevCellSize[0] - S.cellSize[0], S.prevCellSize[1] - S.cellSize[1], S.prevCellSize[2] - S.cellSize[2]);
    S.cellTerm = sqn(dd) / (dt * dt);
  } else S.cellTerm = 0;
}

__global__ void k_end(Dev d) {
  SceneState& S = *d.S;
  if (S.skip) return;
  S.quiet = 0;       // NewtonIntegrator resets quiet_system_flag (:299)
  if (S.periodic) {  // end of NewtonIntegrator::action (:300-302)
    for (int k = 0; k < 3; k++) S.prevCellSize[k] = S.cellSize[k];
    for (int k = 0; k < 9; k++) S.prevVelGrad[k] = S.velGrad[k];
  }
  S.iter++;
  S.time += d.prm->dt;
  S.err[E_STEPS]++;
}

}  // namespace sqdem

// ===========================================================================
// Host side: context, allocation, step sequence, C ABI.
using namespace sqdem;

struct sqdem_ctx {
  int device = 0, precision = SQDEM_FP64, useGraph = 1, contactsPerBody = 16, maxCand = 64;
  int numSMs = 152;
  int lmBlocksPerSM = 4, lmBlocksPerSMmixed = 4, nmBlocksPerSM = 4;
  int shapeSearch = 0, shapePass1 = 0;   // launch shapes set by the caller or the autotuner (0: defaults)
  cudaStream_t stream = nullptr;
  Dev d;
  bool haveBodies = false, haveMats = false, haveParams = false;
  cudaGraph_t graph = nullptr; cudaGraphExec_t exec = nullptr; bool graphValid = false;
  unsigned epoch = 0;   // counts changes of the step's kernel sequence (graphs capturing it are stale)
  std::string err;
  std::vector<void*> allocs;
  sqdem_params params;
  int recordFull = 0;
  int lmSpread = 1;
  int periodicFix = 0;   // sqdem_set_periodic_fix
  int contactModel = SQDEM_CONTACT_LINEAR;
  bool servoOn = false;
  std::vector<int> kind, wallIds, matIds, isSphere, axisSense;
  std::vector<double> shape5;
  int nMats = 0;
  std::vector<double4> hostMats; std::vector<double2> hostMatsB, hostMatsE;
  long long launches = 0, launchesPerStep = 0;
  cudaEvent_t ev[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  float stageMs[3] = {0, 0, 0};
  float searchMs[2] = {0, 0};   // eager steps: search kernel, then the mixed form's FP64 fallback kernel
  bool timingSearch = false;
};

static sqdem_status fail(sqdem_ctx* c, sqdem_status s, const std::string& m) {
  if (c) c->err = m;
  return s;
}
#define CK(call)                                                                                     \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess) return fail(c, SQDEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
static cudaError_t dalloc(sqdem_ctx* c, T** p, size_t n) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, sizeof(T) * (n ? n : 1));
  if (e == cudaSuccess) { c->allocs.push_back(q); cudaMemsetAsync(q, 0, sizeof(T) * (n ? n : 1), c->stream); }
  *p = (T*)q;
  return e;
}
static void freeAll(sqdem_ctx* c) {
  if (c->exec) { cudaGraphExecDestroy(c->exec); c->exec = nullptr; }
  if (c->graph) { cudaGraphDestroy(c->graph); c->graph = nullptr; }
  c->graphValid = false; c->epoch++;
  for (void* p : c->allocs) cudaFree(p);
  c->allocs.clear();
}
// blocks for n items (at least one: every kernel bounds its items, and a zero grid is a launch error)
static inline int nblk(long n, int bs) { return std::max(1, (int)((n + bs - 1) / bs)); }

static sqdem_status allocTable(sqdem_ctx* c, Table& t, int cap) {
  CK(dalloc(c, &t.owner, cap)); CK(dalloc(c, &t.partner, cap)); CK(dalloc(c, &t.flags, cap));
  CK(dalloc(c, &t.angle, cap)); CK(dalloc(c, &t.depth, cap)); CK(dalloc(c, &t.normal, cap));
  CK(dalloc(c, &t.shear, cap)); CK(dalloc(c, &t.nforce, cap)); CK(dalloc(c, &t.phys, cap));
  CK(dalloc(c, &t.F, cap)); CK(dalloc(c, &t.cp, cap)); CK(dalloc(c, &t.cd, cap));
  CK(dalloc(c, &t.p1, cap)); CK(dalloc(c, &t.p2, cap)); CK(dalloc(c, &t.shearInc, cap));
  CK(dalloc(c, &t.twist, cap)); CK(dalloc(c, &t.ortho, cap)); CK(dalloc(c, &t.relVn, cap)); CK(dalloc(c, &t.relVs, cap));
  CK(dalloc(c, &t.hmCurv, cap)); CK(dalloc(c, &t.hmEll, cap)); CK(dalloc(c, &t.hmSum, cap));
  return SQDEM_OK;
}

static int* gateRun(sqdem_ctx* c) { return (int*)((char*)c->d.S + offsetof(SceneState, runCollider)); }

static void launchScan(sqdem_ctx* c, const int* in, int n, int* out, const int* gate) {
  int nb = nblk(n + 1, SCAN_TILE);
  k_scan_reduce<<<nb, SCAN_BS, 0, c->stream>>>(in, n, c->d.scanTmp, gate);
  k_scan_blocks<<<1, SCAN_BS, 0, c->stream>>>(c->d.scanTmp, nb, gate);
  k_scan_apply<<<nb, SCAN_BS, 0, c->stream>>>(in, n, c->d.scanTmp, out, gate);
  c->launches += 3;
}

// Resident blocks per SM of the search kernel the context launches.
static int maxSearchBlocksPerSM(const sqdem_ctx* c) {
  if (c->contactModel == SQDEM_CONTACT_HERTZ_MINDLIN) return c->nmBlocksPerSM;
  return c->precision == SQDEM_MIXED ? c->lmBlocksPerSMmixed : c->lmBlocksPerSM;
}
static int searchBlocksPerSM(const sqdem_ctx* c) {
  const int mx = maxSearchBlocksPerSM(c);
  return c->shapeSearch > 0 ? std::min(c->shapeSearch, mx) : mx;
}
static const int PASS1_BLOCKS_PER_SM = 16;   // grid-stride blocks of pass 1 per SM (default)

// the FP64 search kernel build for a grid of `grid` blocks: the three-blocks-per-SM build when
// the grid asks for more than two blocks per SM
static void launchLmFP64(const sqdem_ctx* c, int grid, cudaStream_t s, const Dev& d, int mode) {
  if (grid > 2 * c->numSMs) k_contacts_lm<3><<<grid, LM_BS, 0, s>>>(d, mode);
  else k_contacts_lm<1><<<grid, LM_BS, 0, s>>>(d, mode);
}

// The contact stage on c->stream: pass 1, then the searches of the selected contact model
// (and, for Hertz-Mindlin, the finish pass of the contacts found touching).
static void launchContactStage(sqdem_ctx* c, const Dev& d, int grid) {
  cudaStream_t s = c->stream;
  const int p1 = c->shapePass1 > 0 ? c->shapePass1 : PASS1_BLOCKS_PER_SM;
  k_contacts_pre<<<std::min(nblk(d.Pcap, 128), c->numSMs * p1), 128, 0, s>>>(d);
  if (c->contactModel == SQDEM_CONTACT_HERTZ_MINDLIN) {
    k_contacts_nm<<<grid, LM_BS, 0, s>>>(d);
    k_contacts_nm_finish<<<std::min(nblk(d.Pcap, 128), c->numSMs * 8), 128, 0, s>>>(d);
    c->launches += 3;
  } else {
    if (c->precision == SQDEM_MIXED) {
      // double-float searches, then the FP64 kernel on the long-search queue and the searches
      // the double-float kernels deferred
      k_body_ff<<<nblk(d.N, 256), 256, 0, s>>>(d);
      if (c->timingSearch) cudaEventRecord(c->ev[4], s);
      k_contacts_lm_ff<<<grid, LM_BS, 0, s>>>(d);
      if (c->timingSearch) cudaEventRecord(c->ev[5], s);
      k_contacts_lm_ff_finish<<<std::min(nblk(d.Pcap, 128), c->numSMs * 8), 128, 0, s>>>(d);
      // one block per SM: one warp per scheduler, so that the FP64 pipe serves each warp's
      // chain of dependent evaluations alone (these searches are long; more warps per
      // scheduler lengthen every round of the longest one)
      launchLmFP64(c, c->numSMs, s, d, LM_DEFERRED);
      if (c->timingSearch) cudaEventRecord(c->ev[6], s);
      c->launches += 5;
    } else {
      if (c->timingSearch) cudaEventRecord(c->ev[4], s);
      launchLmFP64(c, grid, s, d, LM_FP64);
      if (c->timingSearch) { cudaEventRecord(c->ev[5], s); cudaEventRecord(c->ev[6], s); }
      c->launches += 2;
    }
  }
}

// One timestep of kernels on c->stream.
static void enqueueStep(sqdem_ctx* c, bool timed) {
  Dev& d = c->d;
  cudaStream_t s = c->stream;
  const int* gate = gateRun(c);
  const int N = d.N;
  if (timed) cudaEventRecord(c->ev[0], s);
  k_gate<<<1, 1, 0, s>>>(d);
  k_bounds<<<nblk(N, 256), 256, 0, s>>>(d);
  k_grid_setup<<<1, 1, 0, s>>>(d);
  k_zero_cells<<<std::min(nblk(d.Gmax + 1, 256), 4096), 256, 0, s>>>(d);
  k_cell_count<<<nblk(N, 256), 256, 0, s>>>(d);
  c->launches += 5;
  launchScan(c, d.cellCount, d.Gmax, d.cellStart, gate);
  k_cell_scatter<<<nblk(N, 256), 256, 0, s>>>(d);
  k_candidates<<<nblk(N, 128), 128, 0, s>>>(d);
  c->launches += 2;
  launchScan(c, d.rowCount, N, d.rowStartNew, gate);
  const int tblBlocks = std::min(nblk(d.Pcap, 256), c->numSMs * 8);
  k_check_capacity<<<1, 1, 0, s>>>(d);
  k_merge<<<nblk(N, 128), 128, 0, s>>>(d);
  k_copy_back<<<tblBlocks, 256, 0, s>>>(d);
  k_commit<<<1, 1, 0, s>>>(d);
  k_pcount<<<tblBlocks, 256, 0, s>>>(d);
  c->launches += 5;
  launchScan(c, d.pCount, N, d.pStart, gate);
  k_pscatter<<<tblBlocks, 256, 0, s>>>(d);
  k_psort<<<nblk(N, 256), 256, 0, s>>>(d);
  c->launches += 2;
  if (d.W > 0) {
    k_wall_count<<<d.wallChunks, 256, 0, s>>>(d);
    k_wall_lists<<<d.wallChunks, 256, 0, s>>>(d);
    c->launches += 2;
  }
  if (timed) cudaEventRecord(c->ev[1], s);
  // LM grid: all resident blocks, fewer for a small table (at most one lane per 4 entries)
  const int lmFull = c->numSMs * searchBlocksPerSM(c);
  launchContactStage(c, d, std::max(1, std::min(lmFull, nblk(d.Pcap, LM_BS * 4))));
  if (timed) cudaEventRecord(c->ev[2], s);
  if (d.W > 0) { k_wall_forces<<<d.W, 128, 0, s>>>(d); c->launches++; }
  if (c->servoOn) {   // CompressionEngine between InteractionLoop and NewtonIntegrator
    k_servo_gate<<<1, 1, 0, s>>>(d);
    k_servo_sums<<<d.svBlocks, 128, 0, s>>>(d, -1, 1);
    k_servo<<<1, 1, 0, s>>>(d);
    c->launches += 3;
  }
  k_newton_begin<<<1, 1, 0, s>>>(d);
  k_integrate<<<nblk(N, 256), 256, 0, s>>>(d);
  k_end<<<1, 1, 0, s>>>(d);
  c->launches += 3;
  if (timed) cudaEventRecord(c->ev[3], s);
}

static sqdem_status ensureGraph(sqdem_ctx* c) {
  if (c->graphValid) return SQDEM_OK;
  if (c->exec) { cudaGraphExecDestroy(c->exec); c->exec = nullptr; }
  if (c->graph) { cudaGraphDestroy(c->graph); c->graph = nullptr; }
  long long l0 = c->launches;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  enqueueStep(c, false);
  CK(cudaStreamEndCapture(c->stream, &c->graph));
  c->launchesPerStep = c->launches - l0;
  c->launches = l0;
  CK(cudaGraphInstantiate(&c->exec, c->graph, 0));
  c->graphValid = true;
  return SQDEM_OK;
}

static double hostH0(sqdem_ctx* c) {
  double rm = 0;
  for (size_t i = 0; i < c->kind.size(); i++)
    if (c->kind[i] == SQDEM_SUPERQUADRIC) {
      const double* s = &c->shape5[5 * i];
      double r = std::max(s[0], std::max(s[1], s[2]));
      if (s[3] < 1.0 || s[4] < 1.0) r *= std::pow(2.0, 0.5);
      rm = std::max(rm, r);
    }
  double vd = std::max(c->params.verletDist, 0.0);
  double h = 2.0 * (rm + vd);
  return h * (1.0 + 1e-9) + 1e-300;
}

static sqdem_status uploadParams(sqdem_ctx* c) {
  Params P;
  std::memset(&P, 0, sizeof(P));
  P.dt = c->params.dt;
  for (int k = 0; k < 3; k++) P.g[k] = c->params.gravity[k];
  P.damping = c->params.damping; P.verletDist = c->params.verletDist;
  P.minSweepDistFactor = c->params.minSweepDistFactor; P.targetInterv = c->params.targetInterv;
  P.sortAxis = c->params.sortAxis; P.isSuperquadrics = c->params.isSuperquadrics;
  P.exactAsphericalRot = c->params.exactAsphericalRot; P.recordFull = c->recordFull;
  P.lmSpread = c->lmSpread;
  P.contactModel = c->contactModel;
  P.periodicFix = c->periodicFix;
  // 32+ iterations in both forms (from 64 in the mixed form was measured no faster: the
  // double-float kernel then deferred more searches past 50 iterations, run again in FP64)
  P.vlongBucket = (int)VLONG_ITERS_BUCKET;
  P.h0 = hostH0(c);
  CK(cudaMemcpyAsync(c->d.prm, &P, sizeof(P), cudaMemcpyHostToDevice, c->stream));
  return SQDEM_OK;
}

// Superquadrics::Initial (Superquadrics.cpp:47-93) with the Lanczos log-gamma of
// lib/base/Math.hpp:192-212 (Numerical Recipes 3rd ed. coefficients, as the reference).
static double gammlnH(const double xx) {
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
static double betaH(double z, double w) { return std::exp(gammlnH(z) + gammlnH(w) - gammlnH(z + w)); }

static bool finiteRows(const double* a, int n, int stride, int cols) {
  for (int i = 0; i < n; i++)
    for (int k = 0; k < cols; k++)
      if (!std::isfinite(a[(size_t)i * stride + k])) return false;
  return true;
}

extern "C" {

sqdem_status sqdem_shape_props(double rx, double ry, double rz, double e1, double e2, double* out5) {
  if (!out5 || !(rx > 0) || !(ry > 0) || !(rz > 0) || !(e1 > 0) || !(e2 > 0)) return SQDEM_ERR_ARG;
  double r_max = (rx > ry) ? rx : ry;
  r_max = r_max > rz ? r_max : rz;
  if ((e1 < 1.0) || (e2 < 1.0)) r_max *= std::pow(2.0, 0.5);
  double a = rx * ry * rz * e1 * e2;
  double beta1 = betaH(1.5 * e1, 0.5 * e1) * betaH(0.5 * e2, 2. * e2 + 1);
  double beta2 = betaH(0.5 * e1, 0.5 * e1 + 1) * betaH(1.5 * e2, e2 + 1);
  out5[0] = 2. * a * betaH(e1 * 0.5, e1 * 0.5) * betaH(e2 * 0.5 + 1, e2);
  out5[1] = 0.5 * a * (std::pow(ry, 2.) * beta1 + 4. * std::pow(rz, 2.) * beta2);
  out5[2] = 0.5 * a * (std::pow(rx, 2.) * beta1 + 4. * std::pow(rz, 2.) * beta2);
  out5[3] = 0.5 * a * (std::pow(rx, 2.) + std::pow(ry, 2.)) * beta1;
  out5[4] = r_max;
  return SQDEM_OK;
}

sqdem_status sqdem_create(sqdem_ctx** out, const sqdem_config* cfg) {
  if (!out) return SQDEM_ERR_ARG;
  sqdem_ctx* c = new sqdem_ctx();
  *out = c;
  if (cfg) {
    c->device = cfg->device; c->precision = cfg->precision; c->useGraph = cfg->use_graph;
    if (cfg->contacts_per_body > 0) c->contactsPerBody = cfg->contacts_per_body;
  }
  if (c->precision != SQDEM_FP64 && c->precision != SQDEM_MIXED) return fail(c, SQDEM_ERR_ARG, "unknown precision");
  CK(cudaSetDevice(c->device));
  CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CK(cudaDeviceGetAttribute(&c->numSMs, cudaDevAttrMultiProcessorCount, c->device));
  {
    int nb = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_contacts_lm<3>, LM_BS, 0));
    c->lmBlocksPerSM = nb > 0 ? nb : 1;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_contacts_lm_ff, LM_BS, 0));
    c->lmBlocksPerSMmixed = nb > 0 ? nb : 1;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_contacts_nm, LM_BS, 0));
    c->nmBlocksPerSM = nb > 0 ? nb : 1;
  }
  for (int i = 0; i < 7; i++) CK(cudaEventCreate(&c->ev[i]));
  std::memset(&c->d, 0, sizeof(Dev));
  std::memset(&c->params, 0, sizeof(c->params));
  c->params.dt = 1e-5; c->params.damping = 0.2; c->params.verletDist = -0.5; c->params.targetInterv = 50;
  c->params.minSweepDistFactor = 0.1; c->params.sortAxis = 0; c->params.isSuperquadrics = 1;
  c->params.exactAsphericalRot = 1;
  return SQDEM_OK;
}

void sqdem_destroy(sqdem_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  freeAll(c);
  for (int i = 0; i < 7; i++) if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* sqdem_last_error(sqdem_ctx* c) { return c ? c->err.c_str() : "null context"; }

sqdem_status sqdem_set_materials(sqdem_ctx* c, int n, const double* Kn, const double* Ks, const double* fa,
                                 const double* bn, const double* bs, const double* rho) {
  if (!c || n <= 0 || !Kn || !Ks || !fa || !bn || !bs || !rho) return fail(c, SQDEM_ERR_ARG, "bad materials");
  if (c->haveMats && n != c->nMats) return fail(c, SQDEM_ERR_ARG, "material count cannot change");
  CK(cudaSetDevice(c->device));
  std::vector<double4>& m = c->hostMats; std::vector<double2>& mb = c->hostMatsB;
  m.resize(n); mb.resize(n);
  if ((int)c->hostMatsE.size() != n) c->hostMatsE.assign(n, make_double2(29e9, 0.15));   // SuperquadricsMat2 defaults
  for (int i = 0; i < n; i++) { m[i] = make_double4(Kn[i], Ks[i], fa[i], rho[i]); mb[i] = make_double2(bn[i], bs[i]); }
  c->nMats = n; c->haveMats = true;
  if (c->haveBodies) {
    CK(cudaMemcpyAsync(c->d.mats, m.data(), sizeof(double4) * n, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d.matsB, mb.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return SQDEM_OK;
}

sqdem_status sqdem_set_params(sqdem_ctx* c, const sqdem_params* p) {
  if (!c || !p) return fail(c, SQDEM_ERR_ARG, "null params");
  if (!(p->dt > 0)) return fail(c, SQDEM_ERR_ARG, "dt must be positive");
  if (p->sortAxis < 0 || p->sortAxis > 2) return fail(c, SQDEM_ERR_ARG, "sortAxis must be 0, 1 or 2");
  if (p->isSuperquadrics != 1)
    return fail(c, SQDEM_ERR_ARG, "NewtonIntegrator.isSuperquadrics must be 1 for superellipsoid scenes");
  CK(cudaSetDevice(c->device));
  const bool vdChanged = !c->haveParams || p->verletDist != c->params.verletDist;
  c->params = *p;
  c->haveParams = true;
  if (c->haveBodies) {
    sqdem_status s = uploadParams(c);
    if (s) return s;
    if (vdChanged) {
      double vd = p->verletDist;
      CK(cudaMemcpyAsync((char*)c->d.S + offsetof(SceneState, verletDistCur), &vd, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
  }
  return SQDEM_OK;
}

static void packState(sqdem_ctx* c, int n, const double* st, std::vector<double4>* v) {
  // v: pos, ori, vel, angVel, angMom
  for (int i = 0; i < n; i++) {
    const double* o = st + (size_t)i * SQDEM_BODY_STRIDE;
    v[0][i] = make_double4(o[0], o[1], o[2], 0);
    v[1][i] = make_double4(o[3], o[4], o[5], o[6]);
    v[2][i] = make_double4(o[7], o[8], o[9], 0);
    v[3][i] = make_double4(o[10], o[11], o[12], 0);
    v[4][i] = make_double4(o[13], o[14], o[15], 0);
  }
  (void)c;
}

sqdem_status sqdem_set_bodies(sqdem_ctx* c, int n, const int* kind, const double* shape5, const int* was,
                              const int* mat, const int* isSphere, const double* state) {
  if (!c || n <= 0 || !kind || !mat || !state) return fail(c, SQDEM_ERR_ARG, "bad bodies");
  if (n >= (1 << 30)) return fail(c, SQDEM_ERR_CAPACITY, "at most 2^30 - 1 bodies");
  if (!c->haveMats) return fail(c, SQDEM_ERR_STATE, "set materials first");
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  freeAll(c);
  c->haveBodies = false;
  CK(dalloc(c, &c->d.mats, c->nMats)); CK(dalloc(c, &c->d.matsB, c->nMats)); CK(dalloc(c, &c->d.matsE, c->nMats));
  CK(cudaMemcpyAsync(c->d.mats, c->hostMats.data(), sizeof(double4) * c->nMats, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d.matsB, c->hostMatsB.data(), sizeof(double2) * c->nMats, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d.matsE, c->hostMatsE.data(), sizeof(double2) * c->nMats, cudaMemcpyHostToDevice, c->stream));
  c->kind.assign(kind, kind + n);
  c->matIds.assign(mat, mat + n);
  c->shape5.assign(5 * (size_t)n, 0.0);
  c->isSphere.assign(n, 0); c->axisSense.assign(2 * (size_t)n, 0);
  c->wallIds.clear();
  int NP = 0;
  for (int i = 0; i < n; i++) {
    if (mat[i] < 0 || mat[i] >= c->nMats) return fail(c, SQDEM_ERR_ARG, "material id out of range");
    if (kind[i] == SQDEM_WALL) {
      if (!was) return fail(c, SQDEM_ERR_ARG, "wall axis/sense missing");
      int ax = was[2 * i], se = was[2 * i + 1];
      if (ax < 0 || ax > 2 || se < -1 || se > 1) return fail(c, SQDEM_ERR_ARG, "bad wall axis/sense");
      c->axisSense[2 * i] = ax; c->axisSense[2 * i + 1] = se;
      c->wallIds.push_back(i);
    } else if (kind[i] == SQDEM_SUPERQUADRIC) {
      if (!shape5) return fail(c, SQDEM_ERR_ARG, "shape missing");
      for (int k = 0; k < 5; k++) c->shape5[5 * i + k] = shape5[5 * i + k];
      for (int k = 0; k < 5; k++)
        if (!(shape5[5 * i + k] > 0)) return fail(c, SQDEM_ERR_ARG, "shape parameters must be positive");
      if (shape5[5 * i + 3] >= 2.0 || shape5[5 * i + 4] >= 2.0) return fail(c, SQDEM_ERR_ARG, "eps must be < 2");
      c->isSphere[i] = isSphere ? (isSphere[i] != 0) : 0;
      NP++;
    } else return fail(c, SQDEM_ERR_ARG, "unknown body kind");
  }
  if (!finiteRows(state, n, SQDEM_BODY_STRIDE, 16)) return fail(c, SQDEM_ERR_ARG, "non-finite body state");
  if ((int)c->wallIds.size() > MAX_WALLS) return fail(c, SQDEM_ERR_CAPACITY, "more than 64 walls");
  Dev& d = c->d;
  d.N = n; d.NP = NP; d.W = (int)c->wallIds.size();
  d.MAXC = c->maxCand;
  d.Pcap = (int)std::min<long long>((long long)c->contactsPerBody * NP + 64, 0x7fffffffLL - 1024);
  d.Gmax = std::max(8 * NP, 1 << 12);
  CK(dalloc(c, &d.prm, 1)); CK(dalloc(c, &d.S, 1));
  CK(dalloc(c, &d.pos, n)); CK(dalloc(c, &d.ori, n)); CK(dalloc(c, &d.vel, n)); CK(dalloc(c, &d.angVel, n));
  CK(dalloc(c, &d.angMom, n)); CK(dalloc(c, &d.inertia, n)); CK(dalloc(c, &d.shpA, n)); CK(dalloc(c, &d.shpB, n));
  CK(dalloc(c, &d.mass, n)); CK(dalloc(c, &d.info, n)); CK(dalloc(c, &d.blocked, n)); CK(dalloc(c, &d.damped, n));
  CK(dalloc(c, &d.aspherical, n));
  CK(dalloc(c, &d.bmin, n)); CK(dalloc(c, &d.bmax, n)); CK(dalloc(c, &d.ref, n)); CK(dalloc(c, &d.pmin, n));
  CK(dalloc(c, &d.pmax, n)); CK(dalloc(c, &d.force, n)); CK(dalloc(c, &d.torque, n));
  CK(dalloc(c, &d.walls, std::max(d.W, 1)));
  sqdem_status s;
  if ((s = allocTable(c, d.A, d.Pcap))) return s;
  if ((s = allocTable(c, d.B, d.Pcap))) return s;
  CK(dalloc(c, &d.rowStart, n + 1)); CK(dalloc(c, &d.rowStartNew, n + 1)); CK(dalloc(c, &d.rowCount, n + 1));
  CK(dalloc(c, &d.cand, (size_t)n * d.MAXC)); CK(dalloc(c, &d.candCount, n));
  CK(dalloc(c, &d.pCount, n + 1)); CK(dalloc(c, &d.pStart, n + 1)); CK(dalloc(c, &d.pFill, n + 1));
  CK(dalloc(c, &d.pList, d.Pcap));
  CK(dalloc(c, &d.wCount, 2 * std::max(d.W, 1))); CK(dalloc(c, &d.wList, d.Pcap));
  d.wallChunks = std::max(1, std::min(WALL_CHUNKS, nblk(d.Pcap, 4096)));
  CK(dalloc(c, &d.wBlk, (size_t)d.wallChunks * std::max(d.W, 1)));
  d.svBlocks = std::max(1, std::min(nblk(d.Pcap, 128), c->numSMs * 2));
  CK(dalloc(c, &d.wallKn, std::max(d.W, 1))); CK(dalloc(c, &d.svPart, (size_t)d.svBlocks * SV_PART));
  c->servoOn = false;
  CK(dalloc(c, &d.ww, std::max(d.W * d.W, 1)));
  CK(dalloc(c, &d.lmQueue, d.Pcap));
  CK(dalloc(c, &d.fbQueue, d.Pcap));
  CK(dalloc(c, &d.bodyFF, d.N));
  d.qCap = d.Pcap;
  CK(dalloc(c, &d.bodyCell, n)); CK(dalloc(c, &d.cellCount, d.Gmax + 1)); CK(dalloc(c, &d.cellStart, d.Gmax + 1));
  CK(dalloc(c, &d.cellFill, d.Gmax + 1)); CK(dalloc(c, &d.cellBodies, n)); CK(dalloc(c, &d.cellBox, 2 * (size_t)n));
  CK(dalloc(c, &d.scanTmp, nblk((long)std::max(std::max(d.Gmax, d.Pcap), d.N) + 2, SCAN_TILE) + 2));
  // host-side body arrays
  std::vector<double4> v[5];
  for (int k = 0; k < 5; k++) v[k].resize(n);
  packState(c, n, state, v);
  std::vector<double4> inertia(n), shpA(n), shpB(n), bmin(n), bmax(n), ref(n);
  std::vector<double> mass(n);
  std::vector<int4> info(n);
  std::vector<unsigned> blocked(n);
  std::vector<int> damped(n, 1), asph(n);
  const double nan = std::numeric_limits<double>::quiet_NaN();
  for (int i = 0; i < n; i++) {
    const double* o = state + (size_t)i * SQDEM_BODY_STRIDE;
    mass[i] = o[33];
    inertia[i] = make_double4(o[34], o[35], o[36], 0);
    bmin[i] = make_double4(0, 0, 0, 0);
    bmax[i] = make_double4(0, 0, 0, 0);
    if (kind[i] == SQDEM_SUPERQUADRIC) {
      double props[5];
      sqdem_shape_props(shape5[5 * i], shape5[5 * i + 1], shape5[5 * i + 2], shape5[5 * i + 3], shape5[5 * i + 4], props);
      shpA[i] = make_double4(shape5[5 * i], shape5[5 * i + 1], shape5[5 * i + 2], props[4]);
      shpB[i] = make_double4(shape5[5 * i + 3], shape5[5 * i + 4], 0, 0);
      info[i] = make_int4(KIND_SQ, mat[i], c->isSphere[i], 0);
      blocked[i] = 0; asph[i] = 1;
      ref[i] = make_double4(nan, nan, nan, 1.0);   // Aabb created with the body, refPos NaN
    } else {
      shpA[i] = make_double4(0, 0, 0, 0); shpB[i] = make_double4(0, 0, 0, 0);
      info[i] = make_int4(KIND_WALL, mat[i], 0, c->axisSense[2 * i] | ((c->axisSense[2 * i + 1] + 1) << 4));
      blocked[i] = DOF_ALL; asph[i] = 0;
      ref[i] = make_double4(nan, nan, nan, 0.0);   // no bound until the first collider pass
    }
  }
  auto up = [&](void* dst, const void* src, size_t bytes) { return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream); };
  CK(up(d.pos, v[0].data(), sizeof(double4) * n)); CK(up(d.ori, v[1].data(), sizeof(double4) * n));
  CK(up(d.vel, v[2].data(), sizeof(double4) * n)); CK(up(d.angVel, v[3].data(), sizeof(double4) * n));
  CK(up(d.angMom, v[4].data(), sizeof(double4) * n));
  CK(up(d.inertia, inertia.data(), sizeof(double4) * n)); CK(up(d.shpA, shpA.data(), sizeof(double4) * n));
  CK(up(d.shpB, shpB.data(), sizeof(double4) * n)); CK(up(d.mass, mass.data(), sizeof(double) * n));
  CK(up(d.info, info.data(), sizeof(int4) * n)); CK(up(d.blocked, blocked.data(), sizeof(unsigned) * n));
  CK(up(d.damped, damped.data(), sizeof(int) * n)); CK(up(d.aspherical, asph.data(), sizeof(int) * n));
  CK(up(d.bmin, bmin.data(), sizeof(double4) * n)); CK(up(d.bmax, bmax.data(), sizeof(double4) * n));
  CK(up(d.ref, ref.data(), sizeof(double4) * n)); CK(up(d.pmin, bmin.data(), sizeof(double4) * n));
  CK(up(d.pmax, bmax.data(), sizeof(double4) * n));
  if (d.W) CK(up(d.walls, c->wallIds.data(), sizeof(int) * d.W));
  SceneState S;
  std::memset(&S, 0, sizeof(S));
  S.maxVelocitySq = nan; S.fastestBodyMaxDist = -1; S.verletDistCur = c->params.verletDist;
  S.haltAt = -1;
  CK(up(d.S, &S, sizeof(S)));
  c->haveBodies = true;
  c->graphValid = false; c->epoch++;
  if ((s = uploadParams(c))) return s;
  CK(cudaStreamSynchronize(c->stream));
  return SQDEM_OK;
}

sqdem_status sqdem_step(sqdem_ctx* c, int nsteps) {
  if (!c) return SQDEM_ERR_ARG;
  if (!c->haveBodies || !c->haveMats) return fail(c, SQDEM_ERR_STATE, "bodies and materials must be set before stepping");
  if (nsteps < 0) return fail(c, SQDEM_ERR_ARG, "negative step count");
  CK(cudaSetDevice(c->device));
  if (c->useGraph) {
    sqdem_status s = ensureGraph(c);
    if (s) return s;
    for (int i = 0; i < nsteps; i++) CK(cudaGraphLaunch(c->exec, c->stream));
    c->launches += c->launchesPerStep * nsteps;
  } else {
    float acc[5] = {0, 0, 0, 0, 0};
    c->timingSearch = c->contactModel != SQDEM_CONTACT_HERTZ_MINDLIN;
    for (int i = 0; i < nsteps; i++) {
      enqueueStep(c, true);
      CK(cudaEventSynchronize(c->ev[3]));
      float t;
      cudaEventElapsedTime(&t, c->ev[0], c->ev[1]); acc[0] += t;
      cudaEventElapsedTime(&t, c->ev[1], c->ev[2]); acc[1] += t;
      cudaEventElapsedTime(&t, c->ev[2], c->ev[3]); acc[2] += t;
      if (c->timingSearch) {
        cudaEventElapsedTime(&t, c->ev[4], c->ev[5]); acc[3] += t;
        cudaEventElapsedTime(&t, c->ev[5], c->ev[6]); acc[4] += t;
      }
    }
    c->timingSearch = false;
    for (int k = 0; k < 3; k++) c->stageMs[k] = acc[k];
    c->searchMs[0] = acc[3]; c->searchMs[1] = acc[4];
  }
  CK(cudaGetLastError());
  return SQDEM_OK;
}

sqdem_status sqdem_sync(sqdem_ctx* c, sqdem_report* r) {
  if (!c) return SQDEM_ERR_ARG;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  if (!c->haveBodies) { if (r) std::memset(r, 0, sizeof(*r)); return SQDEM_OK; }
  unsigned long long e[E_NUM];
  CK(cudaMemcpy(e, (char*)c->d.S + offsetof(SceneState, err), sizeof(e), cudaMemcpyDeviceToHost));
  unsigned long long z[E_NUM]; std::memset(z, 0, sizeof(z));
  CK(cudaMemcpy((char*)c->d.S + offsetof(SceneState, err), z, sizeof(z), cudaMemcpyHostToDevice));
  if (r) {
    r->nan_normals = (long long)e[E_NAN_NORMAL]; r->nan_forces = (long long)e[E_NAN_FORCE];
    r->lm_calls = (long long)e[E_LM_CALLS]; r->lm_iterations = (long long)e[E_LM_ITERS];
    r->lm_maxiter = (long long)e[E_LM_MAX]; r->overflow = (long long)e[E_OVERFLOW];
    r->collider_runs = (long long)e[E_COLLIDER_RUNS]; r->steps = (long long)e[E_STEPS];
    r->evals_fp32 = (long long)e[E_EVAL32]; r->evals_fp64 = (long long)e[E_EVAL64];
    r->lm_rounds_max = (long long)e[E_ROUNDS_MAX];
    r->fallback_fp64 = (long long)e[E_FALLBACK];
    r->lm_rounds_max_ff = (long long)e[E_ROUNDS_MAX_FF];
    r->long_queue = (long long)e[E_LONG_QUEUE];
  }
  if (e[E_OVERFLOW]) return fail(c, SQDEM_ERR_CAPACITY, "contact table or candidate buffer overflow; increase contacts_per_body");
  return SQDEM_OK;
}

sqdem_status sqdem_get_body_state(sqdem_ctx* c, double* out) {
  if (!c || !out) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  CK(cudaSetDevice(c->device));
  const int n = c->d.N;
  std::vector<double4> pos(n), ori(n), vel(n), av(n), am(n), f(n), t(n), mn(n), mx(n), rf(n), in(n);
  std::vector<double> mass(n);
  auto dn = [&](void* dst, const void* src, size_t bytes) { return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream); };
  CK(dn(pos.data(), c->d.pos, 32 * n)); CK(dn(ori.data(), c->d.ori, 32 * n)); CK(dn(vel.data(), c->d.vel, 32 * n));
  CK(dn(av.data(), c->d.angVel, 32 * n)); CK(dn(am.data(), c->d.angMom, 32 * n)); CK(dn(f.data(), c->d.force, 32 * n));
  CK(dn(t.data(), c->d.torque, 32 * n)); CK(dn(mn.data(), c->d.bmin, 32 * n)); CK(dn(mx.data(), c->d.bmax, 32 * n));
  CK(dn(rf.data(), c->d.ref, 32 * n)); CK(dn(in.data(), c->d.inertia, 32 * n)); CK(dn(mass.data(), c->d.mass, 8 * n));
  CK(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < n; i++) {
    double* o = out + (size_t)i * SQDEM_BODY_STRIDE;
    o[0] = pos[i].x; o[1] = pos[i].y; o[2] = pos[i].z;
    o[3] = ori[i].x; o[4] = ori[i].y; o[5] = ori[i].z; o[6] = ori[i].w;
    o[7] = vel[i].x; o[8] = vel[i].y; o[9] = vel[i].z;
    o[10] = av[i].x; o[11] = av[i].y; o[12] = av[i].z;
    o[13] = am[i].x; o[14] = am[i].y; o[15] = am[i].z;
    o[16] = f[i].x; o[17] = f[i].y; o[18] = f[i].z;
    o[19] = t[i].x; o[20] = t[i].y; o[21] = t[i].z;
    o[22] = mn[i].x; o[23] = mn[i].y; o[24] = mn[i].z;
    o[25] = mx[i].x; o[26] = mx[i].y; o[27] = mx[i].z;
    o[28] = rf[i].x; o[29] = rf[i].y; o[30] = rf[i].z;
    o[31] = mn[i].w; o[32] = mx[i].w; o[33] = mass[i];
    o[34] = in[i].x; o[35] = in[i].y; o[36] = in[i].z;
  }
  return SQDEM_OK;
}

sqdem_status sqdem_put_body_state(sqdem_ctx* c, const double* in) {
  if (!c || !in) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  if (!finiteRows(in, c->d.N, SQDEM_BODY_STRIDE, 16))
    return fail(c, SQDEM_ERR_ARG, "non-finite position, orientation or velocity");
  CK(cudaSetDevice(c->device));
  const int n = c->d.N;
  std::vector<double4> v[5];
  for (int k = 0; k < 5; k++) v[k].resize(n);
  packState(c, n, in, v);
  std::vector<double4> mn(n), mx(n), rf(n);
  for (int i = 0; i < n; i++) {
    const double* o = in + (size_t)i * SQDEM_BODY_STRIDE;
    mn[i] = make_double4(o[22], o[23], o[24], o[31]);
    mx[i] = make_double4(o[25], o[26], o[27], o[32]);
    bool hasBound = (c->kind[i] == SQDEM_SUPERQUADRIC) || !std::isnan(o[28]);
    rf[i] = make_double4(o[28], o[29], o[30], hasBound ? 1.0 : 0.0);
  }
  auto up = [&](void* dst, const void* src, size_t bytes) { return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream); };
  CK(up(c->d.pos, v[0].data(), 32 * n)); CK(up(c->d.ori, v[1].data(), 32 * n)); CK(up(c->d.vel, v[2].data(), 32 * n));
  CK(up(c->d.angVel, v[3].data(), 32 * n)); CK(up(c->d.angMom, v[4].data(), 32 * n));
  CK(up(c->d.bmin, mn.data(), 32 * n)); CK(up(c->d.bmax, mx.data(), 32 * n)); CK(up(c->d.ref, rf.data(), 32 * n));
  CK(up(c->d.pmin, mn.data(), 32 * n)); CK(up(c->d.pmax, mx.data(), 32 * n));
  CK(cudaStreamSynchronize(c->stream));
  return SQDEM_OK;
}

sqdem_status sqdem_get_kinematics(sqdem_ctx* c, double* out16) {
  if (!c || !out16) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  CK(cudaSetDevice(c->device));
  const int n = c->d.N;
  // five double4 planes -> 16 doubles per body, copied straight from device memory
  CK(cudaMemcpy2DAsync(out16 + 0, 16 * 8, c->d.pos, 32, 24, n, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpy2DAsync(out16 + 3, 16 * 8, c->d.ori, 32, 32, n, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpy2DAsync(out16 + 7, 16 * 8, c->d.vel, 32, 24, n, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpy2DAsync(out16 + 10, 16 * 8, c->d.angVel, 32, 24, n, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpy2DAsync(out16 + 13, 16 * 8, c->d.angMom, 32, 24, n, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SQDEM_OK;
}
sqdem_status sqdem_put_kinematics(sqdem_ctx* c, const double* in16) {
  if (!c || !in16) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  if (!finiteRows(in16, c->d.N, 16, 16)) return fail(c, SQDEM_ERR_ARG, "non-finite kinematic state");
  CK(cudaSetDevice(c->device));
  const int n = c->d.N;
  CK(cudaMemcpy2DAsync(c->d.pos, 32, in16 + 0, 16 * 8, 24, n, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpy2DAsync(c->d.ori, 32, in16 + 3, 16 * 8, 32, n, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpy2DAsync(c->d.vel, 32, in16 + 7, 16 * 8, 24, n, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpy2DAsync(c->d.angVel, 32, in16 + 10, 16 * 8, 24, n, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpy2DAsync(c->d.angMom, 32, in16 + 13, 16 * 8, 24, n, cudaMemcpyHostToDevice, c->stream));
  return SQDEM_OK;
}

static sqdem_status readScene(sqdem_ctx* c, SceneState& S) {
  CK(cudaMemcpyAsync(&S, c->d.S, sizeof(S), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SQDEM_OK;
}

sqdem_status sqdem_num_interactions(sqdem_ctx* c, int include_potential, long* n) {
  if (!c || !n) return SQDEM_ERR_ARG;
  if (!c->haveBodies) { *n = 0; return SQDEM_OK; }
  CK(cudaSetDevice(c->device));
  SceneState S; sqdem_status s = readScene(c, S); if (s) return s;
  if (include_potential) { *n = (long)S.P + S.nWW; return SQDEM_OK; }
  std::vector<unsigned> fl(S.P);
  if (S.P) CK(cudaMemcpy(fl.data(), c->d.A.flags, 4 * (size_t)S.P, cudaMemcpyDeviceToHost));
  long k = 0;
  for (int i = 0; i < S.P; i++) k += ((fl[i] & (F_GEOM | F_PHYS)) == (F_GEOM | F_PHYS));
  *n = k;
  return SQDEM_OK;
}

sqdem_status sqdem_get_interactions(sqdem_ctx* c, int include_potential, double* out, long cap, long* nout) {
  if (!c || !nout) return SQDEM_ERR_ARG;
  if (!c->haveBodies) { *nout = 0; return SQDEM_OK; }
  CK(cudaSetDevice(c->device));
  SceneState S; sqdem_status s = readScene(c, S); if (s) return s;
  const int P = S.P;
  const Table& T = c->d.A;
  std::vector<int> ow(P), pa(P); std::vector<unsigned> fl(P); std::vector<double2> an(P); std::vector<double> de(P);
  std::vector<double4> nm(P), sh(P), nf(P), ph(P), cp(P), p1(P), p2(P), si(P), tw(P), orr(P), rn(P), rs(P), hc(P), he(P);
  std::vector<double2> hs(P);
  std::vector<int4> cdv(P);
  std::vector<int2> ww(S.nWW);
  if (P) {
    CK(cudaMemcpy(ow.data(), T.owner, 4 * (size_t)P, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(pa.data(), T.partner, 4 * (size_t)P, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(fl.data(), T.flags, 4 * (size_t)P, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(an.data(), T.angle, 16 * (size_t)P, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(de.data(), T.depth, 8 * (size_t)P, cudaMemcpyDeviceToHost));
    const size_t b4 = 32 * (size_t)P;
    CK(cudaMemcpy(nm.data(), T.normal, b4, cudaMemcpyDeviceToHost)); CK(cudaMemcpy(sh.data(), T.shear, b4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(nf.data(), T.nforce, b4, cudaMemcpyDeviceToHost)); CK(cudaMemcpy(ph.data(), T.phys, b4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(cp.data(), T.cp, b4, cudaMemcpyDeviceToHost)); CK(cudaMemcpy(p1.data(), T.p1, b4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(p2.data(), T.p2, b4, cudaMemcpyDeviceToHost)); CK(cudaMemcpy(si.data(), T.shearInc, b4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(tw.data(), T.twist, b4, cudaMemcpyDeviceToHost)); CK(cudaMemcpy(orr.data(), T.ortho, b4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(rn.data(), T.relVn, b4, cudaMemcpyDeviceToHost)); CK(cudaMemcpy(rs.data(), T.relVs, b4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(hc.data(), T.hmCurv, b4, cudaMemcpyDeviceToHost)); CK(cudaMemcpy(he.data(), T.hmEll, b4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(hs.data(), T.hmSum, 16 * (size_t)P, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(cdv.data(), T.cd, sizeof(int4) * (size_t)P, cudaMemcpyDeviceToHost));
  }
  if (S.nWW) CK(cudaMemcpy(ww.data(), c->d.ww, sizeof(int2) * S.nWW, cudaMemcpyDeviceToHost));
  long k = 0;
  auto put3 = [](double* o, double4 v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; };
  for (int i = 0; i < P; i++) {
    const bool real = (fl[i] & (F_GEOM | F_PHYS)) == (F_GEOM | F_PHYS);
    if (!include_potential && !real) continue;
    if (out && k < cap) {
      double* o = out + (size_t)k * SQDEM_INTR_STRIDE;
      std::memset(o, 0, sizeof(double) * SQDEM_INTR_STRIDE);
      const bool ownerId1 = (fl[i] & F_OWNER_ID1) != 0;
      o[0] = ownerId1 ? ow[i] : pa[i]; o[1] = ownerId1 ? pa[i] : ow[i];
      o[2] = real; o[3] = (fl[i] & F_GEOM) ? 1 : 0; o[4] = de[i]; o[5] = an[i].x; o[6] = an[i].y;
      put3(o + 7, cp[i]); put3(o + 10, nm[i]); put3(o + 13, si[i]); put3(o + 16, p1[i]); put3(o + 19, p2[i]);
      o[22] = (fl[i] & F_SHEARNEW) ? 1 : 0;
      o[23] = ph[i].x; o[24] = ph[i].y; o[25] = ph[i].z;
      put3(o + 26, nf[i]); put3(o + 29, sh[i]); put3(o + 32, tw[i]); put3(o + 35, orr[i]); put3(o + 38, rn[i]); put3(o + 41, rs[i]);
      o[44] = cdv[i].x; o[45] = cdv[i].y; o[46] = cdv[i].z;   // stored for (id1, id2)
      o[47] = hc[i].x; o[48] = hc[i].y; o[49] = hc[i].z; o[50] = hc[i].w;
      o[51] = he[i].x; o[52] = he[i].y; o[53] = he[i].z; o[54] = he[i].w; o[55] = hs[i].x; o[56] = hs[i].y;
    }
    k++;
  }
  if (include_potential)
    for (int i = 0; i < S.nWW; i++) {
      if (out && k < cap) {
        double* o = out + (size_t)k * SQDEM_INTR_STRIDE;
        std::memset(o, 0, sizeof(double) * SQDEM_INTR_STRIDE);
        o[0] = ww[i].x; o[1] = ww[i].y; o[22] = 1;
      }
      k++;
    }
  *nout = k;
  if (out && k > cap) return fail(c, SQDEM_ERR_ARG, "output capacity too small");
  return SQDEM_OK;
}

sqdem_status sqdem_put_interactions(sqdem_ctx* c, long n, const double* in) {
  if (!c || n < 0 || (n && !in)) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  CK(cudaSetDevice(c->device));
  const int N = c->d.N;
  struct Rec { int owner, partner; long idx; };
  std::vector<Rec> recs;
  std::vector<int2> ww;
  for (long i = 0; i < n; i++) {
    const double* o = in + (size_t)i * SQDEM_INTR_STRIDE;
    int a = (int)o[0], b = (int)o[1];
    if (a < 0 || b < 0 || a >= N || b >= N || a == b) return fail(c, SQDEM_ERR_ARG, "bad interaction ids");
    bool wa = c->kind[a] == SQDEM_WALL, wb = c->kind[b] == SQDEM_WALL;
    if (wa && wb) { ww.push_back(make_int2(std::min(a, b), std::max(a, b))); continue; }
    int owner = wa ? b : (wb ? a : std::min(a, b));
    int partner = owner == a ? b : a;
    recs.push_back(Rec{owner, partner, i});
  }
  std::sort(recs.begin(), recs.end(), [](const Rec& x, const Rec& y) {
    return x.owner != y.owner ? x.owner < y.owner : x.partner < y.partner;
  });
  for (size_t i = 1; i < recs.size(); i++)
    if (recs[i].owner == recs[i - 1].owner && recs[i].partner == recs[i - 1].partner)
      return fail(c, SQDEM_ERR_ARG, "duplicate interaction");
  const int P = (int)recs.size();
  if (P > c->d.Pcap) return fail(c, SQDEM_ERR_CAPACITY, "too many interactions for the table");
  std::vector<int> ow(P), pa(P), rowStart(N + 1, 0);
  std::vector<unsigned> fl(P); std::vector<double2> an(P); std::vector<double> de(P);
  std::vector<double4> nm(P), sh(P), nf(P), ph(P), cp(P), p1(P), p2(P), si(P), tw(P), orr(P), rn(P), rs(P), F(P), hc(P), he(P);
  std::vector<double2> hs(P);
  std::vector<int4> cdv(P);
  auto g3 = [](const double* o) { return make_double4(o[0], o[1], o[2], 0); };
  for (int e = 0; e < P; e++) {
    const double* o = in + (size_t)recs[e].idx * SQDEM_INTR_STRIDE;
    ow[e] = recs[e].owner; pa[e] = recs[e].partner;
    rowStart[ow[e] + 1]++;
    unsigned f = 0;
    if (o[3] != 0) f |= F_GEOM;
    if (o[2] != 0) f |= F_GEOM | F_PHYS;
    if (o[22] != 0) f |= F_SHEARNEW;
    if ((int)o[0] == ow[e]) f |= F_OWNER_ID1;
    fl[e] = f;
    de[e] = o[4]; an[e] = make_double2(o[5], o[6]);
    cp[e] = g3(o + 7); nm[e] = g3(o + 10); si[e] = g3(o + 13); p1[e] = g3(o + 16); p2[e] = g3(o + 19);
    ph[e] = make_double4(o[23], o[24], o[25], 0);
    nf[e] = g3(o + 26); sh[e] = g3(o + 29); tw[e] = g3(o + 32); orr[e] = g3(o + 35); rn[e] = g3(o + 38); rs[e] = g3(o + 41);
    F[e] = make_double4(0, 0, 0, 0);
    cdv[e] = make_int4((int)o[44], (int)o[45], (int)o[46], 0);
    hc[e] = make_double4(o[47], o[48], o[49], o[50]); he[e] = make_double4(o[51], o[52], o[53], o[54]);
    hs[e] = make_double2(o[55], o[56]);
  }
  for (int i = 0; i < N; i++) rowStart[i + 1] += rowStart[i];
  // partner incidence lists (ascending entry index) and wall lists
  std::vector<int> pStart(N + 1, 0), pList(P), wCount(2 * std::max(c->d.W, 1), 0), wList(P);
  for (int e = 0; e < P; e++) if (c->kind[pa[e]] == SQDEM_SUPERQUADRIC) pStart[pa[e] + 1]++;
  for (int i = 0; i < N; i++) pStart[i + 1] += pStart[i];
  {
    std::vector<int> fill(N, 0);
    for (int e = 0; e < P; e++) if (c->kind[pa[e]] == SQDEM_SUPERQUADRIC) pList[pStart[pa[e]] + fill[pa[e]]++] = e;
    int off = 0;
    for (int w = 0; w < c->d.W; w++) {
      int wid = c->wallIds[w], cnt = 0;
      wCount[c->d.W + w] = off;
      for (int e = 0; e < P; e++) if (pa[e] == wid) { wList[off + cnt] = e; cnt++; }
      wCount[w] = cnt; off += cnt;
    }
  }
  const Table& T = c->d.A;
  auto up = [&](void* dst, const void* src, size_t bytes) { return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream) : cudaSuccess; };
  CK(up(T.owner, ow.data(), 4 * (size_t)P)); CK(up(T.partner, pa.data(), 4 * (size_t)P)); CK(up(T.flags, fl.data(), 4 * (size_t)P));
  CK(up(T.angle, an.data(), 16 * (size_t)P)); CK(up(T.depth, de.data(), 8 * (size_t)P));
  const size_t b4 = 32 * (size_t)P;
  CK(up(T.normal, nm.data(), b4)); CK(up(T.shear, sh.data(), b4)); CK(up(T.nforce, nf.data(), b4)); CK(up(T.phys, ph.data(), b4));
  CK(up(T.cp, cp.data(), b4)); CK(up(T.p1, p1.data(), b4)); CK(up(T.p2, p2.data(), b4)); CK(up(T.shearInc, si.data(), b4));
  CK(up(T.twist, tw.data(), b4)); CK(up(T.ortho, orr.data(), b4)); CK(up(T.relVn, rn.data(), b4)); CK(up(T.relVs, rs.data(), b4));
  CK(up(T.F, F.data(), b4));
  CK(up(T.hmCurv, hc.data(), b4)); CK(up(T.hmEll, he.data(), b4)); CK(up(T.hmSum, hs.data(), 16 * (size_t)P));
  CK(up(T.cd, cdv.data(), sizeof(int4) * (size_t)P));
  CK(up(c->d.rowStart, rowStart.data(), 4 * (size_t)(N + 1)));
  CK(up(c->d.pStart, pStart.data(), 4 * (size_t)(N + 1))); CK(up(c->d.pList, pList.data(), 4 * (size_t)P));
  CK(up(c->d.wCount, wCount.data(), 4 * wCount.size())); CK(up(c->d.wList, wList.data(), 4 * (size_t)P));
  if (!ww.empty()) CK(up(c->d.ww, ww.data(), sizeof(int2) * ww.size()));
  int Pi = P, nWW = (int)ww.size();
  CK(up((char*)c->d.S + offsetof(SceneState, P), &Pi, sizeof(int)));
  CK(up((char*)c->d.S + offsetof(SceneState, nWW), &nWW, sizeof(int)));
  CK(cudaStreamSynchronize(c->stream));
  return SQDEM_OK;
}

sqdem_status sqdem_get_scalars(sqdem_ctx* c, double* o) {
  if (!c || !o) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  CK(cudaSetDevice(c->device));
  SceneState S; sqdem_status s = readScene(c, S); if (s) return s;
  double mv = S.newtonRan ? (S.maxDispCode == 2 ? 2.0 : (S.maxDispCode == 1 ? 0.5 : 0.0)) : S.maxVelocitySq;
  o[0] = (double)S.iter; o[1] = mv; o[2] = S.fastestBodyMaxDist; o[3] = S.strideActive; o[4] = S.newtonFound;
  o[5] = S.verletDistCur; o[6] = S.numReinit; o[7] = (double)S.colliderRuns; o[8] = S.bbInit;
  return SQDEM_OK;
}
sqdem_status sqdem_put_scalars(sqdem_ctx* c, const double* o) {
  if (!c || !o) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  CK(cudaSetDevice(c->device));
  SceneState S; sqdem_status s = readScene(c, S); if (s) return s;
  S.iter = (long long)o[0]; S.maxVelocitySq = o[1]; S.newtonRan = 0; S.maxDispCode = 0;
  S.fastestBodyMaxDist = o[2]; S.strideActive = o[3] != 0; S.newtonFound = o[4] != 0; S.verletDistCur = o[5];
  S.bbInit = o[8] != 0;
  CK(cudaMemcpyAsync(c->d.S, &S, sizeof(S), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SQDEM_OK;
}

sqdem_status sqdem_search_times(sqdem_ctx* c, double* out2) {
  if (!c || !out2) return SQDEM_ERR_ARG;
  out2[0] = c->searchMs[0]; out2[1] = c->searchMs[1];
  return SQDEM_OK;
}

sqdem_status sqdem_stage_times(sqdem_ctx* c, double* out3) {
  if (!c || !out3) return SQDEM_ERR_ARG;
  for (int k = 0; k < 3; k++) out3[k] = c->stageMs[k];
  return SQDEM_OK;
}

long long sqdem_launch_count(sqdem_ctx* c) { return c ? c->launches : 0; }

// Device time of nsteps timesteps: cudaEvents recorded on the context stream around the
// graph replays (or eager launches).
sqdem_status sqdem_time_steps(sqdem_ctx* c, int nsteps, double* ms) {
  if (!c || !ms || nsteps < 0) return SQDEM_ERR_ARG;
  CK(cudaSetDevice(c->device));
  if (c->useGraph) { sqdem_status s = ensureGraph(c); if (s) return s; }
  CK(cudaEventRecord(c->ev[0], c->stream));
  if (c->useGraph) {
    for (int i = 0; i < nsteps; i++) CK(cudaGraphLaunch(c->exec, c->stream));
    c->launches += c->launchesPerStep * nsteps;
  } else for (int i = 0; i < nsteps; i++) enqueueStep(c, false);
  CK(cudaEventRecord(c->ev[3], c->stream));
  CK(cudaEventSynchronize(c->ev[3]));
  float t = 0;
  CK(cudaEventElapsedTime(&t, c->ev[0], c->ev[3]));
  *ms = t;
  return SQDEM_OK;
}

// End-to-end timing through the host interface: every step uploads the kinematic state
// from host memory (16 doubles per body), advances one timestep and reads the state back;
// the two host buffers alternate (step i reads the buffer step i-1 wrote, starting from in16)
// so the trajectory continues.  Pinned host buffers make the copies asynchronous.
sqdem_status sqdem_time_e2e(sqdem_ctx* c, int nsteps, const double* in16, double* out16, double* ms) {
  if (!c || !ms || !in16 || !out16 || nsteps < 0) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  CK(cudaSetDevice(c->device));
  if (c->useGraph) { sqdem_status s = ensureGraph(c); if (s) return s; }
  const int n = c->d.N;
  CK(cudaEventRecord(c->ev[0], c->stream));
  double* bufs[2] = {const_cast<double*>(in16), out16};
  for (int i = 0; i < nsteps; i++) {
    const double* src = bufs[i & 1];
    double* dst = bufs[(i + 1) & 1];
    CK(cudaMemcpy2DAsync(c->d.pos, 32, src + 0, 16 * 8, 24, n, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpy2DAsync(c->d.ori, 32, src + 3, 16 * 8, 32, n, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpy2DAsync(c->d.vel, 32, src + 7, 16 * 8, 24, n, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpy2DAsync(c->d.angVel, 32, src + 10, 16 * 8, 24, n, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpy2DAsync(c->d.angMom, 32, src + 13, 16 * 8, 24, n, cudaMemcpyHostToDevice, c->stream));
    if (c->useGraph) { CK(cudaGraphLaunch(c->exec, c->stream)); c->launches += c->launchesPerStep; }
    else enqueueStep(c, false);
    CK(cudaMemcpy2DAsync(dst + 0, 16 * 8, c->d.pos, 32, 24, n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpy2DAsync(dst + 3, 16 * 8, c->d.ori, 32, 32, n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpy2DAsync(dst + 7, 16 * 8, c->d.vel, 32, 24, n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpy2DAsync(dst + 10, 16 * 8, c->d.angVel, 32, 24, n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpy2DAsync(dst + 13, 16 * 8, c->d.angMom, 32, 24, n, cudaMemcpyDeviceToHost, c->stream));
  }
  CK(cudaEventRecord(c->ev[3], c->stream));
  CK(cudaEventSynchronize(c->ev[3]));
  float t = 0;
  CK(cudaEventElapsedTime(&t, c->ev[0], c->ev[3]));
  *ms = t;
  return SQDEM_OK;
}

// Device time of the contact kernel (narrowphase + law) alone, averaged over nrep launches
// on the current state (the state is advanced: the kernel updates contact history).
sqdem_status sqdem_time_contacts(sqdem_ctx* c, int nrep, double* ms) {
  if (!c || !ms || nrep <= 0) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  CK(cudaSetDevice(c->device));
  Dev& d = c->d;
  CK(cudaEventRecord(c->ev[1], c->stream));
  for (int i = 0; i < nrep; i++) {
    k_reset_queue<<<1, 1, 0, c->stream>>>(d);
    launchContactStage(c, d, c->numSMs * searchBlocksPerSM(c));
  }
  CK(cudaEventRecord(c->ev[2], c->stream));
  CK(cudaEventSynchronize(c->ev[2]));
  CK(cudaGetLastError());
  float t = 0;
  CK(cudaEventElapsedTime(&t, c->ev[1], c->ev[2]));
  *ms = t / nrep;
  c->launches += 3 * nrep;
  return SQDEM_OK;
}

// Periodic cell: Cell::setHSize (columns of hSize9, row-major, are the base vectors) and
// Cell::setVelGrad (applied at the next NewtonIntegrator pass); walls are not supported in a
// periodic scene.
sqdem_status sqdem_set_periodic(sqdem_ctx* c, const double* hSize9, const double* velGrad9) {
  if (!c || !hSize9) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "set bodies first");
  if (c->d.W > 0) return fail(c, SQDEM_ERR_ARG, "walls are not supported in a periodic scene");
  CK(cudaSetDevice(c->device));
  SceneState S; sqdem_status st = readScene(c, S); if (st) return st;
  S.periodic = 1; S.homoDeform = 1;
  double t[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  for (int k = 0; k < 9; k++) { S.hSize[k] = hSize9[k]; S.trsf[k] = t[k]; }
  for (int i = 0; i < 3; i++) {
    const double a = hSize9[i], b = hSize9[3 + i], cc = hSize9[6 + i];
    S.cellSize[i] = std::sqrt(a * a + (b * b + cc * cc));
    S.prevRunCellSize[i] = S.cellSize[i];
    S.prevCellSize[i] = std::numeric_limits<double>::quiet_NaN();
  }
  if (velGrad9) { for (int k = 0; k < 9; k++) S.nextVelGrad[k] = velGrad9[k]; S.velGradChanged = 1; }
  S.bbInit = 0;
  CK(cudaMemcpyAsync(c->d.S, &S, sizeof(S), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SQDEM_OK;
}
sqdem_status sqdem_set_velgrad(sqdem_ctx* c, const double* velGrad9) {
  if (!c || !velGrad9) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "set bodies first");
  CK(cudaSetDevice(c->device));
  SceneState S; sqdem_status st = readScene(c, S); if (st) return st;
  for (int k = 0; k < 9; k++) S.nextVelGrad[k] = velGrad9[k];
  S.velGradChanged = 1;
  CK(cudaMemcpyAsync(c->d.S, &S, sizeof(S), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SQDEM_OK;
}
// hSize9 velGrad9 prevVelGrad9 size3 prevCellSize3 (33 doubles)
sqdem_status sqdem_get_cell(sqdem_ctx* c, double* o) {
  if (!c || !o) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  CK(cudaSetDevice(c->device));
  SceneState S; sqdem_status st = readScene(c, S); if (st) return st;
  for (int k = 0; k < 9; k++) { o[k] = S.hSize[k]; o[9 + k] = S.velGrad[k]; o[18 + k] = S.prevVelGrad[k]; }
  for (int k = 0; k < 3; k++) { o[27 + k] = S.cellSize[k]; o[30 + k] = S.prevCellSize[k]; }
  return SQDEM_OK;
}
sqdem_status sqdem_put_cell(sqdem_ctx* c, const double* o) {
  if (!c || !o) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  CK(cudaSetDevice(c->device));
  SceneState S; sqdem_status st = readScene(c, S); if (st) return st;
  for (int k = 0; k < 9; k++) { S.hSize[k] = o[k]; S.velGrad[k] = o[9 + k]; S.prevVelGrad[k] = o[18 + k]; S.nextVelGrad[k] = 0; }
  for (int k = 0; k < 3; k++) { S.cellSize[k] = o[27 + k]; S.prevCellSize[k] = o[30 + k]; S.prevRunCellSize[k] = o[27 + k]; }
  S.velGradChanged = 0;
  CK(cudaMemcpyAsync(c->d.S, &S, sizeof(S), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SQDEM_OK;
}

// ---------------------------------------------------------------------------
// Contact stage without allocation.
//
// Some callers cannot call cudaMalloc at the point where they advance the contacts: host
// frameworks that own all device memory through their own pool and forbid raw allocations
// after start-up, or real-time loops that must not block in the allocator.  For them this
// entry point runs one pass of the contact stage (pre-pass, Levenberg-Marquardt kernel,
// contact physics and law) on the context's state with its work queue (scratch) in
// g_static_lm_queue instead of a buffer owned by the context.  It calls no cudaMalloc,
// cudaFree or allocating library routine.
//
// Limits and rules:
//  * the context's contact table may hold at most SQDEM_STATIC_QUEUE_MAX (1,048,576)
//    entries: a context created with a larger table capacity (contacts_per_body x particles)
//    is rejected with SQDEM_ERR_CAPACITY before anything is launched.  The check reads only
//    that host-side capacity, never the current table size on the device, so it cannot pass
//    on a stale size while earlier work is still queued on the context stream; the queue
//    never holds more entries than the table;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and keeps it for later calls; make that
//    first call before any stream capture.  A device reset (cudaDeviceReset) invalidates the
//    kept address: do not use the library across one;
//  * all calls share the one array, which keeps the last call's contents; nothing in it needs
//    to start at zero (the queue counters live in the context and are reset by the call), but
//    calls that overlap on the GPU (other streams or contexts at the same time) race on it;
//  * the launches are asynchronous on the context stream, like sqdem_step, and ordered after
//    the work already queued there.
static std::mutex g_static_queue_mutex;
static int* g_static_queue_addr[128];
static bool g_static_queue_ready[128];

static sqdem_status staticQueueAddress(sqdem_ctx* c, int** out) {
  if (c->device < 0 || c->device >= 128) return fail(c, SQDEM_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_static_queue_mutex);
  if (!g_static_queue_ready[c->device]) {
    CK(cudaSetDevice(c->device));
    int* ptr = nullptr;
    CK(cudaGetSymbolAddress((void**)&ptr, g_static_lm_queue));
    g_static_queue_addr[c->device] = ptr;
    g_static_queue_ready[c->device] = true;
  }
  *out = g_static_queue_addr[c->device];
  return SQDEM_OK;
}

sqdem_status sqdem_contacts_static_queue(sqdem_ctx* c) {
  if (!c) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "bodies must be set before the contact stage");
  if (c->d.Pcap > SQDEM_STATIC_QUEUE_MAX)
    return fail(c, SQDEM_ERR_CAPACITY, "contact table capacity is " + std::to_string(c->d.Pcap) +
                " entries; sqdem_contacts_static_queue handles at most " + std::to_string(SQDEM_STATIC_QUEUE_MAX) +
                " (create the context with fewer contacts per body or fewer particles)");
  CK(cudaSetDevice(c->device));
  int* queue = nullptr;
  sqdem_status st = staticQueueAddress(c, &queue);
  if (st) return st;
  Dev d = c->d;
  d.lmQueue = queue;
  d.qCap = SQDEM_STATIC_QUEUE_MAX;
  k_reset_queue<<<1, 1, 0, c->stream>>>(d);
  c->launches += 1;
  launchContactStage(c, d, c->numSMs * searchBlocksPerSM(c));
  CK(cudaGetLastError());
  return SQDEM_OK;
}

// Switch between CUDA-graph replay (1) and eager launches with per-stage event timing (0).
sqdem_status sqdem_set_use_graph(sqdem_ctx* c, int on) {
  if (!c) return SQDEM_ERR_ARG;
  c->useGraph = on ? 1 : 0;
  return SQDEM_OK;
}

// Record the full contact geometry (point1/2, shearInc, twist/orthonormal axes, relative
// velocities) in the table every step; off by default (extra HBM writes).
sqdem_status sqdem_set_record_full(sqdem_ctx* c, int on) {
  if (!c) return SQDEM_ERR_ARG;
  c->recordFull = on ? 1 : 0;
  if (c->haveBodies) { sqdem_status s = uploadParams(c); if (s) return s; CK(cudaStreamSynchronize(c->stream)); }
  return SQDEM_OK;
}

sqdem_status sqdem_set_periodic_fix(sqdem_ctx* c, int on) {
  if (!c) return SQDEM_ERR_ARG;
  c->periodicFix = on ? 1 : 0;
  c->graphValid = false;
  if (c->haveBodies) { sqdem_status s = uploadParams(c); if (s) return s; CK(cudaStreamSynchronize(c->stream)); }
  return SQDEM_OK;
}

sqdem_status sqdem_set_lm_spread(sqdem_ctx* c, int on) {
  if (!c) return SQDEM_ERR_ARG;
  c->lmSpread = on ? 1 : 0;
  if (c->haveBodies) { sqdem_status s = uploadParams(c); if (s) return s; CK(cudaStreamSynchronize(c->stream)); }
  return SQDEM_OK;
}

// ---------------------------------------------------------------------------
// Launch shapes of the contact stage and their autotuner.  The shapes change no result (each
// search is a per-contact computation taken from a shared queue; forces are gathered in table
// order), only the time.
sqdem_status sqdem_set_launch_shape(sqdem_ctx* c, int search_blocks_per_sm, int pass1_blocks_per_sm) {
  if (!c || search_blocks_per_sm < 0 || pass1_blocks_per_sm < 0 || pass1_blocks_per_sm > 64) return SQDEM_ERR_ARG;
  if (search_blocks_per_sm != c->shapeSearch || pass1_blocks_per_sm != c->shapePass1) {
    c->shapeSearch = search_blocks_per_sm; c->shapePass1 = pass1_blocks_per_sm;
    c->graphValid = false; c->epoch++;
  }
  return SQDEM_OK;
}

// Time every candidate shape on the scene itself: two rounds over the candidates, `steps`
// timesteps each (CUDA events on the context stream), the minimum per candidate kept.  Since
// shapes change no result these are ordinary timesteps: the scene advances by
// candidates x (2 x steps + 1) steps, as it would with the default shape.
sqdem_status sqdem_autotune(sqdem_ctx* c, int steps, sqdem_tune* out) {
  if (!c || steps <= 0) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  const int mx = maxSearchBlocksPerSM(c);
  const int p1s[4] = {4, 8, 16, 32};
  std::vector<double> t(4 * (size_t)mx, 1e300);
  sqdem_status s;
  for (int round = 0; round < 2; round++)
    for (int sb = 1; sb <= mx; sb++)
      for (int k = 0; k < 4; k++) {
        if ((s = sqdem_set_launch_shape(c, sb, p1s[k]))) return s;
        if (round == 0 && (s = sqdem_step(c, 1))) return s;   // graph capture outside the timing
        double ms = 0;
        if ((s = sqdem_time_steps(c, steps, &ms))) return s;
        double& b = t[4 * (size_t)(sb - 1) + k];
        b = std::min(b, ms);
      }
  size_t bi = 0;
  for (size_t i = 1; i < t.size(); i++) if (t[i] < t[bi]) bi = i;
  const int bs = (int)(bi / 4) + 1, bp = p1s[bi % 4];
  if ((s = sqdem_set_launch_shape(c, bs, bp))) return s;
  if (out) { out->search_blocks_per_sm = bs; out->pass1_blocks_per_sm = bp; out->ms_per_step = t[bi] / steps; out->candidates = (int)t.size(); }
  return SQDEM_OK;
}

sqdem_status sqdem_set_contact_model(sqdem_ctx* c, int model) {
  if (!c) return SQDEM_ERR_ARG;
  if (model != SQDEM_CONTACT_LINEAR && model != SQDEM_CONTACT_HERTZ_MINDLIN)
    return fail(c, SQDEM_ERR_ARG, "contact model must be SQDEM_CONTACT_LINEAR or SQDEM_CONTACT_HERTZ_MINDLIN");
  if (model != c->contactModel) { c->contactModel = model; c->graphValid = false; c->epoch++; }
  if (c->haveBodies) { CK(cudaSetDevice(c->device)); sqdem_status s = uploadParams(c); if (s) return s; CK(cudaStreamSynchronize(c->stream)); }
  return SQDEM_OK;
}

int sqdem_contact_model(sqdem_ctx* c) { return c ? c->contactModel : -1; }
int sqdem_num_materials(sqdem_ctx* c) { return (c && c->haveMats) ? c->nMats : 0; }

sqdem_status sqdem_set_material_moduli(sqdem_ctx* c, int n, const double* G, const double* nu) {
  if (!c || !G || !nu) return SQDEM_ERR_ARG;
  if (!c->haveMats || n != c->nMats) return fail(c, SQDEM_ERR_ARG, "moduli need one (G, nu) per material, after sqdem_set_materials");
  for (int i = 0; i < n; i++)
    if (!(G[i] > 0) || !std::isfinite(G[i]) || !std::isfinite(nu[i])) return fail(c, SQDEM_ERR_ARG, "G must be positive and finite, nu finite");
  for (int i = 0; i < n; i++) c->hostMatsE[i] = make_double2(G[i], nu[i]);
  if (c->haveBodies) {
    CK(cudaSetDevice(c->device));
    CK(cudaMemcpyAsync(c->d.matsE, c->hostMatsE.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return SQDEM_OK;
}

sqdem_status sqdem_get_material_moduli(sqdem_ctx* c, double* G, double* nu) {
  if (!c || !G || !nu) return SQDEM_ERR_ARG;
  if (!c->haveMats) return fail(c, SQDEM_ERR_STATE, "no materials");
  for (int i = 0; i < c->nMats; i++) { G[i] = c->hostMatsE[i].x; nu[i] = c->hostMatsE[i].y; }
  return SQDEM_OK;
}


// ---------------------------------------------------------------------------
// Boundary controller (CompressionEngine), quiet flag, Shop reductions.
sqdem_status sqdem_set_servo(sqdem_ctx* c, const double* g) {
  if (!c || !g) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "set bodies first");
  CK(cudaSetDevice(c->device));
  ServoDev C;
  std::memset(&C, 0, sizeof(C));
  const bool on = g[0] != 0;
  if (on) {
    for (int k = 0; k < 6; k++)
      if ((int)c->kind.size() <= k || c->kind[k] != SQDEM_WALL || (int)c->wallIds.size() <= k || c->wallIds[k] != k)
        return fail(c, SQDEM_ERR_ARG, "CompressionEngine needs bodies 0-5 to be the six walls (left, right, front, back, bottom, top)");
    for (int k = 0; k < 30; k++) if (!std::isfinite(g[k])) return fail(c, SQDEM_ERR_ARG, "non-finite servo parameter");
    if (!(g[13] >= 1) || !(g[14] >= 1)) return fail(c, SQDEM_ERR_ARG, "echo_interval and savedata_interval must be >= 1");
    C.z_servo = g[1] != 0; C.continueFlag = g[2] != 0; C.hydroStrain = g[3] != 0; C.shearMode = (int)g[4];
    for (int k = 0; k < 6; k++) C.activated[k] = g[5 + k] != 0;
    C.iterate_num_max = (unsigned)g[11]; C.solve_num_max = (unsigned)g[12]; C.echo_interval = (unsigned)g[13];
    C.savedata_interval = (unsigned)g[14]; C.ramp_interval = (unsigned)g[15]; C.ramp_chunks = (unsigned)g[16];
    C.goalx = g[17]; C.goaly = g[18]; C.goalz = g[19];
    C.gain_alpha = g[20]; C.target_strain = g[21]; C.f_threshold = g[22]; C.fmin_threshold = g[23];
    C.unbf_tol = g[24]; C.max_vel = g[25]; C.hydroStrainRate = g[26];
    C.width0 = g[27]; C.height0 = g[28]; C.depth0 = g[29];
    C.firstRun = 1; C.UnbalancedForce = 1;
    double pv = 0, props[5];
    for (size_t i = 0; i < c->kind.size(); i++)
      if (c->kind[i] == SQDEM_SUPERQUADRIC) {
        const double* s5 = &c->shape5[5 * i];
        sqdem_shape_props(s5[0], s5[1], s5[2], s5[3], s5[4], props);
        pv += props[0];
      }
    C.pvol = pv;
  }
  C.enabled = on ? 1 : 0;
  CK(cudaMemcpyAsync((char*)c->d.S + offsetof(SceneState, sv), &C, sizeof(C), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (c->servoOn != on) { c->servoOn = on; c->graphValid = false; c->epoch++; }
  return SQDEM_OK;
}

sqdem_status sqdem_get_servo(sqdem_ctx* c, double* o) {
  if (!c || !o) return SQDEM_ERR_ARG;
  for (int k = 0; k < SQDEM_SERVO_STATE; k++) o[k] = 0;
  if (!c->haveBodies) return SQDEM_OK;
  CK(cudaSetDevice(c->device));
  SceneState S; sqdem_status st = readScene(c, S); if (st) return st;
  const ServoDev& C = S.sv;
  const double v[34] = {C.width, C.depth, C.height, C.x_area, C.y_area, C.z_area, C.wsxx, C.wsyy, C.wszz,
                        C.wsxx_left, C.wsxx_right, C.wsyy_front, C.wsyy_back, C.wszz_bottom, C.wszz_top,
                        C.gain_x, C.gain_x1, C.gain_y, C.gain_y1, C.gain_z, C.gain_z1, C.UnbalancedForce,
                        C.particlesVolume, C.Init_boxVolume, C.Current_boxVolume, C.strain2,
                        (double)C.iterate_num, (double)C.solve_num, (double)C.rampNum, (double)C.Flag_ForceTarget,
                        (double)C.firstRun, C.width0, C.height0, C.depth0};
  if (C.enabled) for (int k = 0; k < 34; k++) o[k] = v[k];
  o[34] = (double)S.haltAt; o[35] = S.quiet ? 1 : 0;
  return SQDEM_OK;
}

sqdem_status sqdem_put_servo(sqdem_ctx* c, const double* o) {
  if (!c || !o) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  CK(cudaSetDevice(c->device));
  SceneState S; sqdem_status st = readScene(c, S); if (st) return st;
  ServoDev& C = S.sv;
  if (C.enabled) {
    C.width = o[0]; C.depth = o[1]; C.height = o[2]; C.x_area = o[3]; C.y_area = o[4]; C.z_area = o[5];
    C.wsxx = o[6]; C.wsyy = o[7]; C.wszz = o[8]; C.wsxx_left = o[9]; C.wsxx_right = o[10]; C.wsyy_front = o[11];
    C.wsyy_back = o[12]; C.wszz_bottom = o[13]; C.wszz_top = o[14];
    C.gain_x = o[15]; C.gain_x1 = o[16]; C.gain_y = o[17]; C.gain_y1 = o[18]; C.gain_z = o[19]; C.gain_z1 = o[20];
    C.UnbalancedForce = o[21]; C.particlesVolume = o[22]; C.Init_boxVolume = o[23]; C.Current_boxVolume = o[24];
    C.strain2 = o[25]; C.iterate_num = (unsigned)o[26]; C.solve_num = (unsigned)o[27]; C.rampNum = (unsigned)o[28];
    C.Flag_ForceTarget = o[29] != 0; C.firstRun = o[30] != 0; C.width0 = o[31]; C.height0 = o[32]; C.depth0 = o[33];
    CK(cudaMemcpyAsync((char*)c->d.S + offsetof(SceneState, sv), &C, sizeof(C), cudaMemcpyHostToDevice, c->stream));
  }
  long long halt = (long long)o[34];
  int quiet = o[35] != 0;
  CK(cudaMemcpyAsync((char*)c->d.S + offsetof(SceneState, haltAt), &halt, sizeof(halt), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync((char*)c->d.S + offsetof(SceneState, quiet), &quiet, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SQDEM_OK;
}

sqdem_status sqdem_set_quiet(sqdem_ctx* c, int on) {
  if (!c) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  CK(cudaSetDevice(c->device));
  int q = on ? 1 : 0;
  CK(cudaMemcpyAsync((char*)c->d.S + offsetof(SceneState, quiet), &q, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SQDEM_OK;
}

// block partials of k_servo_sums summed in block order
static sqdem_status svSums(sqdem_ctx* c, int need, double* tot) {
  k_servo_sums<<<c->d.svBlocks, 128, 0, c->stream>>>(c->d, need, 0);
  CK(cudaGetLastError());
  std::vector<double> part((size_t)c->d.svBlocks * SV_PART);
  CK(cudaMemcpyAsync(part.data(), c->d.svPart, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < SV_PART; k++) {
    double s = 0;
    for (int b = 0; b < c->d.svBlocks; b++) s += part[(size_t)b * SV_PART + k];
    tot[k] = s;
  }
  return SQDEM_OK;
}

sqdem_status sqdem_unbalanced_force(sqdem_ctx* c, int use_max, double* out) {
  if (!c || !out) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  CK(cudaSetDevice(c->device));
  if (!use_max) {
    double tot[SV_PART];
    sqdem_status s = svSums(c, 2, tot); if (s) return s;
    *out = tot[10] / (tot[9] * 2.0);
    return SQDEM_OK;
  }
  // largest |F + m g| over dynamic bodies (first in id order), over the sum of |Fn + Fs| of its
  // contacts with a non-zero normal force
  const int n = c->d.N;
  std::vector<double4> F(n); std::vector<double> m(n); std::vector<unsigned> bl(n);
  CK(cudaMemcpy(F.data(), c->d.force, sizeof(double4) * n, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(m.data(), c->d.mass, sizeof(double) * n, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(bl.data(), c->d.blocked, sizeof(unsigned) * n, cudaMemcpyDeviceToHost));
  double maxF = 0; int idMax = -1;
  for (int b = 0; b < n; b++) {
    if (bl[b] == DOF_ALL) continue;
    const double x = F[b].x + m[b] * c->params.gravity[0], y = F[b].y + m[b] * c->params.gravity[1],
                 z = F[b].z + m[b] * c->params.gravity[2];
    const double f = std::sqrt(x * x + (y * y + z * z));
    if (f > maxF) { maxF = f; idMax = b; }
  }
  SceneState S; sqdem_status st = readScene(c, S); if (st) return st;
  const int P = S.P;
  std::vector<int> ow(P), pa(P); std::vector<unsigned> fl(P); std::vector<double4> nf(P), sh(P);
  if (P) {
    CK(cudaMemcpy(ow.data(), c->d.A.owner, 4 * (size_t)P, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(pa.data(), c->d.A.partner, 4 * (size_t)P, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(fl.data(), c->d.A.flags, 4 * (size_t)P, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(nf.data(), c->d.A.nforce, sizeof(double4) * P, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(sh.data(), c->d.A.shear, sizeof(double4) * P, cudaMemcpyDeviceToHost));
  }
  double maxCF = 0;
  for (int e = 0; e < P; e++) {
    if ((fl[e] & (F_GEOM | F_PHYS)) != (F_GEOM | F_PHYS)) continue;
    if (!(ow[e] == idMax || pa[e] == idMax)) continue;
    const double nn = std::sqrt(nf[e].x * nf[e].x + (nf[e].y * nf[e].y + nf[e].z * nf[e].z));
    if (nn == 0) continue;
    const double x = nf[e].x + sh[e].x, y = nf[e].y + sh[e].y, z = nf[e].z + sh[e].z;
    maxCF += std::sqrt(x * x + (y * y + z * z));
  }
  *out = maxF / maxCF;
  return SQDEM_OK;
}

sqdem_status sqdem_get_stress(sqdem_ctx* c, double volume, double* out9) {
  if (!c || !out9) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  CK(cudaSetDevice(c->device));
  SceneState S; sqdem_status st = readScene(c, S); if (st) return st;
  if (volume == 0) {
    if (S.periodic) {
      const double* A = S.hSize;
      volume = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) + A[2] * (A[3] * A[7] - A[4] * A[6]);
    } else volume = 1;
  }
  double tot[SV_PART];
  sqdem_status s = svSums(c, 1, tot); if (s) return s;
  for (int k = 0; k < 9; k++) out9[k] = tot[11 + k] / volume;
  return SQDEM_OK;
}

// ---------------------------------------------------------------------------
// Snapshot / restore: the whole state of a context as one byte blob (materials, parameters,
// bodies with bounds and previous-pass bounds, the contact table with its history in table
// order, and the scene words: iteration, collider and integrator bookkeeping, periodic cell,
// CompressionEngine).  A context restored from it continues bit for bit as the original
// would.  The blob records the library's state-record sizes; a blob from a build with other
// sizes is refused.
static const char SNAP_MAGIC[8] = {'S', 'Q', 'D', 'E', 'M', 'S', 'N', '2'};
struct SnapHeader {
  char magic[8];
  unsigned long long sceneBytes, servoBytes, paramsBytes;
  long long N, nMats, nRec;
  int recordFull, lmSpread, servoOn, contactModel;
};

sqdem_status sqdem_snapshot(sqdem_ctx* c, void* buf, size_t* size) {
  if (!c || !size) return SQDEM_ERR_ARG;
  if (!c->haveBodies) return fail(c, SQDEM_ERR_STATE, "no bodies");
  CK(cudaSetDevice(c->device));
  const long long N = c->d.N;
  long nRec = 0;
  sqdem_status s = sqdem_num_interactions(c, 1, &nRec);
  if (s) return s;
  const size_t need = sizeof(SnapHeader) + sizeof(sqdem_params) + sizeof(double) * 8 * c->nMats +
                      N * (sizeof(int) * 5 + sizeof(double) * 5) + sizeof(double) * SQDEM_BODY_STRIDE * N +
                      sizeof(double4) * 2 * N + sizeof(double) * SQDEM_INTR_STRIDE * nRec + sizeof(SceneState);
  if (!buf) { *size = need; return SQDEM_OK; }
  if (*size < need) { *size = need; return fail(c, SQDEM_ERR_CAPACITY, "snapshot buffer too small"); }
  char* w = (char*)buf;
  auto put = [&](const void* src, size_t bytes) { std::memcpy(w, src, bytes); w += bytes; };
  SnapHeader h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, SNAP_MAGIC, 8);
  h.sceneBytes = sizeof(SceneState); h.servoBytes = sizeof(ServoDev); h.paramsBytes = sizeof(sqdem_params);
  h.N = N; h.nMats = c->nMats; h.nRec = nRec;
  h.recordFull = c->recordFull; h.lmSpread = c->lmSpread; h.servoOn = c->servoOn ? 1 : 0; h.contactModel = c->contactModel;
  put(&h, sizeof(h));
  put(&c->params, sizeof(sqdem_params));
  for (int i = 0; i < c->nMats; i++) {
    const double m[8] = {c->hostMats[i].x, c->hostMats[i].y, c->hostMats[i].z, c->hostMatsB[i].x, c->hostMatsB[i].y,
                         c->hostMats[i].w, c->hostMatsE[i].x, c->hostMatsE[i].y};
    put(m, sizeof(m));
  }
  put(c->kind.data(), sizeof(int) * N);
  put(c->axisSense.data(), sizeof(int) * 2 * N);
  put(c->matIds.data(), sizeof(int) * N);
  put(c->isSphere.data(), sizeof(int) * N);
  put(c->shape5.data(), sizeof(double) * 5 * N);
  std::vector<double> st(SQDEM_BODY_STRIDE * N);
  if ((s = sqdem_get_body_state(c, st.data()))) return s;
  put(st.data(), sizeof(double) * st.size());
  std::vector<double4> pm(2 * N);
  CK(cudaMemcpy(pm.data(), c->d.pmin, sizeof(double4) * N, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(pm.data() + N, c->d.pmax, sizeof(double4) * N, cudaMemcpyDeviceToHost));
  put(pm.data(), sizeof(double4) * 2 * N);
  std::vector<double> rec(SQDEM_INTR_STRIDE * (size_t)nRec);
  long got = 0;
  if ((s = sqdem_get_interactions(c, 1, rec.data(), nRec, &got))) return s;
  put(rec.data(), sizeof(double) * rec.size());
  SceneState S;
  if ((s = readScene(c, S))) return s;
  put(&S, sizeof(S));
  *size = need;
  return SQDEM_OK;
}

sqdem_status sqdem_restore(sqdem_ctx* c, const void* buf, size_t size) {
  if (!c || !buf) return SQDEM_ERR_ARG;
  const char* r = (const char*)buf;
  const char* end = r + size;
  auto get = [&](void* dst, size_t bytes) -> bool {
    if (r + bytes > end) return false;
    std::memcpy(dst, r, bytes); r += bytes; return true;
  };
  SnapHeader h;
  if (!get(&h, sizeof(h)) || std::memcmp(h.magic, SNAP_MAGIC, 8) != 0)
    return fail(c, SQDEM_ERR_ARG, "not a snapshot of this library");
  if (h.sceneBytes != sizeof(SceneState) || h.servoBytes != sizeof(ServoDev) || h.paramsBytes != sizeof(sqdem_params))
    return fail(c, SQDEM_ERR_ARG, "snapshot written by a build with other state records");
  if (h.N <= 0 || h.nMats <= 0 || h.nRec < 0 || h.N >= (1LL << 30)) return fail(c, SQDEM_ERR_ARG, "corrupt snapshot header");
  const long long N = h.N;
  sqdem_params P;
  if (!get(&P, sizeof(P))) return fail(c, SQDEM_ERR_ARG, "truncated snapshot");
  std::vector<double> m(8 * h.nMats);
  if (!get(m.data(), sizeof(double) * m.size())) return fail(c, SQDEM_ERR_ARG, "truncated snapshot");
  std::vector<int> kind(N), was(2 * N), mat(N), sph(N);
  std::vector<double> s5(5 * N), st(SQDEM_BODY_STRIDE * N), rec(SQDEM_INTR_STRIDE * (size_t)h.nRec);
  std::vector<double4> pm(2 * N);
  SceneState S;
  if (!get(kind.data(), 4 * N) || !get(was.data(), 8 * N) || !get(mat.data(), 4 * N) || !get(sph.data(), 4 * N) ||
      !get(s5.data(), 40 * N) || !get(st.data(), sizeof(double) * st.size()) || !get(pm.data(), sizeof(double4) * 2 * N) ||
      !get(rec.data(), sizeof(double) * rec.size()) || !get(&S, sizeof(S)))
    return fail(c, SQDEM_ERR_ARG, "truncated snapshot");
  std::vector<double> Kn(h.nMats), Ks(h.nMats), fa(h.nMats), bn(h.nMats), bs(h.nMats), rho(h.nMats), G(h.nMats), nu(h.nMats);
  for (long long i = 0; i < h.nMats; i++) {
    Kn[i] = m[8 * i]; Ks[i] = m[8 * i + 1]; fa[i] = m[8 * i + 2]; bn[i] = m[8 * i + 3]; bs[i] = m[8 * i + 4]; rho[i] = m[8 * i + 5];
    G[i] = m[8 * i + 6]; nu[i] = m[8 * i + 7];
  }
  if (h.contactModel != SQDEM_CONTACT_LINEAR && h.contactModel != SQDEM_CONTACT_HERTZ_MINDLIN)
    return fail(c, SQDEM_ERR_ARG, "corrupt snapshot header");
  c->haveMats = false;
  sqdem_status s;
  if ((s = sqdem_set_materials(c, (int)h.nMats, Kn.data(), Ks.data(), fa.data(), bn.data(), bs.data(), rho.data()))) return s;
  if ((s = sqdem_set_material_moduli(c, (int)h.nMats, G.data(), nu.data()))) return s;
  if ((s = sqdem_set_params(c, &P))) return s;
  c->recordFull = h.recordFull; c->lmSpread = h.lmSpread; c->contactModel = h.contactModel;
  if ((s = sqdem_set_bodies(c, (int)N, kind.data(), s5.data(), was.data(), mat.data(), sph.data(), st.data()))) return s;
  if ((s = sqdem_put_body_state(c, st.data()))) return s;
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpy(c->d.pmin, pm.data(), sizeof(double4) * N, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->d.pmax, pm.data() + N, sizeof(double4) * N, cudaMemcpyHostToDevice));
  if ((s = sqdem_put_interactions(c, (long)h.nRec, rec.data()))) return s;
  std::memset(S.err, 0, sizeof(S.err));
  CK(cudaMemcpyAsync(c->d.S, &S, sizeof(S), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->servoOn = h.servoOn != 0;
  c->graphValid = false; c->epoch++;
  return uploadParams(c);
}

// ---------------------------------------------------------------------------
// Batches of independent scenes (specimens): one context per scene, one CUDA graph that runs
// one step of every scene as parallel branches, so that the scenes' kernels share the GPU.
// Each scene's kernels and results are exactly those of a context stepped alone.
}  // extern "C"
struct BatchPtrs { double4 *pos, *ori, *vel, *angVel, *angMom; long long off; int n; };

__global__ void k_batch_kin(const BatchPtrs* P, int ns, double* kin, long long rows, int toDevice) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows; r += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = ns - 1;
    while (lo < hi) { const int mid = (lo + hi + 1) >> 1; if (P[mid].off <= r) lo = mid; else hi = mid - 1; }
    const BatchPtrs& s = P[lo];
    const int b = (int)(r - s.off);
    double* k = kin + r * 16;
    if (toDevice) {
      s.pos[b] = make_double4(k[0], k[1], k[2], 0); s.ori[b] = make_double4(k[3], k[4], k[5], k[6]);
      s.vel[b] = make_double4(k[7], k[8], k[9], 0); s.angVel[b] = make_double4(k[10], k[11], k[12], 0);
      s.angMom[b] = make_double4(k[13], k[14], k[15], 0);
    } else {
      const double4 p = s.pos[b], o = s.ori[b], v = s.vel[b], w = s.angVel[b], m = s.angMom[b];
      k[0] = p.x; k[1] = p.y; k[2] = p.z; k[3] = o.x; k[4] = o.y; k[5] = o.z; k[6] = o.w;
      k[7] = v.x; k[8] = v.y; k[9] = v.z; k[10] = w.x; k[11] = w.y; k[12] = w.z; k[13] = m.x; k[14] = m.y; k[15] = m.z;
    }
  }
}

struct sqdem_batch {
  int device = 0;
  std::vector<sqdem_ctx*> scenes;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraph_t graph = nullptr; cudaGraphExec_t exec = nullptr;
  std::vector<unsigned> epochs;
  long long launchesPerStep = 0;
  BatchPtrs* dPtrs = nullptr; double* dKin = nullptr; long long rows = 0;
  std::string err;
};

static sqdem_status bfail(sqdem_batch* b, sqdem_status s, const std::string& m) {
  if (b) b->err = m;
  return s;
}
#define BK(call)                                                                                     \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess) return bfail(B, SQDEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

static void batchFreeGraph(sqdem_batch* B) {
  if (B->exec) { cudaGraphExecDestroy(B->exec); B->exec = nullptr; }
  if (B->graph) { cudaGraphDestroy(B->graph); B->graph = nullptr; }
  B->epochs.clear();
}

static sqdem_status batchReady(sqdem_batch* B) {
  for (size_t i = 0; i < B->scenes.size(); i++) {
    const sqdem_ctx* c = B->scenes[i];
    if (!c->haveBodies || !c->haveMats) return bfail(B, SQDEM_ERR_STATE, "scene " + std::to_string(i) + ": bodies and materials must be set");
  }
  bool stale = B->exec == nullptr || B->epochs.size() != B->scenes.size();
  for (size_t i = 0; !stale && i < B->scenes.size(); i++) stale = B->epochs[i] != B->scenes[i]->epoch;
  if (!stale) return SQDEM_OK;
  batchFreeGraph(B);
  BK(cudaSetDevice(B->device));
  BK(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
  BK(cudaEventRecord(B->fork, B->stream));
  long long l = 0;
  for (size_t i = 0; i < B->scenes.size(); i++) {
    sqdem_ctx* c = B->scenes[i];
    BK(cudaStreamWaitEvent(c->stream, B->fork, 0));
    const long long l0 = c->launches;
    enqueueStep(c, false);
    l += c->launches - l0;
    c->launches = l0;
    BK(cudaEventRecord(B->join[i], c->stream));
    BK(cudaStreamWaitEvent(B->stream, B->join[i], 0));
  }
  BK(cudaStreamEndCapture(B->stream, &B->graph));
  BK(cudaGraphInstantiate(&B->exec, B->graph, 0));
  B->launchesPerStep = l;
  for (sqdem_ctx* c : B->scenes) B->epochs.push_back(c->epoch);
  return SQDEM_OK;
}

extern "C" {

sqdem_status sqdem_batch_create(sqdem_batch** out, int n_scenes, const sqdem_config* cfg) {
  if (!out || n_scenes <= 0) return SQDEM_ERR_ARG;
  sqdem_batch* B = new sqdem_batch();
  *out = B;
  B->device = cfg ? cfg->device : 0;
  BK(cudaSetDevice(B->device));
  BK(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
  BK(cudaEventCreateWithFlags(&B->fork, cudaEventDisableTiming));
  BK(cudaEventCreate(&B->t0)); BK(cudaEventCreate(&B->t1));
  B->join.resize(n_scenes);
  for (int i = 0; i < n_scenes; i++) {
    BK(cudaEventCreateWithFlags(&B->join[i], cudaEventDisableTiming));
    sqdem_ctx* c = nullptr;
    sqdem_status s = sqdem_create(&c, cfg);
    B->scenes.push_back(c);
    if (s) return bfail(B, s, "scene " + std::to_string(i) + ": " + (c ? c->err : std::string("create failed")));
    if (c->device != B->device) return bfail(B, SQDEM_ERR_ARG, "all scenes of a batch share one device");
  }
  return SQDEM_OK;
}

void sqdem_batch_destroy(sqdem_batch* B) {
  if (!B) return;
  cudaSetDevice(B->device);
  if (B->stream) cudaStreamSynchronize(B->stream);
  batchFreeGraph(B);
  if (B->dPtrs) cudaFree(B->dPtrs);
  if (B->dKin) cudaFree(B->dKin);
  for (cudaEvent_t e : B->join) cudaEventDestroy(e);
  if (B->fork) cudaEventDestroy(B->fork);
  if (B->t0) cudaEventDestroy(B->t0);
  if (B->t1) cudaEventDestroy(B->t1);
  for (sqdem_ctx* c : B->scenes) sqdem_destroy(c);
  if (B->stream) cudaStreamDestroy(B->stream);
  delete B;
}

const char* sqdem_batch_last_error(sqdem_batch* B) { return B ? B->err.c_str() : "null batch"; }

int sqdem_batch_size(sqdem_batch* B) { return B ? (int)B->scenes.size() : 0; }

sqdem_status sqdem_batch_scene(sqdem_batch* B, int i, sqdem_ctx** ctx) {
  if (!B || !ctx || i < 0 || i >= (int)B->scenes.size()) return SQDEM_ERR_ARG;
  *ctx = B->scenes[i];
  return SQDEM_OK;
}

sqdem_status sqdem_batch_step(sqdem_batch* B, int nsteps) {
  if (!B || nsteps < 0) return SQDEM_ERR_ARG;
  BK(cudaSetDevice(B->device));
  // work queued on a scene's own stream (uploads) precedes the batch's steps
  for (sqdem_ctx* c : B->scenes) BK(cudaStreamSynchronize(c->stream));
  sqdem_status s = batchReady(B);
  if (s) return s;
  for (int i = 0; i < nsteps; i++) BK(cudaGraphLaunch(B->exec, B->stream));
  BK(cudaGetLastError());
  return SQDEM_OK;
}

// Waits for the batch, then reads every scene's report (summed into total, lm_rounds_max the
// largest); returns the first scene error (SQDEM_ERR_CAPACITY on an overflow).
sqdem_status sqdem_batch_sync(sqdem_batch* B, sqdem_report* total) {
  if (!B) return SQDEM_ERR_ARG;
  BK(cudaSetDevice(B->device));
  BK(cudaStreamSynchronize(B->stream));
  if (total) std::memset(total, 0, sizeof(*total));
  sqdem_status first = SQDEM_OK;
  for (size_t i = 0; i < B->scenes.size(); i++) {
    sqdem_report r;
    sqdem_status s = sqdem_sync(B->scenes[i], &r);
    if (s && !first) { first = s; B->err = "scene " + std::to_string(i) + ": " + B->scenes[i]->err; }
    if (total) {
      total->nan_normals += r.nan_normals; total->nan_forces += r.nan_forces; total->lm_calls += r.lm_calls;
      total->lm_iterations += r.lm_iterations; total->lm_maxiter += r.lm_maxiter; total->overflow += r.overflow;
      total->collider_runs += r.collider_runs; total->steps += r.steps; total->evals_fp32 += r.evals_fp32;
      total->evals_fp64 += r.evals_fp64; total->lm_rounds_max = std::max(total->lm_rounds_max, r.lm_rounds_max);
      total->fallback_fp64 += r.fallback_fp64; total->lm_rounds_max_ff = std::max(total->lm_rounds_max_ff, r.lm_rounds_max_ff);
      total->long_queue += r.long_queue;
    }
  }
  return first;
}

sqdem_status sqdem_batch_time_steps(sqdem_batch* B, int nsteps, double* ms) {
  if (!B || !ms || nsteps < 0) return SQDEM_ERR_ARG;
  BK(cudaSetDevice(B->device));
  for (sqdem_ctx* c : B->scenes) BK(cudaStreamSynchronize(c->stream));
  sqdem_status s = batchReady(B);
  if (s) return s;
  BK(cudaEventRecord(B->t0, B->stream));
  for (int i = 0; i < nsteps; i++) BK(cudaGraphLaunch(B->exec, B->stream));
  BK(cudaEventRecord(B->t1, B->stream));
  BK(cudaEventSynchronize(B->t1));
  float t = 0;
  BK(cudaEventElapsedTime(&t, B->t0, B->t1));
  *ms = t;
  return SQDEM_OK;
}

// End to end through host buffers: every step copies the kinematics of all scenes' bodies
// (16 doubles per body in scene order, the sqdem_get_kinematics layout) to the device,
// steps all scenes, and copies them back; in16 and out16 alternate as in sqdem_time_e2e.
sqdem_status sqdem_batch_time_e2e(sqdem_batch* B, int nsteps, const double* in16, double* out16, double* ms) {
  if (!B || !ms || !in16 || !out16 || nsteps < 0) return SQDEM_ERR_ARG;
  BK(cudaSetDevice(B->device));
  for (sqdem_ctx* c : B->scenes) BK(cudaStreamSynchronize(c->stream));
  sqdem_status s = batchReady(B);
  if (s) return s;
  const int ns = (int)B->scenes.size();
  long long rows = 0;
  std::vector<BatchPtrs> hp(ns);
  for (int i = 0; i < ns; i++) {
    const Dev& d = B->scenes[i]->d;
    hp[i] = BatchPtrs{d.pos, d.ori, d.vel, d.angVel, d.angMom, rows, d.N};
    rows += d.N;
  }
  if (!B->dPtrs) BK(cudaMalloc(&B->dPtrs, sizeof(BatchPtrs) * ns));
  if (B->rows != rows) {
    if (B->dKin) BK(cudaFree(B->dKin));
    BK(cudaMalloc(&B->dKin, sizeof(double) * 16 * (size_t)rows));
    B->rows = rows;
  }
  BK(cudaMemcpyAsync(B->dPtrs, hp.data(), sizeof(BatchPtrs) * ns, cudaMemcpyHostToDevice, B->stream));
  const int grid = std::max(1, std::min(nblk(rows, 256), 4096));
  const size_t bytes = sizeof(double) * 16 * (size_t)rows;
  double* bufs[2] = {const_cast<double*>(in16), out16};
  BK(cudaEventRecord(B->t0, B->stream));
  for (int i = 0; i < nsteps; i++) {
    BK(cudaMemcpyAsync(B->dKin, bufs[i & 1], bytes, cudaMemcpyHostToDevice, B->stream));
    k_batch_kin<<<grid, 256, 0, B->stream>>>(B->dPtrs, ns, B->dKin, rows, 1);
    BK(cudaGraphLaunch(B->exec, B->stream));
    k_batch_kin<<<grid, 256, 0, B->stream>>>(B->dPtrs, ns, B->dKin, rows, 0);
    BK(cudaMemcpyAsync(bufs[(i + 1) & 1], B->dKin, bytes, cudaMemcpyDeviceToHost, B->stream));
  }
  BK(cudaEventRecord(B->t1, B->stream));
  BK(cudaEventSynchronize(B->t1));
  float t = 0;
  BK(cudaEventElapsedTime(&t, B->t0, B->t1));
  *ms = t;
  return SQDEM_OK;
}

long long sqdem_batch_launch_count(sqdem_batch* B) { return B ? B->launchesPerStep : 0; }
}  // extern "C"
