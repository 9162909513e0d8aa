// Double-float ("ff") arithmetic on the FP32 pipes, and the Disfunction evaluation of the
// mixed-precision narrowphase written with it.
//
// GB300 issues FP64 at 1/64 of its FP32 rate, and a Disfunction evaluation
// (pkg/dem/Superquadrics_Ig2.cpp:622-687) costs ~18 pow + 4 atan2 + 6 sincos in FP64.  The
// mixed form evaluates it instead in double-float arithmetic: a value is the unevaluated sum
// hi + lo of two floats (~48 significant bits), built from the error-free transformations of
// Knuth (two-sum), Dekker (fast two-sum) and the FMA two-product.  Its own elementary
// functions (below; no CUDA math routine is used):
//   * log2: x = 2^e m, m near c = 1 + j/32 (table of log2 c), log2 m = log2 c +
//     2 atanh((m - c)/(m + c)) / ln 2, the series to the 7th power;
//   * exp2: x = n + j/32 + g with |g| <= 1/64 (table of 2^(j/32)), e^(g ln 2) by its Taylor
//     polynomial to the 6th power;
//   * sincos of a double angle: Cody-Waite reduction by pi/2 in four parts, then j/32 + d with
//     |d| <= 1/64 (table of sin, cos j/32) and the Taylor polynomials of sin d, cos d.
// Table values are the exact values rounded to hi = nearest float, lo = nearest float to the
// remainder (computed to 40 digits).  Every routine is __host__ __device__ and uses only IEEE
// float +, -, *, /, fmaf and exact bit operations, so a host build with -ffp-contract=off
// gives the device's results bit for bit (the CPU tests rely on that).
//
// The support point is computed without the surface angles: for phi0 = atan2(Y, X),
// |cos phi0| = X / hypot(X, Y) and |sin phi0| = Y / hypot(X, Y), so every power pow(q, e) of
// Normal2Phi + getSurface becomes exp2 of a sum of logarithms of ratios, which keeps the
// arguments of exp2 small where the result is not.  The reference's FP64 code rounds the angles
// to doubles before taking their cosines, which leaves an absolute error of ~1e-16 in a cosine
// next to an odd multiple of pi/2 (and a sine next to pi); there the small value the FP64 code
// obtains is reproduced from the rounding it applies (fp64RoundedOffset).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include "sq_device.cuh"

#ifdef __CUDACC__
#define FFH __host__ __device__ __forceinline__
// the elementary functions (and the double-float division and square root) are called, not
// inlined: one evaluation calls them ~40 times, and inlined copies overflow the instruction
// cache (warps then stall on instruction fetch); calling the additions and products too was
// measured slower at 12,800 particles (the calls' own instructions)
#define FFN static __host__ __device__ __noinline__
#else
#define FFH inline
#define FFN static inline
#endif

#ifdef __CUDA_ARCH__
#define FF_TABLE(name, n) static __device__ const float name##_t[n] = name##_V;
#else
#define FF_TABLE(name, n) static const float name##_t[n] = name##_V;
#endif
#define FFT(name, i) (name##_t[i])

namespace sqdem {

#define FF_EXP2_HI_V \
  { \
  0.7071067690849304f, 0.7225903868675232f, 0.7384130954742432f, 0.7545822262763977f, 0.7711054086685181f, \
  0.7879904508590698f, 0.8052451610565186f, 0.8228777647018433f, 0.8408964276313782f, 0.8593096733093262f, \
  0.8781260848045349f, 0.8973545432090759f, 0.9170040488243103f, 0.9370838403701782f, 0.9576032757759094f, \
  0.9785720705986023f, 1.0f, 1.0218971967697144f, 1.0442737340927124f, 1.0671404600143433f, \
  1.0905077457427979f, 1.114386796951294f, 1.1387885808944702f, 1.1637248992919922f, 1.1892070770263672f, \
  1.215247392654419f, 1.2418577671051025f, 1.2690509557724f, 1.2968395948410034f, 1.3252366781234741f, \
  1.3542555570602417f, 1.3839099407196045f, 1.4142135381698608f \
  }
FF_TABLE(FF_EXP2_HI, 33)
#define FF_EXP2_LO_V \
  { \
  1.2101617485882343e-08f, 1.662099968768871e-08f, -2.250449426810519e-08f, -1.2479686617439256e-08f, \
  4.035452416673024e-09f, -2.830512713103417e-08f, 4.918108587048664e-09f, -2.5624860455764065e-08f, \
  -1.2377663338725142e-08f, -2.4248087981959543e-08f, -4.617885185353998e-09f, -5.707522454656555e-09f, \
  -5.619638976384067e-09f, -2.331502813035513e-08f, 4.922664054163306e-09f, -8.510902205216553e-09f, 0.0f, \
  -4.811559861650494e-08f, 4.8334701574503924e-08f, -5.9337519786595294e-08f, -1.3077539939843064e-08f, \
  -5.435540018083884e-08f, 5.386222312608879e-08f, -4.051441493402308e-08f, 3.797635272917432e-08f, \
  -3.267394887984665e-08f, 4.496838101886169e-08f, 1.419333317542737e-09f, -4.018999533172973e-08f, \
  -3.496373324196611e-08f, -1.0123349269974824e-08f, -5.875577357983275e-08f, 2.4203234971764687e-08f \
  }
FF_TABLE(FF_EXP2_LO, 33)
#define FF_LOG2C_HI_V \
  { \
  -0.678071916103363f, -0.6076825857162476f, -0.5405683517456055f, -0.476438045501709f, \
  -0.41503751277923584f, -0.3561438024044037f, -0.2995602786540985f, -0.24511249363422394f, \
  -0.19264507293701172f, -0.14201900362968445f, -0.09310940653085709f, -0.04580368846654892f, 0.0f, \
  0.0443941205739975f, 0.08746284246444702f, 0.12928301095962524f, 0.1699250042438507f, 0.20945335924625397f, \
  0.24792751669883728f, 0.28540220856666565f, 0.32192808389663696f, 0.3575519919395447f, \
  0.39231741428375244f, 0.42626476287841797f, 0.45943161845207214f, 0.49185308814048767f, 0.523561954498291f, \
  0.5545888543128967f, 0.5849624872207642f \
  }
FF_TABLE(FF_LOG2C_HI, 29)
#define FF_LOG2C_LO_V \
  { \
  1.0990725662907153e-08f, 8.495008252396019e-09f, -2.961709810733737e-08f, 1.5587218182844254e-09f, \
  1.3500391915499677e-08f, -7.820871950059427e-09f, -3.2048093068226535e-09f, -4.202307390954729e-09f, \
  -5.005384107192867e-09f, -1.2427434636919088e-09f, 2.13937556559074e-09f, -1.1465758342765753e-09f, 0.0f, \
  -1.215544109811617e-09f, -1.2141075922400546e-09f, 5.9853411116250754e-09f, -2.8015383346513545e-09f, \
  6.382695705298147e-09f, -3.2552518458572877e-09f, 1.0295583052766233e-08f, 1.0990725662907153e-08f, \
  1.2678539107469078e-08f, 8.495008252396019e-09f, -8.176320065444997e-09f, 1.8522511302521139e-10f, \
  8.189187106211193e-09f, 1.5587218182844254e-09f, -2.635259344074825e-09f, 1.3500391915499677e-08f \
  }
FF_TABLE(FF_LOG2C_LO, 29)
#define FF_SIN_HI_V \
  { \
  -0.7260086536407471f, -0.7041674852371216f, -0.681638777256012f, -0.6584444046020508f, \
  -0.6346070766448975f, -0.6101500988006592f, -0.5850972533226013f, -0.5594731569290161f, \
  -0.5333026647567749f, -0.5066114664077759f, -0.4794255495071411f, -0.45177146792411804f, \
  -0.4236762523651123f, -0.3951673209667206f, -0.36627253890037537f, -0.33702006936073303f, \
  -0.30743852257728577f, -0.27755674719810486f, -0.24740396440029144f, -0.21700957417488098f, \
  -0.186403289437294f, -0.15561498701572418f, -0.1246747300028801f, -0.09361273050308228f, \
  -0.0624593161046505f, -0.03124491311609745f, 0.0f, 0.03124491311609745f, 0.0624593161046505f, \
  0.09361273050308228f, 0.1246747300028801f, 0.15561498701572418f, 0.186403289437294f, 0.21700957417488098f, \
  0.24740396440029144f, 0.27755674719810486f, 0.30743852257728577f, 0.33702006936073303f, \
  0.36627253890037537f, 0.3951673209667206f, 0.4236762523651123f, 0.45177146792411804f, 0.4794255495071411f, \
  0.5066114664077759f, 0.5333026647567749f, 0.5594731569290161f, 0.5850972533226013f, 0.6101500988006592f, \
  0.6346070766448975f, 0.6584444046020508f, 0.681638777256012f, 0.7041674852371216f, 0.7260086536407471f \
  }
FF_TABLE(FF_SIN_HI, 53)
#define FF_SIN_LO_V \
  { \
  -1.6199654950810327e-09f, -2.6217412241180682e-08f, 1.723267750719515e-08f, 4.691483201924029e-09f, \
  -3.37037175945909e-09f, 2.1724867238503975e-08f, -1.9617861113374602e-08f, 2.568164880756285e-08f, \
  -8.779244886625293e-09f, 1.1593518145502912e-08f, 1.0902938107903992e-08f, -3.5675657983347264e-09f, \
  -4.838825784503342e-09f, -9.274213397247877e-09f, 9.814328016943819e-09f, 3.384799662775606e-10f, \
  7.996904471951893e-09f, -4.448231560871818e-09f, 5.145768700032249e-09f, -6.920129358434224e-09f, \
  -7.324975737077466e-09f, -5.757831988972839e-09f, -3.3823475131811165e-09f, -7.324306161571315e-10f, \
  -1.737729737882887e-09f, -8.69228633515462e-10f, 0.0f, 8.69228633515462e-10f, 1.737729737882887e-09f, \
  7.324306161571315e-10f, 3.3823475131811165e-09f, 5.757831988972839e-09f, 7.324975737077466e-09f, \
  6.920129358434224e-09f, -5.145768700032249e-09f, 4.448231560871818e-09f, -7.996904471951893e-09f, \
  -3.384799662775606e-10f, -9.814328016943819e-09f, 9.274213397247877e-09f, 4.838825784503342e-09f, \
  3.5675657983347264e-09f, -1.0902938107903992e-08f, -1.1593518145502912e-08f, 8.779244886625293e-09f, \
  -2.568164880756285e-08f, 1.9617861113374602e-08f, -2.1724867238503975e-08f, 3.37037175945909e-09f, \
  -4.691483201924029e-09f, -1.723267750719515e-08f, 2.6217412241180682e-08f, 1.6199654950810327e-09f \
  }
FF_TABLE(FF_SIN_LO, 53)
#define FF_COS_HI_V \
  { \
  0.6876855492591858f, 0.7100338935852051f, 0.7316888570785522f, 0.7526293992996216f, 0.7728349566459656f, \
  0.7922858595848083f, 0.8109630942344666f, 0.8288484811782837f, 0.8459244966506958f, 0.8621744513511658f, \
  0.8775825500488281f, 0.8921337127685547f, 0.9058136940002441f, 0.9186091423034668f, 0.9305076003074646f, \
  0.9414974451065063f, 0.9515679478645325f, 0.9607092142105103f, 0.9689124226570129f, 0.9761694669723511f, \
  0.9824733138084412f, 0.9878177642822266f, 0.9921976923942566f, 0.9956086874008179f, 0.9980475306510925f, \
  0.9995117783546448f, 1.0f, 0.9995117783546448f, 0.9980475306510925f, 0.9956086874008179f, \
  0.9921976923942566f, 0.9878177642822266f, 0.9824733138084412f, 0.9761694669723511f, 0.9689124226570129f, \
  0.9607092142105103f, 0.9515679478645325f, 0.9414974451065063f, 0.9305076003074646f, 0.9186091423034668f, \
  0.9058136940002441f, 0.8921337127685547f, 0.8775825500488281f, 0.8621744513511658f, 0.8459244966506958f, \
  0.8288484811782837f, 0.8109630942344666f, 0.7922858595848083f, 0.7728349566459656f, 0.7526293992996216f, \
  0.7316888570785522f, 0.7100338935852051f, 0.6876855492591858f \
  }
FF_TABLE(FF_COS_HI, 53)
#define FF_COS_LO_V \
  { \
  1.2961319129090043e-08f, -1.0019125085136693e-08f, 1.1795268761716216e-08f, -2.6881554759938808e-08f, \
  -1.0493494073671172e-08f, 9.237019482633002e-11f, 2.5270750825256982e-08f, 6.431041921217684e-09f, \
  2.5803721381834066e-09f, 2.858371495051415e-08f, 1.1841544633739431e-08f, -1.3401559861847545e-08f, \
  -1.0574307651722847e-08f, 1.3491451511526975e-08f, 2.1604849465006737e-08f, 1.8021374614818342e-08f, \
  1.8363972842383447e-10f, 2.880505078906026e-08f, -9.463682060228962e-10f, 6.896283988311325e-09f, \
  -7.071859209339948e-10f, 1.9534246220587193e-08f, -2.516492791926339e-08f, -9.428161584779104e-10f, \
  -1.9950993745965206e-08f, -1.9869508705028238e-08f, 0.0f, -1.9869508705028238e-08f, \
  -1.9950993745965206e-08f, -9.428161584779104e-10f, -2.516492791926339e-08f, 1.9534246220587193e-08f, \
  -7.071859209339948e-10f, 6.896283988311325e-09f, -9.463682060228962e-10f, 2.880505078906026e-08f, \
  1.8363972842383447e-10f, 1.8021374614818342e-08f, 2.1604849465006737e-08f, 1.3491451511526975e-08f, \
  -1.0574307651722847e-08f, -1.3401559861847545e-08f, 1.1841544633739431e-08f, 2.858371495051415e-08f, \
  2.5803721381834066e-09f, 6.431041921217684e-09f, 2.5270750825256982e-08f, 9.237019482633002e-11f, \
  -1.0493494073671172e-08f, -2.6881554759938808e-08f, 1.1795268761716216e-08f, -1.0019125085136693e-08f, \
  1.2961319129090043e-08f \
  }
FF_TABLE(FF_COS_LO, 53)
#define FF_LN2_HI 0.6931471824645996f
#define FF_LN2_LO -1.9046542121259336e-09f
#define FF_INV_LN2_HI 1.4426950216293335f
#define FF_INV_LN2_LO 1.925963033500011e-08f
#define FF_TWO_THIRDS_HI 0.6666666865348816f
#define FF_TWO_THIRDS_LO -1.9868215517249155e-08f
#define FF_SIXTH_HI 0.1666666716337204f
#define FF_SIXTH_LO -4.967053879312289e-09f
#define FF_PIO2_1 1.5703125f
#define FF_PIO2_2 0.0004837512969970703f
#define FF_PIO2_3 7.549790126404332e-08f
#define FF_PIO2_4 -1.7151245100058819e-15f

struct ff { float hi, lo; };

FFH ff mkff(float h, float l) { ff r; r.hi = h; r.lo = l; return r; }
FFH ff ffFromD(double d) { const float h = (float)d; return mkff(h, (float)(d - (double)h)); }
FFH double ffToD(ff a) { return (double)a.hi + (double)a.lo; }
FFH int ffBits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_int(x);
#else
  int i; memcpy(&i, &x, 4); return i;
#endif
}
FFH float ffFloat(int i) {
#ifdef __CUDA_ARCH__
  return __int_as_float(i);
#else
  float x; memcpy(&x, &i, 4); return x;
#endif
}
FFH float pow2i(int n) { return ffFloat((n + 127) << 23); }   // 2^n, -126 <= n <= 127

// Error-free transformations.
FFH ff twoSum(float a, float b) {
  const float s = a + b, bb = s - a;
  return mkff(s, (a - (s - bb)) + (b - bb));
}
FFH ff fastTwoSum(float a, float b) {   // |a| >= |b| or a == 0
  const float s = a + b;
  return mkff(s, b - (s - a));
}
FFH ff twoProd(float a, float b) {
  const float p = a * b;
  return mkff(p, fmaf(a, b, -p));
}

FFH ff ffNeg(ff a) { return mkff(-a.hi, -a.lo); }
FFH ff ffAbs(ff a) { return a.hi < 0.f ? ffNeg(a) : a; }
FFH bool ffGt(ff a, ff b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
FFH ff ffAdd(ff a, ff b) {   // accurate sum (both parts two-summed)
  ff s = twoSum(a.hi, b.hi);
  const ff t = twoSum(a.lo, b.lo);
  s = fastTwoSum(s.hi, s.lo + t.hi);
  return fastTwoSum(s.hi, s.lo + t.lo);
}
FFH ff ffSub(ff a, ff b) { return ffAdd(a, ffNeg(b)); }
FFH ff ffAddF(ff a, float b) {
  const ff s = twoSum(a.hi, b);
  return fastTwoSum(s.hi, s.lo + a.lo);
}
FFH ff ffMul(ff a, ff b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fastTwoSum(p, e);
}
FFH ff ffMulF(ff a, float b) {
  const float p = a.hi * b;
  return fastTwoSum(p, fmaf(a.lo, b, fmaf(a.hi, b, -p)));
}
// a / b: a first quotient from the float reciprocal, then two corrections from the exact
// remainders.
FFN ff ffDiv(ff a, ff b) {
  const float inv = 1.0f / b.hi;
  const float q1 = a.hi * inv;
  ff r = ffSub(a, ffMulF(b, q1));
  const float q2 = r.hi * inv;
  r = ffSub(r, ffMulF(b, q2));
  const float q3 = r.hi * inv;
  return ffAddF(fastTwoSum(q1, q2), q3);
}

// sqrt(a) for a >= 0: the float root and one correction from the exact remainder.
FFN ff ffSqrt(ff a) {
  if (!(a.hi > 0.f)) return mkff(a.hi == 0.f ? 0.f : NAN, 0.f);
  const float s = sqrtf(a.hi);
  const ff r = ffSub(a, twoProd(s, s));
  return fastTwoSum(s, r.hi / (2.f * s));
}

// log2 of a positive double-float whose high part is a normal float.
FFN ff ffLog2(ff x) {
  int e = ((ffBits(x.hi) >> 23) & 0xff) - 127;   // x.hi in [2^e, 2^(e+1))
  const float sc = pow2i(-e);
  ff m = mkff(x.hi * sc, x.lo * sc);            // m.hi in [1, 2), exact scaling
  if (m.hi > 1.41421356f) { m.hi *= 0.5f; m.lo *= 0.5f; e += 1; }
  const float jf = rintf((m.hi - 1.f) * 32.f);   // -9..13
  const float c = 1.f + jf * 0.03125f;
  const ff t = ffDiv(ffAddF(m, -c), ffAddF(m, c));   // m.hi - c is exact; |t| <= 0.0112
  const ff t2 = ffMul(t, t);
  const float t2f = t2.hi;
  // ln(m / c) = 2 atanh(t) = t (2 + t^2 (2/3 + t^2 (2/5 + t^2 2/7)))
  ff p = ffAddF(mkff(FF_TWO_THIRDS_HI, FF_TWO_THIRDS_LO), t2f * (0.4f + t2f * 0.285714298f));
  p = ffMul(ffAddF(ffMul(p, t2), 2.f), t);
  p = ffMul(p, mkff(FF_INV_LN2_HI, FF_INV_LN2_LO));
  const int j = (int)jf + 12;
  p = ffAdd(p, mkff(FFT(FF_LOG2C_HI, j), FFT(FF_LOG2C_LO, j)));
  return ffAddF(p, (float)e);
}

// 2^x for a double-float x.  Results below 2^-126 keep only their high part (and become 0
// below 2^-149): the callers use such values only as negligible terms.
FFN ff ffExp2(ff x) {
  if (x.hi < -149.f) return mkff(0.f, 0.f);
  if (x.hi > 127.f) return mkff(INFINITY, 0.f);
  const float n = rintf(x.hi);
  const ff f = twoSum(x.hi - n, x.lo);            // x.hi - n exact; |f| <= 1/2
  const float jf = rintf(f.hi * 32.f);            // -16..16
  const ff g = twoSum(f.hi - jf * 0.03125f, f.lo);   // exact difference; |g| <= 1/64
  const ff t = ffMul(g, mkff(FF_LN2_HI, FF_LN2_LO));
  const float tf = t.hi;
  // e^t = 1 + t (1 + t (1/2 + t (1/6 + t/24 + t^2/120 + t^3/720)))
  ff p = ffAddF(mkff(FF_SIXTH_HI, FF_SIXTH_LO), tf * (0.0416666679f + tf * (0.00833333377f + tf * 0.00138888892f)));
  p = ffAddF(ffMul(p, t), 0.5f);
  p = ffAddF(ffMul(p, t), 1.f);
  p = ffAddF(ffMul(p, t), 1.f);
  const int j = (int)jf + 16;
  p = ffMul(p, mkff(FFT(FF_EXP2_HI, j), FFT(FF_EXP2_LO, j)));
  const int ni = (int)n;
  if (ni >= -126) { const float s = pow2i(ni); return mkff(p.hi * s, p.lo * s); }
  const float s1 = pow2i(-126), s2 = pow2i(ni + 126 < -126 ? -126 : ni + 126);
  return mkff(p.hi * s1 * s2, 0.f);
}

// sin and cos of a double-float angle |x| < 6000; ok = false (NaN, larger angles) otherwise.
struct FFSinCos { ff s, c; bool ok; };
FFN FFSinCos ffSinCosV(ff x) {
  FFSinCos out;
  ff& s = out.s;
  ff& c = out.c;
  out.ok = true;
  if (!(fabsf(x.hi) < 6000.f)) { s = c = mkff(NAN, 0.f); out.ok = false; return out; }
  const float k = rintf(x.hi * 0.636619772f);
  // r = x - k pi/2 (k P1 and k P2 exact: 12 trailing zero bits; x.hi - k P1 exact)
  ff r = twoSum(x.hi - k * FF_PIO2_1, -k * FF_PIO2_2);
  r = ffAdd(r, mkff(x.lo, 0.f));
  r = ffSub(r, twoProd(k, FF_PIO2_3));
  r = ffAddF(r, -k * FF_PIO2_4);
  const float jf = rintf(r.hi * 32.f);            // -26..26
  const ff d = twoSum(r.hi - jf * 0.03125f, r.lo);   // |d| <= 1/64
  const ff d2 = ffMul(d, d);
  const float d2f = d2.hi;
  // sin d = d (1 - d^2 (1/6 - d^2/120 + d^4/5040)), cos d = 1 - d^2 (1/2 - d^2/24 + d^4/720)
  ff sd = ffAddF(mkff(FF_SIXTH_HI, FF_SIXTH_LO), -d2f * (0.00833333377f - d2f * 0.000198412701f));
  sd = ffMul(ffAddF(ffNeg(ffMul(sd, d2)), 1.f), d);
  ff cd = twoSum(0.5f, -d2f * (0.0416666679f - d2f * 0.00138888892f));
  cd = ffAddF(ffNeg(ffMul(cd, d2)), 1.f);
  const int j = (int)jf + 26;
  const ff Sj = mkff(FFT(FF_SIN_HI, j), FFT(FF_SIN_LO, j)), Cj = mkff(FFT(FF_COS_HI, j), FFT(FF_COS_LO, j));
  const ff sv = ffAdd(ffMul(Sj, cd), ffMul(Cj, sd));
  const ff cv = ffSub(ffMul(Cj, cd), ffMul(Sj, sd));
  switch (((int)k) & 3) {
    case 0: s = sv; c = cv; break;
    case 1: s = cv; c = ffNeg(sv); break;
    case 2: s = ffNeg(sv); c = ffNeg(cv); break;
    default: s = ffNeg(cv); c = sv; break;
  }
  return out;
}
FFH bool ffSinCos(ff x, ff& s, ff& c) {
  const FFSinCos r = ffSinCosV(x);
  s = r.s;
  c = r.c;
  return r.ok;
}
FFH bool ffSinCos(double a, ff& s, ff& c) { return ffSinCos(ffFromD(a), s, c); }

// ---------------------------------------------------------------------------
// Disfunction in double-float, in the frame of body A translated to A's centre.
struct FFShape {
  ff rx, ry, rz;
  ff e1, e2, a1, i1, i2;   // eps1, eps2, 2 - eps1, 1/(2 - eps1), 1/(2 - eps2): the FP64 values
  ff R[9];                 // rotation matrix (local -> global), row-major
  float rmax, pad;         // bounding radius (float) and padding to 9 float4
};
struct FFPair { FFShape A, B; ff pB[3]; };   // pB: centre of B (with its periodic shift) - centre of A

FFH void ffShapeInit(FFShape& f, const SqShape& s) {
  f.rx = ffFromD(s.rx); f.ry = ffFromD(s.ry); f.rz = ffFromD(s.rz);
  f.e1 = ffFromD(s.e1); f.e2 = ffFromD(s.e2); f.a1 = ffFromD(s.a1); f.i1 = ffFromD(s.i1); f.i2 = ffFromD(s.i2);
  for (int k = 0; k < 9; k++) f.R[k] = ffFromD(s.R.m[k]);
  f.rmax = (float)s.rmax; f.pad = 0.f;
}
FFH void ffPairInit(FFPair& P, const SqShape& A, const SqShape& B) {
  ffShapeInit(P.A, A);
  ffShapeInit(P.B, B);
  P.pB[0] = ffFromD(B.pos.x - A.pos.x);
  P.pB[1] = ffFromD(B.pos.y - A.pos.y);
  P.pB[2] = ffFromD(B.pos.z - A.pos.z);
}
FFH ff ffDot3(ff a0, ff a1, ff a2, ff b0, ff b1, ff b2) {
  return ffAdd(ffMul(a0, b0), ffAdd(ffMul(a1, b1), ffMul(a2, b2)));
}

// The reference takes the cosine (sine) of an angle next to an odd multiple of pi/2 (next to
// pi) after atan2 has rounded the angle to a double, so the small value it obtains is the sine
// of the rounded distance to that multiple: with delta the exact distance (signed towards the
// multiple's double, fl(pi/2) = pi/2 - T, spacing u = 2^-52 there; fl(pi) = pi - 2T,
// u = 2^-51), the rounded angle is fl(pi/2) + rint(v) u with v = (T - delta) / u, and the
// small value is sin(y), y = delta + (v - rint(v)) u.  This routine returns y for
// T / u = 0.275765943415... (the same for pi/2 with 2^-52 and pi with 2^-51), assuming a
// correctly rounded atan2.  delta <= 2^-10 here, where v has at least 4 fractional bits in
// double-float; an error of rint(v) by one changes the value by 2^-52 relative to delta.
FFH ff fp64RoundedOffset(ff delta, float invU, float u) {
  const ff v = ffSub(mkff(0.275765955f, -1.20331265e-08f), ffMulF(delta, invU));
  const float a = rintf(v.hi);
  const float b = rintf((v.hi - a) + v.lo);
  const float frac = ((v.hi - a) - b) + v.lo;
  return ffAddF(delta, frac * u);
}
// sin(y) for |y| <= 2^-9
FFH ff ffSinSmall(ff y) {
  const ff y2 = ffMul(y, y);
  const float y2f = y2.hi;
  return ffMul(y, ffAddF(ffNeg(ffMul(y2, mkff(FF_SIXTH_HI - y2f * 0.00833333377f, FF_SIXTH_LO))), 1.f));
}
// atan(r) for 0 < r <= 2^-10
FFH ff ffAtanSmall(ff r) {
  const ff r2 = ffMul(r, r);
  const float r2f = r2.hi;
  return ffMul(r, ffAddF(ffNeg(ffMulF(r2, 0.333333343f - r2f * 0.2f)), 1.f));
}

// Superquadrics::Normal2Phi followed by getSurface (pkg/dem/Superquadrics.cpp:269-307,110-120)
// without the surface angles: the local surface point of s whose outward normal is parallel to
// the local direction n.  Where an angle falls within 2^-10 of a multiple of pi/2 at which the
// reference's cosine or sine is small, that small value is the one the reference's FP64 rounding
// gives (fp64RoundedOffset).  ill: a normal component below 1e-30 (exactly axis-aligned
// directions, where the reference's sgn(0) = 0 conventions apply) or a non-finite value.
FFH void ffSupportBody(const FFShape& s, ff nx, ff ny, ff nz, ff q[3], bool& ill) {
  ff ax = ffMul(s.rx, nx), ay = ffMul(s.ry, ny), az = ffMul(s.rz, nz);
  const float sx = ax.hi < 0.f ? -1.f : 1.f, sy = ay.hi < 0.f ? -1.f : 1.f, sz = az.hi < 0.f ? -1.f : 1.f;
  ax = ffAbs(ax); ay = ffAbs(ay); az = ffAbs(az);
  if (!(ax.hi > 1e-30f && ay.hi > 1e-30f && az.hi > 1e-30f)) {
    ill = true;
    q[0] = q[1] = q[2] = mkff(0.f, 0.f);
    return;
  }
  const float SMALL = -10.f;   // log2 of the ratio below which the FP64 rounding is emulated
  // phi0 = atan2(sy Y, sx X), X = ax^i1, Y = ay^i1; rho = min/max of X, Y
  const bool yGtX = ffGt(ay, ax);
  const ff d0 = ffMul(s.i1, ffLog2(yGtX ? ffDiv(ax, ay) : ffDiv(ay, ax)));   // log2 rho <= 0
  const ff rho = ffExp2(d0);
  const ff L = ffMulF(ffLog2(ffAddF(ffMul(rho, rho), 1.f)), 0.5f);         // log2 hypot(1, rho)
  ff lc = ffNeg(L), ls = ffNeg(L);          // log2 |cos phi0|, log2 |sin phi0|
  float sc0 = sx, ss0 = sy;                 // their signs
  if (yGtX) {                               // phi0 next to +-pi/2: cos is the small one
    if (d0.hi < SMALL) {
      const ff y = fp64RoundedOffset(ffMulF(ffAtanSmall(rho), sx), 4503599627370496.f, 2.22044605e-16f);
      lc = ffLog2(ffAbs(ffSinSmall(y)));
      sc0 = y.hi < 0.f ? -1.f : 1.f;
      if (y.hi == 0.f) ill = true;
    } else lc = ffSub(d0, L);
  } else if (sx < 0.f && d0.hi < SMALL) {  // phi0 next to +-pi: sin is the small one
    const ff y = fp64RoundedOffset(ffAtanSmall(rho), 2251799813685248.f, 4.44089210e-16f);
    ls = ffLog2(ffAbs(ffSinSmall(y)));
    ss0 = y.hi < 0.f ? -sy : sy;
    if (y.hi == 0.f) ill = true;
  } else ls = ffSub(d0, L);
  // phi1 = atan2(sz Z, W), Z = (az |cos phi0|^a1)^i2, W = ax^i2
  const ff d1 = ffMul(s.i2, ffAdd(ffLog2(ffDiv(az, ax)), ffMul(s.a1, lc)));  // log2 (Z / W)
  const bool zGtW = d1.hi > 0.f;
  const ff nd1 = zGtW ? ffNeg(d1) : d1;
  const ff rho1 = ffExp2(nd1);
  const ff L1 = ffMulF(ffLog2(ffAddF(ffMul(rho1, rho1), 1.f)), 0.5f);
  ff lc1 = ffNeg(L1), ls1 = ffNeg(L1);
  if (zGtW) {                               // phi1 next to +-pi/2: cos is the small one
    if (nd1.hi < SMALL) {
      const ff y = fp64RoundedOffset(ffAtanSmall(rho1), 4503599627370496.f, 2.22044605e-16f);
      lc1 = ffLog2(ffAbs(ffSinSmall(y)));
      if (y.hi == 0.f) ill = true;
    } else lc1 = ffSub(nd1, L1);
  } else ls1 = ffSub(nd1, L1);
  // getSurface: (rx |c0|^e1 |c1|^e2, ry |s0|^e1 |c1|^e2, rz |s1|^e2) with the signs of cos/sin
  const ff ec1 = ffMul(s.e2, lc1);
  q[0] = ffMulF(ffMul(s.rx, ffExp2(ffAdd(ffMul(s.e1, lc), ec1))), sc0);
  q[1] = ffMulF(ffMul(s.ry, ffExp2(ffAdd(ffMul(s.e1, ls), ec1))), ss0);
  q[2] = ffMulF(ffMul(s.rz, ffExp2(ffMul(s.e2, ls1))), sz);
}

struct FFSup { ff q0, q1, q2; bool ill; };
FFN FFSup ffSupportV(const FFShape& s, ff nx, ff ny, ff nz) {
  FFSup out;
  out.ill = false;
  ff q[3];
  bool& ill = out.ill;
  ffSupportBody(s, nx, ny, nz, q, ill);
  out.q0 = q[0]; out.q1 = q[1]; out.q2 = q[2];
  return out;
}
FFH void ffSupport(const FFShape& s, ff nx, ff ny, ff nz, ff q[3], bool& ill) {
  const FFSup r = ffSupportV(s, nx, ny, nz);
  q[0] = r.q0; q[1] = r.q1; q[2] = r.q2;
  if (r.ill) ill = true;
}

// One evaluation: support points of A along c(pa) and of B along -c(pa), relative to A's
// centre; d = p2 - p1, sep = c . d (the reference's stop_flag is sep > 0).
struct FFEval {
  ff c[3], p1[3], p2[3], d[3], sep;
  bool ill;
};
FFH void ffDisfunction(const FFShape& A, const FFShape& B, const ff pB[3], ff pa0, ff pa1, FFEval& r) {
  ff s0, c0, s1, c1;
  const bool ok0 = ffSinCos(pa0, s0, c0), ok1 = ffSinCos(pa1, s1, c1);
  r.ill = !(ok0 && ok1);
  r.c[0] = ffMul(c0, c1); r.c[1] = ffMul(s0, c1); r.c[2] = s1;
  ff q[3];
  // A: local normal R_A^T c
  ffSupport(A, ffDot3(A.R[0], A.R[3], A.R[6], r.c[0], r.c[1], r.c[2]),
            ffDot3(A.R[1], A.R[4], A.R[7], r.c[0], r.c[1], r.c[2]),
            ffDot3(A.R[2], A.R[5], A.R[8], r.c[0], r.c[1], r.c[2]), q, r.ill);
  for (int i = 0; i < 3; i++) r.p1[i] = ffDot3(A.R[3 * i], A.R[3 * i + 1], A.R[3 * i + 2], q[0], q[1], q[2]);
  // B: local normal -R_B^T c
  ffSupport(B, ffNeg(ffDot3(B.R[0], B.R[3], B.R[6], r.c[0], r.c[1], r.c[2])),
            ffNeg(ffDot3(B.R[1], B.R[4], B.R[7], r.c[0], r.c[1], r.c[2])),
            ffNeg(ffDot3(B.R[2], B.R[5], B.R[8], r.c[0], r.c[1], r.c[2])), q, r.ill);
  for (int i = 0; i < 3; i++)
    r.p2[i] = ffAdd(ffDot3(B.R[3 * i], B.R[3 * i + 1], B.R[3 * i + 2], q[0], q[1], q[2]), pB[i]);
  for (int i = 0; i < 3; i++) r.d[i] = ffSub(r.p2[i], r.p1[i]);
  r.sep = ffDot3(r.c[0], r.c[1], r.c[2], r.d[0], r.d[1], r.d[2]);
  if (!(fabsf(r.sep.hi) < INFINITY)) r.ill = true;   // non-finite: the FP64 path decides
}
FFH void ffDisfunction(const FFPair& P, double pa0, double pa1, FFEval& r) {
  ffDisfunction(P.A, P.B, P.pB, ffFromD(pa0), ffFromD(pa1), r);
}

}  // namespace sqdem
