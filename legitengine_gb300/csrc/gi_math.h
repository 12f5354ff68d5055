// gi_math.h -- float transcendental functions with a fixed evaluation order.
//
// The reference's shaders (bin/data/Shaders/glsl/SSVGI/indirectLighting.frag,
// Common/directLighting.frag) call GLSL atan/log/pow/sin/cos/exp, whose rounding
// is whatever the Vulkan driver's compiler emits: nothing pins it.  This header
// fixes one evaluation: every function below is a short sequence of IEEE-754
// single-precision adds, multiplies, divisions, square roots and explicit fmaf,
// so that the host compiler (built with -ffp-contract=off) and nvcc (built with
// --fmad=false, no fast-math) produce the same bits for the same input.  The
// CUDA kernels and the CPU restatement both use it; the tests bound its error
// against libm in double precision.
//
// Methods (all from the public literature, coefficients are Taylor/atanh series
// terms 1/k! and 1/(2k+1)):
// Division inside these functions, as in all library code, is a * rcp(b)
// (div_ below).
//   log:  x = m * 2^e, m in (sqrt(1/2), sqrt(2)];  ln m = 2 atanh(s),
//         s = (m-1)/(m+1), series to s^11.
//   exp:  Cody & Waite (1980) two-constant reduction x = n ln2 + r, |r| <= ln2/2,
//         Taylor series of e^r to r^8.
//   exp2: x = n + f, |f| <= 1/2, e^(f ln2) by the same series.
//   atan2: octant reduction to t in [0,1], then t > tan(pi/12) is mapped by
//         atan(t) = pi/6 + atan((t sqrt3 - 1)/(t + sqrt3)); Taylor series to t^15.
//   sin/cos: Cody & Waite three-constant reduction by pi/2, Taylor series to
//         r^9 (sin) and r^10 (cos) on |r| <= pi/4.
#pragma once

#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define GI_HD __host__ __device__ __forceinline__
#else
#define GI_HD static inline
#endif

namespace gi {

GI_HD uint32_t f2u(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
#endif
}

GI_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, 4);
  return x;
#endif
}

GI_HD float fma_(float a, float b, float c) { return fmaf(a, b, c); }

// Correctly rounded reciprocal (IEEE-754 1/b, round to nearest even).
GI_HD float rcp_(float b) {
#if defined(__CUDA_ARCH__)
  return __frcp_rn(b);
#else
  return 1.0f / b;
#endif
}

// fp32 division as evaluated everywhere in this library and its restatement:
// a times the correctly rounded reciprocal of b (two roundings; GLSL allows
// 2.5 ulp for division, and shader compilers emit this form).
GI_HD float div_(float a, float b) { return a * rcp_(b); }

static constexpr float kInf = __builtin_huge_valf();
static constexpr float kPi = 3.14159274101257324f;       // float nearest pi
static constexpr float kPiO2 = 1.57079637050628662f;     // float nearest pi/2
static constexpr float kPiO6 = 0.52359879016876221f;     // float nearest pi/6
static constexpr float kSqrt3 = 1.73205077648162842f;
static constexpr float kTanPiO12 = 0.26794919371604919f; // 2 - sqrt(3)
static constexpr float kSqrt2 = 1.41421353816986084f;
static constexpr float kLn2Hi = 0.693145751953125f;      // 16 significant bits
static constexpr float kLn2Lo = 1.42860676533018700e-06f;
static constexpr float kLog2e = 1.44269502162933350f;
static constexpr float kTwoOPi = 0.63661974668502808f;
static constexpr float kPiO2_1 = 1.5703125f;             // 9 significant bits
static constexpr float kPiO2_2 = 4.83826792333275080e-04f;
static constexpr float kPiO2_3 = 2.56328291925456140e-12f;

// Scale by 2^n for n in [-252, 254] by two exact multiplications.
GI_HD float ldexp_(float x, int n) {
  int n1 = n / 2;
  int n2 = n - n1;
  float s1 = u2f((uint32_t)(n1 + 127) << 23);
  float s2 = u2f((uint32_t)(n2 + 127) << 23);
  return (x * s1) * s2;
}

// ln(m) for m in (sqrt(1/2), sqrt(2)] by 2*atanh((m-1)/(m+1)).
GI_HD float log_core(float m) {
  float s = div_(m - 1.0f, m + 1.0f);
  float z = s * s;
  float p = fma_(z, 1.0f / 11.0f, 1.0f / 9.0f);
  p = fma_(z, p, 1.0f / 7.0f);
  p = fma_(z, p, 1.0f / 5.0f);
  p = fma_(z, p, 1.0f / 3.0f);
  float s2 = s + s;
  return fma_(s2 * z, p, s2);
}

// Split a positive finite x into m * 2^e with m in (sqrt(1/2), sqrt(2)].
GI_HD float split_exp(float x, int* e) {
  uint32_t u = f2u(x);
  int bias = 0;
  if (u < 0x00800000u) {  // subnormal: scale up by 2^24 (exact)
    x = x * 16777216.0f;
    u = f2u(x);
    bias = -24;
  }
  int ex = (int)(u >> 23) - 127 + bias;
  float m = u2f((u & 0x007fffffu) | 0x3f800000u);
  if (m > kSqrt2) {
    m = m * 0.5f;
    ex += 1;
  }
  *e = ex;
  return m;
}

GI_HD float logf_(float x) {
  if (x != x) return x;
  if (x < 0.0f) return u2f(0x7fc00000u);
  if (x == 0.0f) return -kInf;
  if (x == kInf) return kInf;
  int e;
  float m = split_exp(x, &e);
  float lm = log_core(m);
  float fe = (float)e;
  return fe * kLn2Hi + fma_(fe, kLn2Lo, lm);
}

GI_HD float log2f_(float x) {
  if (x != x) return x;
  if (x < 0.0f) return u2f(0x7fc00000u);
  if (x == 0.0f) return -kInf;
  if (x == kInf) return kInf;
  int e;
  float m = split_exp(x, &e);
  float lm = log_core(m);
  return fma_(lm, kLog2e, (float)e);
}

// e^r for |r| <= ~0.35 by the Taylor series to r^8.
GI_HD float exp_core(float r) {
  float p = fma_(r, 1.0f / 40320.0f, 1.0f / 5040.0f);
  p = fma_(r, p, 1.0f / 720.0f);
  p = fma_(r, p, 1.0f / 120.0f);
  p = fma_(r, p, 1.0f / 24.0f);
  p = fma_(r, p, 1.0f / 6.0f);
  p = fma_(r, p, 0.5f);
  p = fma_(r, p, 1.0f);
  return fma_(r, p, 1.0f);
}

GI_HD float expf_(float x) {
  if (x != x) return x;
  if (x > 88.8f) return kInf;
  if (x < -104.0f) return 0.0f;
  float n = rintf(x * kLog2e);
  float r = fma_(-n, kLn2Hi, x);  // exact: n * kLn2Hi has <= 24 bits
  r = fma_(-n, kLn2Lo, r);
  return ldexp_(exp_core(r), (int)n);
}

GI_HD float exp2f_(float x) {
  if (x != x) return x;
  if (x >= 128.0f) return kInf;
  if (x < -150.0f) return 0.0f;
  float n = rintf(x);
  float f = x - n;  // exact
  float r = fma_(f, kLn2Hi, f * kLn2Lo);
  return ldexp_(exp_core(r), (int)n);
}

// pow(b, y) for b >= 0 as exp2(y * log2(b)); pow(0, y>0) = 0.
GI_HD float powf_(float b, float y) {
  if (b == 0.0f) return y > 0.0f ? 0.0f : (y == 0.0f ? 1.0f : kInf);
  if (b == 1.0f) return 1.0f;
  return exp2f_(y * log2f_(b));
}

// atan(t) for |t| <= tan(pi/12), Taylor series to t^15.
GI_HD float atan_core(float t) {
  float z = t * t;
  float p = fma_(z, -1.0f / 15.0f, 1.0f / 13.0f);
  p = fma_(z, p, -1.0f / 11.0f);
  p = fma_(z, p, 1.0f / 9.0f);
  p = fma_(z, p, -1.0f / 7.0f);
  p = fma_(z, p, 1.0f / 5.0f);
  p = fma_(z, p, -1.0f / 3.0f);
  return fma_(t * z, p, t);
}

GI_HD bool signbit_(float x) { return (f2u(x) >> 31) != 0u; }

GI_HD float copysign_(float a, float s) {
  return u2f((f2u(a) & 0x7fffffffu) | (f2u(s) & 0x80000000u));
}

// atan2 with the IEEE-754 special cases (signed zeros and infinities).
GI_HD float atan2f_(float y, float x) {
  if (x != x || y != y) return x + y;
  float ax = fabsf(x), ay = fabsf(y);
  float a;
  if (ax == kInf && ay == kInf) {
    a = signbit_(x) ? 3.0f * (kPi * 0.25f) : kPi * 0.25f;
    return copysign_(a, y);
  }
  if (ay == 0.0f && ax == 0.0f) {
    a = signbit_(x) ? kPi : 0.0f;
    return copysign_(a, y);
  }
  bool swap = ay > ax;
  float num = swap ? ax : ay;
  float den = swap ? ay : ax;
  float t = div_(num, den);  // in [0, 1] (up to one rounding above 1)
  float base = 0.0f;
  if (t > kTanPiO12) {
    t = div_(t * kSqrt3 - 1.0f, t + kSqrt3);
    base = kPiO6;
  }
  a = base + atan_core(t);
  if (swap) a = kPiO2 - a;
  if (signbit_(x)) a = kPi - a;
  return copysign_(a, y);
}

GI_HD void sincos_core(float r, float* s, float* c) {
  float z = r * r;
  float ps = fma_(z, 1.0f / 362880.0f, -1.0f / 5040.0f);
  ps = fma_(z, ps, 1.0f / 120.0f);
  ps = fma_(z, ps, -1.0f / 6.0f);
  *s = fma_(r * z, ps, r);
  float pc = fma_(z, -1.0f / 3628800.0f, 1.0f / 40320.0f);
  pc = fma_(z, pc, -1.0f / 720.0f);
  pc = fma_(z, pc, 1.0f / 24.0f);
  pc = fma_(z, pc, -0.5f);
  *c = fma_(z, pc, 1.0f);
}

// sin and cos of x for |x| < 2^15 (the callers pass angles within a few turns).
GI_HD void sincosf_(float x, float* s, float* c) {
  if (x != x || fabsf(x) == kInf) {
    *s = u2f(0x7fc00000u);
    *c = *s;
    return;
  }
  float k = rintf(x * kTwoOPi);
  float r = fma_(-k, kPiO2_1, x);
  r = fma_(-k, kPiO2_2, r);
  r = fma_(-k, kPiO2_3, r);
  float sr, cr;
  sincos_core(r, &sr, &cr);
  int q = ((int)k) & 3;
  switch (q) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
  }
}

GI_HD float sinf_(float x) { float s, c; sincosf_(x, &s, &c); return s; }
GI_HD float cosf_(float x) { float s, c; sincosf_(x, &s, &c); return c; }

}  // namespace gi
