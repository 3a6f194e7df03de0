// ear_math.cuh -- scalar math shared by the sm_103a kernels and the
// library's host code.  Everything here is IEEE single precision with a
// fixed operation order; translation units that need results bit-identical
// to the CPU restatement are compiled with --fmad=false (device) and
// -ffp-contract=off (host).
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define EAR_HD __host__ __device__ __forceinline__
#else
#define EAR_HD inline
#endif

#ifndef __CUDACC__
#include <cmath>
#include <cstring>
#endif

namespace ear {

EAR_HD uint32_t f2u(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}
EAR_HD float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}
EAR_HD float f_sqrt(float x) {
#ifdef __CUDA_ARCH__
  return __fsqrt_rn(x);
#else
  return std::sqrt(x);
#endif
}
EAR_HD float f_rint(float x) {
#ifdef __CUDA_ARCH__
  return rintf(x);
#else
  return std::rint(x);
#endif
}
EAR_HD float f_ceil(float x) {
#ifdef __CUDA_ARCH__
  return ceilf(x);
#else
  return std::ceil(x);
#endif
}
EAR_HD float f_abs(float x) { return u2f(f2u(x) & 0x7fffffffu); }

struct V3 {
  float x, y, z;
};
EAR_HD V3 mk(float x, float y, float z) { return V3{x, y, z}; }
EAR_HD V3 sub(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
EAR_HD V3 neg(V3 a) { return V3{a.x * -1.0f, a.y * -1.0f, a.z * -1.0f}; }
EAR_HD float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
EAR_HD V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
EAR_HD float length(V3 a) { return f_sqrt(dot(a, a)); }
EAR_HD V3 normalized(V3 a) {
  const float l = length(a);
  if (l != 0.0f) return V3{a.x / l, a.y / l, a.z / l};
  return a;
}
// v - 2 (v.n) n
EAR_HD V3 reflect(V3 v, V3 n) {
  const float d = dot(v, n);
  return V3{v.x - 2.0f * (d * n.x), v.y - 2.0f * (d * n.y), v.z - 2.0f * (d * n.z)};
}

// True for zero, subnormal, infinite and NaN values (fpclassify != FP_NORMAL).
EAR_HD bool invalid_float(float x) {
  const uint32_t e = (f2u(x) >> 23) & 0xffu;
  return e == 0u || e == 0xffu;
}

// x^y for x >= 0: exp2(y * log2 x).  log uses the atanh series
// ln m = 2 (s + s^3/3 + ... + s^11/11), s = (m-1)/(m+1), m in [1/sqrt2, sqrt2);
// exp2 splits z = n + f, |f| <= 1/2, evaluates e^(f ln2) by its degree-7
// Taylor polynomial and scales by 2^n with at most one rounding.  Negative x
// gives NaN (the bases on this path are never negative).
EAR_HD float powf_portable(float x, float y) {
  const float kInf = u2f(0x7f800000u);
  if (x == 1.0f || y == 0.0f) return 1.0f;
  if (x != x || y != y) return u2f(0x7fc00000u);
  if (x < 0.0f) return u2f(0x7fc00000u);
  if (x == 0.0f) return y > 0.0f ? 0.0f : kInf;
  if (x == kInf) return y > 0.0f ? kInf : 0.0f;
  uint32_t b = f2u(x);
  int e = (int)(b >> 23);
  if (e == 0) {
    b = f2u(x * 16777216.0f);
    e = (int)(b >> 23) - 24;
  }
  e -= 127;
  float m = u2f((b & 0x007fffffu) | 0x3f800000u);
  if (m > 1.41421354f) {
    m = m * 0.5f;
    e += 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  float p = 0.0909090936f;
  p = p * s2 + 0.111111112f;
  p = p * s2 + 0.142857149f;
  p = p * s2 + 0.200000003f;
  p = p * s2 + 0.333333343f;
  const float two_s = s + s;
  const float ln_m = two_s + two_s * (s2 * p);
  const float log2x = (float)e + ln_m * 1.44269502f;
  const float z = y * log2x;
  if (z > 128.0f) return kInf;
  if (z < -150.0f) return 0.0f;
  const float n = f_rint(z);
  const float f = z - n;
  const float g = f * 0.693147182f;
  float q = 1.98412698e-4f;
  q = q * g + 1.38888889e-3f;
  q = q * g + 8.33333377e-3f;
  q = q * g + 4.16666679e-2f;
  q = q * g + 0.166666672f;
  q = q * g + 0.5f;
  q = q * g + 1.0f;
  q = q * g + 1.0f;
  const int ni = (int)n;
  if (ni > 127) return (q * u2f(0x7f000000u)) * 2.0f;
  if (ni >= -126) return q * u2f((uint32_t)(ni + 127) << 23);
  return (q * u2f((uint32_t)(ni + 64 + 127) << 23)) * 5.42101086e-20f;
}

// x^y in the kernels: powf_portable, or -- in the fast kernels
// (FAST = true, device code) -- exp2(y log2 x) on the special-function unit,
// a few ulp from it: statistically identical, not bit-identical.  y = 0 and
// x = 1 give 1 as powf_portable does; the bases on this path are >= 0.
template <bool FAST>
EAR_HD float pow_sel(float x, float y) {
#ifdef __CUDA_ARCH__
  if (FAST) {
    if (y == 0.0f || x == 1.0f) return 1.0f;
    return exp2f(y * __log2f(x));
  }
#endif
  return powf_portable(x, y);
}

// Philox-4x32-10 (Salmon et al., "Parallel random numbers: as easy as
// 1, 2, 3", SC'11).
struct U4 {
  uint32_t x, y, z, w;
};
EAR_HD void mulhilo(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
#ifdef __CUDA_ARCH__
  *hi = __umulhi(a, b);
  *lo = a * b;
#else
  const uint64_t p = (uint64_t)a * b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
#endif
}
EAR_HD U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                        uint32_t k1) {
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo(0xD2511F53u, c0, &hi0, &lo0);
    mulhilo(0xCD9E8D57u, c2, &hi1, &lo1);
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  return U4{c0, c1, c2, c3};
}
// 24 random bits -> [0, 1 - 2^-24], exact in float.
EAR_HD float uniform24(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-8f; }

// RNG counter layout (one Philox block per draw group):
//   c0 = ray bits 0..31, c1 = ray bits 32..47 | band << 16 | stream << 24,
//   c2 = bounce | try << 16, c3 = context; key = seed.
EAR_HD U4 rng_block(uint32_t k0, uint32_t k1, uint32_t context, uint32_t band, uint64_t ray,
                    uint32_t stream, uint32_t bounce, uint32_t tr) {
  const uint32_t c1 = (uint32_t)((ray >> 32) & 0xffffu) | (band << 16) | (stream << 24);
  return philox4x32_10((uint32_t)ray, c1, bounce | (tr << 16), context, k0, k1);
}

constexpr int kMaxTries = 256;
constexpr float kFourPi = 4.0f * 3.14159265f;  // SHERE_SURFACE(1)
EAR_HD float inv_hemi_2(float r) { return 2.0f / (kFourPi * r * r); }
EAR_HD float inv_sphere_2(float r) { return 1.0f / (kFourPi * r * r); }

// Derived per-band material constants (Material::Material /
// Material::Bounce).  Returns false for an invalid material.
struct MatDerived {
  float survival[3];
  float p_reflect[3];
  float spec[3];
  uint32_t always_reflect;  // bit b
};

}  // namespace ear
