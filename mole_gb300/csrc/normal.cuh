// normal.cuh -- bit-reproducible FP32 Box-Muller normals.
//
// Every operation is an explicitly rounded IEEE single-precision add, mul,
// fma, div or sqrt (no contraction is left to the compiler), so a host
// implementation that performs the same operation sequence produces the same
// bits. log uses m = u / 2^e with m in [sqrt(1/2), sqrt(2)) and the series
// ln m = 2 atanh(s) = 2 (s + s^3/3 + ... + s^9/9), s = (m - 1)/(m + 1),
// |s| <= 0.1716; sin and cos of an angle in [0, pi/2] use their Taylor series
// through x^11 and x^12. Errors are below 1e-7 relative.
#pragma once

#include <stdint.h>

namespace mole {

#define MOLE_FADD(a, b) __fadd_rn(a, b)
#define MOLE_FSUB(a, b) __fsub_rn(a, b)
#define MOLE_FMUL(a, b) __fmul_rn(a, b)
#define MOLE_FFMA(a, b, c) __fmaf_rn(a, b, c)
#define MOLE_FDIV(a, b) __fdiv_rn(a, b)
#define MOLE_FSQRT(a) __fsqrt_rn(a)
#define MOLE_AS_UINT(f) __float_as_uint(f)
#define MOLE_AS_FLOAT(u) __uint_as_float(u)

__device__ __forceinline__ float repro_log01(float u) {
  uint32_t bits = MOLE_AS_UINT(u);
  int e = (int)((bits >> 23) & 0xffu) - 127;
  float m = MOLE_AS_FLOAT((bits & 0x7fffffu) | 0x3f800000u);
  if (m > 1.41421356f) {
    m = MOLE_FMUL(m, 0.5f);
    e += 1;
  }
  const float s = MOLE_FDIV(MOLE_FSUB(m, 1.0f), MOLE_FADD(m, 1.0f));
  const float s2 = MOLE_FMUL(s, s);
  float p = MOLE_FFMA(s2, 0.111111112f, 0.142857149f);
  p = MOLE_FFMA(p, s2, 0.2f);
  p = MOLE_FFMA(p, s2, 0.333333343f);
  p = MOLE_FFMA(p, s2, 1.0f);
  const float t = MOLE_FMUL(s, p);
  return MOLE_FFMA((float)e, 0.693147182f, MOLE_FADD(t, t));
}

// sin and cos of x in [0, pi/2]
__device__ __forceinline__ void repro_sincos_q(float x, float& s, float& c) {
  const float x2 = MOLE_FMUL(x, x);
  float ps = MOLE_FFMA(x2, -2.50521084e-8f, 2.75573192e-6f);
  ps = MOLE_FFMA(ps, x2, -1.98412698e-4f);
  ps = MOLE_FFMA(ps, x2, 8.33333333e-3f);
  ps = MOLE_FFMA(ps, x2, -1.66666667e-1f);
  ps = MOLE_FFMA(ps, x2, 1.0f);
  s = MOLE_FMUL(x, ps);
  float pc = MOLE_FFMA(x2, 2.08767570e-9f, -2.75573192e-7f);
  pc = MOLE_FFMA(pc, x2, 2.48015873e-5f);
  pc = MOLE_FFMA(pc, x2, -1.38888889e-3f);
  pc = MOLE_FFMA(pc, x2, 4.16666667e-2f);
  pc = MOLE_FFMA(pc, x2, -0.5f);
  c = MOLE_FFMA(pc, x2, 1.0f);
}

// Two N(0,1) deviates from 32 random bits each: the radius from the top 24
// bits of a, the quadrant from the top 2 bits of b and the angle inside the
// quadrant from its next 24 bits.
__device__ __forceinline__ void repro_box_muller(uint32_t a, uint32_t b, float& z0, float& z1) {
  const float u = MOLE_FMUL(MOLE_FADD((float)(a >> 8), 0.5f), 5.96046448e-8f);  // 2^-24
  const float r = MOLE_FSQRT(MOLE_FMUL(-2.0f, repro_log01(u)));
  const float f = MOLE_FMUL(MOLE_FADD((float)((b >> 6) & 0xffffffu), 0.5f), 5.96046448e-8f);
  const float x = MOLE_FMUL(f, 1.57079637f);
  float s, c;
  repro_sincos_q(x, s, c);
  const uint32_t q = b >> 30;
  float cs = c, sn = s;
  if (q == 1u) {
    cs = -s;
    sn = c;
  } else if (q == 2u) {
    cs = -c;
    sn = -s;
  } else if (q == 3u) {
    cs = s;
    sn = -c;
  }
  z0 = MOLE_FMUL(r, cs);
  z1 = MOLE_FMUL(r, sn);
}

}  // namespace mole
