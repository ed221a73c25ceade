// fp64.cuh -- FP64 reciprocal, reciprocal square root and exponential that
// each take two FP64-pipe instructions.
//
// GB300 issues one FP64 warp instruction per 64 cycles per SM sub-partition
// (1/62 of its FP32 rate), and a hardware float <-> double conversion takes a
// slot of that pipe like a DFMA. The library's reciprocal and reciprocal
// square root take five FP64-pipe instructions each, its exp fifteen and a
// division eight (smsp__inst_executed_pipe_fp64 per call, measured). The
// functions below do the approximation on the FP32 pipe, the one correction
// that needs 53-bit arithmetic as FP64 FMAs, and every other step (splitting
// a double into FP32 pieces, building an exact double from FP32 pieces or
// from an integer product) with integer operations:
//
//   rcp64(x)    Newton-Raphson from the FP32 approximation y0 ~ 1/x: with
//               e = 1 - x y0 (one FMA, exact to rounding), 1/x = y0 (1 + e +
//               e^2 + ...); y0 e^2 is below 2^-42 y0 and is formed in FP32,
//               added into the zero low bits of y0's double, and the result
//               is fma(y0, e, y0 + y0 e^2): 2 FP64 instructions, within 1 ulp.
//   rsqrt64(x)  the same for x^-1/2 (Markstein, "IA-64 and Elementary
//               Functions", 2000, ch. 6): e = 1 - x y0^2 with y0^2 exact as a
//               double (built from the FP32 product and its FMA remainder),
//               x^-1/2 = y0 (1 + e/2 + 3 e^2 / 8 + ...): 2 FP64 instructions.
//   exp64(x)    Tang's table-driven method (P. T. P. Tang, "Table-driven
//               implementation of the exponential function in IEEE
//               floating-point arithmetic", ACM TOMS 15(2), 1989): x = n ln2/64
//               + r with n L1 (L1 the 36-bit head of ln2/64) an exact double
//               built from the integer product, r1 = x - n L1 by one FMA, r1
//               split into FP32 pieces, the tail n L2 subtracted and e^r - 1
//               evaluated in double-float on the FP32 pipe, and
//               e^x = 2^(n >> 6) (T + T q), T = 2^((n & 63)/64), by one FMA:
//               2 FP64 instructions, within 2 ulp.
//   expab64(a, b) = e^(a b) with the product fused into the reduction.
//
// Outside the ranges where the FP32 pieces stay normal the functions return
// the library's result (a branch that valid walker data does not take). The
// constants are derived from exact arithmetic by
// mole_gb300/gen_exp_constants.py (checked by the tests). The integer helpers
// are host-callable so that the CPU tests check them.
#pragma once

#include <stdint.h>
#include <string.h>

#include "df64.cuh"

#if defined(__CUDACC__)
#define MOLE_HD __host__ __device__ __forceinline__
#else
#define MOLE_HD inline
#endif

namespace mole {

MOLE_HD uint32_t f_bits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}
MOLE_HD float f_from(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}
MOLE_HD uint64_t d_bits(double d) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u;
  memcpy(&u, &d, 8);
  return u;
#endif
}
MOLE_HD double d_from(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double d;
  memcpy(&d, &u, 8);
  return d;
#endif
}
MOLE_HD int clz32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __clz((int)x);
#else
  return x ? __builtin_clz(x) : 32;
#endif
}
MOLE_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

// Bits of the double equal to a normal float (exponent rebiased, significand
// shifted); callers guarantee a normal argument.
MOLE_HD uint64_t f2d_bits_normal(uint32_t fb) {
  return ((uint64_t)(fb & 0x80000000u) << 32) | ((uint64_t)(((fb >> 23) & 0xFFu) + 896u) << 52) |
         ((uint64_t)(fb & 0x7FFFFFu) << 29);
}

// h + l as a double, for a normalised double-float pair: h a normal float and
// |l| <= ulp(h) / 2 (l of either sign, possibly zero; a subnormal l is taken
// as zero). The sum is exact when it fits 53 bits (l the FMA remainder of a
// product of two floats) and rounded to nearest otherwise (ties away from
// zero). l is added to the bit pattern of h as an integer multiple of the
// double ulp of h's binade (half that ulp when h is a power of two and l
// lowers it into the binade below); no carry leaves h's binade because
// |l| <= ulp(h) / 2.
MOLE_HD double dbl_add_small(float h, float l) {
  const uint32_t hb = f_bits(h), lb = f_bits(l);
  const int eh = (int)((hb >> 23) & 0xFFu), el = (int)((lb >> 23) & 0xFFu);
  const uint64_t H = f2d_bits_normal(hb);
  if (el == 0) return d_from(H);
  const bool opposite = ((hb ^ lb) >> 31) != 0u;
  const bool down = opposite && (hb & 0x7FFFFFu) == 0u;
  // l = ml 2^(el - 150); ulp of the double h = 2^(eh - 179) (2^(eh - 180) below a power of two)
  const int sh = el - eh + 29 + (down ? 1 : 0);
  const uint32_t ml = (lb & 0x7FFFFFu) | 0x800000u;
  uint64_t k;
  if (sh >= 0) k = (uint64_t)ml << (sh > 8 ? 8 : sh);  // sh <= 6 under the precondition
  else if (sh > -25) k = (uint64_t)((ml + (1u << (-sh - 1))) >> (-sh));
  else k = 0;
  return d_from(opposite ? H - k : H + k);
}

// The exact double of a normal float (integer-built, no conversion instruction).
MOLE_HD double dbl_of_float(float f) { return d_from(f2d_bits_normal(f_bits(f))); }

// Splits a double into (h, l): h its top 24 significant bits (a float, toward
// zero), l the remaining 29 bits rounded to a float (|l| < 2^-23 |h|, relative
// error 2^-24 of l). For |d| < 2^-100 both are zero; |d| must be below 2^100.
MOLE_HD void split_double(double d, float& h, float& l) {
  const uint64_t b = d_bits(d);
  const uint32_t hi = (uint32_t)(b >> 32);
  const int e = (int)((hi >> 20) & 0x7FFu) - 1023;
  if (e < -100) {
    h = 0.f;
    l = 0.f;
    return;
  }
  const uint32_t s = hi & 0x80000000u;
  h = f_from(s | (uint32_t)(e + 127) << 23 | (uint32_t)((b >> 29) & 0x7FFFFFu));
  const uint32_t m = (uint32_t)(b & 0x1FFFFFFFu);  // the low 29 bits: value m 2^(e - 52)
  if (m == 0u) {
    l = 0.f;
    return;
  }
  const int len = 32 - clz32(m);  // m = 1.xxx 2^(len - 1)
  const int fe = len - 1 + e - 52 + 127;
  if (fe <= 0) {
    l = 0.f;
    return;
  }
  uint32_t mant;
  if (len > 24) mant = (m + (1u << (len - 25))) >> (len - 24);  // round to 24 bits
  else mant = m << (24 - len);
  // rounding up may carry to 2^24: the exponent field absorbs it
  l = f_from(s | (((uint32_t)fe << 23) + (mant - 0x800000u)));
}

// n L1 as an exact double for |n| < 2^16, L1 = the head of ln2/64 with 36
// significant bits (|n| L1 < 2^52 units of 2^-42: exact).
constexpr uint64_t kExpL1Int = 0xB17217F7Dull;  // L1 = kExpL1Int 2^-42 = 0x1.62e42fefap-7
MOLE_HD double exp_nl1(int n) {
  if (n == 0) return 0.0;
  const uint64_t p = (uint64_t)(n < 0 ? -n : n) * kExpL1Int;
  const int lz = clz64(p);
  const uint64_t mant = ((p << lz) << 1) >> 12;
  const uint64_t ex = (uint64_t)(63 - lz - 42 + 1023);
  return d_from((n < 0 ? 0x8000000000000000ull : 0ull) | (ex << 52) | mant);
}

// u01(x) - 1/2 = (x + 1/2) 2^-32 - 1/2 = (2x + 1 - 2^32) 2^-33 exactly (an odd
// integer below 2^32 in magnitude), built with integer operations.
MOLE_HD double u01_centered(uint32_t x) {
  const int64_t m = 2 * (int64_t)x + 1 - 4294967296LL;
  const uint64_t a = (uint64_t)(m < 0 ? -m : m);
  const int lz = clz64(a);
  const uint64_t mant = ((a << lz) << 1) >> 12;
  const uint64_t ex = (uint64_t)(63 - lz - 33 + 1023);
  return d_from((m < 0 ? 0x8000000000000000ull : 0ull) | (ex << 52) | mant);
}

#ifdef __CUDACC__

// The library's results outside the fast paths, as calls: a call is a branch,
// which the compiler cannot if-convert into predicated FP64 instructions that
// would take FP64-pipe slots on every call of the fast path.
static __device__ __noinline__ double rcp64_slow(double x) { return 1.0 / x; }
static __device__ __noinline__ double rsqrt64_slow(double x) { return rsqrt(x); }
static __device__ __noinline__ double exp64_slow(double a, double b) { return exp(a * b); }

// 1/x in FP64 to within 1 ulp: two FP64 instructions. The fast path covers
// 2^-60 < |x| < 2^60, where y0 e^2 stays a normal float down to 2^-53 y0;
// zeros, infinities, NaNs and extreme magnitudes take the library's IEEE
// division.
__device__ __forceinline__ double rcp64(double x) {
  const float xf = d2f_rz(x);
  const float ax = fabsf(xf);
  if (!(ax > 0x1p-60f && ax < 0x1p60f)) return rcp64_slow(x);
  const float y0 = rcp_approx(xf);  // |1 - x y0| < 2^-21 (approximation plus truncation of x)
  const double e = fma(-x, dbl_of_float(y0), 1.0);
  const float ef = d2f_rz(e);
  const float c = __fmul_rn(y0, __fmul_rn(ef, ef));  // y0 e^2, |c| < 2^-42 |y0|
  return fma(dbl_of_float(y0), e, dbl_add_small(y0, c));
}

// x^-1/2 in FP64 to within about 1 ulp: two FP64 instructions. Fast path for
// 2^-60 < x < 2^60 (squared distances of walker data); everything else (zero,
// negative, infinite, extreme) takes the library's rsqrt.
__device__ __forceinline__ double rsqrt64(double x) {
  const float xf = d2f_rz(x);
  if (!(xf > 0x1p-60f && xf < 0x1p60f)) return rsqrt64_slow(x);
  const float y0 = rsqrt_approx(xf);  // |1 - x y0^2| < 2^-21
  const float s = __fmul_rn(y0, y0);
  const float se = __fmaf_rn(y0, y0, -s);  // y0^2 = s + se exactly
  const double e = fma(-x, dbl_add_small(s, se), 1.0);
  const float ef = d2f_rz(e);
  const float c = __fmul_rn(__fmul_rn(0.375f, y0), __fmul_rn(ef, ef));  // 3/8 y0 e^2
  return fma(dbl_of_float(__fmul_rn(0.5f, y0)), e, dbl_add_small(y0, c));
}

// e^(a b), with the product fused into the argument reduction; the FP32
// estimate of a b picks n. Fast path for |a b| < 600 (normal results); the
// library's exp(a * b) elsewhere.
__device__ __forceinline__ double expab64(double a, double b) {
  const float xf = __fmul_rn(d2f_rz(a), d2f_rz(b));  // within 2^-21 relative of a b
  if (!(fabsf(xf) < 600.f)) return exp64_slow(a, b);
  const float n = rintf(__fmul_rn(xf, 92.33248261689366f));  // 64 / ln2
  const int ni = (int)n;
  // r1 = a b - n L1 exactly, rounded once (|r1| < 0.0057: the estimate of a b
  // is within 1.8e-4 of it and n the nearest integer to 64 xf / ln2)
  const double r1 = fma(a, b, -exp_nl1(ni));
  float rh, rl;
  split_double(r1, rh, rl);
  // r = r1 - n L2, L2 = ln2/64 - L1 = kL2h + kL2l, in double-float: n kL2h
  // exactly as p + pe, n kL2l (below 2^-56) folded into pe
  constexpr float kL2h = 0x1.cf79acp-46f;
  constexpr float kL2l = -0x1.b0e264p-73f;
  const float p = __fmul_rn(n, kL2h);
  const float pe = __fmaf_rn(n, kL2l, __fmaf_rn(n, kL2h, -p));
  const df64 s = df_two_sum(rh, -p);
  const df64 r = df_two_sum(s.h, __fadd_rn(s.l, __fsub_rn(rl, pe)));
  // q = e^r - 1 = r + r^2/2 + r^3/6 (double-float) + r^4/24 + r^5/120 + r^6/720 (FP32)
  float t = __fmaf_rn(r.h, 1.0f / 720.0f, 1.0f / 120.0f);
  t = __fmaf_rn(r.h, t, 1.0f / 24.0f);
  const df64 a3 = df_mul(r, t) + df64(0x1.555556p-3f, -0x1.555556p-28f);  // 1/6 + r t
  const df64 b2 = r * a3 + df64(0.5f);
  const df64 q = r + r * (r * b2);
  const double T = __ldg(&kExp2Tab64[ni & 63]);
  const double v = fma(T, fabsf(q.h) < 0x1p-100f ? 0.0 : dbl_add_small(q.h, q.l), T);
  return d_from(d_bits(v) + ((uint64_t)(int64_t)(ni >> 6) << 52));
}
__device__ __forceinline__ double exp64(double x) { return expab64(x, 1.0); }

// The FP64-part reciprocal of the walker code (double; df64 has its own).
__device__ __forceinline__ double recip(double x) { return rcp64(x); }

#endif  // __CUDACC__

}  // namespace mole
