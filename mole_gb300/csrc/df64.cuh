// df64.cuh -- double-float arithmetic on the FP32 pipe.
//
// A df64 value is the unevaluated sum h + l of two FP32 numbers with
// |l| <= ulp(h) / 2: about 48 significant bits, relative rounding near 2^-47
// per operation. GB300 executes FP32 at 62x its FP64 rate, so a
// double-float operation of 7-20 FP32 instructions costs a fraction of one
// native FP64 instruction's pipe time. The walker kernels of the FP64-accurate
// "df64" precision run every one-body, pair, inverse and local-energy term in
// this type; the exponent range is FP32's, which the kernels guard (values
// beyond it make the launch rerun in native FP64).
//
// Error-free transformations (published methods, written here from them):
//   two_sum       Knuth, TAOCP vol. 2, 4.2.2 (six additions, no branch)
//   fast_two_sum  Dekker 1971 (|a| >= |b|)
//   two_prod      via FMA: p = a b, e = fma(a, b, -p)
//   addition      the "sloppy" double-double add of Hida, Li and Bailey (QD, 2001)
//   reciprocal, reciprocal square root: one Newton correction of the FP32
//                 hardware approximation, with the residual formed exactly
//   exp           reduction by ln2/64 (three-part constant), 64-entry table of
//                 2^(j/64), degree-5 polynomial on |r| <= ln2/128
// Every FP32 operation in the transformations uses the _rn intrinsics so that
// the compiler cannot contract or reassociate them.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>

#include "common.cuh"

namespace mole {

struct df64 {
  float h, l;
  df64() = default;
  __host__ __device__ constexpr df64(float hh, float ll) : h(hh), l(ll) {}
  __host__ __device__ constexpr df64(int i) : h((float)i), l(0.f) {}  // exact for |i| < 2^24
  __host__ __device__ constexpr df64(float f) : h(f), l(0.f) {}
  __host__ __device__ df64(double d) : h((float)d), l((float)(d - (double)(float)d)) {}
  __host__ __device__ explicit operator double() const { return (double)h + (double)l; }
  __host__ __device__ explicit operator float() const { return h; }
};

template <class T>
struct is_df64 : std::false_type {};
template <>
struct is_df64<df64> : std::true_type {};

__device__ __forceinline__ df64 df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df64(s, e);
}
__device__ __forceinline__ df64 df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df64(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.h, -a.l); }
__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  const df64 s = df_two_sum(a.h, b.h);
  return df_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return df_fast_two_sum(p, e);
}
// product with an FP32 number
__device__ __forceinline__ df64 df_mul(df64 a, float b) {
  const float p = __fmul_rn(a.h, b);
  float e = __fmaf_rn(a.h, b, -p);
  e = __fmaf_rn(a.l, b, e);
  return df_fast_two_sum(p, e);
}
// exact scaling by a power of two
__device__ __forceinline__ df64 df_scale(df64 a, float pow2) { return df64(__fmul_rn(a.h, pow2), __fmul_rn(a.l, pow2)); }

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// 1 / b: r ~ 1/b.h to 2^-23, e = 1 - b r formed with FMAs (the first one
// exact), 1/b = r (1 + e + e^2 + ...).
__device__ __forceinline__ df64 df_rcp(df64 b) {
  const float r = rcp_approx(b.h);
  float e = __fmaf_rn(-b.h, r, 1.0f);
  e = __fmaf_rn(-b.l, r, e);
  const float t = __fmaf_rn(e, e, e);
  return df_fast_two_sum(r, __fmul_rn(r, t));
}
__device__ __forceinline__ df64 operator/(df64 a, df64 b) {
  // quotient digit q1 = a.h / b, remainder a - q1 b with exact products, q2 = rem / b
  const float r = rcp_approx(b.h);
  const float q1 = __fmul_rn(a.h, r);
  const float p = __fmul_rn(q1, b.h);
  const float pe = __fmaf_rn(q1, b.h, -p);
  float rem = __fsub_rn(a.h, p);  // exact: q1 b.h is within 2^-22 of a.h
  rem = __fsub_rn(rem, pe);
  rem = __fadd_rn(rem, a.l);
  rem = __fmaf_rn(-q1, b.l, rem);
  const float q2 = __fmul_rn(rem, r);
  // second correction of q1 + q2 (r carries 2^-23 relative error)
  float e = __fmaf_rn(-b.h, r, 1.0f);
  e = __fmaf_rn(-b.l, r, e);
  return df_fast_two_sum(q1, __fmaf_rn(q2, e, q2));
}

// a^-1/2 for a > 0: y ~ a.h^-1/2 to 2^-22, e = 1 - a y^2 from exact products,
// a^-1/2 = y (1 + e/2 + 3 e^2 / 8 + ...).
__device__ __forceinline__ df64 df_rsqrt(df64 a) {
  const float y = rsqrt_approx(a.h);
  const float s = __fmul_rn(y, y);
  const float se = __fmaf_rn(y, y, -s);
  const float p = __fmul_rn(a.h, s);
  const float pe = __fmaf_rn(a.h, s, -p);
  float e = __fsub_rn(1.0f, p);  // exact: p is within 2^-21 of 1
  e = __fsub_rn(e, pe);
  e = __fmaf_rn(-a.h, se, e);
  e = __fmaf_rn(-a.l, s, e);
  const float t = __fmul_rn(e, __fmaf_rn(0.375f, e, 0.5f));
  return df_fast_two_sum(y, __fmul_rn(y, t));
}
__device__ __forceinline__ df64 df_sqrt(df64 a) { return a.h > 0.f ? a * df_rsqrt(a) : df64(0.f, 0.f); }

// 2^(j/64), j = 0..63, as df64 pairs in the CTA's shared memory; every kernel
// that evaluates df_exp calls df64_setup() with all its threads first.
static __shared__ float2 g_df64_exp2_tab[64];
__device__ __forceinline__ void df64_setup() {
  for (int j = threadIdx.x; j < 64; j += blockDim.x) {
    const double v = exp2((double)j / 64.0);
    const float h = (float)v;
    g_df64_exp2_tab[j] = make_float2(h, (float)(v - (double)h));
  }
  __syncthreads();
}

// e^x. x = n ln2/64 + r with n = rint(64 x / ln2) (|n| < 2^13, so n L1 is
// exact for the 11-bit head L1 of ln2/64), e^x = 2^(n >> 6) 2^((n & 63)/64) e^r,
// e^r - 1 = r + r^2/2 (double-float) + r^3/6 + r^4/24 + r^5/120 (FP32;
// |r| <= 0.0055 so the truncated r^6/720 is below 2^-54). Results below
// FP32's normal range flush to zero; the kernels treat such magnitudes as
// out of range.
__device__ __forceinline__ df64 df_exp(df64 x) {
  constexpr float kInv = 0x1.715476p+6f;   // 64 / ln2
  constexpr float kL1 = 0x1.63p-7f;        // ln2/64, head (11 bits)
  constexpr float kL2 = -0x1.bd0106p-19f;  // next 24 bits
  constexpr float kL3 = 0x1.cf79acp-46f;   // next 24 bits
  if (x.h < -87.0f) return df64(0.f, 0.f);
  if (x.h > 88.0f) return df64(INFINITY, 0.f);
  const float n = rintf(__fmul_rn(x.h, kInv));
  const float t = __fmaf_rn(-n, kL1, x.h);  // exact
  const float p2 = __fmul_rn(n, kL2);
  const float e2 = __fmaf_rn(n, kL2, -p2);
  const df64 a = df_two_sum(t, -p2);
  const df64 r = df_two_sum(a.h, __fadd_rn(a.l, __fsub_rn(__fsub_rn(x.l, e2), __fmul_rn(n, kL3))));
  // r^2 / 2 in double-float, the cubic tail in FP32
  const float s = __fmul_rn(r.h, r.h);
  const float se = __fmaf_rn(__fadd_rn(r.h, r.h), r.l, __fmaf_rn(r.h, r.h, -s));
  const df64 half_sq(__fmul_rn(s, 0.5f), __fmul_rn(se, 0.5f));
  float c = __fmaf_rn(r.h, 1.0f / 120.0f, 1.0f / 24.0f);
  c = __fmaf_rn(r.h, c, 1.0f / 6.0f);
  const float q = __fmul_rn(__fmul_rn(s, r.h), c);
  df64 E = r + half_sq;
  const df64 eq = df_two_sum(E.h, q);
  E = df_fast_two_sum(eq.h, __fadd_rn(eq.l, E.l));
  const int ni = (int)n;
  const float2 tb = g_df64_exp2_tab[ni & 63];
  const df64 T(tb.x, tb.y);
  const df64 v = T + T * E;
  const int k = ni >> 6;  // floor division
  if (k < -126) return df64(0.f, 0.f);
  return df_scale(v, __int_as_float((k + 127) << 23));
}

__device__ __forceinline__ df64& operator+=(df64& a, df64 b) { return a = a + b; }
__device__ __forceinline__ df64& operator-=(df64& a, df64 b) { return a = a - b; }
__device__ __forceinline__ df64& operator*=(df64& a, df64 b) { return a = a * b; }
__device__ __forceinline__ bool operator>(df64 a, df64 b) { return a.h > b.h || (a.h == b.h && a.l > b.l); }
__device__ __forceinline__ bool operator<(df64 a, df64 b) { return b > a; }
__device__ __forceinline__ bool operator!=(df64 a, df64 b) { return a.h != b.h || a.l != b.l; }

// Uniform in (0, 1) from 32 random bits, exactly the value of u01<double>:
// (x + 1/2) 2^-32 has at most 33 significant bits.
template <>
__device__ __forceinline__ df64 u01<df64>(uint32_t x) {
  const float a = __fmul_rn((float)(x >> 8), 256.0f);
  const float b = __fadd_rn((float)(x & 255u), 0.5f);
  return df_scale(df_two_sum(a, b), 0x1p-32f);
}

// Helpers the walker code uses for both FP64-part types (double, df64).
__device__ __forceinline__ double to_d(double x) { return x; }
__device__ __forceinline__ double to_d(df64 x) { return (double)x; }
__device__ __forceinline__ float mag(double x) { return (float)fabs(x); }
__device__ __forceinline__ float mag(df64 x) { return fabsf(x.h); }
__device__ __forceinline__ bool is_neg(double x) { return x < 0.0; }
__device__ __forceinline__ bool is_neg(df64 x) { return x.h < 0.f; }
__device__ __forceinline__ bool is_zero(double x) { return x == 0.0; }
__device__ __forceinline__ bool is_zero(df64 x) { return x.h == 0.f; }
__device__ __forceinline__ double recip(double x) { return 1.0 / x; }
__device__ __forceinline__ df64 recip(df64 x) { return df_rcp(x); }
__device__ __forceinline__ double twice(double x) { return 2.0 * x; }
__device__ __forceinline__ df64 twice(df64 x) { return df64(__fmul_rn(x.h, 2.f), __fmul_rn(x.l, 2.f)); }

}  // namespace mole
