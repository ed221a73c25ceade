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
//   exp           Tang's table-driven method (P. T. P. Tang, ACM TOMS 15(2),
//                 1989): reduction by ln2/64 (three-part constant), 64-entry
//                 table of 2^(j/64), degree-5 polynomial on |r| <= ln2/128;
//                 the constants and tables are derived from exact arithmetic
//                 by mole_gb300/gen_exp_constants.py (checked by the tests)
// Every FP32 operation in the transformations uses the _rn intrinsics so that
// the compiler cannot contract or reassociate them.
//
// fp64.cuh builds the native FP64 kernels' reciprocal, reciprocal square root
// and exponential on the same pieces.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>

#include "common.cuh"

namespace mole {

// float <-> double conversions and double comparisons each take an FP64-pipe
// slot on GB300 (one warp instruction per 16 cycles per SM), as much as a
// DFMA. The two below build the result with integer operations and selects
// only (no branch the compiler could if-convert into a hardware conversion).
//
// float -> double: exponent rebiased by 1023 - 127, significand shifted into
// place; exact for normal floats, zeros, infinities and NaNs; subnormal
// floats (below 1.2e-38 in magnitude) become zeros of their sign.
__device__ __forceinline__ double f2d(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t s = u & 0x80000000u, e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
  uint32_t hi = s | ((e + 896u) << 20) | (m >> 3);
  uint32_t lo = m << 29;
  hi = e == 0xFFu ? (s | 0x7FF00000u | (m >> 3)) : hi;
  hi = e == 0u ? s : hi;
  lo = e == 0u ? 0u : lo;
  return __hiloint2double((int)hi, (int)lo);
}
// double -> float rounded toward zero (the top 24 significant bits); values
// below FP32's normal range become zeros of their sign, values above it
// infinities, NaNs stay NaNs.
__device__ __forceinline__ float d2f_rz(double d) {
  const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
  const uint32_t s = hi & 0x80000000u, e = (hi >> 20) & 0x7FFu;
  const uint32_t m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
  uint32_t u = s | ((e - 896u) << 23) | m;
  u = e > 1150u ? (s | 0x7F800000u | (e == 0x7FFu ? (m | (lo != 0u)) : 0u)) : u;
  u = e < 897u ? s : u;
  return __uint_as_float(u);
}
// The same for magnitudes below FP32's largest, as positions and their
// differences are: one select fewer, which the register-bound DMC kernels feel.
__device__ __forceinline__ float d2f_rz_small(double d) {
  const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
  const uint32_t s = hi & 0x80000000u, e = (hi >> 20) & 0x7FFu;
  const uint32_t u = s | ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
  return __uint_as_float(e < 897u ? s : u);
}

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

// 2^(j/64), j = 0..63, rounded to FP64 (read through the L1 cache: a warp's
// lanes touch at most 64 distinct 8-byte entries, 4 cache lines).
static __device__ __align__(16) const double kExp2Tab64[64] = {
    0x1.0000000000000p+0, 0x1.02c9a3e778061p+0, 0x1.059b0d3158574p+0, 0x1.0874518759bc8p+0,
    0x1.0b5586cf9890fp+0, 0x1.0e3ec32d3d1a2p+0, 0x1.11301d0125b51p+0, 0x1.1429aaea92de0p+0,
    0x1.172b83c7d517bp+0, 0x1.1a35beb6fcb75p+0, 0x1.1d4873168b9aap+0, 0x1.2063b88628cd6p+0,
    0x1.2387a6e756238p+0, 0x1.26b4565e27cddp+0, 0x1.29e9df51fdee1p+0, 0x1.2d285a6e4030bp+0,
    0x1.306fe0a31b715p+0, 0x1.33c08b26416ffp+0, 0x1.371a7373aa9cbp+0, 0x1.3a7db34e59ff7p+0,
    0x1.3dea64c123422p+0, 0x1.4160a21f72e2ap+0, 0x1.44e086061892dp+0, 0x1.486a2b5c13cd0p+0,
    0x1.4bfdad5362a27p+0, 0x1.4f9b2769d2ca7p+0, 0x1.5342b569d4f82p+0, 0x1.56f4736b527dap+0,
    0x1.5ab07dd485429p+0, 0x1.5e76f15ad2148p+0, 0x1.6247eb03a5585p+0, 0x1.6623882552225p+0,
    0x1.6a09e667f3bcdp+0, 0x1.6dfb23c651a2fp+0, 0x1.71f75e8ec5f74p+0, 0x1.75feb564267c9p+0,
    0x1.7a11473eb0187p+0, 0x1.7e2f336cf4e62p+0, 0x1.82589994cce13p+0, 0x1.868d99b4492edp+0,
    0x1.8ace5422aa0dbp+0, 0x1.8f1ae99157736p+0, 0x1.93737b0cdc5e5p+0, 0x1.97d829fde4e50p+0,
    0x1.9c49182a3f090p+0, 0x1.a0c667b5de565p+0, 0x1.a5503b23e255dp+0, 0x1.a9e6b5579fdbfp+0,
    0x1.ae89f995ad3adp+0, 0x1.b33a2b84f15fbp+0, 0x1.b7f76f2fb5e47p+0, 0x1.bcc1e904bc1d2p+0,
    0x1.c199bdd85529cp+0, 0x1.c67f12e57d14bp+0, 0x1.cb720dcef9069p+0, 0x1.d072d4a07897cp+0,
    0x1.d5818dcfba487p+0, 0x1.da9e603db3285p+0, 0x1.dfc97337b9b5fp+0, 0x1.e502ee78b3ff6p+0,
    0x1.ea4afa2a490dap+0, 0x1.efa1bee615a27p+0, 0x1.f50765b6e4540p+0, 0x1.fa7c1819e90d8p+0,
};
// The same values as double-float pairs.
static __device__ __align__(16) const float kExp2TabDF[64][2] = {
    {0x1.0000000000000p+0f, 0x0.0p+0f}, {0x1.02c9a40000000p+0f, -0x1.887fa00000000p-28f},
    {0x1.059b0e0000000p+0f, -0x1.9d4f520000000p-25f}, {0x1.0874520000000p+0f, -0x1.e2990e0000000p-26f},
    {0x1.0b55860000000p+0f, 0x1.9f31220000000p-25f}, {0x1.0e3ec40000000p+0f, -0x1.a585cc0000000p-25f},
    {0x1.11301e0000000p+0f, -0x1.fdb4960000000p-25f}, {0x1.1429aa0000000p+0f, 0x1.d525bc0000000p-25f},
    {0x1.172b840000000p+0f, -0x1.c157420000000p-27f}, {0x1.1a35be0000000p+0f, 0x1.6df96e0000000p-25f},
    {0x1.1d48740000000p+0f, -0x1.d2e8ca0000000p-25f}, {0x1.2063b80000000p+0f, 0x1.0c519a0000000p-25f},
    {0x1.2387a60000000p+0f, 0x1.ceac480000000p-25f}, {0x1.26b4560000000p+0f, 0x1.789f380000000p-26f},
    {0x1.29e9e00000000p+0f, -0x1.5c04240000000p-25f}, {0x1.2d285a0000000p+0f, 0x1.b900c20000000p-26f},
    {0x1.306fe00000000p+0f, 0x1.4636e20000000p-25f}, {0x1.33c08c0000000p+0f, -0x1.b37d200000000p-25f},
    {0x1.371a740000000p+0f, -0x1.18aac60000000p-25f}, {0x1.3a7db40000000p+0f, -0x1.634c020000000p-25f},
    {0x1.3dea640000000p+0f, 0x1.8246840000000p-25f}, {0x1.4160a20000000p+0f, 0x1.f72e2a0000000p-28f},
    {0x1.44e0860000000p+0f, 0x1.8624b40000000p-30f}, {0x1.486a2c0000000p+0f, -0x1.47d8660000000p-25f},
    {0x1.4bfdae0000000p+0f, -0x1.593abc0000000p-25f}, {0x1.4f9b280000000p+0f, -0x1.2c5a6c0000000p-25f},
    {0x1.5342b60000000p+0f, -0x1.2c56100000000p-25f}, {0x1.56f4740000000p+0f, -0x1.295b040000000p-25f},
    {0x1.5ab07e0000000p+0f, -0x1.5bd5ec0000000p-27f}, {0x1.5e76f20000000p+0f, -0x1.4a5bd60000000p-25f},
    {0x1.6247ec0000000p+0f, -0x1.f8b5500000000p-25f}, {0x1.6623880000000p+0f, 0x1.2a91120000000p-27f},
    {0x1.6a09e60000000p+0f, 0x1.9fcef40000000p-26f}, {0x1.6dfb240000000p+0f, -0x1.cd72e80000000p-27f},
    {0x1.71f75e0000000p+0f, 0x1.1d8bee0000000p-25f}, {0x1.75feb60000000p+0f, -0x1.37b3060000000p-25f},
    {0x1.7a11480000000p+0f, -0x1.829fd00000000p-25f}, {0x1.7e2f340000000p+0f, -0x1.2616340000000p-25f},
    {0x1.82589a0000000p+0f, -0x1.accc7c0000000p-26f}, {0x1.868d9a0000000p+0f, -0x1.2edb440000000p-26f},
    {0x1.8ace540000000p+0f, 0x1.15506e0000000p-27f}, {0x1.8f1aea0000000p+0f, -0x1.baa2320000000p-26f},
    {0x1.93737c0000000p+0f, -0x1.e647440000000p-25f}, {0x1.97d82a0000000p+0f, -0x1.0d8d840000000p-31f},
    {0x1.9c49180000000p+0f, 0x1.51f8480000000p-27f}, {0x1.a0c6680000000p+0f, -0x1.2886a60000000p-26f},
    {0x1.a5503c0000000p+0f, -0x1.b83b540000000p-25f}, {0x1.a9e6b60000000p+0f, -0x1.50c0480000000p-25f},
    {0x1.ae89fa0000000p+0f, -0x1.a94b140000000p-26f}, {0x1.b33a2c0000000p+0f, -0x1.ec3a820000000p-26f},
    {0x1.b7f7700000000p+0f, -0x1.a094380000000p-25f}, {0x1.bcc1ea0000000p+0f, -0x1.f687c60000000p-25f},
    {0x1.c199be0000000p+0f, -0x1.3d56b20000000p-27f}, {0x1.c67f120000000p+0f, 0x1.cafa2a0000000p-25f},
    {0x1.cb720e0000000p+0f, -0x1.8837cc0000000p-27f}, {0x1.d072d40000000p+0f, 0x1.40f1300000000p-25f},
    {0x1.d5818e0000000p+0f, -0x1.822dbc0000000p-27f}, {0x1.da9e600000000p+0f, 0x1.ed99420000000p-27f},
    {0x1.dfc9740000000p+0f, -0x1.908c940000000p-25f}, {0x1.e502ee0000000p+0f, 0x1.e2cffe0000000p-26f},
    {0x1.ea4afa0000000p+0f, 0x1.52486c0000000p-27f}, {0x1.efa1be0000000p+0f, 0x1.cc2b440000000p-25f},
    {0x1.f507660000000p+0f, -0x1.246eb00000000p-26f}, {0x1.fa7c180000000p+0f, 0x1.9e90d80000000p-28f},
};
__device__ __forceinline__ df64 df_exp2_tab(int j) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(kExp2TabDF[j]));
  return df64(v.x, v.y);
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
  // r = t - n L2 - n L3 + x.l: the two large parts exactly, the small ones in FP32
  const df64 a = df_two_sum(t, -p2);
  const df64 b = df_two_sum(a.h, x.l);
  const df64 r = df_fast_two_sum(b.h, __fsub_rn(__fsub_rn(__fadd_rn(a.l, b.l), e2), __fmul_rn(n, kL3)));
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
  const df64 T = df_exp2_tab(ni & 63);
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
__device__ __forceinline__ bool is_pos(double x) { return x > 0.0; }
__device__ __forceinline__ bool is_pos(df64 x) { return x.h > 0.f; }
__device__ __forceinline__ bool is_zero(df64 x) { return x.h == 0.f; }
__device__ __forceinline__ df64 recip(df64 x) { return df_rcp(x); }
__device__ __forceinline__ double twice(double x) { return 2.0 * x; }
// The start of a sum: -0 for double (-0 + a = a for every a, so the first
// addition folds away), zero for df64.
template <class F>
__device__ __forceinline__ F acc_zero() {
  return F(0);
}
template <>
__device__ __forceinline__ double acc_zero<double>() {
  return -0.0;
}
__device__ __forceinline__ df64 twice(df64 x) { return df64(__fmul_rn(x.h, 2.f), __fmul_rn(x.l, 2.f)); }

}  // namespace mole
