// walker.cuh -- per-walker Slater-Jastrow state and operations.
//
// One thread owns one walker. Electron, orbital and spin-block indices are
// compile-time (templates on the spin-block sizes NU, ND), so the walker
// state lives in registers for small N.
//
// The state is the positions, the FP64 inverse Slater matrices and caches of
// every one-body term (orbital values, gradients and Laplacians, the e-n
// Jastrow and potential) and every pair term (u, u'/r, u'' + 2u'/r, 1/r) at
// the current configuration. A proposal computes the moved electron's terms
// once; an accepted move copies them into the caches, so the local energy
// after a sweep is assembled from the caches without a single exp, sqrt or
// division.
//
// Arithmetic type R is double (plain method), float (mixed method) or df64
// (FP64-accurate double-float on the FP32 pipe). The inverse matrices, the
// Sherman-Morrison ratio products, the local-energy assembly and every
// accumulation are FP64 for double and float, and df64 for df64 (type F).
#pragma once

#include "common.cuh"
#include "df64.cuh"
#include "fp64.cuh"
#include "nn.cuh"
#include "normal.cuh"

namespace mole {

// FP32 mirror of what the FP64 kernels' single-precision Metropolis screen
// reads (compact.cuh): 1s-STO systems with at most one electron per spin.
struct ScreenParams {
  float nuc[kMaxNuc * 3];
  float zeta[kMaxBasis];
  float coef[2][kMaxBasis];  // orbital 0 of each spin block
  float rmax;                // largest nuclear coordinate magnitude
  float cusp_anti, cusp_para, ee_b;
};

// System description in kernel-parameter memory (broadcast reads).
template <class R>
struct SysParams {
  int n_nuc;
  int n_basis;
  int nuc_b0[kMaxNuc + 1];  // basis functions of nucleus I are [nuc_b0[I], nuc_b0[I+1])
  int b_kind[kMaxBasis];
  int b_exp[kMaxBasis];  // exponent parameter index of basis function b
  int all_sto1s;         // every basis function is a 1s STO
  R nuc_pos[kMaxNuc * 3];
  R nuc_z[kMaxNuc];
  R b_zeta[kMaxBasis];
  R coef[2][kMaxSpin][kMaxBasis];  // [spin][orbital][basis]
  int ee_on, ee_npoly;
  int ee_scaled;  // ee_kappa > 0: the Pade term of the scaled distance (1 - e^-kappa r) / kappa
  R ee_kappa, cusp_anti, cusp_para, ee_b;
  R ee_m2b;  // -2 ee_b
  R ee_poly[kMaxPoly];
  int en_on;
  R en_a;
  R en_coef[kMaxNuc];
  int nn_on;
  int pot_kind;  // 0 Coulomb, 1 harmonic
  R half_omega2;
  double vnn;  // n-n repulsion constant
  R vnn_r;     // the same in R (read by the df64 form)
  int n_exp, P, off_ee, off_en, off_nn;
  const double* nn_theta;  // device copy of the 9,090 network parameters (neural systems)
  const float* nn_tab;     // quintic tables of the pair networks (neural systems, FP32 form)
  ScreenParams scr;
};

template <class R>
__device__ __forceinline__ R rsqrt_t(R x);
template <>
__device__ __forceinline__ double rsqrt_t<double>(double x) {
  return rsqrt64(x);
}
template <>
__device__ __forceinline__ float rsqrt_t<float>(float x) {
  return rsqrtf(x);
}
template <>
__device__ __forceinline__ df64 rsqrt_t<df64>(df64 x) {
  return df_rsqrt(x);
}
template <class R>
__device__ __forceinline__ R exp_t(R x);
template <>
__device__ __forceinline__ double exp_t<double>(double x) {
  return exp64(x);
}
template <>
__device__ __forceinline__ float exp_t<float>(float x) {
  return __expf(x);
}
template <>
__device__ __forceinline__ df64 exp_t<df64>(df64 x) {
  return df_exp(x);
}
// e^(-z r): in FP64 the product is fused into the argument reduction.
template <class R>
__device__ __forceinline__ R expm_t(R z, R r) {
  return exp_t<R>(-(z * r));
}
template <>
__device__ __forceinline__ double expm_t<double>(double z, double r) {
  return expab64(-z, r);
}
// 1 / x: two FP64 instructions in FP64, IEEE division in FP32, Newton in df64.
template <class R>
__device__ __forceinline__ R recip_t(R x) {
  return (R)1 / x;
}
template <>
__device__ __forceinline__ double recip_t<double>(double x) {
  return rcp64(x);
}
template <>
__device__ __forceinline__ df64 recip_t<df64>(df64 x) {
  return df_rcp(x);
}

// One electron's orbitals of its spin block (value, gradient, Laplacian),
// e-n Jastrow (value, gradient, Laplacian, d/da), e-n potential and the
// exponent derivatives sum_{b in p} coef[k][b] d chi_b / d zeta_p.
template <class R, int n, int NZ>
struct OneBody {
  static constexpr int nm = n > 0 ? n : 1;
  static constexpr int pm = NZ > 0 ? NZ : 1;
  R val[nm];
  R grad[nm][3];
  R lap[nm];
  R dz[nm][pm];
  R jen, gjen[3], ljen, djen;
  R ven;
};

// Neural-Jastrow context of a thread: the CTA's shared weights and this
// thread's hidden-layer jet scratch (element stride `stride`).
template <class R>
struct NnCtx {
  const NnShared<R>* sh;
  R* scr;
  int stride;
};

template <class R, int n, int NZ, bool EN, bool NN = false>
__device__ __forceinline__ void one_body(const SysParams<R>& sp, int spin, const R (&r)[3], OneBody<R, n, NZ>& o,
                                         const NnCtx<R>* nn = nullptr) {
#pragma unroll
  for (int k = 0; k < OneBody<R, n, NZ>::nm; ++k) {
    o.val[k] = 0;
    o.grad[k][0] = o.grad[k][1] = o.grad[k][2] = 0;
    o.lap[k] = 0;
#pragma unroll
    for (int p = 0; p < OneBody<R, n, NZ>::pm; ++p) o.dz[k][p] = 0;
  }
  o.jen = 0;
  o.gjen[0] = o.gjen[1] = o.gjen[2] = 0;
  o.ljen = 0;
  o.djen = 0;
  o.ven = 0;
  #pragma unroll 1
  for (int I = 0; I < sp.n_nuc; ++I) {
    const R d0 = r[0] - sp.nuc_pos[3 * I], d1 = r[1] - sp.nuc_pos[3 * I + 1], d2 = r[2] - sp.nuc_pos[3 * I + 2];
    const R r2 = d0 * d0 + d1 * d1 + d2 * d2;
    const R inv = rsqrt_t<R>(r2);
    const R rr = r2 * inv;
    o.ven -= sp.nuc_z[I] * inv;
    // one basis function b of compile-time kind K (K < 0: read at run time);
    // a system whose basis is all 1s STOs takes a loop without the kind
    // branches, which the compiler would otherwise turn into predicated FP64
    // instructions of every kind
    auto basis = [&](auto kc, int b) {
      constexpr int K = decltype(kc)::value;
      const int kind = K >= 0 ? K : sp.b_kind[b];
      const R z = sp.b_zeta[b];
      const bool gto = kind == kGto1s;
      const R rad = gto ? r2 : rr;
      R e = expm_t<R>(z, rad);
      // with one orbital the coefficient is folded into e: every basis value
      // below is linear in e
      if constexpr (n == 1) e *= sp.coef[spin][0][b];
      // chi, its gradient fr d (+ e along one axis for 2p), its Laplacian
      // la lb, d chi / dz = -rad chi
      R chi, fr, la, lb;
      int ax = -1;
      if (gto) {
        chi = e;
        fr = (R)-2 * z * e;
        la = fr;
        lb = (R)3 - z * r2 - z * r2;  // lap = e (4 z^2 r^2 - 6 z)
      } else if (kind == kSto1s) {
        chi = e;
        la = z * e;
        fr = -la * inv;
        lb = z - (R)2 * inv;  // lap = z e (z - 2 / r)
      } else if (kind == kSto2s) {
        chi = rr * e;
        fr = e * ((R)1 - z * rr) * inv;
        la = e;
        lb = z * z * rr - (R)4 * z + (R)2 * inv;
      } else {
        ax = kind - kSto2px;
        const R da = ax == 0 ? d0 : (ax == 1 ? d1 : d2);
        chi = da * e;
        la = z * chi;
        fr = -la * inv;
        lb = z - (R)4 * inv;  // lap = z chi (z - 4 / r)
      }
      const int ix = sp.b_exp[b];
      if constexpr (n == 1) {
        o.val[0] += chi;
        if (ax < 0) {
          o.grad[0][0] += fr * d0;
          o.grad[0][1] += fr * d1;
          o.grad[0][2] += fr * d2;
        } else {  // 2p: + e along its axis
          o.grad[0][0] += fr * d0 + (ax == 0 ? e : (R)0);
          o.grad[0][1] += fr * d1 + (ax == 1 ? e : (R)0);
          o.grad[0][2] += fr * d2 + (ax == 2 ? e : (R)0);
        }
        o.lap[0] += la * lb;
        if constexpr (NZ > 0) {
#pragma unroll
          for (int p = 0; p < NZ; ++p)
            if (p == ix) o.dz[0][p] -= rad * chi;
        }
      } else {
        const R l = la * lb;
        const R dzb = -rad * chi;
#pragma unroll
        for (int k = 0; k < n; ++k) {
          const R c = sp.coef[spin][k][b];
          const R cf = c * fr;
          o.val[k] += c * chi;
          if (ax < 0) {
            o.grad[k][0] += cf * d0;
            o.grad[k][1] += cf * d1;
            o.grad[k][2] += cf * d2;
          } else {  // 2p: + c e along its axis
            const R ce = c * e;
            o.grad[k][0] += cf * d0 + (ax == 0 ? ce : (R)0);
            o.grad[k][1] += cf * d1 + (ax == 1 ? ce : (R)0);
            o.grad[k][2] += cf * d2 + (ax == 2 ? ce : (R)0);
          }
          o.lap[k] += c * l;
          if constexpr (NZ > 0) {
#pragma unroll
            for (int p = 0; p < NZ; ++p)
              if (p == ix) o.dz[k][p] += c * dzb;
          }
        }
      }
    };
    const int b1 = sp.nuc_b0[I + 1];
    if (sp.all_sto1s) {
      #pragma unroll 1
      for (int b = sp.nuc_b0[I]; b < b1; ++b) basis(std::integral_constant<int, kSto1s>{}, b);
    } else {
      #pragma unroll 1
      for (int b = sp.nuc_b0[I]; b < b1; ++b) basis(std::integral_constant<int, -1>{}, b);
    }
    if (EN) {
      // Pade e-n term A r / (1 + a r): value, gradient A q^2 d / r,
      // Laplacian 2 A q^2 (1/r - a q), d/da -A r^2 q^2, q = 1 / (1 + a r)
      const R A = sp.en_coef[I];
      const R q = recip_t<R>((R)1 + sp.en_a * rr);
      const R Aq = A * q;
      const R Aq2 = Aq * q;
      const R du = Aq2 * inv;
      o.jen += Aq * rr;
      o.gjen[0] += du * d0;
      o.gjen[1] += du * d1;
      o.gjen[2] += du * d2;
      o.ljen += (Aq2 + Aq2) * (inv - sp.en_a * q);
      if constexpr (NZ > 0) o.djen -= Aq2 * rr * rr;
    }
    if constexpr (NN) {
      R y, y1, y2;
      if constexpr (std::is_same<R, float>::value) nn_tab_eval(sp.nn_tab, 2 + I, rr, y, y1, y2);
      else nn_jet<R>(nn->sh->net[1], rr, sp.nuc_z[I], nn->scr, nn->stride, y, y1, y2);
      const R f = y1 * inv;
      o.jen += y;
      o.gjen[0] += f * d0;
      o.gjen[1] += f * d1;
      o.gjen[2] += f * d2;
      o.ljen += y2 + (R)2 * f;
    }
  }
}

// Pair term values: u, f = u'/r, l = u'' + 2u'/r, 1/r, du/db and du/d b_p.
template <class R, int PM>
struct PairVals {
  R u, f, l, inv, db;
  R rs;  // scaled distance R(r) of the Pade term
};

// Pade pair term (theory/jastrow.tex:15-126) at separation d = r_i - r_j,
// plus the e-e network when NN.
template <class R, int PM, bool NN = false>
__device__ __forceinline__ void pair_vals(const SysParams<R>& sp, bool same, R d0, R d1, R d2, PairVals<R, PM>& v,
                                          const NnCtx<R>* nn = nullptr) {
  const R r2 = d0 * d0 + d1 * d1 + d2 * d2;
  const R inv = rsqrt_t<R>(r2);
  const R r = r2 * inv;
  v.inv = inv;
  v.db = 0;
  v.rs = r;
  R yn = 0, fn = 0, ln = 0;  // the e-e network's u, u'/r, u'' + 2u'/r
  if constexpr (NN) {
    R y, y1, y2;
    if constexpr (std::is_same<R, float>::value) nn_tab_eval(sp.nn_tab, same ? 0 : 1, r, y, y1, y2);
    else nn_jet<R>(nn->sh->net[0], r, same ? (R)1 : (R)0, nn->scr, nn->stride, y, y1, y2);
    yn = y;
    fn = y1 * inv;
    ln = y2 + (R)2 * fn;
  }
  if (!sp.ee_on) {
    v.u = yn;
    v.f = fn;
    v.l = ln;
    return;
  }
  const R cusp = same ? sp.cusp_para : sp.cusp_anti;
  R val, f, l;
  if (sp.ee_scaled) {
    // Pade term of the scaled distance Rs = (1 - e^-kappa r) / kappa
    const R e = exp_t<R>(-sp.ee_kappa * r);
    const R Rs = ((R)1 - e) / sp.ee_kappa;
    const R Rp = e, Rpp = -sp.ee_kappa * e;
    const R q = recip_t<R>((R)1 + sp.ee_b * Rs);
    val = cusp * Rs * q;
    R uR = cusp * q * q;
    R uRR = (R)-2 * cusp * sp.ee_b * q * q * q;
    if constexpr (PM > 0) v.db = -cusp * Rs * Rs * q * q;
    R Rk = Rs, Rk2 = 1;  // R^(p-1), R^(p-2)
    #pragma unroll 1
    for (int i = 0; i < sp.ee_npoly; ++i) {
      const R p = (R)(i + 2), c = sp.ee_poly[i];
      val += c * Rk * Rs;
      uR += p * c * Rk;
      uRR += p * (p - (R)1) * c * Rk2;
      Rk2 = Rk;
      Rk *= Rs;
    }
    f = uR * Rp * inv;
    l = uRR * Rp * Rp + uR * Rpp + (R)2 * f;
    v.rs = Rs;
  } else {
    // u = c r q, u' = c q^2, u'' = -2 b c q^3, du/db = -c r^2 q^2, q = 1 / (1 + b r)
    const R q = recip_t<R>((R)1 + sp.ee_b * r);
    const R cq = cusp * q;
    R uR = cq * q;
    val = cq * r;
    R uRR = sp.ee_m2b * q * uR;
    if constexpr (PM > 0) v.db = -(r2 * uR);
    R Rk = r, Rk2 = 1;  // r^(p-1), r^(p-2)
    #pragma unroll 1
    for (int i = 0; i < sp.ee_npoly; ++i) {
      const R p = (R)(i + 2), c = sp.ee_poly[i];
      val += c * Rk * r;
      uR += p * c * Rk;
      uRR += p * (p - (R)1) * c * Rk2;
      Rk2 = Rk;
      Rk *= r;
    }
    f = uR * inv;
    l = uRR + (R)2 * f;
  }
  if constexpr (NN) {
    v.u = yn + val;
    v.f = fn + f;
    v.l = ln + l;
  } else {
    v.u = val;
    v.f = f;
    v.l = l;
  }
}

// The Metropolis test ratio^2 exp(x) > u, u = u01(ubits) >= 2^-33. With
// |x| < 80 and 1e-30 < ratio^2 < 1e30 the FP32 value of ratio^2 exp(x) (from
// ratio and x truncated to 24 bits) is within 3e-5 relative of the exact one
// while it is a normal float, and it
// under- (over-) flows only when the exact value is below 1e-38 (above
// 3e38), i.e. far below (above) any u; so where it is clear of u by 1e-3
// relative it decides exactly as the FP64 test. Everything else takes the
// FP64 expression. Same decisions as FP64, the FP64 exp skipped in all but
// borderline and extreme cases.
// The FP64 expression of the test, as a call (a branch the compiler cannot
// turn into predicated FP64 instructions on the screened path).
static __device__ __noinline__ bool metropolis_fp64(double ratio, double x, uint32_t ubits) {
  return ratio * ratio * exp(x) > u01<double>(ubits);
}
// The test for x = 2 dj, the doubling done in FP32 (exact) and, in the
// borderline case, in FP64.
__device__ __forceinline__ bool metropolis_accept_dj(double ratio, double dj, uint32_t ubits) {
  const float rf = d2f_rz(ratio), xf = 2.f * d2f_rz(dj);
  const float r2 = rf * rf;
  if (fabsf(xf) < 80.f && r2 > 1e-30f && r2 < 1e30f) {
    const float uf = u01<float>(ubits);
    const float d = r2 * __expf(xf) - uf;
    if (fabsf(d) > 1e-3f * uf) return d > 0.f;
  }
  return metropolis_fp64(ratio, dj + dj, ubits);
}
__device__ __forceinline__ bool metropolis_accept(double ratio, double x, uint32_t ubits) {
  const float rf = d2f_rz(ratio), xf = d2f_rz(x);  // truncated: no FP64-pipe conversion
  const float r2 = rf * rf;
  if (fabsf(xf) < 80.f && r2 > 1e-30f && r2 < 1e30f) {
    const float uf = u01<float>(ubits);
    const float d = r2 * __expf(xf) - uf;
    if (fabsf(d) > 1e-3f * uf) return d > 0.f;
  }
  return ratio * ratio * exp(x) > u01<double>(ubits);
}
// The same test for double-float ratio and exponent: the high words are the
// values rounded to FP32, so the screen above holds unchanged; borderline
// cases decide in FP64 on the double-float values.
__device__ __forceinline__ bool metropolis_accept(df64 ratio, df64 x, uint32_t ubits) {
  const float r2 = ratio.h * ratio.h;
  if (fabsf(x.h) < 80.f && r2 > 1e-30f && r2 < 1e30f) {
    const float uf = u01<float>(ubits);
    const float d = r2 * __expf(x.h) - uf;
    if (fabsf(d) > 1e-3f * uf) return d > 0.f;
  }
  const double rd = (double)ratio;
  return rd * rd * exp((double)x) > u01<double>(ubits);
}

// Pivot magnitude of the Gauss-Jordan elimination.
__device__ __forceinline__ double piv_mag(double x) { return fabs(x); }
__device__ __forceinline__ float piv_mag(df64 x) { return fabsf(x.h); }

// In-register Gauss-Jordan inverse with partial pivoting; row swaps are
// predicated so that every index stays compile-time.
template <int n, class T>
__device__ __forceinline__ bool gj_invert(T (&a)[n * n], T (&inv)[n * n], double* lndet, double* sign) {
#pragma unroll
  for (int i = 0; i < n * n; ++i) inv[i] = (i / n == i % n) ? T(1) : T(0);
  double ld = 0.0, sg = 1.0;
  bool ok = true;
#pragma unroll
  for (int col = 0; col < n; ++col) {
    int piv = col;
    auto best = piv_mag(a[col * n + col]);
#pragma unroll
    for (int r = col + 1; r < n; ++r)
      if (piv_mag(a[r * n + col]) > best) {
        best = piv_mag(a[r * n + col]);
        piv = r;
      }
#pragma unroll
    for (int r = col + 1; r < n; ++r)
      if (r == piv) {
#pragma unroll
        for (int j = 0; j < n; ++j) {
          T t = a[col * n + j];
          a[col * n + j] = a[r * n + j];
          a[r * n + j] = t;
          t = inv[col * n + j];
          inv[col * n + j] = inv[r * n + j];
          inv[r * n + j] = t;
        }
        sg = -sg;
      }
    const T p = a[col * n + col];
    ok = ok && !is_zero(p);
    if (lndet) ld += log(fabs(to_d(p)));
    if (is_neg(p)) sg = -sg;
    const T ip = recip(p);
#pragma unroll
    for (int j = 0; j < n; ++j) {
      a[col * n + j] *= ip;
      inv[col * n + j] *= ip;
    }
#pragma unroll
    for (int r = 0; r < n; ++r) {
      if (r == col) continue;
      const T f = a[r * n + col];
#pragma unroll
      for (int j = 0; j < n; ++j) {
        a[r * n + j] -= f * a[col * n + j];
        inv[r * n + j] -= f * inv[col * n + j];
      }
    }
  }
  if (lndet) *lndet = ld;
  if (sign) *sign = sg;
  return ok;
}

// Walker state and moves for spin blocks of NU up and ND down electrons;
// PM > 0 also caches what the first PM parameter derivatives need; EN
// compiles the e-n Jastrow term in (its caches fold away when it is off).
template <int NU, int ND, class R, int PM, bool EN, bool NN = false>
struct Walker {
  NnCtx<R> nn;  // shared-memory weights and jet scratch when NN
  static constexpr int N = NU + ND;
  static constexpr int NDm = ND > 0 ? ND : 1;
  static constexpr int NMAX = NU > NDm ? NU : NDm;
  static constexpr int NP = N * (N - 1) / 2;
  static constexpr int NPm = NP > 0 ? NP : 1;
  static constexpr int PMC = PM > 0 ? PM : 1;
  // exponent-derivative slots cached: one for the two-parameter kernel
  static constexpr int NZ = PM == 0 ? 0 : (PM == 2 ? 1 : PM);
  static constexpr int NZC = NZ > 0 ? NZ : 1;
  using SP = SysParams<R>;
  // FP64-part type: double, or df64 in the double-float form
  static constexpr bool DF = is_df64<R>::value;
  using F = typename std::conditional<DF, df64, double>::type;

  // R -> F and F -> R for the FP32 form without FP64-pipe conversions (f2d is
  // exact; d2f_rz truncates to 24 bits); identities otherwise
  static __device__ __forceinline__ F to_f(R v) {
    if constexpr (F32) return f2d(v);
    else return (F)v;
  }
  static __device__ __forceinline__ R to_r(F v) {
    if constexpr (F32) return d2f_rz_small(v);  // positions: below FP32's largest
    else return (R)v;
  }

  F x[N][3];
  F bu[NU * NU];    // inverse of the up Slater matrix, bu[k*NU+i]
  F bd[NDm * NDm];  // inverse of the down Slater matrix
  // df64 form: set when a value left the range where double-float keeps
  // FP64 accuracy (the launch is then rerun in native FP64)
  bool oor = false;
  // The FP32 form's drift-diffusion move computes drifts and Green's-function
  // sums in FP32 from an FP32 copy of the inverses (set at every refresh and
  // every accepted drift move); ratios and updates stay on the FP64 ones.
  static constexpr bool F32 = std::is_same<R, float>::value;
  using D = typename std::conditional<F32, float, F>::type;  // drift arithmetic
  float bfu[F32 ? NU * NU : 1];
  float bfd[F32 ? NDm * NDm : 1];
  // one-body caches
  R og[N][NMAX][3], ol[N][NMAX];
  R odz[N][NMAX][NZC];
  R jen[N], gjen[N][3], ljen[N], djen[N], ven[N];
  // pair caches, pair (i, j), i < j
  R pu[NPm], pf[NPm], pl[NPm], pinv[NPm], pdb[NPm], prs[NPm];

  static constexpr __device__ int pidx(int i, int j) {
    return i < j ? i * N - i * (i + 1) / 2 + (j - i - 1) : j * N - j * (j + 1) / 2 + (i - j - 1);
  }
  static constexpr __device__ bool same_spin(int i, int j) { return (i < NU) == (j < NU); }

  __device__ __forceinline__ void load(const double* pos, int W, int w) {
#pragma unroll
    for (int e = 0; e < N; ++e)
#pragma unroll
      for (int c = 0; c < 3; ++c) x[e][c] = F(pos[(size_t)(3 * e + c) * W + w]);
  }
  __device__ __forceinline__ void store(double* pos, int W, int w) const {
#pragma unroll
    for (int e = 0; e < N; ++e)
#pragma unroll
      for (int c = 0; c < 3; ++c) pos[(size_t)(3 * e + c) * W + w] = to_d(x[e][c]);
  }
  __device__ __forceinline__ void rpos(int e, R (&r)[3]) const {
    r[0] = to_r(x[e][0]);
    r[1] = to_r(x[e][1]);
    r[2] = to_r(x[e][2]);
  }

  template <int e, int n>
  __device__ __forceinline__ void put_one_body(const OneBody<R, n, NZ>& o) {
#pragma unroll
    for (int k = 0; k < n; ++k) {
      og[e][k][0] = o.grad[k][0];
      og[e][k][1] = o.grad[k][1];
      og[e][k][2] = o.grad[k][2];
      ol[e][k] = o.lap[k];
      if constexpr (NZ > 0)
#pragma unroll
        for (int p = 0; p < NZ; ++p) odz[e][k][p] = o.dz[k][p];
    }
    jen[e] = o.jen;
    gjen[e][0] = o.gjen[0];
    gjen[e][1] = o.gjen[1];
    gjen[e][2] = o.gjen[2];
    ljen[e] = o.ljen;
    djen[e] = o.djen;
    ven[e] = o.ven;
  }
  __device__ __forceinline__ void put_pair(int p, const PairVals<R, PM>& v) {
    pu[p] = v.u;
    pf[p] = v.f;
    pl[p] = v.l;
    pinv[p] = v.inv;
    if constexpr (PM > 0) {
      pdb[p] = v.db;
      prs[p] = v.rs;
    }
  }

  // Rebuilds the inverses in FP64 from fresh orbital values and every cache.
  // Returns false on a singular block.
  __device__ bool refresh(const SP& sp, double* lndet, double* sign) {
    F au[NU * NU], ad[NDm * NDm];
    static_for<0, N>([&](auto ec) {
      constexpr int e = decltype(ec)::value;
      constexpr bool isup = e < NU;
      constexpr int n = isup ? NU : ND;
      constexpr int i = isup ? e : e - NU;
      R r[3];
      rpos(e, r);
      OneBody<R, n, NZ> o;
      one_body<R, n, NZ, EN, NN>(sp, isup ? 0 : 1, r, o, &nn);
#pragma unroll
      for (int k = 0; k < n; ++k) {
        if constexpr (isup) au[i * NU + k] = (F)o.val[k];
        else ad[i * NDm + k] = (F)o.val[k];
      }
      put_one_body<e, n>(o);
    });
    double l1 = 0.0, s1 = 1.0, l2 = 0.0, s2 = 1.0;
    bool ok = gj_invert<NU>(au, bu, lndet ? &l1 : nullptr, &s1);
    if constexpr (ND > 0) ok = gj_invert<ND>(ad, bd, lndet ? &l2 : nullptr, &s2) && ok;
    if constexpr (F32) {
#pragma unroll
      for (int k = 0; k < NU * NU; ++k) bfu[k] = d2f_rz(bu[k]);
#pragma unroll
      for (int k = 0; k < (ND > 0 ? ND * ND : 0); ++k) bfd[k] = d2f_rz(bd[k]);
    }
    if constexpr (DF) check_range<NU>(bu), check_range<ND>(bd);
    F J = F(0);
#pragma unroll
    for (int e = 0; e < N; ++e) J += (F)jen[e];
    static_for<0, N>([&](auto ic) {
      constexpr int i = decltype(ic)::value;
      static_for<i + 1, N>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        PairVals<R, PM> v;
        pair_vals<R, PM, NN>(sp, same_spin(i, j), (R)(x[i][0] - x[j][0]), (R)(x[i][1] - x[j][1]),
                             (R)(x[i][2] - x[j][2]), v, &nn);
        put_pair(pidx(i, j), v);
        J += (F)v.u;
      });
    });
    if (lndet) *lndet = l1 + l2 + to_d(J);
    if (sign) *sign = s1 * s2;
    return ok;
  }

  // df64 form: inverse entries beyond 2^96 mean orbital values near the
  // bottom of FP32's exponent range, where double-float loses digits
  template <int n, class B>
  __device__ __forceinline__ void check_range(const B& b) {
    if constexpr (n > 0) {
      bool in = true;  // NaN compares false, so it counts as out of range
#pragma unroll
      for (int k = 0; k < n * n; ++k) in = in && (piv_mag(b[k]) < 0x1p96f);
      if (!in) oor = true;
    }
  }

  // grad ln det at electron j from the caches and the inverse B
  template <int j>
  __device__ __forceinline__ void det_grad(F (&g)[3]) const {
    constexpr bool isup = j < NU;
    constexpr int n = isup ? NU : ND;
    constexpr int i = isup ? j : j - NU;
    constexpr int ld = isup ? NU : NDm;
    const F* B = isup ? bu : bd;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      F s = F(0);
#pragma unroll
      for (int k = 0; k < n; ++k) s += to_f(og[j][k][c]) * B[k * ld + i];
      g[c] = s;
    }
  }
  // grad ln det at electron j in the drift arithmetic (FP32 copy of B in the FP32 form)
  template <int j>
  __device__ __forceinline__ void det_grad_d(D (&g)[3]) const {
    if constexpr (F32) {
      constexpr bool isup = j < NU;
      constexpr int n = isup ? NU : ND;
      constexpr int i = isup ? j : j - NU;
      constexpr int ld = isup ? NU : NDm;
      const float* B = isup ? bfu : bfd;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < n; ++k) s += og[j][k][c] * B[k * ld + i];
        g[c] = s;
      }
    } else {
      det_grad<j>(g);
    }
  }
  // grad J at electron j from the caches
  template <int j>
  __device__ __forceinline__ void jas_grad(R (&g)[3]) const {
    g[0] = gjen[j][0];
    g[1] = gjen[j][1];
    g[2] = gjen[j][2];
#pragma unroll
    for (int m = 0; m < N; ++m) {
      if (m == j) continue;
      const R f = pf[pidx(j, m)];
      g[0] += f * to_r(x[j][0] - x[m][0]);
      g[1] += f * to_r(x[j][1] - x[m][1]);
      g[2] += f * to_r(x[j][2] - x[m][2]);
    }
  }

  // One Metropolis move of electron e; returns 1 when accepted.
  template <int MOVE, int e>
  __device__ __forceinline__ int move(const SP& sp, R step, uint64_t seed, uint32_t wid, uint32_t t) {
    constexpr bool isup = e < NU;
    constexpr int n = isup ? NU : ND;
    constexpr int i = isup ? e : e - NU;
    constexpr bool DRIFT = MOVE == kMoveDiffuse;
    constexpr int ld = isup ? NU : NDm;
    F* B = isup ? bu : bd;

    // drift at the current configuration (diffuse moves)
    D vcur[N][3];
    if constexpr (DRIFT) {
      static_for<0, N>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        D gdj[3];
        R gjj[3];
        det_grad_d<j>(gdj);
        jas_grad<j>(gjj);
#pragma unroll
        for (int c = 0; c < 3; ++c) vcur[j][c] = gdj[c] + (D)gjj[c];
      });
    }

    const uint4 ra = draw4(seed, wid, t, 2u * e, kTagMove);
    F dx[3];
    F xn[3];
    R uacc;
    uint32_t ubits;
    // FP64 box and Gaussian moves: x + step v with one rounding (v = u - 1/2
    // exactly, or the FP32 normal)
    constexpr bool FMA_PROPOSAL = std::is_same<R, double>::value && !DRIFT;
    if constexpr (FMA_PROPOSAL && MOVE == kMoveBox) {
      xn[0] = fma(step, u01_centered(ra.x), x[e][0]);
      xn[1] = fma(step, u01_centered(ra.y), x[e][1]);
      xn[2] = fma(step, u01_centered(ra.z), x[e][2]);
      ubits = ra.w;
    } else if constexpr (FMA_PROPOSAL) {
      float z0, z1, z2, z3;
      repro_box_muller(ra.x, ra.y, z0, z1);
      repro_box_muller(ra.z, ra.w, z2, z3);
      const uint4 rb = draw4(seed, wid, t, 2u * e + 1u, kTagMove);
      ubits = rb.x;
      xn[0] = fma(step, f2d(z0), x[e][0]);
      xn[1] = fma(step, f2d(z1), x[e][1]);
      xn[2] = fma(step, f2d(z2), x[e][2]);
    } else if constexpr (MOVE == kMoveBox) {
      dx[0] = (F)(step * (u01<R>(ra.x) - (R)0.5));
      dx[1] = (F)(step * (u01<R>(ra.y) - (R)0.5));
      dx[2] = (F)(step * (u01<R>(ra.z) - (R)0.5));
      uacc = u01<R>(ra.w);
      ubits = ra.w;
    } else {
      float z0, z1, z2, z3;
      repro_box_muller(ra.x, ra.y, z0, z1);
      repro_box_muller(ra.z, ra.w, z2, z3);
      const uint4 rb = draw4(seed, wid, t, 2u * e + 1u, kTagMove);
      uacc = u01<R>(rb.x);
      ubits = rb.x;
      if constexpr (MOVE == kMoveGauss && DF) {
        dx[0] = df_mul(step, z0);
        dx[1] = df_mul(step, z1);
        dx[2] = df_mul(step, z2);
      } else if constexpr (MOVE == kMoveGauss) {
        dx[0] = (double)step * f2d(z0);
        dx[1] = (double)step * f2d(z1);
        dx[2] = (double)step * f2d(z2);
      } else if constexpr (DF) {
        const F sq = df_sqrt(step);
        dx[0] = step * vcur[e][0] + df_mul(sq, z0);
        dx[1] = step * vcur[e][1] + df_mul(sq, z1);
        dx[2] = step * vcur[e][2] + df_mul(sq, z2);
      } else if constexpr (F32) {
        const float sq = sqrtf(step);
        dx[0] = f2d(step * vcur[e][0] + sq * z0);
        dx[1] = f2d(step * vcur[e][1] + sq * z1);
        dx[2] = f2d(step * vcur[e][2] + sq * z2);
      } else {
        const double sq = sqrt((double)step);
        dx[0] = (double)step * vcur[e][0] + sq * (double)z0;
        dx[1] = (double)step * vcur[e][1] + sq * (double)z1;
        dx[2] = (double)step * vcur[e][2] + sq * (double)z2;
      }
    }
    if constexpr (!FMA_PROPOSAL) {
      xn[0] = x[e][0] + dx[0];
      xn[1] = x[e][1] + dx[1];
      xn[2] = x[e][2] + dx[2];
    }
    const R rn[3] = {to_r(xn[0]), to_r(xn[1]), to_r(xn[2])};  // as every other FP32 position
    OneBody<R, n, NZ> o;
    one_body<R, n, NZ, EN, NN>(sp, isup ? 0 : 1, rn, o, &nn);
    F ratio = F(0);
#pragma unroll
    for (int k = 0; k < n; ++k) ratio += to_f(o.val[k]) * B[k * ld + i];

    // new pair terms of electron e (without one-body Jastrow terms the sum
    // starts at -0, so that its first addition folds away)
    R dJ;
    if constexpr (EN || NN) dJ = o.jen - jen[e];
    else dJ = acc_zero<R>();
    PairVals<R, PM> pv[N];
    static_for<0, N>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      if constexpr (j != e) {
        pair_vals<R, PM, NN>(sp, same_spin(e, j), rn[0] - to_r(x[j][0]), rn[1] - to_r(x[j][1]), rn[2] - to_r(x[j][2]), pv[j],
                             &nn);
        dJ += pv[j].u - pu[pidx(e, j)];
      }
    });

    bool acc;
    F bn[n * n];
    float bnf[F32 ? n * n : 1];
    if constexpr (!DRIFT) {
      if constexpr (std::is_same<R, double>::value) {
        acc = metropolis_accept_dj(ratio, dJ, ubits);
      } else if constexpr (DF) {
        acc = metropolis_accept(ratio, twice(dJ), ubits);
      } else {
        // ratio^2 e^(2 dJ) > u screened in FP32 (the truncated ratio is within
        // 2^-23, the product within about 2.4e-7 relative), the FP64
        // expression deciding only within 1e-3 of u: the same decisions
        const float ef = exp_t<R>((R)2 * dJ);
        const float rf = d2f_rz(ratio);
        const float r2 = rf * rf;
        const float dd = r2 * ef - uacc;
        if (r2 > 1e-30f && r2 < 1e30f && ef < 1e30f && fabsf(dd) > 1e-3f * uacc) acc = dd > 0.f;
        else acc = ratio * ratio * f2d(ef) > f2d(uacc);
      }
    } else {
      // tentative inverse after replacing row i
      F v[n];
#pragma unroll
      for (int j = 0; j < n; ++j) {
        F s = F(0);
#pragma unroll
        for (int k = 0; k < n; ++k) s += to_f(o.val[k]) * B[k * ld + j];
        v[j] = s;
      }
      const F ir = recip(ratio);
#pragma unroll
      for (int k = 0; k < n; ++k) {
        const F ck = B[k * ld + i] * ir;
#pragma unroll
        for (int j = 0; j < n; ++j) bn[k * n + j] = B[k * ld + j] - ck * (v[j] - (j == i ? F(1) : F(0)));
      }
      if constexpr (F32)
#pragma unroll
        for (int k = 0; k < n * n; ++k) bnf[k] = d2f_rz(bn[k]);
      // Green's function ratio over every electron (metrop.rs:182-195) with
      // the drift at the proposed configuration
      D hi = 0, lo = 0;
      static_for<0, N>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        constexpr bool jup = j < NU;
        D vn[3];
        // determinant part
        if constexpr (jup == isup) {
          constexpr int ij = jup ? j : j - NU;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            D g = 0;
#pragma unroll
            for (int k = 0; k < n; ++k) {
              if constexpr (F32) g += (j == e ? o.grad[k][c] : og[j][k][c]) * bnf[k * n + ij];
              else g += (F)(j == e ? o.grad[k][c] : og[j][k][c]) * bn[k * n + ij];
            }
            vn[c] = g;
          }
        } else {
          det_grad_d<j>(vn);
        }
        // Jastrow part
        R gj[3];
        if constexpr (j == e) {
          gj[0] = o.gjen[0];
          gj[1] = o.gjen[1];
          gj[2] = o.gjen[2];
#pragma unroll
          for (int m = 0; m < N; ++m) {
            if (m == e) continue;
            gj[0] += pv[m].f * (rn[0] - to_r(x[m][0]));
            gj[1] += pv[m].f * (rn[1] - to_r(x[m][1]));
            gj[2] += pv[m].f * (rn[2] - to_r(x[m][2]));
          }
        } else {
          jas_grad<j>(gj);
          const R fo = pf[pidx(j, e)], fn = pv[j].f;
          gj[0] += fn * (to_r(x[j][0]) - rn[0]) - fo * to_r(x[j][0] - x[e][0]);
          gj[1] += fn * (to_r(x[j][1]) - rn[1]) - fo * to_r(x[j][1] - x[e][1]);
          gj[2] += fn * (to_r(x[j][2]) - rn[2]) - fo * to_r(x[j][2] - x[e][2]);
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const D dj = (j == e) ? to_r(dx[c]) : (D)0;  // D is R in every form
          const D a = -dj - (D)step * (vn[c] + (D)gj[c]);
          const D b = dj - (D)step * vcur[j][c];
          hi += a * a;
          lo += b * b;
        }
      });
      const D la = (D)2 * (D)dJ - (hi - lo) / ((D)2 * (D)step);
      acc = is_pos(ratio) && metropolis_accept(ratio, to_f(la), ubits);
    }
    if (!acc) return 0;

    // commit
    x[e][0] = xn[0];
    x[e][1] = xn[1];
    x[e][2] = xn[2];
    put_one_body<e, n>(o);
    static_for<0, N>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      if constexpr (j != e) put_pair(pidx(e, j), pv[j]);
    });
    if constexpr (DRIFT) {
#pragma unroll
      for (int k = 0; k < n * n; ++k) B[(k / n) * ld + (k % n)] = bn[k];
      if constexpr (DF) {
        bool in = true;
#pragma unroll
        for (int k = 0; k < n * n; ++k) in = in && (piv_mag(bn[k]) < 0x1p96f);
        if (!in) oor = true;
      }
      if constexpr (F32) {
        float* Bf = isup ? bfu : bfd;
#pragma unroll
        for (int k = 0; k < n * n; ++k) Bf[(k / n) * ld + (k % n)] = bnf[k];
      }
    } else {
      if constexpr (n == 1) {
        // a 1 x 1 block: the inverse is the reciprocal of the new orbital value
        B[0] = recip(to_f(o.val[0]));
        if constexpr (DF)
          if (!(piv_mag(B[0]) < 0x1p96f)) oor = true;
      } else {
      // Sherman-Morrison row update (FP64)
      F v[n], col[n];
#pragma unroll
      for (int j = 0; j < n; ++j) {
        F s = F(0);
#pragma unroll
        for (int k = 0; k < n; ++k) s += to_f(o.val[k]) * B[k * ld + j];
        v[j] = s;
      }
      const F ir = recip(ratio);
#pragma unroll
      for (int k = 0; k < n; ++k) col[k] = B[k * ld + i] * ir;
#pragma unroll
      for (int k = 0; k < n; ++k)
#pragma unroll
        for (int j = 0; j < n; ++j) B[k * ld + j] -= col[k] * (v[j] - (j == i ? F(1) : F(0)));
      if constexpr (DF) {
        bool in = true;
#pragma unroll
        for (int k = 0; k < n; ++k)
#pragma unroll
          for (int j = 0; j < n; ++j) in = in && (piv_mag(B[k * ld + j]) < 0x1p96f);
        if (!in) oor = true;
      }
      }
    }
    return 1;
  }

  template <int MOVE>
  __device__ __forceinline__ int sweep(const SP& sp, R step, uint64_t seed, uint32_t wid, uint32_t t) {
    int acc = 0;
    static_for<0, N>([&](auto ec) { acc += move<MOVE, decltype(ec)::value>(sp, step, seed, wid, t); });
    return acc;
  }

  // Local energy E_L = -1/2 sum_i lap_i psi / psi + V in log-derivative form,
  // assembled from the caches. With PM > 0 also O_k = d ln psi / d theta_k
  // for the first PM parameters. grad (optional) receives grad ln psi [N][3];
  // lapout receives sum_i lap_i psi / psi.
  __device__ F local_energy(const SP& sp, F (&O)[PMC], double* grad, double* lapout) const {
    // pair gradient vectors u'(r)/r (x_i - x_j), i < j, formed once: electron
    // i's Jastrow gradient takes +, electron j's takes -
    R gp[NPm][3];
    static_for<0, N>([&](auto ic) {
      constexpr int i = decltype(ic)::value;
      static_for<i + 1, N>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        constexpr int p = pidx(i, j);
#pragma unroll
        for (int c = 0; c < 3; ++c) gp[p][c] = pf[p] * to_r(x[i][c] - x[j][c]);
      });
    });
    // sums start at -0 so that the first addition folds away (-0 + a = a)
    F lap = acc_zero<F>(), V = acc_zero<F>();
    if constexpr (PM > 0)
#pragma unroll
      for (int p = 0; p < PM; ++p) O[p] = acc_zero<F>();
    F djs = acc_zero<F>();
    static_for<0, N>([&](auto ec) {
      constexpr int e = decltype(ec)::value;
      constexpr bool isup = e < NU;
      constexpr int n = isup ? NU : ND;
      constexpr int i = isup ? e : e - NU;
      constexpr int ld = isup ? NU : NDm;
      const F* B = isup ? bu : bd;
      F gD[3], lD = F(0);
      det_grad<e>(gD);
#pragma unroll
      for (int k = 0; k < n; ++k) lD += to_f(ol[e][k]) * B[k * ld + i];
      // Jastrow gradient and Laplacian at electron e from the caches
      R gJ[3], lJ;
      if constexpr (EN) {
        gJ[0] = gjen[e][0];
        gJ[1] = gjen[e][1];
        gJ[2] = gjen[e][2];
        lJ = ljen[e];
      } else {
        gJ[0] = gJ[1] = gJ[2] = 0;  // replaced by the first pair term when there is one
        lJ = 0;
      }
      static_for<0, N>([&](auto mc) {
        constexpr int m = decltype(mc)::value;
        if constexpr (m != e) {
          constexpr int p = pidx(e, m);
          constexpr bool first = !EN && m == (e == 0 ? 1 : 0);
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const R g = e < m ? gp[p][c] : -gp[p][c];
            if constexpr (first) gJ[c] = g;
            else gJ[c] += g;
          }
          if constexpr (first) lJ = pl[p];
          else lJ += pl[p];
        }
      });
      F dot = F(0), gj2 = F(0);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const F gj = to_f(gJ[c]);
        dot += gD[c] * gj;
        gj2 += gj * gj;
        if (grad) grad[3 * e + c] = to_d(gD[c] + gj);
      }
      lap += lD + to_f(lJ) + twice(dot) + gj2;
      V += to_f(ven[e]);  // -sum_I Z_I / r_iI (zero charges in the harmonic well)
      if constexpr (PM > 0) {
        // exponent derivatives: the first NZ slots
#pragma unroll
        for (int p = 0; p < NZ; ++p) {
          F s = F(0);
#pragma unroll
          for (int k = 0; k < n; ++k) s += to_f(odz[e][k][p]) * B[k * ld + i];
          O[p] += s;
        }
        if constexpr (EN) djs += to_f(djen[e]);
      }
    });
    if (sp.pot_kind == 0) {
#pragma unroll
      for (int p = 0; p < NP; ++p) V += to_f(pinv[p]);
      if constexpr (DF) V += sp.vnn_r;
      else V += sp.vnn;
    }
    // the harmonic well (pot_kind 1) as a loop of at most one trip: a branch
    // rather than FP64 instructions predicated off in every Coulomb system
    #pragma unroll 1
    for (int h = 0; h < sp.pot_kind; ++h)
#pragma unroll
      for (int e = 0; e < N; ++e)
        V += to_f(sp.half_omega2) * (x[e][0] * x[e][0] + x[e][1] * x[e][1] + x[e][2] * x[e][2]);
    if constexpr (PM > 0) {
      F dudb = acc_zero<F>();
      F dpoly[kMaxPoly] = {acc_zero<F>(), acc_zero<F>(), acc_zero<F>(), acc_zero<F>()};
#pragma unroll
      for (int p = 0; p < NP; ++p) dudb += to_f(pdb[p]);
      if (sp.ee_npoly > 0) {
        // d u / d b_(q+3) = R^(q+2)
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          const F rs = to_f(prs[p]);
          F rk = rs * rs;
#pragma unroll
          for (int q = 0; q < kMaxPoly; ++q) {
            if (q < sp.ee_npoly) dpoly[q] += rk;
            rk *= rs;
          }
        }
      }
#pragma unroll
      for (int p = 0; p < PM; ++p) {
        if (p >= sp.n_exp) O[p] = F(0);  // slots past the exponents hold Jastrow derivatives
        if (sp.ee_on && p == sp.off_ee) O[p] = dudb;
#pragma unroll
        for (int q = 0; q < kMaxPoly; ++q)
          if (sp.ee_on && q < sp.ee_npoly && p == sp.off_ee + 1 + q) O[p] = dpoly[q];
        if (EN && p == sp.off_en) O[p] = djs;
      }
    }
    if (lapout) *lapout = to_d(lap);
    if constexpr (DF) return V - df_scale(lap, 0.5f);
    else return -0.5 * lap + V;
  }
};

}  // namespace mole
