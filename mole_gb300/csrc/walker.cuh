// walker.cuh -- per-walker Slater-Jastrow state and operations.
//
// One thread owns one walker. All electron, orbital and spin-block indices
// are compile-time (templates on the spin-block sizes NU, ND), so the walker
// state -- positions, the FP64 inverse Slater matrices and the Jastrow caches
// -- lives in registers for small N and in L1-resident local memory for the
// largest systems.
//
// Arithmetic type R is double (plain method) or float (mixed method). The
// inverse matrices, Sherman-Morrison ratio products, the local-energy
// assembly and every accumulation stay FP64 in both.
#pragma once

#include "common.cuh"

namespace mole {

// System description in kernel-parameter memory (broadcast reads).
template <class R>
struct SysParams {
  int n_nuc;
  int n_basis;
  int nuc_b0[kMaxNuc + 1];  // basis functions of nucleus I are [nuc_b0[I], nuc_b0[I+1])
  int b_kind[kMaxBasis];
  int b_exp[kMaxBasis];  // exponent parameter index of basis function b
  R nuc_pos[kMaxNuc * 3];
  R nuc_z[kMaxNuc];
  R b_zeta[kMaxBasis];
  R coef[2][kMaxSpin][kMaxBasis];  // [spin][orbital][basis]
  int ee_on, ee_npoly;
  R ee_kappa, cusp_anti, cusp_para, ee_b;
  R ee_poly[kMaxPoly];
  int en_on;
  R en_a;
  R en_coef[kMaxNuc];
  int nn_on;
  int pot_kind;  // 0 Coulomb, 1 harmonic
  R half_omega2;
  double vnn;    // n-n repulsion constant
  int n_exp, P, off_ee, off_en, off_nn;
};

template <class R>
__device__ __forceinline__ R rsqrt_t(R x);
template <>
__device__ __forceinline__ double rsqrt_t<double>(double x) {
  return rsqrt(x);
}
template <>
__device__ __forceinline__ float rsqrt_t<float>(float x) {
  return rsqrtf(x);
}
template <class R>
__device__ __forceinline__ R exp_t(R x);
template <>
__device__ __forceinline__ double exp_t<double>(double x) {
  return exp(x);
}
template <>
__device__ __forceinline__ float exp_t<float>(float x) {
  return __expf(x);
}

// Orbitals of one spin block, e-n Jastrow and e-n potential for one electron.
template <class R, int n>
struct OneElec {
  static constexpr int nm = n > 0 ? n : 1;
  R val[nm];
  R grad[nm][3];
  R lap[nm];
  R jen, gjen[3], ljen;  // e-n Jastrow value, gradient, laplacian
  R ven;                 // sum_I -Z_I / r_I
  R djen_da;             // d(e-n Jastrow)/da
};

// GRAD/LAP: derivative orders wanted. POT: accumulate the e-n potential.
// DZ: accumulate d ln det / d zeta into dz[PM] with weights
// w_b = sum_k coef[k][b] * bcol[k] (bcol = column of the inverse for this electron).
template <class R, int n, bool GRAD, bool LAP, bool POT, int PM>
__device__ __forceinline__ void one_elec(const SysParams<R>& sp, int spin, const R (&r)[3], OneElec<R, n>& o,
                                         const double* bcol, double* dz) {
#pragma unroll
  for (int k = 0; k < OneElec<R, n>::nm; ++k) {
    o.val[k] = 0;
    if (GRAD)
#pragma unroll
      for (int c = 0; c < 3; ++c) o.grad[k][c] = 0;
    if (LAP) o.lap[k] = 0;
  }
  o.jen = 0;
  o.gjen[0] = o.gjen[1] = o.gjen[2] = 0;
  o.ljen = 0;
  o.ven = 0;
  o.djen_da = 0;
  for (int I = 0; I < sp.n_nuc; ++I) {
    const R d0 = r[0] - sp.nuc_pos[3 * I], d1 = r[1] - sp.nuc_pos[3 * I + 1], d2 = r[2] - sp.nuc_pos[3 * I + 2];
    const R r2 = d0 * d0 + d1 * d1 + d2 * d2;
    const R inv = rsqrt_t<R>(r2);
    const R rr = r2 * inv;
    if (POT) o.ven -= sp.nuc_z[I] * inv;
    const int b1 = sp.nuc_b0[I + 1];
    for (int b = sp.nuc_b0[I]; b < b1; ++b) {
      const int kind = sp.b_kind[b];
      const R z = sp.b_zeta[b];
      R chi, g0 = 0, g1 = 0, g2 = 0, l = 0, rad;
      if (kind == kGto1s) {
        const R e = exp_t<R>(-z * r2);
        chi = e;
        if (GRAD) {
          const R f = (R)-2 * z * e;
          g0 = f * d0; g1 = f * d1; g2 = f * d2;
        }
        if (LAP) l = e * ((R)4 * z * z * r2 - (R)6 * z);
        rad = r2;
      } else {
        const R e = exp_t<R>(-z * rr);
        rad = rr;
        if (kind == kSto1s) {
          chi = e;
          if (GRAD) {
            const R f = -z * e * inv;
            g0 = f * d0; g1 = f * d1; g2 = f * d2;
          }
          if (LAP) l = e * (z * z - (R)2 * z * inv);
        } else if (kind == kSto2s) {
          chi = rr * e;
          if (GRAD) {
            const R f = e * ((R)1 - z * rr) * inv;
            g0 = f * d0; g1 = f * d1; g2 = f * d2;
          }
          if (LAP) l = e * (z * z * rr - (R)4 * z + (R)2 * inv);
        } else {
          const R da = kind == kSto2px ? d0 : (kind == kSto2py ? d1 : d2);
          chi = da * e;
          if (GRAD) {
            const R f = -z * da * e * inv;
            g0 = f * d0; g1 = f * d1; g2 = f * d2;
            if (kind == kSto2px) g0 += e;
            else if (kind == kSto2py) g1 += e;
            else g2 += e;
          }
          if (LAP) l = da * e * (z * z - (R)4 * z * inv);
        }
      }
#pragma unroll
      for (int k = 0; k < n; ++k) {
        const R c = sp.coef[spin][k][b];
        o.val[k] += c * chi;
        if (GRAD) {
          o.grad[k][0] += c * g0;
          o.grad[k][1] += c * g1;
          o.grad[k][2] += c * g2;
        }
        if (LAP) o.lap[k] += c * l;
      }
      if constexpr (PM > 0) {
        double w = 0.0;
#pragma unroll
        for (int k = 0; k < n; ++k) w += (double)sp.coef[spin][k][b] * bcol[k];
        const double dzb = -(double)rad * (double)chi * w;
        const int ix = sp.b_exp[b];
#pragma unroll
        for (int p = 0; p < PM; ++p)
          if (p == ix) dz[p] += dzb;
      }
    }
    if (sp.en_on) {
      const R A = sp.en_coef[I];
      const R q = (R)1 / ((R)1 + sp.en_a * rr);
      o.jen += A * rr * q;
      if (GRAD) {
        const R du = A * q * q * inv;
        o.gjen[0] += du * d0;
        o.gjen[1] += du * d1;
        o.gjen[2] += du * d2;
      }
      if (LAP) o.ljen += (R)-2 * A * sp.en_a * q * q * q + (R)2 * A * q * q * inv;
      if constexpr (PM > 0) o.djen_da += -A * rr * rr * q * q;
    }
  }
}

// Pade pair term u(r) and its radial derivatives (theory/jastrow.tex:15-105);
// dudb/dpoly are the parameter derivatives (jastrow.tex:107-126).
template <class R, bool DER, bool PAR>
__device__ __forceinline__ void pade_pair(const SysParams<R>& sp, bool same, R r, R& u, R& du, R& d2u, R& dudb,
                                          R* dpoly) {
  const R cusp = same ? sp.cusp_para : sp.cusp_anti;
  R Rs = r, Rp = 1, Rpp = 0;
  if (sp.ee_kappa > (R)0) {
    const R e = exp_t<R>(-sp.ee_kappa * r);
    Rs = ((R)1 - e) / sp.ee_kappa;
    Rp = e;
    Rpp = -sp.ee_kappa * e;
  }
  const R q = (R)1 / ((R)1 + sp.ee_b * Rs);
  R val = cusp * Rs * q;
  R uR = cusp * q * q;
  R uRR = (R)-2 * cusp * sp.ee_b * q * q * q;
  if (PAR) dudb = -cusp * Rs * Rs * q * q;
  R Rk = Rs, Rk2 = 1;  // R^(p-1), R^(p-2)
  for (int i = 0; i < sp.ee_npoly; ++i) {
    const R p = (R)(i + 2), c = sp.ee_poly[i];
    val += c * Rk * Rs;
    uR += p * c * Rk;
    uRR += p * (p - (R)1) * c * Rk2;
    if (PAR) dpoly[i] = Rk * Rs;
    Rk2 = Rk;
    Rk *= Rs;
  }
  u = val;
  if (DER) {
    du = uR * Rp;
    d2u = uRR * Rp * Rp + uR * Rpp;
  }
}

// In-register Gauss-Jordan inverse with partial pivoting; row swaps are
// predicated so that every index stays compile-time.
template <int n>
__device__ __forceinline__ bool gj_invert(double (&a)[n * n], double (&inv)[n * n], double* lndet, double* sign) {
#pragma unroll
  for (int i = 0; i < n * n; ++i) inv[i] = (i / n == i % n) ? 1.0 : 0.0;
  double ld = 0.0, sg = 1.0;
  bool ok = true;
#pragma unroll
  for (int col = 0; col < n; ++col) {
    int piv = col;
    double best = fabs(a[col * n + col]);
#pragma unroll
    for (int r = col + 1; r < n; ++r)
      if (fabs(a[r * n + col]) > best) {
        best = fabs(a[r * n + col]);
        piv = r;
      }
#pragma unroll
    for (int r = col + 1; r < n; ++r)
      if (r == piv) {
#pragma unroll
        for (int j = 0; j < n; ++j) {
          double t = a[col * n + j];
          a[col * n + j] = a[r * n + j];
          a[r * n + j] = t;
          t = inv[col * n + j];
          inv[col * n + j] = inv[r * n + j];
          inv[r * n + j] = t;
        }
        sg = -sg;
      }
    const double p = a[col * n + col];
    ok = ok && (p != 0.0);
    if (lndet) ld += log(fabs(p));
    if (p < 0.0) sg = -sg;
    const double ip = 1.0 / p;
#pragma unroll
    for (int j = 0; j < n; ++j) {
      a[col * n + j] *= ip;
      inv[col * n + j] *= ip;
    }
#pragma unroll
    for (int r = 0; r < n; ++r) {
      if (r == col) continue;
      const double f = a[r * n + col];
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

// Walker state and moves for spin blocks of NU up and ND down electrons.
template <int NU, int ND, class R>
struct Walker {
  static constexpr int N = NU + ND;
  static constexpr int NDm = ND > 0 ? ND : 1;
  static constexpr int NP = N * (N - 1) / 2;
  static constexpr int NPm = NP > 0 ? NP : 1;
  using SP = SysParams<R>;

  double x[N][3];
  double bu[NU * NU];    // inverse of the up Slater matrix, bu[k*NU+i]
  double bd[NDm * NDm];  // inverse of the down Slater matrix
  R upair[NPm];          // cached u(r_ij), i < j
  R jen[N];              // cached e-n Jastrow per electron
  // drift caches (diffuse moves only)
  R dphi[N][(NU > NDm ? NU : NDm)][3];  // grad of own-block orbitals at each electron
  double gd[N][3];                      // grad ln det per electron
  R gj[N][3];                           // grad J per electron

  static constexpr __device__ int pidx(int i, int j) { return i * N - i * (i + 1) / 2 + (j - i - 1); }
  static constexpr __device__ bool same_spin(int i, int j) { return (i < NU) == (j < NU); }

  __device__ __forceinline__ void load(const double* pos, int W, int w) {
#pragma unroll
    for (int e = 0; e < N; ++e)
#pragma unroll
      for (int c = 0; c < 3; ++c) x[e][c] = pos[(size_t)(3 * e + c) * W + w];
  }
  __device__ __forceinline__ void store(double* pos, int W, int w) const {
#pragma unroll
    for (int e = 0; e < N; ++e)
#pragma unroll
      for (int c = 0; c < 3; ++c) pos[(size_t)(3 * e + c) * W + w] = x[e][c];
  }
  __device__ __forceinline__ void rpos(int e, R (&r)[3]) const {
    r[0] = (R)x[e][0];
    r[1] = (R)x[e][1];
    r[2] = (R)x[e][2];
  }

  // Rebuilds the inverses in FP64 from fresh orbital values, the Jastrow
  // caches and (DRIFT) the drift caches. Returns false on a singular block.
  template <bool DRIFT>
  __device__ bool refresh(const SP& sp, double* lndet, double* sign) {
    double au[NU * NU], ad[NDm * NDm];
    static_for<0, N>([&](auto ec) {
      constexpr int e = decltype(ec)::value;
      constexpr bool isup = e < NU;
      constexpr int n = isup ? NU : ND;
      constexpr int i = isup ? e : e - NU;
      R r[3];
      rpos(e, r);
      OneElec<R, n> o;
      one_elec<R, n, DRIFT, false, false, 0>(sp, isup ? 0 : 1, r, o, nullptr, nullptr);
#pragma unroll
      for (int k = 0; k < n; ++k) {
        if constexpr (isup) au[i * NU + k] = (double)o.val[k];
        else ad[i * NDm + k] = (double)o.val[k];
        if (DRIFT)
#pragma unroll
          for (int c = 0; c < 3; ++c) dphi[e][k][c] = o.grad[k][c];
      }
      jen[e] = o.jen;
      if (DRIFT)
#pragma unroll
        for (int c = 0; c < 3; ++c) gj[e][c] = o.gjen[c];
    });
    double l1 = 0.0, s1 = 1.0, l2 = 0.0, s2 = 1.0;
    bool ok = gj_invert<NU>(au, bu, lndet ? &l1 : nullptr, &s1);
    if constexpr (ND > 0) ok = gj_invert<ND>(ad, bd, lndet ? &l2 : nullptr, &s2) && ok;
    double J = 0.0;
#pragma unroll
    for (int e = 0; e < N; ++e) J += (double)jen[e];
    if (sp.ee_on) {
      static_for<0, N>([&](auto ic) {
        constexpr int i = decltype(ic)::value;
        static_for<i + 1, N>([&](auto jc) {
          constexpr int j = decltype(jc)::value;
          const R d0 = (R)(x[i][0] - x[j][0]), d1 = (R)(x[i][1] - x[j][1]), d2 = (R)(x[i][2] - x[j][2]);
          const R r2 = d0 * d0 + d1 * d1 + d2 * d2;
          const R inv = rsqrt_t<R>(r2);
          R u, du, d2u, db;
          pade_pair<R, DRIFT, false>(sp, same_spin(i, j), r2 * inv, u, du, d2u, db, nullptr);
          upair[pidx(i, j)] = u;
          J += (double)u;
          if (DRIFT) {
            const R f = du * inv;
            gj[i][0] += f * d0; gj[i][1] += f * d1; gj[i][2] += f * d2;
            gj[j][0] -= f * d0; gj[j][1] -= f * d1; gj[j][2] -= f * d2;
          }
        });
      });
    }
    if (DRIFT) {
      static_for<0, N>([&](auto ec) {
        constexpr int e = decltype(ec)::value;
        constexpr bool isup = e < NU;
        constexpr int n = isup ? NU : ND;
        constexpr int i = isup ? e : e - NU;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          double g = 0.0;
#pragma unroll
          for (int k = 0; k < n; ++k) g += (double)dphi[e][k][c] * (isup ? bu[k * NU + i] : bd[k * NDm + i]);
          gd[e][c] = g;
        }
      });
    }
    if (lndet) *lndet = l1 + l2 + J;
    if (sign) *sign = s1 * s2;
    return ok;
  }

  // One Metropolis move of electron e; returns 1 when accepted.
  template <int MOVE, int e>
  __device__ __forceinline__ int move(const SP& sp, R step, uint64_t seed, uint32_t wid, uint32_t t) {
    constexpr bool isup = e < NU;
    constexpr int n = isup ? NU : ND;
    constexpr int i = isup ? e : e - NU;
    constexpr bool DRIFT = MOVE == kMoveDiffuse;
    double* B = isup ? bu : bd;
    constexpr int ld = isup ? NU : NDm;

    const uint4 ra = draw4(seed, wid, t, 2u * e, kTagMove);
    R dx[3];
    R uacc;
    if constexpr (MOVE == kMoveBox) {
      dx[0] = step * (u01<R>(ra.x) - (R)0.5);
      dx[1] = step * (u01<R>(ra.y) - (R)0.5);
      dx[2] = step * (u01<R>(ra.z) - (R)0.5);
      uacc = u01<R>(ra.w);
    } else {
      R z0, z1, z2, z3;
      box_muller(ra.x, ra.y, z0, z1);
      box_muller(ra.z, ra.w, z2, z3);
      const uint4 rb = draw4(seed, wid, t, 2u * e + 1u, kTagMove);
      uacc = u01<R>(rb.x);
      if constexpr (MOVE == kMoveGauss) {
        dx[0] = step * z0; dx[1] = step * z1; dx[2] = step * z2;
      } else {
        const R sq = sqrt(step);
        dx[0] = step * ((R)gd[e][0] + gj[e][0]) + sq * z0;
        dx[1] = step * ((R)gd[e][1] + gj[e][1]) + sq * z1;
        dx[2] = step * ((R)gd[e][2] + gj[e][2]) + sq * z2;
      }
    }
    double xn[3] = {x[e][0] + (double)dx[0], x[e][1] + (double)dx[1], x[e][2] + (double)dx[2]};
    R rn[3] = {(R)xn[0], (R)xn[1], (R)xn[2]};
    OneElec<R, n> o;
    one_elec<R, n, DRIFT, false, false, 0>(sp, isup ? 0 : 1, rn, o, nullptr, nullptr);
    double ratio = 0.0;
#pragma unroll
    for (int k = 0; k < n; ++k) ratio += (double)o.val[k] * B[k * ld + i];

    // Jastrow change; new pair values and (DRIFT) pair gradients
    R dJ = o.jen - jen[e];
    R unew[N];
    R gpn[N][3], gpo[N][3];  // grad_e u(e,j) new / old
    if (sp.ee_on) {
      static_for<0, N>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        if constexpr (j != e) {
          const R d0 = rn[0] - (R)x[j][0], d1 = rn[1] - (R)x[j][1], d2 = rn[2] - (R)x[j][2];
          const R r2 = d0 * d0 + d1 * d1 + d2 * d2;
          const R inv = rsqrt_t<R>(r2);
          R u, du, d2u, db;
          pade_pair<R, DRIFT, false>(sp, same_spin(e, j), r2 * inv, u, du, d2u, db, nullptr);
          unew[j] = u;
          dJ += u - upair[e < j ? pidx(e, j) : pidx(j, e)];
          if constexpr (DRIFT) {
            gpn[j][0] = du * inv * d0; gpn[j][1] = du * inv * d1; gpn[j][2] = du * inv * d2;
            const R o0 = (R)(x[e][0] - x[j][0]), o1 = (R)(x[e][1] - x[j][1]), o2 = (R)(x[e][2] - x[j][2]);
            const R or2 = o0 * o0 + o1 * o1 + o2 * o2;
            const R oinv = rsqrt_t<R>(or2);
            R ou, odu, od2u;
            pade_pair<R, true, false>(sp, same_spin(e, j), or2 * oinv, ou, odu, od2u, db, nullptr);
            gpo[j][0] = odu * oinv * o0; gpo[j][1] = odu * oinv * o1; gpo[j][2] = odu * oinv * o2;
          }
        }
      });
    }

    bool acc;
    double bn[n > 0 ? n * n : 1];
    double gdn[N][3];
    R gjn[N][3];
    if constexpr (!DRIFT) {
      const double p = ratio * ratio * (double)exp_t<R>((R)2 * dJ);
      acc = p > (double)uacc;
    } else {
      // tentative inverse after replacing row i
      double v[n];
#pragma unroll
      for (int j = 0; j < n; ++j) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < n; ++k) s += (double)o.val[k] * B[k * ld + j];
        v[j] = s;
      }
      const double ir = 1.0 / ratio;
#pragma unroll
      for (int k = 0; k < n; ++k) {
        const double ck = B[k * ld + i] * ir;
#pragma unroll
        for (int j = 0; j < n; ++j) bn[k * n + j] = B[k * ld + j] - ck * (v[j] - (j == i ? 1.0 : 0.0));
      }
      // drift at the proposed configuration, all electrons
      static_for<0, N>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        constexpr bool jup = j < NU;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if constexpr (jup == isup) {
            constexpr int ij = jup ? j : j - NU;
            double g = 0.0;
#pragma unroll
            for (int k = 0; k < n; ++k) g += (double)(j == e ? o.grad[k][c] : dphi[j][k][c]) * bn[k * n + ij];
            gdn[j][c] = g;
          } else {
            gdn[j][c] = gd[j][c];
          }
          if constexpr (j == e) {
            R g = o.gjen[c];
            if (sp.ee_on)
#pragma unroll
              for (int m = 0; m < N; ++m)
                if (m != e) g += gpn[m][c];
            gjn[j][c] = g;
          } else {
            gjn[j][c] = gj[j][c];
            if (sp.ee_on) gjn[j][c] += gpo[j][c] - gpn[j][c];
          }
        }
      });
      // Green's function ratio over every electron (metrop.rs:182-195)
      double hi = 0.0, lo = 0.0;
#pragma unroll
      for (int j = 0; j < N; ++j)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const double dj = (j == e) ? (double)dx[c] : 0.0;
          const double a = -dj - (double)step * (gdn[j][c] + (double)gjn[j][c]);
          const double b = dj - (double)step * (gd[j][c] + (double)gj[j][c]);
          hi += a * a;
          lo += b * b;
        }
      const double la = 2.0 * (double)dJ - (hi - lo) / (2.0 * (double)step);
      const double p = ratio * ratio * exp(la);
      acc = (ratio > 0.0) && (p > (double)uacc);
    }
    if (!acc) return 0;

    // commit
    x[e][0] = xn[0]; x[e][1] = xn[1]; x[e][2] = xn[2];
    jen[e] = o.jen;
    if (sp.ee_on) {
#pragma unroll
      for (int j = 0; j < N; ++j)
        if (j != e) upair[e < j ? pidx(e, j) : pidx(j, e)] = unew[j];
    }
    if constexpr (DRIFT) {
#pragma unroll
      for (int k = 0; k < n * n; ++k) B[(k / n) * ld + (k % n)] = bn[k];
#pragma unroll
      for (int k = 0; k < n; ++k)
#pragma unroll
        for (int c = 0; c < 3; ++c) dphi[e][k][c] = o.grad[k][c];
#pragma unroll
      for (int j = 0; j < N; ++j)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          gd[j][c] = gdn[j][c];
          gj[j][c] = gjn[j][c];
        }
    } else {
      // Sherman-Morrison row update (FP64)
      double v[n], col[n];
#pragma unroll
      for (int j = 0; j < n; ++j) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < n; ++k) s += (double)o.val[k] * B[k * ld + j];
        v[j] = s;
      }
      const double ir = 1.0 / ratio;
#pragma unroll
      for (int k = 0; k < n; ++k) col[k] = B[k * ld + i] * ir;
#pragma unroll
      for (int k = 0; k < n; ++k)
#pragma unroll
        for (int j = 0; j < n; ++j) B[k * ld + j] -= col[k] * (v[j] - (j == i ? 1.0 : 0.0));
    }
    return 1;
  }

  template <int MOVE>
  __device__ __forceinline__ int sweep(const SP& sp, R step, uint64_t seed, uint32_t wid, uint32_t t) {
    int acc = 0;
    static_for<0, N>([&](auto ec) { acc += move<MOVE, decltype(ec)::value>(sp, step, seed, wid, t); });
    return acc;
  }

  // Local energy E_L = -1/2 sum_i lap_i psi / psi + V in log-derivative form.
  // If PM > 0 also O_k = d ln psi / d theta_k for the first PM parameters.
  // grad (optional) receives grad ln psi [N][3]; lap receives sum_i lap_i psi/psi.
  template <int PM>
  __device__ double local_energy(const SP& sp, double (&O)[PM > 0 ? PM : 1], double* grad, double* lapout) {
    double lap = 0.0, V = 0.0;
    if constexpr (PM > 0)
#pragma unroll
      for (int p = 0; p < PM; ++p) O[p] = 0.0;
    double gD[N][3];
    R gJ[N][3];
    R lJ[N];
    double lD[N];
    double djen = 0.0;
    static_for<0, N>([&](auto ec) {
      constexpr int e = decltype(ec)::value;
      constexpr bool isup = e < NU;
      constexpr int n = isup ? NU : ND;
      constexpr int i = isup ? e : e - NU;
      const double* B = isup ? bu : bd;
      constexpr int ld = isup ? NU : NDm;
      R r[3];
      rpos(e, r);
      OneElec<R, n> o;
      double bcol[n > 0 ? n : 1];
#pragma unroll
      for (int k = 0; k < n; ++k) bcol[k] = B[k * ld + i];
      one_elec<R, n, true, true, true, PM>(sp, isup ? 0 : 1, r, o, bcol, O);
      double l = 0.0;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        double g = 0.0;
#pragma unroll
        for (int k = 0; k < n; ++k) g += (double)o.grad[k][c] * bcol[k];
        gD[e][c] = g;
        gJ[e][c] = o.gjen[c];
      }
#pragma unroll
      for (int k = 0; k < n; ++k) l += (double)o.lap[k] * bcol[k];
      lD[e] = l;
      lJ[e] = o.ljen;
      V += (double)o.ven;
      djen += (double)o.djen_da;
    });
    if (sp.pot_kind == 1) {
      V = 0.0;
#pragma unroll
      for (int e = 0; e < N; ++e)
        V += (double)sp.half_omega2 * (x[e][0] * x[e][0] + x[e][1] * x[e][1] + x[e][2] * x[e][2]);
    }
    double dudb = 0.0;
    double dpoly[kMaxPoly] = {0.0, 0.0, 0.0, 0.0};
    static_for<0, N>([&](auto ic) {
      constexpr int i = decltype(ic)::value;
      static_for<i + 1, N>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        const R d0 = (R)(x[i][0] - x[j][0]), d1 = (R)(x[i][1] - x[j][1]), d2 = (R)(x[i][2] - x[j][2]);
        const R r2 = d0 * d0 + d1 * d1 + d2 * d2;
        const R inv = rsqrt_t<R>(r2);
        if (sp.pot_kind == 0) V += (double)inv;
        if (sp.ee_on) {
          R u, du, d2u, db, dp[kMaxPoly];
          pade_pair<R, true, (PM > 0)>(sp, same_spin(i, j), r2 * inv, u, du, d2u, db, dp);
          const R f = du * inv;
          gJ[i][0] += f * d0; gJ[i][1] += f * d1; gJ[i][2] += f * d2;
          gJ[j][0] -= f * d0; gJ[j][1] -= f * d1; gJ[j][2] -= f * d2;
          const R lj = d2u + (R)2 * f;
          lJ[i] += lj;
          lJ[j] += lj;
          if constexpr (PM > 0) {
            dudb += (double)db;
            for (int p = 0; p < sp.ee_npoly; ++p) dpoly[p] += (double)dp[p];
          }
        }
      });
    });
#pragma unroll
    for (int e = 0; e < N; ++e) {
      double dot = 0.0, gj2 = 0.0;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double gj = (double)gJ[e][c];
        dot += gD[e][c] * gj;
        gj2 += gj * gj;
        if (grad) grad[3 * e + c] = gD[e][c] + gj;
      }
      lap += lD[e] + (double)lJ[e] + 2.0 * dot + gj2;
    }
    if constexpr (PM > 0) {
#pragma unroll
      for (int p = 0; p < PM; ++p) {
        if (sp.ee_on && p == sp.off_ee) O[p] += dudb;
        if (sp.ee_on && p > sp.off_ee && p <= sp.off_ee + sp.ee_npoly) {
#pragma unroll
          for (int q = 0; q < kMaxPoly; ++q)
            if (p == sp.off_ee + 1 + q) O[p] += dpoly[q];
        }
        if (sp.en_on && p == sp.off_en) O[p] += djen;
      }
    }
    if (lapout) *lapout = lap;
    if (sp.pot_kind == 0) V += sp.vnn;
    return -0.5 * lap + V;
  }
};

}  // namespace mole
