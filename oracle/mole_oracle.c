/*
 * mole_oracle.c -- CPU FP64 oracle for the mole walker hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the reference the GPU path is compared with, never shipped or
 * called by it. Reference citations are file:line inside Jvanrhijn/mole.
 *
 * Independence from the GPU path: determinants here are formed densely and
 * factorised by Gauss-Jordan elimination with partial pivoting at every call
 * (no Sherman-Morrison), the Jastrow is recomputed from all pairs, and the
 * Philox generator is a separate implementation of Salmon et al., "Parallel
 * random numbers: as easy as 1, 2, 3" (SC'11).
 */
#include "mole_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define TAG_MOVE 0x4d4f5645u /* 'MOVE' */
#define TAG_INIT 0x494e4954u /* 'INIT' */
#define TAG_COMB 0x434f4d42u /* 'COMB' */

/* ------------------------------------------------------------------ RNG */

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int round = 0; round < 10; ++round) {
    if (round > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static void draw4(uint64_t seed, uint32_t a, uint32_t b, uint32_t c, uint32_t tag, uint32_t out[4]) {
  uint32_t ctr[4] = {a, b, c, tag};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  orc_philox4x32_10(ctr, key, out);
}

static double u01(uint32_t x) { return ((double)x + 0.5) * (1.0 / 4294967296.0); }

/* Box-Muller pair from two uniforms */
static void box_muller(uint32_t a, uint32_t b, double* z0, double* z1) {
  double r = sqrt(-2.0 * log(u01(a)));
  double t = 2.0 * M_PI * u01(b);
  *z0 = r * cos(t);
  *z1 = r * sin(t);
}

/* Single-precision Box-Muller whose every operation is an IEEE-rounded add,
 * mul, fma, div or sqrt, in a fixed order (this file is compiled with
 * -ffp-contract=off): ln u from u = m 2^e, m in [sqrt(1/2), sqrt(2)),
 * ln m = 2 atanh(s), s = (m-1)/(m+1), series through s^9; sin/cos of an angle
 * in one quadrant from their Taylor series through x^11 / x^12. The GPU path
 * draws its proposal normals the same way, so both produce the same bits. */
static float f32_log01(float u) {
  uint32_t bits;
  memcpy(&bits, &u, 4);
  int e = (int)((bits >> 23) & 0xffu) - 127;
  uint32_t mb = (bits & 0x7fffffu) | 0x3f800000u;
  float m;
  memcpy(&m, &mb, 4);
  if (m > 1.41421356f) {
    m = m * 0.5f;
    e += 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  float p = fmaf(s2, 0.111111112f, 0.142857149f);
  p = fmaf(p, s2, 0.2f);
  p = fmaf(p, s2, 0.333333343f);
  p = fmaf(p, s2, 1.0f);
  const float t = s * p;
  return fmaf((float)e, 0.693147182f, t + t);
}

static void f32_sincos_q(float x, float* s, float* c) {
  const float x2 = x * x;
  float ps = fmaf(x2, -2.50521084e-8f, 2.75573192e-6f);
  ps = fmaf(ps, x2, -1.98412698e-4f);
  ps = fmaf(ps, x2, 8.33333333e-3f);
  ps = fmaf(ps, x2, -1.66666667e-1f);
  ps = fmaf(ps, x2, 1.0f);
  *s = x * ps;
  float pc = fmaf(x2, 2.08767570e-9f, -2.75573192e-7f);
  pc = fmaf(pc, x2, 2.48015873e-5f);
  pc = fmaf(pc, x2, -1.38888889e-3f);
  pc = fmaf(pc, x2, 4.16666667e-2f);
  pc = fmaf(pc, x2, -0.5f);
  *c = fmaf(pc, x2, 1.0f);
}

static void f32_box_muller(uint32_t a, uint32_t b, float* z0, float* z1) {
  const float u = ((float)(a >> 8) + 0.5f) * 5.96046448e-8f;
  const float r = sqrtf(-2.0f * f32_log01(u));
  const float f = ((float)((b >> 6) & 0xffffffu) + 0.5f) * 5.96046448e-8f;
  const float x = f * 1.57079637f;
  float s, c;
  f32_sincos_q(x, &s, &c);
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
  *z0 = r * cs;
  *z1 = r * sn;
}

void orc_normal_pair(uint32_t a, uint32_t b, float* z) { f32_box_muller(a, b, &z[0], &z[1]); }

void orc_init_positions(int W, int N, uint64_t seed, int kind, double width, double* pos) {
  for (int w = 0; w < W; ++w)
    for (int e = 0; e < N; ++e) {
      uint32_t u[4];
      draw4(seed, (uint32_t)w, (uint32_t)e, 0u, TAG_INIT, u);
      double* p = pos + ((size_t)w * N + e) * 3;
      if (kind == 0) {
        double z0, z1, z2, z3;
        box_muller(u[0], u[1], &z0, &z1);
        box_muller(u[2], u[3], &z2, &z3);
        p[0] = width * z0; p[1] = width * z1; p[2] = width * z2;
      } else {
        for (int k = 0; k < 3; ++k) p[k] = width * (2.0 * u01(u[k]) - 1.0);
      }
    }
}

/* ------------------------------------------------------- parameter layout */

static int off_ee(const orc_system* s) { return s->n_exp; }
static int off_en(const orc_system* s) { return off_ee(s) + (s->ee_on ? 1 + s->ee_npoly : 0); }
static int off_nn(const orc_system* s) { return off_en(s) + (s->en_on ? 1 : 0); }
int orc_num_params(const orc_system* s) { return off_nn(s) + (s->nn_on ? ORC_NN_P : 0); }

/* -------------------------------------------------------------- basis */

static void basis_eval(const orc_system* s, const double* zeta, int b, const double* r, double* v,
                       double g[3], double* lap, double* dz) {
  const double* c = s->nuc_pos + 3 * s->b_center[b];
  double d[3] = {r[0] - c[0], r[1] - c[1], r[2] - c[2]};
  double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  double z = zeta[s->b_exp[b]];
  int kind = s->b_kind[b];
  if (kind == ORC_GTO_1S) {
    double e = exp(-z * r2);
    *v = e;
    for (int k = 0; k < 3; ++k) g[k] = -2.0 * z * e * d[k];
    *lap = e * (4.0 * z * z * r2 - 6.0 * z);
    *dz = -r2 * e;
    return;
  }
  double rr = sqrt(r2);
  double e = exp(-z * rr);
  if (kind == ORC_STO_1S) {
    *v = e;
    for (int k = 0; k < 3; ++k) g[k] = -z * e * d[k] / rr;
    *lap = e * (z * z - 2.0 * z / rr);
  } else if (kind == ORC_STO_2S) {
    *v = rr * e;
    for (int k = 0; k < 3; ++k) g[k] = e * (1.0 - z * rr) * d[k] / rr;
    *lap = e * (z * z * rr - 4.0 * z + 2.0 / rr);
  } else {
    int a = kind - ORC_STO_2PX;
    *v = d[a] * e;
    for (int k = 0; k < 3; ++k) g[k] = e * ((k == a ? 1.0 : 0.0) - z * d[a] * d[k] / rr);
    *lap = d[a] * e * (z * z - 4.0 * z / rr);
  }
  *dz = -rr * (*v);
}

/* Gauss-Jordan inverse with partial pivoting: A (n x n, row-major) ->
 * inv, returns ln|det| and sign; -1 on exact singularity. */
static int gj_inverse(int n, const double* A, double* inv, double* lndet, double* sign) {
  double a[ORC_MAX_SPIN * ORC_MAX_SPIN * 2];
  int m = 2 * n;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < m; ++j) a[i * m + j] = j < n ? A[i * n + j] : (j - n == i ? 1.0 : 0.0);
  double ld = 0.0, sg = 1.0;
  for (int col = 0; col < n; ++col) {
    int piv = col;
    for (int i = col + 1; i < n; ++i)
      if (fabs(a[i * m + col]) > fabs(a[piv * m + col])) piv = i;
    if (a[piv * m + col] == 0.0) return -1;
    if (piv != col) {
      for (int j = 0; j < m; ++j) {
        double t = a[col * m + j];
        a[col * m + j] = a[piv * m + j];
        a[piv * m + j] = t;
      }
      sg = -sg;
    }
    double p = a[col * m + col];
    ld += log(fabs(p));
    if (p < 0) sg = -sg;
    for (int j = 0; j < m; ++j) a[col * m + j] /= p;
    for (int i = 0; i < n; ++i) {
      if (i == col) continue;
      double f = a[i * m + col];
      if (f == 0.0) continue;
      for (int j = 0; j < m; ++j) a[i * m + j] -= f * a[col * m + j];
    }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) inv[i * n + j] = a[i * m + n + j];
  *lndet = ld;
  *sign = sg;
  return 0;
}

/* ------------------------------------------------------------ Jastrow */

/* Pade e-e term of theory/jastrow.tex:15-29 with b1 = cusp, b2 = b and
 * polynomial coefficients b_{p+1}, p = 2..npoly+1, in the scaled distance
 * R = (1 - exp(-kappa r)) / kappa (R = r when kappa = 0). Radial
 * derivatives follow jastrow.tex:32-105; parameter derivatives 107-126. */
static void pade_ee(double r, double cusp, double b, double kappa, int npoly, const double* poly,
                    double* u, double* du, double* d2u, double* dudb, double* dudpoly) {
  double R, Rp, Rpp;
  if (kappa > 0.0) {
    double e = exp(-kappa * r);
    R = (1.0 - e) / kappa;
    Rp = e;
    Rpp = -kappa * e;
  } else {
    R = r;
    Rp = 1.0;
    Rpp = 0.0;
  }
  double q = 1.0 / (1.0 + b * R);
  double val = cusp * R * q;
  double uR = cusp * q * q;
  double uRR = -2.0 * cusp * b * q * q * q;
  double Rk = R; /* R^(p-1) */
  for (int i = 0; i < npoly; ++i) {
    int p = i + 2;
    double Rpm2 = Rk / R; /* R^(p-2) */
    val += poly[i] * Rk * R;
    uR += p * poly[i] * Rk;
    uRR += p * (p - 1) * poly[i] * Rpm2;
    if (dudpoly) dudpoly[i] = Rk * R;
    Rk *= R;
  }
  *u = val;
  *du = uR * Rp;
  *d2u = uRR * Rp * Rp + uR * Rpp;
  if (dudb) *dudb = -cusp * R * R * q * q;
}

/* Pairwise MLP y(x(r)) = w3 . tanh(W2 tanh(W1 x + b1) + b2) + b3 with
 * features x = [r, exp(-r), s r, s exp(-r)]. Returns y, dy/dr, d2y/dr2 and,
 * if dth is non-NULL, adds dy/dtheta into dth (same layout as th). */
static void nn_pair(const double* th, double r, double s, double* y, double* dy, double* d2y,
                    double* dth) {
  const double* W1 = th;
  const double* b1 = W1 + ORC_NN_H * ORC_NN_IN;
  const double* W2 = b1 + ORC_NN_H;
  const double* b2 = W2 + ORC_NN_H * ORC_NN_H;
  const double* w3 = b2 + ORC_NN_H;
  const double* b3 = w3 + ORC_NN_H;
  double er = exp(-r);
  double x[4] = {r, er, s * r, s * er};
  double x1[4] = {1.0, -er, s, -s * er};
  double x2[4] = {0.0, er, 0.0, s * er};
  double h1[ORC_NN_H], h1p[ORC_NN_H], h1pp[ORC_NN_H];
  for (int a = 0; a < ORC_NN_H; ++a) {
    double z = b1[a], zp = 0.0, zpp = 0.0;
    for (int c = 0; c < 4; ++c) {
      z += W1[a * 4 + c] * x[c];
      zp += W1[a * 4 + c] * x1[c];
      zpp += W1[a * 4 + c] * x2[c];
    }
    double t = tanh(z), sd = 1.0 - t * t;
    h1[a] = t;
    h1p[a] = sd * zp;
    h1pp[a] = sd * zpp - 2.0 * t * sd * zp * zp;
  }
  double out = b3[0], outp = 0.0, outpp = 0.0;
  double delta2[ORC_NN_H], h2[ORC_NN_H];
  for (int a = 0; a < ORC_NN_H; ++a) {
    double z = b2[a], zp = 0.0, zpp = 0.0;
    for (int c = 0; c < ORC_NN_H; ++c) {
      z += W2[a * ORC_NN_H + c] * h1[c];
      zp += W2[a * ORC_NN_H + c] * h1p[c];
      zpp += W2[a * ORC_NN_H + c] * h1pp[c];
    }
    double t = tanh(z), sd = 1.0 - t * t;
    h2[a] = t;
    out += w3[a] * t;
    outp += w3[a] * sd * zp;
    outpp += w3[a] * (sd * zpp - 2.0 * t * sd * zp * zp);
    delta2[a] = w3[a] * sd;
  }
  *y = out;
  *dy = outp;
  *d2y = outpp;
  if (!dth) return;
  double* gW1 = dth;
  double* gb1 = gW1 + ORC_NN_H * ORC_NN_IN;
  double* gW2 = gb1 + ORC_NN_H;
  double* gb2 = gW2 + ORC_NN_H * ORC_NN_H;
  double* gw3 = gb2 + ORC_NN_H;
  double* gb3 = gw3 + ORC_NN_H;
  gb3[0] += 1.0;
  for (int a = 0; a < ORC_NN_H; ++a) {
    gw3[a] += h2[a];
    gb2[a] += delta2[a];
    for (int c = 0; c < ORC_NN_H; ++c) gW2[a * ORC_NN_H + c] += delta2[a] * h1[c];
  }
  for (int c = 0; c < ORC_NN_H; ++c) {
    double d1 = 0.0;
    for (int a = 0; a < ORC_NN_H; ++a) d1 += W2[a * ORC_NN_H + c] * delta2[a];
    d1 *= 1.0 - h1[c] * h1[c];
    gb1[c] += d1;
    for (int k = 0; k < 4; ++k) gW1[c * 4 + k] += d1 * x[k];
  }
}

/* ------------------------------------------------------------ evaluator */

int orc_eval(const orc_system* s, const double* theta, const double* pos, orc_eval_out* out,
             double* O) {
  const int N = s->n_up + s->n_dn;
  const int P = orc_num_params(s);
  if (O) memset(O, 0, sizeof(double) * (size_t)P);
  double gD[ORC_MAX_ELEC * 3] = {0}, lD[ORC_MAX_ELEC] = {0};
  double gJ[ORC_MAX_ELEC * 3] = {0}, lJ[ORC_MAX_ELEC] = {0};
  double lnpsi = 0.0, sign = 1.0;

  /* Slater determinants, one per spin block */
  for (int blk = 0; blk < 2; ++blk) {
    int n = blk == 0 ? s->n_up : s->n_dn;
    int e0 = blk == 0 ? 0 : s->n_up;
    const double* C = blk == 0 ? s->coef_up : s->coef_dn;
    if (n == 0) continue;
    double A[ORC_MAX_SPIN * ORC_MAX_SPIN], inv[ORC_MAX_SPIN * ORC_MAX_SPIN];
    double chi[ORC_MAX_SPIN][ORC_MAX_BASIS], gchi[ORC_MAX_SPIN][ORC_MAX_BASIS][3];
    double lchi[ORC_MAX_SPIN][ORC_MAX_BASIS], dzchi[ORC_MAX_SPIN][ORC_MAX_BASIS];
    for (int i = 0; i < n; ++i)
      for (int b = 0; b < s->n_basis; ++b)
        basis_eval(s, theta, b, pos + 3 * (e0 + i), &chi[i][b], gchi[i][b], &lchi[i][b],
                   &dzchi[i][b]);
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < n; ++k) {
        double v = 0.0;
        for (int b = 0; b < s->n_basis; ++b) v += C[k * ORC_MAX_BASIS + b] * chi[i][b];
        A[i * n + k] = v;
      }
    double ld, sg;
    if (gj_inverse(n, A, inv, &ld, &sg) != 0) return -1;
    lnpsi += ld;
    sign *= sg;
    for (int i = 0; i < n; ++i) {
      int e = e0 + i;
      for (int b = 0; b < s->n_basis; ++b) {
        double wgt = 0.0; /* sum_k C[k][b] inv[k][i] */
        for (int k = 0; k < n; ++k) wgt += C[k * ORC_MAX_BASIS + b] * inv[k * n + i];
        for (int c = 0; c < 3; ++c) gD[3 * e + c] += wgt * gchi[i][b][c];
        lD[e] += wgt * lchi[i][b];
        if (O) O[s->b_exp[b]] += wgt * dzchi[i][b];
      }
    }
  }

  /* Jastrow */
  double J = 0.0;
  const double* nnth = s->nn_on ? theta + off_nn(s) : NULL;
  double* nnO = (O && s->nn_on) ? O + off_nn(s) : NULL;
  for (int i = 0; i < N; ++i)
    for (int j = i + 1; j < N; ++j) {
      const double* ri = pos + 3 * i;
      const double* rj = pos + 3 * j;
      double d[3] = {ri[0] - rj[0], ri[1] - rj[1], ri[2] - rj[2]};
      double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      int same = (i < s->n_up) == (j < s->n_up);
      double u = 0.0, du = 0.0, d2u = 0.0;
      if (s->ee_on) {
        double dudb, dpoly[ORC_MAX_POLY];
        int o = off_ee(s);
        pade_ee(r, same ? s->cusp_para : s->cusp_anti, theta[o], s->ee_kappa, s->ee_npoly,
                theta + o + 1, &u, &du, &d2u, &dudb, dpoly);
        if (O) {
          O[o] += dudb;
          for (int p = 0; p < s->ee_npoly; ++p) O[o + 1 + p] += dpoly[p];
        }
      }
      if (s->nn_on) {
        double y, dy, d2y;
        nn_pair(nnth, r, same ? 1.0 : 0.0, &y, &dy, &d2y, nnO);
        u += y; du += dy; d2u += d2y;
      }
      J += u;
      for (int c = 0; c < 3; ++c) {
        gJ[3 * i + c] += du * d[c] / r;
        gJ[3 * j + c] -= du * d[c] / r;
      }
      lJ[i] += d2u + 2.0 * du / r;
      lJ[j] += d2u + 2.0 * du / r;
    }
  for (int i = 0; i < N; ++i)
    for (int I = 0; I < s->n_nuc; ++I) {
      if (!s->en_on && !s->nn_on) break;
      const double* ri = pos + 3 * i;
      const double* R = s->nuc_pos + 3 * I;
      double d[3] = {ri[0] - R[0], ri[1] - R[1], ri[2] - R[2]};
      double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      double u = 0.0, du = 0.0, d2u = 0.0;
      if (s->en_on) {
        double A = s->en_coef[I], a = theta[off_en(s)];
        double q = 1.0 / (1.0 + a * r);
        u = A * r * q;
        du = A * q * q;
        d2u = -2.0 * A * a * q * q * q;
        if (O) O[off_en(s)] += -A * r * r * q * q;
      }
      if (s->nn_on) {
        double y, dy, d2y;
        nn_pair(nnth + ORC_NN_NET_P, r, (double)s->nuc_z[I], &y, &dy, &d2y,
                nnO ? nnO + ORC_NN_NET_P : NULL);
        u += y; du += dy; d2u += d2y;
      }
      J += u;
      for (int c = 0; c < 3; ++c) gJ[3 * i + c] += du * d[c] / r;
      lJ[i] += d2u + 2.0 * du / r;
    }
  lnpsi += J;

  /* assemble */
  double lap = 0.0;
  for (int i = 0; i < N; ++i) {
    double dot = 0.0, gj2 = 0.0;
    for (int c = 0; c < 3; ++c) {
      out->grad[3 * i + c] = gD[3 * i + c] + gJ[3 * i + c];
      dot += gD[3 * i + c] * gJ[3 * i + c];
      gj2 += gJ[3 * i + c] * gJ[3 * i + c];
    }
    lap += lD[i] + lJ[i] + 2.0 * dot + gj2;
  }
  double V = 0.0;
  if (s->pot_kind == ORC_POT_HARMONIC) {
    for (int i = 0; i < 3 * N; ++i) V += 0.5 * s->omega * s->omega * pos[i] * pos[i];
  } else {
    for (int i = 0; i < N; ++i) {
      for (int I = 0; I < s->n_nuc; ++I) {
        const double* R = s->nuc_pos + 3 * I;
        double d0 = pos[3 * i] - R[0], d1 = pos[3 * i + 1] - R[1], d2 = pos[3 * i + 2] - R[2];
        V -= s->nuc_z[I] / sqrt(d0 * d0 + d1 * d1 + d2 * d2);
      }
      for (int j = i + 1; j < N; ++j) {
        double d0 = pos[3 * i] - pos[3 * j], d1 = pos[3 * i + 1] - pos[3 * j + 1],
               d2 = pos[3 * i + 2] - pos[3 * j + 2];
        V += 1.0 / sqrt(d0 * d0 + d1 * d1 + d2 * d2);
      }
    }
    /* n-n repulsion constant, src/operator/src/operator.rs:42-49 */
    for (int I = 0; I < s->n_nuc; ++I)
      for (int K = I + 1; K < s->n_nuc; ++K) {
        const double* a = s->nuc_pos + 3 * I;
        const double* b = s->nuc_pos + 3 * K;
        double d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
        V += (double)(s->nuc_z[I] * s->nuc_z[K]) / sqrt(d0 * d0 + d1 * d1 + d2 * d2);
      }
  }
  out->lnpsi = lnpsi;
  out->sign = sign;
  out->lap_over_psi = lap;
  out->vpot = V;
  out->eloc = -0.5 * lap + V;
  return 0;
}

/* ---------------------------------------- reference example wavefunctions */

static double nrm(const double* x) { return sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]); }

/* 1-electron STO exp(-a|x|): value, gradient, laplacian, d/da, as in
 * examples/hydrogen_molecule.rs:43-57 and examples/dmc.rs:106-128. */
static double sto(double a, const double* x, double* g, double* lap, double* da) {
  double n = nrm(x), v = exp(-a * n);
  if (g)
    for (int k = 0; k < 3; ++k) g[k] = -a * v / n * x[k];
  if (lap) *lap = a * v / n * (a * n - 2.0);
  if (da) *da = -n * v;
  return v;
}

double orc_ref_wf(int kind, const double* par, const double* pos, double* grad, double* lap,
                  double* dpar) {
  if (kind == ORC_REF_HELIUM) {
    /* examples/helium_atom_singlet.rs:63-104 */
    double a = par[0], n1 = nrm(pos), n2 = nrm(pos + 3);
    double v = exp(-a * (n1 + n2));
    if (grad)
      for (int k = 0; k < 3; ++k) {
        grad[k] = -a / n1 * v * pos[k];
        grad[3 + k] = -a / n2 * v * pos[3 + k];
      }
    if (lap) *lap = a / n1 * v * (a * n1 - 2.0) + a / n2 * v * (a * n2 - 2.0);
    if (dpar) dpar[0] = -v * (n1 + n2);
    return v;
  }
  if (kind == ORC_REF_STO_H) {
    /* examples/dmc.rs:106-133 */
    return sto(par[0], pos, grad, lap, dpar);
  }
  if (kind == ORC_REF_H2_HL) {
    /* examples/hydrogen_molecule.rs:91-153; par = {alpha, separation} along x */
    double a = par[0], h = 0.5 * par[1];
    double x1m[3] = {pos[0] - h, pos[1], pos[2]}, x1p[3] = {pos[0] + h, pos[1], pos[2]};
    double x2m[3] = {pos[3] - h, pos[4], pos[5]}, x2p[3] = {pos[3] + h, pos[4], pos[5]};
    double g1m[3], g1p[3], g2m[3], g2p[3], l1m, l1p, l2m, l2p, d1m, d1p, d2m, d2p;
    double v1m = sto(a, x1m, g1m, &l1m, &d1m), v1p = sto(a, x1p, g1p, &l1p, &d1p);
    double v2m = sto(a, x2m, g2m, &l2m, &d2m), v2p = sto(a, x2p, g2p, &l2p, &d2p);
    double v = v1m * v2p + v1p * v2m;
    if (grad)
      for (int k = 0; k < 3; ++k) {
        grad[k] = v2p * g1m[k] + v2m * g1p[k];
        grad[3 + k] = v1p * g2m[k] + v1m * g2p[k];
      }
    if (lap) *lap = (v2p * l1m + v2m * l1p) + (v1p * l2m + v1m * l2p);
    if (dpar) dpar[0] = v1m * d2p + d1m * v2p + v1p * d2m + d1p * v2m;
    return v;
  }
  if (kind == ORC_REF_H2ION) {
    /* tests/hydrogen_molecular_ion_lcao.rs:66-92; par = {alpha, separation} */
    double a = par[0], h = 0.5 * par[1];
    double r1[3] = {pos[0] - h, pos[1], pos[2]}, r2[3] = {pos[0] + h, pos[1], pos[2]};
    double g1[3], g2[3], l1, l2;
    double v1 = sto(a, r1, g1, &l1, NULL), v2 = sto(a, r2, g2, &l2, NULL);
    if (grad)
      for (int k = 0; k < 3; ++k) grad[k] = v1 * g2[k] + v2 * g1[k];
    if (lap)
      *lap = v1 * l2 + v2 * l1 + 2.0 * (g1[0] * g2[0] + g1[1] * g2[1] + g1[2] * g2[2]);
    if (dpar) dpar[0] = 0.0;
    return v1 * v2;
  }
  /* ORC_REF_GAUSSIAN: examples/custom_operator.rs:301-316 (1 electron) */
  double a = par[0], n = nrm(pos);
  double v = exp(-(n / a) * (n / a));
  if (grad)
    for (int k = 0; k < 3; ++k) grad[k] = -2.0 * v / (a * a) * pos[k];
  if (lap) *lap = v * (4.0 * n * n - 6.0 * a * a) / (a * a * a * a);
  if (dpar) dpar[0] = v * 2.0 * n * n / (a * a * a); /* tests/sho_optimize.rs:73-78 */
  return v;
}

double orc_ref_eloc(int kind, const double* par, const double* pos, int n_nuc, const double* nuc_pos,
                    const int32_t* nuc_z, int harmonic, double omega) {
  int N = (kind == ORC_REF_HELIUM || kind == ORC_REF_H2_HL) ? 2 : 1;
  double lap;
  double psi = orc_ref_wf(kind, par, pos, NULL, &lap, NULL);
  /* KineticEnergy::act_on = -1/2 lap psi (operator.rs:122-124) */
  double t = -0.5 * lap;
  if (harmonic) {
    /* HarmonicHamiltonian::act_on (examples/custom_operator.rs:51-60):
     * 1/2 omega^2 |x|^2 psi, |x| the Frobenius norm of the whole cfg */
    double x2 = 0.0;
    for (int i = 0; i < 3 * N; ++i) x2 += pos[i] * pos[i];
    return (t + 0.5 * omega * omega * x2 * psi) / psi;
  }
  /* IonicPotential::value (operator.rs:22-33) + repulsion constant (42-49) */
  double vion = 0.0;
  for (int I = 0; I < n_nuc; ++I)
    for (int j = 0; j < N; ++j) {
      double d[3] = {pos[3 * j] - nuc_pos[3 * I], pos[3 * j + 1] - nuc_pos[3 * I + 1],
                     pos[3 * j + 2] - nuc_pos[3 * I + 2]};
      vion -= (double)nuc_z[I] / nrm(d);
    }
  for (int I = 0; I < n_nuc; ++I)
    for (int K = I + 1; K < n_nuc; ++K) {
      double d[3] = {nuc_pos[3 * K] - nuc_pos[3 * I], nuc_pos[3 * K + 1] - nuc_pos[3 * I + 1],
                     nuc_pos[3 * K + 2] - nuc_pos[3 * I + 2]};
      vion += (double)(nuc_z[I] * nuc_z[K]) / nrm(d);
    }
  /* ElectronicPotential::value (operator.rs:76-86) */
  double vee = 0.0;
  for (int i = 0; i < N; ++i)
    for (int j = i + 1; j < N; ++j) {
      double d[3] = {pos[3 * i] - pos[3 * j], pos[3 * i + 1] - pos[3 * j + 1],
                     pos[3 * i + 2] - pos[3 * j + 2]};
      vee += 1.0 / nrm(d);
    }
  /* ElectronicHamiltonian::act_on / psi (operator.rs:181-183, samplers.rs:89-90) */
  return (t + vion * psi + vee * psi) / psi;
}

/* ---------------------------------------------------------------- moves */

typedef struct {
  double lnpsi, sign;
  double grad[ORC_MAX_ELEC * 3];
} wstate;

static int eval_state(const orc_system* s, const double* th, const double* pos, wstate* w) {
  orc_eval_out o;
  if (orc_eval(s, th, pos, &o, NULL) != 0) return -1;
  w->lnpsi = o.lnpsi;
  w->sign = o.sign;
  memcpy(w->grad, o.grad, sizeof(w->grad));
  return 0;
}

/* One single-electron move of electron e; returns 1 if accepted.
 * Box: x_e += U(-L/2, L/2)^3, accept if min(psi'^2/psi^2, 1) > u
 *      (src/metropolis/src/metrop.rs:60-82).
 * Gauss: x_e += N(0, sigma^2)^3, same symmetric acceptance.
 * Diffuse: x_e += tau grad ln psi_e + N(0, tau)^3; reject on a sign change;
 *      accept with the Green's-function ratio over ALL electrons
 *      (src/metropolis/src/metrop.rs:150-198), evaluated in log form. */
static int move_electron(const orc_system* s, const double* th, int N, double* pos, wstate* cur,
                         int e, int move, double step, uint64_t seed, uint32_t walker,
                         uint32_t t) {
  uint32_t ua[4], ub[4];
  draw4(seed, walker, t, (uint32_t)(2 * e), TAG_MOVE, ua);
  double prop[ORC_MAX_ELEC * 3];
  memcpy(prop, pos, sizeof(double) * 3 * N);
  double dx[3] = {0.0, 0.0, 0.0};
  double uacc;
  /* box and Gaussian moves: x + step v rounded once (fma; u - 1/2 is exact) */
  if (move == ORC_MOVE_BOX) {
    for (int k = 0; k < 3; ++k) prop[3 * e + k] = fma(step, u01(ua[k]) - 0.5, prop[3 * e + k]);
    uacc = u01(ua[3]);
  } else {
    float z[4];
    f32_box_muller(ua[0], ua[1], &z[0], &z[1]);
    f32_box_muller(ua[2], ua[3], &z[2], &z[3]);
    draw4(seed, walker, t, (uint32_t)(2 * e + 1), TAG_MOVE, ub);
    uacc = u01(ub[0]);
    if (move == ORC_MOVE_GAUSS) {
      for (int k = 0; k < 3; ++k) prop[3 * e + k] = fma(step, (double)z[k], prop[3 * e + k]);
    } else {
      double sq = sqrt(step);
      for (int k = 0; k < 3; ++k) dx[k] = step * cur->grad[3 * e + k] + sq * (double)z[k];
      for (int k = 0; k < 3; ++k) prop[3 * e + k] += dx[k];
    }
  }
  wstate nw;
  if (eval_state(s, th, prop, &nw) != 0) return 0;
  double logA = 2.0 * (nw.lnpsi - cur->lnpsi);
  if (move == ORC_MOVE_DIFFUSE) {
    if (nw.sign != cur->sign) return 0;
    double hi = 0.0, lo = 0.0;
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < 3; ++k) {
        double dj = prop[3 * j + k] - pos[3 * j + k];
        double a = -dj - step * nw.grad[3 * j + k];
        double b = dj - step * cur->grad[3 * j + k];
        hi += a * a;
        lo += b * b;
      }
    logA += -(hi - lo) / (2.0 * step);
  }
  int acc = logA >= 0.0 ? 1 : exp(logA) > uacc;
  if (acc) {
    memcpy(pos, prop, sizeof(double) * 3 * N);
    *cur = nw;
  }
  return acc;
}

int orc_vmc_run(const orc_system* s, const double* th, int W, double* pos, const orc_vmc_opts* o,
                double* mom, double* tb, double* sO, double* sEO, double* sOO) {
  const int N = s->n_up + s->n_dn;
  const int P = orc_num_params(s);
  const int nb = o->n_steps / o->block_size;
  memset(mom, 0, sizeof(double) * ORC_NMOM);
  if (tb) memset(tb, 0, sizeof(double) * (size_t)nb);
  if (o->sr) {
    memset(sO, 0, sizeof(double) * (size_t)P);
    memset(sEO, 0, sizeof(double) * (size_t)P);
    memset(sOO, 0, sizeof(double) * (size_t)P * P);
  }
  double* O = (double*)malloc(sizeof(double) * (size_t)(P > 0 ? P : 1));
  for (int w = 0; w < W; ++w) {
    double* p = pos + (size_t)w * N * 3;
    wstate cur;
    if (eval_state(s, th, p, &cur) != 0) {
      free(O);
      return -1;
    }
    double bsum = 0.0;
    for (int it = 0; it < o->n_eq + o->n_steps; ++it) {
      uint32_t t = o->step0 + (uint32_t)it;
      for (int e = 0; e < N; ++e) {
        mom[ORC_MOM_ACCEPT] += move_electron(s, th, N, p, &cur, e, o->move, o->step, o->seed,
                                             o->walker0 + (uint32_t)w, t);
        mom[ORC_MOM_PROPOSED] += 1.0;
      }
      if (it < o->n_eq) continue;
      orc_eval_out ev;
      if (orc_eval(s, th, p, &ev, o->sr ? O : NULL) != 0) {
        free(O);
        return -1;
      }
      double E = ev.eloc;
      int k = it - o->n_eq;
      mom[ORC_MOM_COUNT] += 1.0;
      mom[ORC_MOM_SUM_E] += E;
      mom[ORC_MOM_SUM_E2] += E * E;
      bsum += E;
      if ((k + 1) % o->block_size == 0) {
        double m = bsum / o->block_size;
        mom[ORC_MOM_SUM_BLOCK2] += m * m;
        mom[ORC_MOM_NBLOCKS] += 1.0;
        if (tb) tb[k / o->block_size] += bsum;
        bsum = 0.0;
      }
      if (o->sr)
        for (int a = 0; a < P; ++a) {
          sO[a] += O[a];
          sEO[a] += E * O[a];
          for (int b = 0; b < P; ++b) sOO[a * P + b] += O[a] * O[b];
        }
    }
  }
  free(O);
  return 0;
}

/* ----------------------------------------------------------------- DMC */

/* Drift-diffusion sweep with accept/reject and weight update per walker
 * (src/dmc/src/dmc.rs:87-128), then a stochastic comb: walker k of the new
 * population is the parent j whose cumulative weight interval contains
 * (k + u) * sum(w) / W, u from one uniform; all new weights are equal. */
double orc_dmc_step(const orc_system* s, const double* th, int W, double* pos, double* eloc,
                    double tau, double e_ref, uint64_t seed, uint32_t step, double* accepted,
                    double* proposed, int* parent) {
  const int N = s->n_up + s->n_dn;
  double* w = (double*)malloc(sizeof(double) * (size_t)W);
  double ens = 0.0;
  for (int k = 0; k < W; ++k) {
    double* p = pos + (size_t)k * N * 3;
    wstate cur;
    eval_state(s, th, p, &cur);
    double e_old = eloc[k];
    ens += e_old;
    for (int e = 0; e < N; ++e) {
      *accepted += move_electron(s, th, N, p, &cur, e, ORC_MOVE_DIFFUSE, tau, seed, (uint32_t)k, step);
      *proposed += 1.0;
    }
    orc_eval_out ev;
    orc_eval(s, th, p, &ev, NULL);
    eloc[k] = ev.eloc;
    w[k] = exp(-tau * (0.5 * (e_old + ev.eloc) - e_ref));
  }
  ens /= W;
  /* comb */
  double* cum = (double*)malloc(sizeof(double) * (size_t)W);
  double acc = 0.0;
  for (int k = 0; k < W; ++k) {
    acc += w[k];
    cum[k] = acc;
  }
  uint32_t u[4];
  draw4(seed, 0u, step, 0u, TAG_COMB, u);
  double uu = u01(u[0]);
  int j = 0;
  for (int k = 0; k < W; ++k) {
    double target = ((double)k + uu) * (acc / W);
    while (j < W - 1 && cum[j] <= target) ++j;
    parent[k] = j;
  }
  double* np = (double*)malloc(sizeof(double) * (size_t)W * N * 3);
  double* ne = (double*)malloc(sizeof(double) * (size_t)W);
  for (int k = 0; k < W; ++k) {
    memcpy(np + (size_t)k * N * 3, pos + (size_t)parent[k] * N * 3, sizeof(double) * N * 3);
    ne[k] = eloc[parent[k]];
  }
  memcpy(pos, np, sizeof(double) * (size_t)W * N * 3);
  memcpy(eloc, ne, sizeof(double) * (size_t)W);
  free(np);
  free(ne);
  free(cum);
  free(w);
  return ens;
}
