// compact.cuh -- FP64 Metropolis moves whose FP64 work is packed across the
// warps of a CTA.
//
// GB300 issues one FP64 warp instruction per 64 cycles per SM sub-partition,
// and a warp instruction takes that slot whatever the number of active lanes
// (measured: an FMA chain run by 1, 8, 16 or 32 lanes of every warp takes the
// same time). With one walker per thread, the FP64 evaluation of a proposal
// (orbitals, pair term, new inverse) therefore costs every warp the same
// whether 30 % of its lanes will reject the move or not. Here each move is
// done in three phases:
//
//   1. every thread screens its own proposal in FP32: the acceptance
//      ratio^2 e^(2 dJ) against the uniform u, with a bound on the FP32
//      error (below). Clearly rejected proposals are done; the others
//      (accepted, or too close to call) take a slot;
//   2. the slots are numbered across the CTA (warp ballots and a prefix over
//      the warps) and their inputs (the walker's id, the moving electron's
//      and its partner's FP64 positions) written to shared memory; thread k
//      then evaluates slot k in FP64 -- the proposal drawn again from the
//      walker's random stream, its orbitals, pair term and new inverse --
//      so the FP64 instructions run on ceil(slots / 32) warps instead of
//      all of them;
//   3. the owner reads its slot back, decides the close calls with the FP64
//      test (metropolis_accept_dj, exactly as the one-thread-per-walker
//      kernel) and commits.
//
// The FP64 arithmetic of a slot is the same code, on the same operands, as
// Walker::move's, and the screen's error bound makes every decision equal to
// the FP64 one: the trajectories are those of the one-thread-per-walker
// kernel, bit for bit.
//
// Layout: two 7-warp CTAs per SM (216 walkers each at 65,536 walkers) at most
// 128 registers, so that the 14 warps fit the four SM sub-partitions'
// 16,384-register files. Measured on H2 (65,536 walkers, Gaussian 0.4,
// two-parameter SR sums): FP64-pipe instructions per walker-step 211 -> 181,
// the launch 53.5 -> 51.5 ms; the gain is bounded because a sub-partition
// holds only ~3.5 walker warps, so its FP64 work shrinks by whole warps, and
// the FP64 pipe idles while both CTAs screen (pipe busy 80 % -> 71 %). Four
// 4-warp CTAs (201 instructions, 55.7 ms) and three 5-warp CTAs (196, 54.4
// ms) did worse.
//
// Scope: the FP64 box and Gaussian moves of systems with at most one electron
// per spin (He, H2, H, H2+), a basis of 1s STOs, the Pade e-e term without
// scaled distance or polynomial terms, no e-n Jastrow, Coulomb potential --
// the host picks this kernel only then, and only for ensembles of at least
// half a wave (smaller ones keep more CTAs busy with 64-walker CTAs).
//
// FP32 error bound of the screen. Positions enter as their top 24 bits, so
// every coordinate, difference and distance carries an absolute error below
// dr = 2^-21 (|x| + |R| + 2 r) (truncation 2^-23, roundings 2^-24, the
// approximate rsqrt 2^-22.9). A 1s term c e^(-z r) then has relative error
// below 2^-20 (1 + z (xm + Rmax + 2 r)) (z dr, the argument's rounding and
// ex2.approx's 2^-22.5, the coefficient's rounding); the screen uses 2^-19,
// twice that. The ratio phi B takes their magnitude sum over |phi| (so a
// cancelling sum widens the bound) plus 2^-22 for B's truncation. The pair
// term u = c r / (1 + b r) has |du/dr| = |c| q^2 <= |c|, so its error is below
// |c| dr_pair + 2^-20 |u|; the cached old u enters truncated (2^-23). The
// logarithms (lg2.approx, 2^-22 absolute, and the product's rounding) add
// 2^-20 (1 + |ln ratio^2| + |ln u|). ln(1 + d) <= 1.34 d for d <= 1/4 gives
// tol = 3 d_ratio + 2 d_J + d_log; outside d_ratio <= 1/4, normal magnitudes
// and coordinates below 10^3 the move is a close call.
#pragma once

#include "walker.cuh"

namespace mole {

constexpr int kCompactBlock = 224;  // 7 warps; two CTAs per SM hold 65,536 walkers in one wave
constexpr int kCompactMinBlocks = 2;
enum { kScrReject = 0, kScrAccept = 1, kScrUnsure = 2 };

// Shared-memory slots of one move, field-major (slot k of field f at f[f][k]).
// Inputs (x_e, x_partner) occupy fields 0..5 and are overwritten in place by
// the outputs: xn[3], val, 1/val, grad[3], lap, dz (with SR sums), ven and,
// with two electrons, the pair's u, u'/r, u'' + 2u'/r, 1/r (+ du/db, r).
template <int N, int PM>
struct CompactSlots {
  static constexpr int NZ = PM == 0 ? 0 : 1;
  static constexpr int NPV = N == 2 ? (PM > 0 ? 6 : 4) : 0;
  static constexpr int NF = 10 + NZ + NPV;
  double f[NF][kCompactBlock];
  uint32_t wid[kCompactBlock];
  int wcnt[kCompactBlock / 32];
};

// u - 1/2 = (x - 2^31 + 1/2) 2^-32 in FP32 for the screen (relative error
// 2^-24 of the exact value, also near u = 1/2).
__device__ __forceinline__ float u01c_f(uint32_t x) {
  return __fmaf_rn((float)(int32_t)(x ^ 0x80000000u), 0x1p-32f, 0x1p-33f);
}

// Phase 1: the FP32 screen of electron e's proposal; sets ubits (the
// acceptance uniform's bits) for the FP64 close call.
template <int NU, int ND, int MOVE, int e, class Wk>
__device__ __forceinline__ int screen_move(const Wk& wk, const SysParams<double>& sp, float stepf, uint64_t seed,
                                           uint32_t wid, uint32_t t, uint32_t& ubits) {
  constexpr int N = NU + ND;
  constexpr bool isup = e < NU;
  const ScreenParams& q = sp.scr;
  const uint4 ra = draw4(seed, wid, t, 2u * e, kTagMove);
  float v0, v1, v2;
  if constexpr (MOVE == kMoveBox) {
    v0 = u01c_f(ra.x);
    v1 = u01c_f(ra.y);
    v2 = u01c_f(ra.z);
    ubits = ra.w;
  } else {
    float z3;
    repro_box_muller(ra.x, ra.y, v0, v1);
    repro_box_muller(ra.z, ra.w, v2, z3);
    ubits = draw4(seed, wid, t, 2u * e + 1u, kTagMove).x;
  }
  const float xo0 = d2f_rz(wk.x[e][0]), xo1 = d2f_rz(wk.x[e][1]), xo2 = d2f_rz(wk.x[e][2]);
  const float x0 = fmaf(stepf, v0, xo0), x1 = fmaf(stepf, v1, xo1), x2 = fmaf(stepf, v2, xo2);
  const float xm = fmaxf(fmaxf(fmaxf(fabsf(x0), fabsf(x1)), fabsf(x2)), fmaxf(fmaxf(fabsf(xo0), fabsf(xo1)), fabsf(xo2)));
  // the new orbital value and the magnitude sum of its terms' error bounds
  float phi = 0.f, err = 0.f;
  #pragma unroll 1
  for (int I = 0; I < sp.n_nuc; ++I) {
    const float d0 = x0 - q.nuc[3 * I], d1 = x1 - q.nuc[3 * I + 1], d2 = x2 - q.nuc[3 * I + 2];
    const float r2 = fmaf(d0, d0, fmaf(d1, d1, d2 * d2));
    const float r = r2 * rsqrt_approx(r2);
    const int b1 = sp.nuc_b0[I + 1];
    #pragma unroll 1
    for (int b = sp.nuc_b0[I]; b < b1; ++b) {
      const float z = q.zeta[b];
      const float ce = q.coef[isup ? 0 : 1][b] * __expf(-z * r);
      phi += ce;
      err = fmaf(fabsf(ce), fmaf(z, xm + q.rmax + 2.f * r, 1.f), err);
    }
  }
  const float bf = d2f_rz(isup ? wk.bu[0] : wk.bd[0]);
  const float ratio = phi * bf;
  // |ratio error| / |ratio|
  const float dr = fmaf(0x1p-19f, err / fabsf(phi), 0x1p-22f);
  float dJ = 0.f, dj_err = 0.f;
  if constexpr (N == 2) {
    constexpr int j = 1 - e;
    const float xj0 = d2f_rz(wk.x[j][0]), xj1 = d2f_rz(wk.x[j][1]), xj2 = d2f_rz(wk.x[j][2]);
    const float xjm = fmaxf(fmaxf(fabsf(xj0), fabsf(xj1)), fabsf(xj2));
    const float d0 = x0 - xj0, d1 = x1 - xj1, d2 = x2 - xj2;
    const float r2 = fmaf(d0, d0, fmaf(d1, d1, d2 * d2));
    const float r = r2 * rsqrt_approx(r2);
    const float c = Wk::same_spin(e, j) ? q.cusp_para : q.cusp_anti;
    const float un = c * r * rcp_approx(fmaf(q.ee_b, r, 1.f));
    const float uo = d2f_rz(wk.pu[0]);
    dJ = un - uo;
    dj_err = fmaf(fabsf(c) * 0x1p-20f, xm + xjm + 2.f * r, 0x1p-20f * (fabsf(un) + fabsf(uo)));
  }
  const float uf = u01<float>(ubits);
  const float lr = __logf(ratio * ratio), lu = __logf(uf);
  const float L = lr + 2.f * dJ - lu;
  const float tol = fmaf(3.f, dr, fmaf(2.f, dj_err, 0x1p-20f * (1.f + fabsf(lr) + fabsf(lu))));
  const bool ok = fabsf(phi) > 1e-30f && fabsf(phi) < 1e30f && dr < 0.25f && xm < 1e3f && fabsf(lr) < 80.f &&
                  fabsf(dJ) < 40.f;
  if (!ok) return kScrUnsure;
  return L > tol ? kScrAccept : (L < -tol ? kScrReject : kScrUnsure);
}

// Phase 2: the FP64 evaluation of slot k (run by thread k).
template <int NU, int ND, int PM, int MOVE, int e, class Wk, class CS>
__device__ __forceinline__ void compact_task(const SysParams<double>& sp, double step, uint64_t seed, uint32_t t, CS& cs,
                                             int k) {
  constexpr int N = NU + ND;
  constexpr bool isup = e < NU;
  constexpr int NZ = CS::NZ;
  const uint32_t wid = cs.wid[k];
  const double xe[3] = {cs.f[0][k], cs.f[1][k], cs.f[2][k]};
  double xj[3] = {0.0, 0.0, 0.0};
  if constexpr (N == 2) {
    xj[0] = cs.f[3][k];
    xj[1] = cs.f[4][k];
    xj[2] = cs.f[5][k];
  }
  // the walker's FP64 proposal, its random numbers drawn again (Walker::move's arithmetic)
  const uint4 ra = draw4(seed, wid, t, 2u * e, kTagMove);
  double xn[3];
  if constexpr (MOVE == kMoveBox) {
    xn[0] = fma(step, u01_centered(ra.x), xe[0]);
    xn[1] = fma(step, u01_centered(ra.y), xe[1]);
    xn[2] = fma(step, u01_centered(ra.z), xe[2]);
  } else {
    float z0, z1, z2, z3;
    repro_box_muller(ra.x, ra.y, z0, z1);
    repro_box_muller(ra.z, ra.w, z2, z3);
    xn[0] = fma(step, f2d(z0), xe[0]);
    xn[1] = fma(step, f2d(z1), xe[1]);
    xn[2] = fma(step, f2d(z2), xe[2]);
  }
  OneBody<double, 1, NZ> o;
  one_body<double, 1, NZ, false, false>(sp, isup ? 0 : 1, xn, o);
  PairVals<double, PM> pv;
  if constexpr (N == 2)
    pair_vals<double, PM, false>(sp, Wk::same_spin(e, 1 - e), xn[0] - xj[0], xn[1] - xj[1], xn[2] - xj[2], pv);
  const double binv = recip(o.val[0]);
  cs.f[0][k] = xn[0];
  cs.f[1][k] = xn[1];
  cs.f[2][k] = xn[2];
  cs.f[3][k] = o.val[0];
  cs.f[4][k] = binv;
  cs.f[5][k] = o.grad[0][0];
  cs.f[6][k] = o.grad[0][1];
  cs.f[7][k] = o.grad[0][2];
  cs.f[8][k] = o.lap[0];
  if constexpr (NZ > 0) cs.f[9][k] = o.dz[0][0];
  cs.f[9 + NZ][k] = o.ven;
  if constexpr (N == 2) {
    cs.f[10 + NZ][k] = pv.u;
    cs.f[11 + NZ][k] = pv.f;
    cs.f[12 + NZ][k] = pv.l;
    cs.f[13 + NZ][k] = pv.inv;
    if constexpr (PM > 0) {
      cs.f[14 + NZ][k] = pv.db;
      cs.f[15 + NZ][k] = pv.rs;
    }
  }
}

// One move of electron e with the packed FP64 evaluation; every thread of
// the CTA calls it (inactive ones screen nothing). Returns 1 when accepted.
template <int NU, int ND, int PM, int MOVE, int e, class Wk, class CS>
__device__ __forceinline__ int compact_move(Wk& wk, const SysParams<double>& sp, double step, float stepf,
                                            uint64_t seed, uint32_t wid, uint32_t t, bool active, CS& cs) {
  constexpr int N = NU + ND;
  constexpr bool isup = e < NU;
  constexpr int NZ = CS::NZ;
  uint32_t ubits = 0;
  const int dec = active ? screen_move<NU, ND, MOVE, e>(wk, sp, stepf, seed, wid, t, ubits) : kScrReject;
  const bool need = dec != kScrReject;
  const unsigned m = __ballot_sync(0xffffffffu, need);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) cs.wcnt[warp] = __popc(m);
  __syncthreads();
  int base = 0, total = 0;
#pragma unroll
  for (int w = 0; w < kCompactBlock / 32; ++w) {
    const int c = cs.wcnt[w];
    base += w < warp ? c : 0;
    total += c;
  }
  const int slot = base + __popc(m & ((1u << lane) - 1u));
  if (need) {
    cs.wid[slot] = wid;
    cs.f[0][slot] = wk.x[e][0];
    cs.f[1][slot] = wk.x[e][1];
    cs.f[2][slot] = wk.x[e][2];
    if constexpr (N == 2) {
      cs.f[3][slot] = wk.x[1 - e][0];
      cs.f[4][slot] = wk.x[1 - e][1];
      cs.f[5][slot] = wk.x[1 - e][2];
    }
  }
  __syncthreads();
  if ((int)threadIdx.x < total) compact_task<NU, ND, PM, MOVE, e, Wk>(sp, step, seed, t, cs, threadIdx.x);
  __syncthreads();
  if (!need) return 0;
  OneBody<double, 1, NZ> o;
  o.val[0] = cs.f[3][slot];
  o.grad[0][0] = cs.f[5][slot];
  o.grad[0][1] = cs.f[6][slot];
  o.grad[0][2] = cs.f[7][slot];
  o.lap[0] = cs.f[8][slot];
  if constexpr (NZ > 0) o.dz[0][0] = cs.f[9][slot];
  o.ven = cs.f[9 + NZ][slot];
  o.jen = 0.0;
  o.gjen[0] = o.gjen[1] = o.gjen[2] = 0.0;
  o.ljen = 0.0;
  o.djen = 0.0;
  PairVals<double, PM> pv;
  if constexpr (N == 2) {
    pv.u = cs.f[10 + NZ][slot];
    pv.f = cs.f[11 + NZ][slot];
    pv.l = cs.f[12 + NZ][slot];
    pv.inv = cs.f[13 + NZ][slot];
    pv.db = 0.0;
    pv.rs = 0.0;
    if constexpr (PM > 0) {
      pv.db = cs.f[14 + NZ][slot];
      pv.rs = cs.f[15 + NZ][slot];
    }
  }
  if (dec == kScrUnsure) {
    // the close call: the FP64 test of Walker::move on the FP64 values
    const double ratio = o.val[0] * (isup ? wk.bu[0] : wk.bd[0]);
    double dJ = acc_zero<double>();
    if constexpr (N == 2) dJ += pv.u - wk.pu[0];
    if (!metropolis_accept_dj(ratio, dJ, ubits)) return 0;
  }
  wk.x[e][0] = cs.f[0][slot];
  wk.x[e][1] = cs.f[1][slot];
  wk.x[e][2] = cs.f[2][slot];
  wk.template put_one_body<e, 1>(o);
  if constexpr (N == 2) wk.put_pair(0, pv);
  if constexpr (isup) wk.bu[0] = cs.f[4][slot];
  else wk.bd[0] = cs.f[4][slot];
  return 1;
}

template <int NU, int ND, int PM, int MOVE, class Wk, class CS>
__device__ __forceinline__ int compact_sweep(Wk& wk, const SysParams<double>& sp, double step, float stepf,
                                             uint64_t seed, uint32_t wid, uint32_t t, bool active, CS& cs) {
  int acc = 0;
  static_for<0, NU + ND>([&](auto ec) {
    acc += compact_move<NU, ND, PM, MOVE, decltype(ec)::value>(wk, sp, step, stepf, seed, wid, t, active, cs);
  });
  return acc;
}

}  // namespace mole
