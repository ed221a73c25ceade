// team.cuh -- FP64 VMC for small ensembles: a team of four warps per 32
// walkers, software-pipelined over the moves.
//
// With one walker per thread a 1,024-walker ensemble is 32 warps, one per
// SM sub-partition in use, and each sweep costs a warp its whole dependent
// FP64 instruction stream: GB300 issues one FP64 warp instruction per 64
// cycles per sub-partition, so the sweep takes (FP64 instructions per
// walker-step) x ~64 cycles whatever the number of walkers per warp. Here the
// stream of each walker is split over four warps on four sub-partitions:
//
//   warp 0  electron 0's moves: the orbital terms of the proposal (value,
//           gradient, Laplacian, exponent derivative, e-n potential), the
//           ratio and the decision;
//   warp 3  the same for electron 1;
//   warp 1  the pair value u of every move and the Jastrow difference;
//   warp 2  the local energy, O_k and every sum of the sweep before (from a
//           double-buffered snapshot in shared memory), with the pair's
//           derivative terms formed from its kept intermediates, while the
//           others run the next sweep.
//
// Move m = it N + e depends on the decision of move m - 1 only through the
// pair term (the other electron's position); electron e's orbital chain
// depends only on e's previous decision, two moves back. So the one-body
// warp of electron e forms its next proposal right after its decision and
// publishes it before the move in between, and runs its chain while the pair
// warp finishes that move: the per-move recurrence is the pair chain and the
// decision, and each orbital chain has two moves' time. The proposal, the
// ratio and the Jastrow difference pass through shared memory (four slots by
// m & 3); move m's named barrier (id 1 + e) joins the pair warp and warp e
// (bar.sync) and the other one-body warp (bar.arrive, once its proposal for
// move m + 1 is written). Each move's random numbers are drawn once, by its
// one-body warp; the acceptance number reaches the pair warp with the
// proposal, and both warps take the same decision from the same ratio,
// Jastrow difference and number. The arithmetic is Walker::move's and
// Walker::local_energy's on the same operands (the periodic rebuild would
// recompute the same values from the same positions, so only its
// singularity test is kept), and the moment sums fuse their products
// explicitly, as the per-thread kernel's do: trajectories and acceptance
// counts are the per-thread kernel's bit for bit, and so are the energies and
// SR sums for H2 and H; with He a few local-energy values differ in the last
// bit (not caused by the periodic rebuild, the walker's distance or the
// split of the value and derivative terms; not otherwise explained).
//
// A move is one dependent chain per warp, and on GB300 a dependent FP64
// instruction costs 64 cycles while an integer or FP32 one costs about 4.
// The move code is therefore straight-line: the nucleus count NB (1 or 2,
// one 1s function each) is a template parameter, the system's constants sit
// in registers, and the next move's random draw (Philox and the unit
// proposal, ~100 integer instructions) is made during the current move's
// chain, in the issue slots the FP64 chain leaves idle.
//
// Scope: FP64 box and Gaussian moves, at most one electron per spin, one 1s
// STO per nucleus (at most 2 nuclei), plain Pade e-e term or none, no e-n
// Jastrow, Coulomb potential; the host picks it for small ensembles.
//
// Named barriers: 1 + e (move of electron e; 96 threads, 64 for the last
// move), 3 + b (snapshot b written: the producers arrive, warp 2 waits),
// 5 + b (snapshot b read: warp 2 arrives, the producers wait before writing
// it again), b = sample parity; 7 (move 0's proposal, before the pair warp's
// first move). With one electron warp 0 runs alone and warps 1 and 3 idle.
#pragma once

#include "walker.cuh"

namespace mole {

constexpr int kTeamThreads = 128;

// Named barriers with compile-time ids (so that the kernel reserves only the
// ids it uses); the _par forms pick id or id + 1.
template <int ID>
__device__ __forceinline__ void named_sync(int n) {
  asm volatile("bar.sync %0, %1;" ::"n"(ID), "r"(n) : "memory");
}
template <int ID>
__device__ __forceinline__ void named_arrive(int n) {
  asm volatile("bar.arrive %0, %1;" ::"n"(ID), "r"(n) : "memory");
}
template <int ID>
__device__ __forceinline__ void named_sync_par(int par, int n) {
  if (par) named_sync<ID + 1>(n);
  else named_sync<ID>(n);
}
template <int ID>
__device__ __forceinline__ void named_arrive_par(int par, int n) {
  if (par) named_arrive<ID + 1>(n);
  else named_arrive<ID>(n);
}

// The system's constants of the team scope, loaded once into registers:
// nucleus I carries basis function I (a 1s STO). Without the e-e term the
// cusps are zero, which makes the pair value, slope and curvature zero.
template <int NB>
struct TeamConst {
  double R[NB][3], z[NB], Z[NB], c[2][NB];
  int ix[NB];
  double cusp_anti, cusp_para, ee_b, ee_m2b;
  __device__ explicit TeamConst(const SysParams<double>& sp) {
#pragma unroll
    for (int I = 0; I < NB; ++I) {
      R[I][0] = sp.nuc_pos[3 * I];
      R[I][1] = sp.nuc_pos[3 * I + 1];
      R[I][2] = sp.nuc_pos[3 * I + 2];
      z[I] = sp.b_zeta[I];
      Z[I] = sp.nuc_z[I];
      c[0][I] = sp.coef[0][0][I];
      c[1][I] = sp.coef[1][0][I];
      ix[I] = sp.b_exp[I];
    }
    cusp_anti = sp.ee_on ? sp.cusp_anti : 0.0;
    cusp_para = sp.ee_on ? sp.cusp_para : 0.0;
    ee_b = sp.ee_b;
    ee_m2b = sp.ee_m2b;
  }
};

// pair_vals<double, PM, false> of the team scope (plain Pade term, no
// polynomial), straight-line, split in two: the value u (keeping r^2, 1/r,
// r, q and c q), which the pair warp needs for each move, and the
// derivative terms from those, which the E_L warp forms once per sweep.
struct TeamPrScr {
  double r2, inv, r, q, cq;
};

template <int NB>
__device__ __forceinline__ double team_pair_value(const TeamConst<NB>& k, bool same, double d0, double d1, double d2,
                                                  TeamPrScr& s) {
  const double r2 = d0 * d0 + d1 * d1 + d2 * d2;
  const double inv = rsqrt_t<double>(r2);
  const double r = r2 * inv;
  const double cusp = same ? k.cusp_para : k.cusp_anti;
  // u = c r q, u' = c q^2, u'' = -2 b c q^3, du/db = -c r^2 q^2, q = 1 / (1 + b r)
  const double q = recip_t<double>(1.0 + k.ee_b * r);
  const double cq = cusp * q;
  s.r2 = r2;
  s.inv = inv;
  s.r = r;
  s.q = q;
  s.cq = cq;
  return cq * r;
}

template <int NB, int PM>
__device__ __forceinline__ void team_pair_derivs(const TeamConst<NB>& k, const TeamPrScr& s, PairVals<double, PM>& v) {
  v.inv = s.inv;
  v.db = 0;
  v.rs = s.r;
  const double uR = s.cq * s.q;
  // u'' is rounded on its own, as pair_vals rounds it (its polynomial loop
  // stands between the product and the sum below): no contraction into l
  const double uRR = __dmul_rn(k.ee_m2b * s.q, uR);
  if constexpr (PM > 0) v.db = -(s.r2 * uR);
  const double f = uR * s.inv;
  v.f = f;
  v.l = uRR + 2.0 * f;
}

// one_body<double, 1, NZ> of the team scope with the nucleus loop unrolled:
// the same operations on the same operands, so the same values.
template <int NB, int NZ>
__device__ __forceinline__ void team_one_body(const TeamConst<NB>& k, int spin, const double (&r)[3],
                                              OneBody<double, 1, NZ>& o) {
  o.val[0] = 0;
  o.grad[0][0] = o.grad[0][1] = o.grad[0][2] = 0;
  o.lap[0] = 0;
#pragma unroll
  for (int p = 0; p < OneBody<double, 1, NZ>::pm; ++p) o.dz[0][p] = 0;
  o.jen = 0;
  o.gjen[0] = o.gjen[1] = o.gjen[2] = 0;
  o.ljen = 0;
  o.djen = 0;
  o.ven = 0;
#pragma unroll
  for (int I = 0; I < NB; ++I) {
    const double d0 = r[0] - k.R[I][0], d1 = r[1] - k.R[I][1], d2 = r[2] - k.R[I][2];
    const double r2 = d0 * d0 + d1 * d1 + d2 * d2;
    const double inv = rsqrt_t<double>(r2);
    const double rr = r2 * inv;
    o.ven -= k.Z[I] * inv;
    const double z = k.z[I];
    const double rad = rr;
    double e = expm_t<double>(z, rad);
    e *= k.c[spin][I];
    const double chi = e;
    const double la = z * e;
    const double fr = -la * inv;
    const double lb = z - 2.0 * inv;  // lap = z e (z - 2 / r)
    o.val[0] += chi;
    o.grad[0][0] += fr * d0;
    o.grad[0][1] += fr * d1;
    o.grad[0][2] += fr * d2;
    o.lap[0] += la * lb;
    if constexpr (NZ > 0) {
#pragma unroll
      for (int p = 0; p < NZ; ++p)
        if (p == k.ix[I]) o.dz[0][p] -= rad * chi;
    }
  }
}

// The unit proposal of one move (Walker::move's draws): box moves u - 1/2
// exactly, Gaussian moves the FP32 normals; and the acceptance bits.
struct TeamUnit {
  double v[3];
  uint32_t ubits;
};
template <int MOVE>
__device__ __forceinline__ TeamUnit team_unit(uint64_t seed, uint32_t w, uint32_t t, int e) {
  TeamUnit u;
  const uint4 ra = draw4(seed, w, t, 2u * e, kTagMove);
  if constexpr (MOVE == kMoveBox) {
    u.v[0] = u01_centered(ra.x);
    u.v[1] = u01_centered(ra.y);
    u.v[2] = u01_centered(ra.z);
    u.ubits = ra.w;
  } else {
    float z0, z1, z2, z3;
    repro_box_muller(ra.x, ra.y, z0, z1);
    repro_box_muller(ra.z, ra.w, z2, z3);
    u.ubits = draw4(seed, w, t, 2u * e + 1u, kTagMove).x;
    u.v[0] = f2d(z0);
    u.v[1] = f2d(z1);
    u.v[2] = f2d(z2);
  }
  return u;
}

// The caches the E_L warp needs, per walker (slot [field][lane]): per
// electron x (3), the orbital value, gradient (3), Laplacian, [exponent
// derivative], e-n potential; the pair's intermediates r^2, 1/r, r, q, c q.
template <int N, int PM>
struct TeamSnap {
  static constexpr int NZ = PM == 0 ? 0 : 1;
  static constexpr int SF = 9 + NZ;
  static constexpr int NF0 = N * SF;
  static constexpr int NF1 = N == 2 ? 5 : 0;
  double f[2][NF0 + NF1][32];
};

template <int NU, int ND, int PM, int NB, int MOVE>
__device__ __forceinline__ void team_body(const SysParams<double>& sp, const VmcArgs& a) {
  using Wk = Walker<NU, ND, double, PM, false, false>;
  constexpr int N = NU + ND;
  constexpr int NZ = Wk::NZ;
  constexpr int NA = n_acc(PM);
  constexpr int NSR = NA - kNMom;
  using Snap = TeamSnap<N, PM>;
  constexpr int SF = Snap::SF;
  // warps taking part in a snapshot barrier: the E_L warp and the producers
  constexpr int kSnapThreads = N == 2 ? 128 : 64;
  __shared__ Snap snap;
  // per-move exchange, slot m & 3 for move m: the ratio (one-body warp), the
  // Jastrow difference (pair warp), the proposal and its acceptance draw
  // (one-body warp, for the pair warp)
  __shared__ double xr[4][32], xdj[4][32], xxn[4][3][32];
  __shared__ uint32_t xub[4][32];
  __shared__ double red[kTeamThreads / 32];
  const int lane = threadIdx.x & 31, role = threadIdx.x >> 5;
  const int w = blockIdx.x * 32 + lane;
  const bool active = w < a.W;
  const double step = a.step;
  const int total = a.n_eq + a.n_steps;
  const int refresh = a.refresh > 0 ? a.refresh : 100;
  const int M = total * N;  // moves of the run; move m = it N + e

  Wk wk;
  wk.nn = NnCtx<double>{nullptr, nullptr, 0};
  if (active) wk.load(a.pos, a.W, w);
  else
#pragma unroll
    for (int e = 0; e < N; ++e) wk.x[e][0] = wk.x[e][1] = wk.x[e][2] = 1.0 + e;
  bool ok = true;
  int naccept = 0;
  // the E_L warp's sums
  double sE = acc_zero<double>(), sE2 = acc_zero<double>(), bsum = acc_zero<double>(), sB2 = 0.0;
  double srv[NSR > 0 ? NSR : 1];
#pragma unroll
  for (int k = 0; k < (NSR > 0 ? NSR : 1); ++k) srv[k] = 0.0;
  bool e_finite = true;
  const TeamConst<NB> kc(sp);

  // One-body warp of electron E: its orbital value chain, decisions and
  // derivative caches. Its next proposal is formed right after its decision
  // and published before the pair warp needs it (the barrier of the move
  // in between).
  auto one_body_warp = [&](auto ec) {
    constexpr int E = decltype(ec)::value;
    constexpr int spin = E < NU ? 0 : 1;
    OneBody<double, 1, NZ> o;
    team_one_body<NB, NZ>(kc, spin, wk.x[E], o);
    double vo = o.val[0];  // the orbital value; 1x1 inverse = 1 / vo
    ok = !is_zero(vo);
    const TeamUnit u0 = team_unit<MOVE>(a.seed, (uint32_t)w, a.step0, E);
    double xn[3];
    xn[0] = fma(step, u0.v[0], wk.x[E][0]);
    xn[1] = fma(step, u0.v[1], wk.x[E][1]);
    xn[2] = fma(step, u0.v[2], wk.x[E][2]);
    uint32_t ub = u0.ubits;
    if (N == 2 && M > 0) {
      xxn[E][0][lane] = xn[0];
      xxn[E][1][lane] = xn[1];
      xxn[E][2][lane] = xn[2];
      xub[E][lane] = ub;
      if (E == 0) named_arrive<7>(64);  // move 0's proposal, before the pair warp's first move
      else named_arrive<1>(96);         // move 1's, at the barrier of move 0
    }
    for (int it = 0; it < total; ++it) {
      const uint32_t t = a.step0 + (uint32_t)it;
      [[maybe_unused]] const int m = it * N + E;
      // this electron's next draw (sweep it + 1), beside the value chain
      const TeamUnit un = team_unit<MOVE>(a.seed, (uint32_t)w, t + 1u, E);
      const double B = recip(vo);
      OneBody<double, 1, NZ> on;
      team_one_body<NB, NZ>(kc, spin, xn, on);
      const double val = on.val[0];
      double ratio = acc_zero<double>();
      ratio += val * B;
      double dJ;
      if constexpr (N == 2) {
        xr[m & 3][lane] = ratio;
        named_sync<1 + E>(m + 1 < M ? 96 : 64);
        dJ = xdj[m & 3][lane];
      } else {
        dJ = acc_zero<double>();
      }
      const bool acc = metropolis_accept_dj(ratio, dJ, ub);
      if (acc) {
        wk.x[E][0] = xn[0];
        wk.x[E][1] = xn[1];
        wk.x[E][2] = xn[2];
        vo = val;
        naccept += 1;
      }
      if (it + 1 < total) {
        xn[0] = fma(step, un.v[0], wk.x[E][0]);
        xn[1] = fma(step, un.v[1], wk.x[E][1]);
        xn[2] = fma(step, un.v[2], wk.x[E][2]);
        ub = un.ubits;
        if constexpr (N == 2) {
          const int s2 = (m + 2) & 3;
          xxn[s2][0][lane] = xn[0];
          xxn[s2][1][lane] = xn[1];
          xxn[s2][2][lane] = xn[2];
          xub[s2][lane] = ub;
          named_arrive<2 - E>(96);  // the barrier of move m + 1 (the other electron's)
        }
      }
      if (acc) o = on;
      // the periodic rebuild recomputes these caches from the same
      // positions by the same arithmetic, so only its singularity test remains
      if ((it + 1) % refresh == 0) ok = !is_zero(vo) && ok;
      if (it < a.n_eq) continue;
      const int k = it - a.n_eq, b = k & 1;
      if (k >= 2) named_sync_par<5>(b, kSnapThreads);
      double(*s)[32] = snap.f[b];
      s[SF * E + 0][lane] = wk.x[E][0];
      s[SF * E + 1][lane] = wk.x[E][1];
      s[SF * E + 2][lane] = wk.x[E][2];
      s[SF * E + 3][lane] = vo;
      s[SF * E + 4][lane] = o.grad[0][0];
      s[SF * E + 5][lane] = o.grad[0][1];
      s[SF * E + 6][lane] = o.grad[0][2];
      s[SF * E + 7][lane] = o.lap[0];
      if constexpr (NZ > 0) s[SF * E + 8][lane] = o.dz[0][0];
      s[SF * E + 8 + NZ][lane] = o.ven;
      named_arrive_par<3>(b, kSnapThreads);
    }
    for (int k = (a.n_steps >= 2 ? a.n_steps - 2 : 0); k < a.n_steps; ++k) named_sync_par<5>(k & 1, kSnapThreads);
  };

  if (role == 0) {
    one_body_warp(std::integral_constant<int, 0>{});
  } else if (role == 3) {
    if constexpr (N == 2) one_body_warp(std::integral_constant<int, 1>{});
  } else if (role == 1) {
    if constexpr (N == 2) {
      // the pair warp: the Jastrow difference of each move, which needs the
      // decision of the move before (the other electron's position)
      TeamPrScr ps;
      double pu = team_pair_value<NB>(kc, Wk::same_spin(0, 1), wk.x[0][0] - wk.x[1][0], wk.x[0][1] - wk.x[1][1],
                                      wk.x[0][2] - wk.x[1][2], ps);
      if (M > 0) named_sync<7>(64);
      for (int it = 0; it < total; ++it) {
        static_for<0, 2>([&](auto ec) {
          constexpr int e = decltype(ec)::value;
          constexpr int j = 1 - e;
          const int m = it * 2 + e, sl = m & 3;
          double xn[3];
          xn[0] = xxn[sl][0][lane];
          xn[1] = xxn[sl][1][lane];
          xn[2] = xxn[sl][2][lane];
          const uint32_t ub = xub[sl][lane];
          TeamPrScr pn;
          const double un = team_pair_value<NB>(kc, Wk::same_spin(e, j), xn[0] - wk.x[j][0], xn[1] - wk.x[j][1],
                                                xn[2] - wk.x[j][2], pn);
          double dJ = acc_zero<double>();
          dJ += un - pu;
          xdj[sl][lane] = dJ;
          named_sync<1 + e>(m + 1 < M ? 96 : 64);
          const double ratio = xr[sl][lane];
          if (metropolis_accept_dj(ratio, dJ, ub)) {
            wk.x[e][0] = xn[0];
            wk.x[e][1] = xn[1];
            wk.x[e][2] = xn[2];
            pu = un;
            ps = pn;
          }
        });
        if (it < a.n_eq) continue;
        const int k = it - a.n_eq, b = k & 1;
        if (k >= 2) named_sync_par<5>(b, kSnapThreads);
        double(*s)[32] = snap.f[b];
        s[Snap::NF0 + 0][lane] = ps.r2;
        s[Snap::NF0 + 1][lane] = ps.inv;
        s[Snap::NF0 + 2][lane] = ps.r;
        s[Snap::NF0 + 3][lane] = ps.q;
        s[Snap::NF0 + 4][lane] = ps.cq;
        named_arrive_par<3>(b, kSnapThreads);
      }
      for (int k = (a.n_steps >= 2 ? a.n_steps - 2 : 0); k < a.n_steps; ++k) named_sync_par<5>(k & 1, kSnapThreads);
    }
  } else {
    // the E_L warp: E_L, O_k and the sums of sampled sweep k from snapshot k & 1
    for (int k = 0; k < a.n_steps; ++k) {
      const int b = k & 1;
      named_sync_par<3>(b, kSnapThreads);
      const double(*s)[32] = snap.f[b];
      double vs[N];
#pragma unroll
      for (int e = 0; e < N; ++e) {
        wk.x[e][0] = s[SF * e + 0][lane];
        wk.x[e][1] = s[SF * e + 1][lane];
        wk.x[e][2] = s[SF * e + 2][lane];
        vs[e] = s[SF * e + 3][lane];
        wk.og[e][0][0] = s[SF * e + 4][lane];
        wk.og[e][0][1] = s[SF * e + 5][lane];
        wk.og[e][0][2] = s[SF * e + 6][lane];
        wk.ol[e][0] = s[SF * e + 7][lane];
        if constexpr (NZ > 0) wk.odz[e][0][0] = s[SF * e + 8][lane];
        wk.ven[e] = s[SF * e + 8 + NZ][lane];
      }
      TeamPrScr ps;
      if constexpr (N == 2) {
        ps.r2 = s[Snap::NF0 + 0][lane];
        ps.inv = s[Snap::NF0 + 1][lane];
        ps.r = s[Snap::NF0 + 2][lane];
        ps.q = s[Snap::NF0 + 3][lane];
        ps.cq = s[Snap::NF0 + 4][lane];
      }
      named_arrive_par<5>(b, kSnapThreads);
      // the 1x1 inverses (the move's own reciprocal of the orbital value)
#pragma unroll
      for (int e = 0; e < N; ++e) {
        if (e < NU) wk.bu[0] = recip(vs[e]);
        else wk.bd[0] = recip(vs[e]);
      }
      if constexpr (N == 2) {
        PairVals<double, PM> pv;
        team_pair_derivs<NB, PM>(kc, ps, pv);
        wk.pf[0] = pv.f;
        wk.pl[0] = pv.l;
        wk.pinv[0] = pv.inv;
        if constexpr (PM > 0) {
          wk.pdb[0] = pv.db;
          wk.prs[0] = pv.rs;
        }
      }
      double O[PM > 0 ? PM : 1];
      const double E = wk.local_energy(sp, O, nullptr, nullptr);
      e_finite = e_finite && (E == E);
      // fused explicitly, as the per-thread kernel's sums are
      sE2 = fma(E, E, sE2);
      bsum += E;
      if constexpr (PM > 0) {
#pragma unroll
        for (int p = 0; p < PM; ++p) {
          srv[p] += O[p];
          srv[PM + p] = fma(E, O[p], srv[PM + p]);
        }
        int qq = 2 * PM;
#pragma unroll
        for (int p = 0; p < PM; ++p)
#pragma unroll
          for (int r = p; r < PM; ++r, ++qq) srv[qq] = fma(O[p], O[r], srv[qq]);
      }
      if ((k + 1) % a.block_size == 0) {
        const double bs = bsum;
        const double m = bs / a.block_size;
        sB2 = fma(m, m, sB2);
        const double v = warp_sum(active ? bs : 0.0);
        if (lane == 0) a.tb_partials[(size_t)blockIdx.x * (a.n_steps / a.block_size) + k / a.block_size] = v;
        sE += bsum;
        bsum = acc_zero<double>();
      }
    }
    sE += bsum;
  }

  // one partial row per CTA (deterministic order, as vmc_body's)
  double acc[kNMom] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (active) {
    if (role == 0 || role == 3) {
      acc[5] = (double)naccept;
      if (!ok) atomicOr(a.status, 2);
    }
    if (role == 0) acc[6] = (double)total * N;
    if (role == (N == 2 ? 1 : 0)) wk.store(a.pos, a.W, w);  // the pair warp holds both positions
    if (role == 2) {
      acc[0] = (double)a.n_steps;
      acc[1] = sE;
      acc[2] = sE2;
      acc[3] = sB2;
      acc[4] = (double)(a.n_steps / a.block_size);
      if (!e_finite || !(sE2 < 1e300)) atomicOr(a.status, 1);
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NA; ++k) {
    double v[1] = {k < kNMom ? acc[k] : ((active && role == 2) ? srv[k - kNMom] : 0.0)};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) a.partials[(size_t)blockIdx.x * NA + k] = v[0];
  }
}

// FP64 VMC with a four-warp team per 32 walkers (box: move 0, else
// Gaussian), NB nuclei with one 1s function each.
template <int NU, int ND, int PM, int NB>
__global__ void __launch_bounds__(kTeamThreads) vmc_team_kernel(const __grid_constant__ SysParams<double> sp,
                                                               const VmcArgs a) {
  if (a.move == kMoveBox) team_body<NU, ND, PM, NB, kMoveBox>(sp, a);
  else team_body<NU, ND, PM, NB, kMoveGauss>(sp, a);
}

}  // namespace mole
