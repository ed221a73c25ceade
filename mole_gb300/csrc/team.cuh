// team.cuh -- FP64 VMC for small ensembles: a team of three warps per 32
// walkers.
//
// With one walker per thread a 1,024-walker ensemble is 32 warps, one per
// SM sub-partition in use, and each sweep costs a warp its whole dependent
// FP64 instruction stream: GB300 issues one FP64 warp instruction per 64
// cycles per sub-partition, so the sweep takes (FP64 instructions per
// walker-step) x ~64 cycles whatever the number of walkers per warp. Here the
// stream of each walker is split over three warps on three sub-partitions:
//
//   warp 0  the moved electron's orbital terms (value, gradient, Laplacian,
//           exponent derivative, e-n potential), the ratio and the new
//           1x1 inverse;
//   warp 1  the same proposal's pair term (u, u'/r, u'' + 2u'/r, 1/r, du/db);
//   warp 2  the local energy, O_k and every sum of the sweep before (from a
//           double-buffered snapshot of the caches in shared memory), while
//           warps 0 and 1 run the next sweep.
//
// Warps 0 and 1 draw the same random numbers, exchange the ratio and the
// Jastrow difference through shared memory (one named barrier per move,
// double-buffered by move parity), take the same decision and commit each its
// own caches; both keep the positions. The arithmetic is Walker::move's and
// Walker::local_energy's on the same operands, so the trajectories, energies
// and sums are the per-thread kernel's, bit for bit.
//
// A move is one dependent chain per warp, and on GB300 a dependent FP64
// instruction costs 64 cycles while an integer or FP32 one costs about 4.
// The move code is therefore straight-line: the nucleus count NB (1 or 2,
// one 1s function each) is a template parameter, the system's constants sit
// in registers, and the next move's random draw (Philox and the unit
// proposal, ~100 integer instructions) is made during the current move, in
// the issue slots the FP64 chain leaves idle.
//
// Scope: FP64 box and Gaussian moves, at most one electron per spin, one 1s
// STO per nucleus (at most 2 nuclei), plain Pade e-e term or none, no e-n
// Jastrow, Coulomb potential; the host picks it for small ensembles.
//
// Named barriers: 1 (warps 0 and 1, each move), 2 + b (snapshot b written:
// warps 0 and 1 arrive, warp 2 waits), 4 + b (snapshot b read: warp 2
// arrives, warps 0 and 1 wait before writing it again); b = sample parity.
#pragma once

#include "walker.cuh"

namespace mole {

constexpr int kTeamThreads = 96;

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

// pair_vals<double, PM, false> of the team scope (plain Pade term, no
// polynomial), straight-line.
template <int NB, int PM>
__device__ __forceinline__ void team_pair(const TeamConst<NB>& k, bool same, double d0, double d1, double d2,
                                          PairVals<double, PM>& v) {
  const double r2 = d0 * d0 + d1 * d1 + d2 * d2;
  const double inv = rsqrt_t<double>(r2);
  const double r = r2 * inv;
  v.inv = inv;
  v.db = 0;
  v.rs = r;
  const double cusp = same ? k.cusp_para : k.cusp_anti;
  // u = c r q, u' = c q^2, u'' = -2 b c q^3, du/db = -c r^2 q^2, q = 1 / (1 + b r)
  const double q = recip_t<double>(1.0 + k.ee_b * r);
  const double cq = cusp * q;
  const double uR = cq * q;
  const double val = cq * r;
  // u'' is rounded on its own, as pair_vals rounds it (its polynomial loop
  // stands between the product and the sum below): no contraction into l
  const double uRR = __dmul_rn(k.ee_m2b * q, uR);
  if constexpr (PM > 0) v.db = -(r2 * uR);
  const double f = uR * inv;
  const double l = uRR + 2.0 * f;
  v.u = val;
  v.f = f;
  v.l = l;
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

// The caches warp 2 needs, per walker (slot [field][lane]).
template <int N, int PM>
struct TeamSnap {
  static constexpr int NZ = PM == 0 ? 0 : 1;
  // x (3N), B (N), og (3N), ol (N), odz (N NZ), ven (N); pair: u, f, l, 1/r, du/db, R
  static constexpr int NF0 = 3 * N + N + 3 * N + N + N * NZ + N;
  static constexpr int NF1 = N == 2 ? 6 : 0;
  double f[2][NF0 + NF1 + 1][32];
};

template <int NU, int ND, int PM, int NB, int MOVE>
__device__ __forceinline__ void team_body(const SysParams<double>& sp, const VmcArgs& a) {
  using Wk = Walker<NU, ND, double, PM, false, false>;
  constexpr int N = NU + ND;
  constexpr int NZ = Wk::NZ;
  constexpr int NA = n_acc(PM);
  constexpr int NSR = NA - kNMom;
  using Snap = TeamSnap<N, PM>;
  __shared__ Snap snap;
  __shared__ double xch[2][2][32];  // [move parity][0: ratio, 1: dJ][lane]
  __shared__ double red[kTeamThreads / 32];
  const int lane = threadIdx.x & 31, role = threadIdx.x >> 5;
  const int w = blockIdx.x * 32 + lane;
  const bool active = w < a.W;
  const double step = a.step;
  const int total = a.n_eq + a.n_steps;
  const int refresh = a.refresh > 0 ? a.refresh : 100;

  Wk wk;
  wk.nn = NnCtx<double>{nullptr, nullptr, 0};
  if (active) wk.load(a.pos, a.W, w);
  else
#pragma unroll
    for (int e = 0; e < N; ++e) wk.x[e][0] = wk.x[e][1] = wk.x[e][2] = 1.0 + e;
  bool ok = true;
  int naccept = 0;
  // warp 2's sums
  double sE = acc_zero<double>(), sE2 = acc_zero<double>(), bsum = acc_zero<double>(), sB2 = 0.0;
  double srv[NSR > 0 ? NSR : 1];
#pragma unroll
  for (int k = 0; k < (NSR > 0 ? NSR : 1); ++k) srv[k] = 0.0;
  bool e_finite = true;

  if (role < 2) {
    ok = wk.refresh(sp, nullptr, nullptr);
    const TeamConst<NB> kc(sp);
    int mv = 0;  // move counter (exchange-buffer parity)
    TeamUnit un = team_unit<MOVE>(a.seed, (uint32_t)w, a.step0, 0);
    for (int it = 0; it < total; ++it) {
      const uint32_t t = a.step0 + (uint32_t)it;
      static_for<0, N>([&](auto ec) {
        constexpr int e = decltype(ec)::value;
        constexpr bool isup = e < NU;
        constexpr int j = N == 2 ? 1 - e : 0;
        // the proposal (Walker::move's draws and arithmetic); the next
        // move's draw is made here too, independent of this move's chain
        const TeamUnit u = un;
        if constexpr (e + 1 < N) un = team_unit<MOVE>(a.seed, (uint32_t)w, t, e + 1);
        else un = team_unit<MOVE>(a.seed, (uint32_t)w, t + 1u, 0);
        double xn[3];
        xn[0] = fma(step, u.v[0], wk.x[e][0]);
        xn[1] = fma(step, u.v[1], wk.x[e][1]);
        xn[2] = fma(step, u.v[2], wk.x[e][2]);
        const uint32_t ubits = u.ubits;
        const int par = mv & 1;
        OneBody<double, 1, NZ> o;
        PairVals<double, PM> pv;
        double ratio, dJ;
        if (role == 0) {
          team_one_body<NB, NZ>(kc, isup ? 0 : 1, xn, o);
          ratio = acc_zero<double>();
          ratio += o.val[0] * (isup ? wk.bu[0] : wk.bd[0]);
          xch[par][0][lane] = ratio;
        } else {
          dJ = acc_zero<double>();
          if constexpr (N == 2) {
            team_pair<NB, PM>(kc, Wk::same_spin(e, j), xn[0] - wk.x[j][0], xn[1] - wk.x[j][1], xn[2] - wk.x[j][2],
                              pv);
            dJ += pv.u - wk.pu[0];
          }
          xch[par][1][lane] = dJ;
        }
        named_sync<1>(64);
        if (role == 0) dJ = xch[par][1][lane];
        else ratio = xch[par][0][lane];
        ++mv;
        if (metropolis_accept_dj(ratio, dJ, ubits)) {
          wk.x[e][0] = xn[0];
          wk.x[e][1] = xn[1];
          wk.x[e][2] = xn[2];
          if (role == 0) {
            naccept += 1;
            wk.template put_one_body<e, 1>(o);
            if constexpr (isup) wk.bu[0] = recip(o.val[0]);
            else wk.bd[0] = recip(o.val[0]);
          } else if constexpr (N == 2) {
            wk.put_pair(0, pv);
          }
        }
      });
      if ((it + 1) % refresh == 0) {
        // each warp rebuilds its own caches (the other's are rebuilt too and not used)
        ok = wk.refresh(sp, nullptr, nullptr) && ok;
      }
      if (it < a.n_eq) continue;
      // snapshot of this sweep for warp 2
      const int k = it - a.n_eq, b = k & 1;
      if (k >= 2) named_sync_par<4>(b, kTeamThreads);
      double(*s)[32] = snap.f[b];
      if (role == 0) {
        int q = 0;
#pragma unroll
        for (int e = 0; e < N; ++e) {
          s[q++][lane] = wk.x[e][0];
          s[q++][lane] = wk.x[e][1];
          s[q++][lane] = wk.x[e][2];
          s[q++][lane] = e < NU ? wk.bu[0] : wk.bd[0];
          s[q++][lane] = wk.og[e][0][0];
          s[q++][lane] = wk.og[e][0][1];
          s[q++][lane] = wk.og[e][0][2];
          s[q++][lane] = wk.ol[e][0];
          if constexpr (NZ > 0) s[q++][lane] = wk.odz[e][0][0];
          s[q++][lane] = wk.ven[e];
        }
      } else if constexpr (N == 2) {
        s[Snap::NF0 + 0][lane] = wk.pu[0];
        s[Snap::NF0 + 1][lane] = wk.pf[0];
        s[Snap::NF0 + 2][lane] = wk.pl[0];
        s[Snap::NF0 + 3][lane] = wk.pinv[0];
        s[Snap::NF0 + 4][lane] = wk.pdb[0];
        s[Snap::NF0 + 5][lane] = wk.prs[0];
      }
      named_arrive_par<2>(b, kTeamThreads);
    }
    // the last two snapshots' releases, so that every barrier completes
    for (int k = (a.n_steps >= 2 ? a.n_steps - 2 : 0); k < a.n_steps; ++k) named_sync_par<4>(k & 1, kTeamThreads);
  } else {
    // warp 2: E_L, O_k and the sums of sampled sweep k from snapshot k & 1
    for (int k = 0; k < a.n_steps; ++k) {
      const int b = k & 1;
      named_sync_par<2>(b, kTeamThreads);
      const double(*s)[32] = snap.f[b];
      int q = 0;
#pragma unroll
      for (int e = 0; e < N; ++e) {
        wk.x[e][0] = s[q++][lane];
        wk.x[e][1] = s[q++][lane];
        wk.x[e][2] = s[q++][lane];
        if (e < NU) wk.bu[0] = s[q++][lane];
        else wk.bd[0] = s[q++][lane];
        wk.og[e][0][0] = s[q++][lane];
        wk.og[e][0][1] = s[q++][lane];
        wk.og[e][0][2] = s[q++][lane];
        wk.ol[e][0] = s[q++][lane];
        if constexpr (NZ > 0) wk.odz[e][0][0] = s[q++][lane];
        wk.ven[e] = s[q++][lane];
      }
      if constexpr (N == 2) {
        wk.pu[0] = s[Snap::NF0 + 0][lane];
        wk.pf[0] = s[Snap::NF0 + 1][lane];
        wk.pl[0] = s[Snap::NF0 + 2][lane];
        wk.pinv[0] = s[Snap::NF0 + 3][lane];
        wk.pdb[0] = s[Snap::NF0 + 4][lane];
        wk.prs[0] = s[Snap::NF0 + 5][lane];
      }
      named_arrive_par<4>(b, kTeamThreads);
      double O[PM > 0 ? PM : 1];
      const double E = wk.local_energy(sp, O, nullptr, nullptr);
      e_finite = e_finite && (E == E);
      sE2 += E * E;
      bsum += E;
      if constexpr (PM > 0) {
#pragma unroll
        for (int p = 0; p < PM; ++p) {
          srv[p] += O[p];
          srv[PM + p] += E * O[p];
        }
        int qq = 2 * PM;
#pragma unroll
        for (int p = 0; p < PM; ++p)
#pragma unroll
          for (int r = p; r < PM; ++r, ++qq) srv[qq] += O[p] * O[r];
      }
      if ((k + 1) % a.block_size == 0) {
        const double bs = bsum;
        const double m = bs / a.block_size;
        sB2 += m * m;
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
    if (role == 0) {
      acc[5] = (double)naccept;
      acc[6] = (double)total * N;
      wk.store(a.pos, a.W, w);
      if (!ok) atomicOr(a.status, 2);
    } else if (role == 2) {
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

// FP64 VMC with a three-warp team per 32 walkers (box: move 0, else
// Gaussian), NB nuclei with one 1s function each.
template <int NU, int ND, int PM, int NB>
__global__ void __launch_bounds__(kTeamThreads) vmc_team_kernel(const __grid_constant__ SysParams<double> sp,
                                                               const VmcArgs a) {
  if (a.move == kMoveBox) team_body<NU, ND, PM, NB, kMoveBox>(sp, a);
  else team_body<NU, ND, PM, NB, kMoveGauss>(sp, a);
}

}  // namespace mole
