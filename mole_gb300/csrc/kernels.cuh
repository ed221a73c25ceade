// kernels.cuh -- VMC, evaluation and DMC kernels over a walker ensemble.
#pragma once

#include "compact.cuh"
#include "walker.cuh"

namespace mole {

// c + a b for the moment sums, fused explicitly in FP64 and FP32 so that every
// kernel rounds them alike (the double-float form's arithmetic is explicit).
template <class F>
__device__ __forceinline__ F fma_acc(F a, F b, F c) {
  return c + a * b;
}
template <>
__device__ __forceinline__ double fma_acc<double>(double a, double b, double c) {
  return fma(a, b, c);
}
template <>
__device__ __forceinline__ float fma_acc<float>(float a, float b, float c) {
  return fmaf(a, b, c);
}

// Threads per CTA for every walker kernel, and the resident CTAs per SM the
// register budget is tuned for: seven 64-walker CTAs per SM hold 65,536
// walkers in one balanced wave on 152 SMs.
constexpr int kBlock = 64;
template <int NU, int ND>
constexpr int min_blocks() {
  return (NU + ND) <= 2 ? 7 : ((NU + ND) <= 4 ? 4 : 2);
}
__host__ __device__ inline int min_blocks_rt(int nu, int nd) {
  return (nu + nd) <= 2 ? 7 : ((nu + nd) <= 4 ? 4 : 2);
}

// VMC grid: with walkers for at least half a wave the grid is a whole number
// of waves of (SMs x resident CTAs) and the walkers are split evenly over the
// CTAs (every SM gets the same number of walkers); smaller ensembles use
// full 64-walker CTAs. Returns the grid and sets *wpc, walkers per CTA.
inline int vmc_grid(int W, int nu, int nd, int n_sm, int* wpc) {
  const int g = (W + kBlock - 1) / kBlock;
  const int cap = n_sm * min_blocks_rt(nu, nd);
  if (n_sm <= 0 || 2 * g < cap) {
    *wpc = kBlock;
    return g;
  }
  const int grid = cap * ((g + cap - 1) / cap);
  *wpc = (W + grid - 1) / grid;
  return grid;
}

// Accumulators per walker: moments first, then SR sums.
constexpr int kNMom = 7;  // count, sumE, sumE2, sumBlock2, nBlocks, accept, proposed
__host__ __device__ constexpr int n_acc(int PM) { return kNMom + (PM > 0 ? 2 * PM + PM * (PM + 1) / 2 : 0); }

struct VmcArgs {
  double* pos;  // SoA [3N][W]
  int W;
  int move;
  double step;
  int n_eq, n_steps, block_size, refresh;
  uint64_t seed;
  uint32_t step0;
  int wpc;              // walkers per CTA (<= blockDim.x): CTA b runs walkers [b wpc, (b + 1) wpc)
  double* partials;     // [gridDim.x][n_acc]
  double* tb_partials;  // [gridDim.x][n_steps / block_size]
  int* status;          // bit 0: non-finite E_L; bit 1: singular determinant; bit 3: df64 range left
};

// The energy sums live in registers; the SR sums, touched once per sweep,
// live in per-thread shared-memory slots srs[k * blockDim.x + tid] to keep
// the walker caches in registers.
extern __shared__ __align__(16) unsigned char mole_dyn_smem[];

// Neural systems: loads both networks into the CTA's dynamic shared memory
// (all threads must call this) and returns this thread's context.
template <class R, bool NN>
__device__ __forceinline__ NnCtx<R> nn_setup(const SysParams<R>& sp) {
  NnCtx<R> c{nullptr, nullptr, 0};
  if constexpr (NN && !std::is_same<R, float>::value) {  // the FP32 form reads the quintic tables instead
    auto* sh = reinterpret_cast<NnShared<R>*>(mole_dyn_smem);
    nn_load<R>(sh, sp.nn_theta);
    R* scr = reinterpret_cast<R*>(mole_dyn_smem + sizeof(NnShared<R>));
    c = NnCtx<R>{sh, scr + threadIdx.x, (int)blockDim.x};
  }
  return c;
}

// BLK: threads per CTA; COMPACT: the FP64 moves with packed FP64 work
// (compact.cuh; R = double, cs its shared-memory slots).
template <int NU, int ND, class R, int PM, bool EN, bool NN, int MOVE, int BLK = kBlock, bool COMPACT = false,
          class CS = int>
__device__ __forceinline__ void vmc_body(const SysParams<R>& sp, const VmcArgs& a, double* red, double* srs,
                                         CS* cs = nullptr) {
  using Wk = Walker<NU, ND, R, PM, EN, NN>;
  using F = typename Wk::F;  // accumulation type: double, or df64 in the double-float form
  constexpr int NA = n_acc(PM);
  constexpr int NSR = NA - kNMom;
  const int w = blockIdx.x * a.wpc + threadIdx.x;
  const int tid = threadIdx.x;
  const bool active = tid < a.wpc && w < a.W;
  F* srf = reinterpret_cast<F*>(srs);  // df64 is 8 bytes like the double slots
  Wk wk;
  wk.nn = nn_setup<R, NN>(sp);
  if (active) wk.load(a.pos, a.W, w);
  else
#pragma unroll
    for (int e = 0; e < Wk::N; ++e) wk.x[e][0] = wk.x[e][1] = wk.x[e][2] = 1.0 + e;
  bool ok = wk.refresh(sp, nullptr, nullptr);
  F sE = F(0), sE2 = F(0), bsum = F(0);
  double sB2 = 0.0;
  int naccept = 0;
#pragma unroll
  for (int k = 0; k < NSR; ++k) srf[k * BLK + tid] = F(0);
  const int total = a.n_eq + a.n_steps;
  const int refresh = a.refresh > 0 ? a.refresh : 100;
  const R step = (R)a.step;
  const float stepf = (float)a.step;
  for (int it = 0; it < total; ++it) {
    const uint32_t t = a.step0 + (uint32_t)it;
    if constexpr (COMPACT)
      naccept += compact_sweep<NU, ND, PM, MOVE>(wk, sp, step, stepf, a.seed, (uint32_t)w, t, active, *cs);
    else
      naccept += wk.template sweep<MOVE>(sp, step, a.seed, (uint32_t)w, t);
    if ((it + 1) % refresh == 0) ok = wk.refresh(sp, nullptr, nullptr) && ok;
    if (it < a.n_eq) continue;
    F O[PM > 0 ? PM : 1];
    const F E = wk.local_energy(sp, O, nullptr, nullptr);
    const int k = it - a.n_eq;
    // the products are fused explicitly: left to the code generator, the
    // choice can differ between kernels, and the team kernel's sums must
    // equal these bit for bit
    sE2 = fma_acc(E, E, sE2);
    bsum += E;  // added to sE at every block end and after the last sweep
    if constexpr (PM > 0) {
#pragma unroll
      for (int p = 0; p < PM; ++p) {
        srf[p * BLK + tid] += O[p];
        srf[(PM + p) * BLK + tid] = fma_acc(E, O[p], srf[(PM + p) * BLK + tid]);
      }
      int q = 2 * PM;
#pragma unroll
      for (int p = 0; p < PM; ++p)
#pragma unroll
        for (int r = p; r < PM; ++r, ++q) srf[q * BLK + tid] = fma_acc(O[p], O[r], srf[q * BLK + tid]);
    }
    if ((k + 1) % a.block_size == 0) {
      const double bs = to_d(bsum);
      const double m = bs / a.block_size;
      sB2 = fma(m, m, sB2);
      double v[1] = {active ? bs : 0.0};
      block_sum<1>(v, red);
      if (threadIdx.x == 0) a.tb_partials[(size_t)blockIdx.x * (a.n_steps / a.block_size) + k / a.block_size] = v[0];
      sE += bsum;
      bsum = F(0);
    }
  }
  sE += bsum;
  const double dE = to_d(sE), dE2 = to_d(sE2);
  double acc[kNMom] = {(double)a.n_steps, dE, dE2, sB2, (double)(a.n_steps / a.block_size), (double)naccept,
                       (double)total * Wk::N};
  if (active) {
    wk.store(a.pos, a.W, w);
    // the df64 form reports every anomaly as out of range: the host reruns
    // the launch in native FP64, which reports its own status
    if (!ok) atomicOr(a.status, Wk::DF ? 8 : 2);
    if (!(dE == dE) || !(dE2 < 1e300)) atomicOr(a.status, Wk::DF ? 8 : 1);
    if (Wk::DF && wk.oor) atomicOr(a.status, 8);
  } else {
#pragma unroll
    for (int k = 0; k < kNMom; ++k) acc[k] = 0.0;
  }
  // deterministic CTA reduction, then one partial row per CTA
#pragma unroll
  for (int k = 0; k < NA; ++k) {
    double v[1] = {k < kNMom ? acc[k] : (active ? to_d(srf[(k - kNMom) * BLK + tid]) : 0.0)};
    block_sum<1>(v, red);
    if (threadIdx.x == 0) a.partials[(size_t)blockIdx.x * NA + k] = v[0];
  }
}


// DRIFT selects the drift-diffusion kernel; otherwise box and Gaussian moves
// share one kernel (uniform branch on a.move).
template <int NU, int ND, class R, int PM, bool DRIFT, bool EN, bool NN = false>
__global__ void __launch_bounds__(kBlock, (min_blocks<NU, ND>())) vmc_kernel(const __grid_constant__ SysParams<R> sp,
                                                                            const VmcArgs a) {
  __shared__ double red[kBlock / 32];
  __shared__ double srs[(n_acc(PM) - kNMom > 0 ? n_acc(PM) - kNMom : 1) * kBlock];
  if constexpr (DRIFT) {
    vmc_body<NU, ND, R, PM, EN, NN, kMoveDiffuse>(sp, a, red, srs);
  } else {
    if (a.move == kMoveBox) vmc_body<NU, ND, R, PM, EN, NN, kMoveBox>(sp, a, red, srs);
    else vmc_body<NU, ND, R, PM, EN, NN, kMoveGauss>(sp, a, red, srs);
  }
}

// FP64 VMC with the packed FP64 moves (compact.cuh): systems with one
// electron per spin block, box (move 0) and Gaussian moves.
template <int NU, int ND, int PM>
// (128 registers: two 7-warp CTAs per SM -- four of their 14 warps share an
// SM sub-partition and its 16,384 registers; launched with kCompactBlock threads)
__global__ void __maxnreg__(128)
    vmc_compact_kernel(const __grid_constant__ SysParams<double> sp, const VmcArgs a) {
  __shared__ double red[kCompactBlock / 32];
  __shared__ double srs[(n_acc(PM) - kNMom > 0 ? n_acc(PM) - kNMom : 1) * kCompactBlock];
  __shared__ CompactSlots<NU + ND, PM> cs;
  if (a.move == kMoveBox)
    vmc_body<NU, ND, double, PM, false, false, kMoveBox, kCompactBlock, true>(sp, a, red, srs, &cs);
  else
    vmc_body<NU, ND, double, PM, false, false, kMoveGauss, kCompactBlock, true>(sp, a, red, srs, &cs);
}

}  // namespace mole
#include "team.cuh"
namespace mole {

// Grid of the packed kernel: whole waves of (SMs x 2) CTAs with the walkers
// split evenly. Sets *wpc (walkers per CTA).
inline int compact_grid(int W, int n_sm, int* wpc) {
  const int cap = n_sm * kCompactMinBlocks;
  const int g = (W + kCompactBlock - 1) / kCompactBlock;
  const int grid = cap * ((g + cap - 1) / cap);
  *wpc = (W + grid - 1) / grid;
  return grid;
}

struct EvalArgs {
  const double* pos;  // SoA [3N][W]
  int W;
  double* lnpsi;      // [W]
  double* sign;       // [W]
  double* grad;       // [W][N][3]
  double* lap;        // [W]
  double* eloc;       // [W]
  double* O;          // [W][ldO] (first min(P, PM, ldO) entries)
  int ldO;
  int* status;
};

template <int NU, int ND, class R, int PM, bool EN, bool NN = false>
__global__ void __launch_bounds__(kBlock) eval_kernel(const __grid_constant__ SysParams<R> sp, const EvalArgs a) {
  using Wk = Walker<NU, ND, R, PM, EN, NN>;
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  Wk wk;
  wk.nn = nn_setup<R, NN>(sp);
  if (w >= a.W) return;
  wk.load(a.pos, a.W, w);
  double ln, sg;
  const bool ok = wk.refresh(sp, &ln, &sg);
  typename Wk::F O[PM > 0 ? PM : 1];
  double g[Wk::N * 3];
  double lap;
  const double E = to_d(wk.local_energy(sp, O, g, &lap));
  // the df64 form reports every anomaly as out of range (the host reruns in FP64)
  if (!ok) atomicOr(a.status, Wk::DF ? 8 : 2);
  if (!(E == E)) atomicOr(a.status, Wk::DF ? 8 : 1);
  if (Wk::DF && wk.oor) atomicOr(a.status, 8);
  a.lnpsi[w] = ln;
  a.sign[w] = sg;
  a.lap[w] = lap;
  a.eloc[w] = E;
#pragma unroll
  for (int k = 0; k < Wk::N * 3; ++k) a.grad[(size_t)w * Wk::N * 3 + k] = g[k];
  if constexpr (PM > 0)
    if (a.O)
      for (int p = 0; p < sp.P && p < PM && p < a.ldO; ++p) a.O[(size_t)w * a.ldO + p] = to_d(O[p]);
}

struct DmcArgs {
  double* pos;         // SoA [3N][W], updated in place
  double* eloc;        // [W] E_L at pos (in: old, out: new)
  double* weight;      // [W] out
  int W;
  double tau;
  const double* e_ref; // device scalar
  double eloc_cut;     // > 0: E_L clipped to e_ref +- eloc_cut in the weight factor
  uint64_t seed;
  const uint64_t* step;  // device step counter
  double* partials;    // [gridDim.x][kDmcPart]: sum E_old, accepted, proposed, walkers on a node
  int* status;
};
constexpr int kDmcPart = 4;

template <int NU, int ND, class R, bool EN, bool NN = false>
__global__ void __launch_bounds__(kBlock, (min_blocks<NU, ND>())) dmc_step_kernel(const __grid_constant__ SysParams<R> sp, const DmcArgs a) {
  using Wk = Walker<NU, ND, R, 0, EN, NN>;
  __shared__ double red[kDmcPart * kBlock / 32];
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = w < a.W;
  const uint32_t t = (uint32_t)(*a.step);
  double v[kDmcPart] = {0.0, 0.0, 0.0, 0.0};
  const NnCtx<R> nnc = nn_setup<R, NN>(sp);
  if (active) {
    Wk wk;
    wk.nn = nnc;
    wk.load(a.pos, a.W, w);
    const double e_old = a.eloc[w];
    v[2] = (double)Wk::N;
    const bool regular = wk.refresh(sp, nullptr, nullptr);
    // the df64 form cannot tell a node from FP32 range loss: the host reruns
    // the steps in native FP64, which decides
    if (Wk::DF && (!regular || wk.oor)) atomicOr(a.status, 8);
    if (!regular) {
      // an exactly singular Slater matrix: psi = 0 at the precision of the
      // orbital values (the walker sits on a node, or an electron is so far
      // out that every orbital underflows), so the walker carries no weight,
      // is left out of this step's energy and is removed by the comb
      a.weight[w] = 0.0;
      v[3] = 1.0;
    } else {
      v[0] = e_old;
      if (!(e_old == e_old)) atomicOr(a.status, 1);
      const int nacc = wk.template sweep<kMoveDiffuse>(sp, (R)a.tau, a.seed, (uint32_t)w, t);
      typename Wk::F O[1];
      const double e_new = to_d(wk.local_energy(sp, O, nullptr, nullptr));
      if (Wk::DF && (wk.oor || !(e_new == e_new))) atomicOr(a.status, 8);
      wk.store(a.pos, a.W, w);
      a.eloc[w] = e_new;
      const double er = *a.e_ref;
      double eo = e_old, en = e_new;
      if (a.eloc_cut > 0.0) {
        eo = fmin(fmax(eo, er - a.eloc_cut), er + a.eloc_cut);
        en = fmin(fmax(en, er - a.eloc_cut), er + a.eloc_cut);
      }
      a.weight[w] = exp(-a.tau * (0.5 * (eo + en) - er));
      if (!(e_new == e_new)) atomicOr(a.status, 1);
      v[1] = (double)nacc;
    }
  }
  block_sum<kDmcPart>(v, red);
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < kDmcPart; ++k) a.partials[(size_t)blockIdx.x * kDmcPart + k] = v[k];
}

}  // namespace mole
