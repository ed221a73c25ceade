// batch.cuh -- a ragged batch of independent Slater-Jastrow systems (different
// electron counts, walker counts and parameters) advanced by ONE persistent
// launch.
//
// The reference runs one Markov chain per Runner::run call
// (src/montecarlo/src/montecarlo.rs:24-46) and parallelises only over chains
// of one system (src/vmc/src/vmc.rs:63-76). Here every (system, walker group)
// is a work item; a persistent grid of CTAs pulls items from a global counter
// (most expensive first) so systems with 2 and 10 electrons share the GPU.
//
// One thread owns one walker. Unlike the fixed-size kernels of walker.cuh the
// spin-block sizes are runtime values (nu, nd <= 5), so the walker state sits
// in shared memory, walker-fastest: slot k of thread t is st[k * blockDim + t]
// (a warp touches 32 consecutive doubles: no bank conflicts). A walker keeps
// only what is expensive to rebuild in FP64 -- its positions and the two
// inverse Slater matrices; orbital, Jastrow and potential terms are
// re-evaluated in the arithmetic type R (FP32 in the mixed form) when needed.
// The inverse, the Sherman-Morrison ratio and update, the local-energy
// assembly and every accumulation stay FP64 in both forms.
#pragma once

#include "kernels.cuh"

namespace mole {

constexpr int kBatchMaxThreads = 256;

// Per-system bookkeeping of a batch.
struct BatchSystem {
  long long pos_off;  // first double of this system's SoA block [3N][W] in the batch buffer
  int W, nu, nd;
  int item0, n_items;  // this system's work items are ids [item0, item0 + n_items)
  double step;         // proposal width (box side or Gaussian sigma)
  uint64_t seed;       // the system's random-stream key
};

struct BatchArgs {
  const void* sys;          // SysParams<R>[n_systems] (device)
  const BatchSystem* info;  // [n_systems]
  const int2* items;        // [n_items] by item id: (system, first walker)
  const int* order;         // [n_items] item ids in dispatch order
  int n_items, n_systems;
  int slots;                // doubles of walker state per thread (max over the systems)
  int rslots;               // R-typed position shadow per thread (3 N max; 0 when R is double)
  double* pos;              // every system's SoA block
  int move, n_eq, n_steps, block_size, refresh;
  uint64_t* step0;          // device sweep counter (the random-stream position)
  unsigned* queue;          // device work counter, zero at launch
  double* partials;         // [n_items][kNMom] by item id
  double* moments;          // [n_systems][kNMom], then the status word (as a double)
  int* status;              // bit 0: non-finite E_L; bit 1: singular determinant
};

// Shared-memory bytes of one CTA: the system image, `slots` doubles per
// walker, the reduction scratch and, in the FP32 form, an FP32 copy of the
// positions (`rslots` floats per walker) so that distances never pass
// through the FP64 pipe.
template <class R>
__host__ __device__ constexpr size_t batch_sp_bytes() {
  return (sizeof(SysParams<R>) + 15) / 16 * 16;
}
template <class R>
__host__ __device__ inline int batch_rslots(int max_elec) {
  return sizeof(R) == sizeof(double) ? 0 : 3 * max_elec;
}
template <class R>
__host__ __device__ inline size_t batch_smem_bytes(int wpb, int slots, int max_elec) {
  return batch_sp_bytes<R>() + (size_t)slots * wpb * sizeof(double) + (size_t)kNMom * (wpb / 32) * sizeof(double) +
         (size_t)batch_rslots<R>(max_elec) * wpb * sizeof(R);
}
// FP64 slots per walker: the positions (FP64 form only; the FP32 form keeps
// its FP64 positions in the global buffer and touches them only on accepted
// moves) and the two inverse matrices.
template <class R>
__host__ __device__ inline int batch_slots(int nu, int nd) {
  return (sizeof(R) == sizeof(double) ? 3 * (nu + nd) : 0) + nu * nu + nd * nd;
}

// R -> double and float -> R without an FP64-pipe conversion (f2d is exact).
template <class R>
__device__ __forceinline__ double up_d(R v) {
  if constexpr (sizeof(R) == sizeof(double)) return v;
  else return f2d(v);
}
template <class R>
__device__ __forceinline__ R from_f(float v) {
  if constexpr (sizeof(R) == sizeof(double)) return f2d(v);
  else return v;
}

// a / b: IEEE in FP64, the SFU reciprocal (2 ulp) in the FP32 form.
template <class R>
__device__ __forceinline__ R div_t(R a, R b) {
  if constexpr (sizeof(R) == sizeof(double)) return a / b;
  else return __fdividef(a, b);
}

// Orbital values of spin block `spin` at r (the first MS orbitals, MS the
// system's larger spin block; the unused ones have zero coefficients) and the
// e-n Jastrow value.
template <class R, int MS>
__device__ __forceinline__ void batch_orbitals(const SysParams<R>& sp, int spin, const R (&r)[3], R (&phi)[MS],
                                               R& jen) {
#pragma unroll
  for (int k = 0; k < MS; ++k) phi[k] = 0;
  jen = 0;
  for (int I = 0; I < sp.n_nuc; ++I) {
    const R d0 = r[0] - sp.nuc_pos[3 * I], d1 = r[1] - sp.nuc_pos[3 * I + 1], d2 = r[2] - sp.nuc_pos[3 * I + 2];
    const R r2 = d0 * d0 + d1 * d1 + d2 * d2;
    const R rr = r2 * rsqrt_t<R>(r2);
    const int b1 = sp.nuc_b0[I + 1];
    for (int b = sp.nuc_b0[I]; b < b1; ++b) {
      const int kind = sp.b_kind[b];
      const R z = sp.b_zeta[b];
      R chi;
      if (kind == kGto1s) {
        chi = exp_t<R>(-z * r2);
      } else {
        const R e = exp_t<R>(-z * rr);
        if (kind == kSto1s) chi = e;
        else if (kind == kSto2s) chi = rr * e;
        else chi = (kind == kSto2px ? d0 : (kind == kSto2py ? d1 : d2)) * e;
      }
#pragma unroll
      for (int k = 0; k < MS; ++k) phi[k] += sp.coef[spin][k][b] * chi;
    }
    if (sp.en_on) jen += div_t<R>(sp.en_coef[I] * rr, (R)1 + sp.en_a * rr);
  }
}

// e-n Jastrow value alone.
template <class R>
__device__ __forceinline__ R batch_jen(const SysParams<R>& sp, const R (&r)[3]) {
  R j = 0;
  for (int I = 0; I < sp.n_nuc; ++I) {
    const R d0 = r[0] - sp.nuc_pos[3 * I], d1 = r[1] - sp.nuc_pos[3 * I + 1], d2 = r[2] - sp.nuc_pos[3 * I + 2];
    const R r2 = d0 * d0 + d1 * d1 + d2 * d2;
    const R rr = r2 * rsqrt_t<R>(r2);
    j += div_t<R>(sp.en_coef[I] * rr, (R)1 + sp.en_a * rr);
  }
  return j;
}

// Pade pair value u(r) (theory/jastrow.tex:15-29), the value part of pair_vals.
template <class R>
__device__ __forceinline__ R batch_pair_u(const SysParams<R>& sp, bool same, R d0, R d1, R d2) {
  if (!sp.ee_on) return 0;
  const R r2 = d0 * d0 + d1 * d1 + d2 * d2;
  const R r = r2 * rsqrt_t<R>(r2);
  R Rs = r;
  if (sp.ee_kappa > (R)0) Rs = div_t<R>((R)1 - exp_t<R>(-sp.ee_kappa * r), sp.ee_kappa);
  R val = div_t<R>((same ? sp.cusp_para : sp.cusp_anti) * Rs, (R)1 + sp.ee_b * Rs);
  R Rk = Rs * Rs;
  for (int i = 0; i < sp.ee_npoly; ++i) {
    val += sp.ee_poly[i] * Rk;
    Rk *= Rs;
  }
  return val;
}

// Walker view: the thread's slots in the CTA's shared state.
template <class R>
struct BatchWalker {
  double* X;   // X[(3e + c) * xs]: the FP64 positions the moves accumulate into
               // (shared slots in the FP64 form, the global SoA buffer in the FP32 form)
  R* Xr;       // the positions in the arithmetic type (X itself when R is double)
  double* Bu;  // inverse of the up Slater matrix, Bu[(k * nu + j) * nt]
  double* Bd;  // inverse of the down Slater matrix
  int nt, xs, nu, nd;
  __device__ __forceinline__ double& x(int e, int c) const { return X[(size_t)(3 * e + c) * xs]; }
  __device__ __forceinline__ R xr(int e, int c) const { return Xr[(3 * e + c) * nt]; }
  __device__ __forceinline__ void set_x(int e, int c, double v) const {
    X[(size_t)(3 * e + c) * xs] = v;
    if constexpr (sizeof(R) != sizeof(double)) Xr[(3 * e + c) * nt] = (R)v;
  }
  __device__ __forceinline__ double* B(int spin) const { return spin ? Bd : Bu; }
};

// Rebuilds both inverses in FP64 from fresh orbital values by Gauss-Jordan
// elimination with partial pivoting (the matrix in registers, padded to
// kMaxSpin x kMaxSpin; the inverse written straight to the shared slots).
template <class R, int MS>
__device__ bool batch_refresh(const SysParams<R>& sp, const BatchWalker<R>& wk) {
  bool ok = true;
  for (int spin = 0; spin < 2; ++spin) {
    const int n = spin ? wk.nd : wk.nu;
    if (n == 0) continue;
    const int e0 = spin ? wk.nu : 0;
    double* inv = wk.B(spin);
    const int nt = wk.nt;
    double a[MS][MS];
#pragma unroll
    for (int i = 0; i < MS; ++i) {
      if (i < n) {
        const R r[3] = {wk.xr(e0 + i, 0), wk.xr(e0 + i, 1), wk.xr(e0 + i, 2)};
        R phi[MS], jen;
        batch_orbitals<R, MS>(sp, spin, r, phi, jen);
#pragma unroll
        for (int k = 0; k < MS; ++k) a[i][k] = up_d<R>(phi[k]);
      } else {
#pragma unroll
        for (int k = 0; k < MS; ++k) a[i][k] = 0.0;
      }
    }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) inv[(i * n + j) * nt] = i == j ? 1.0 : 0.0;
#pragma unroll
    for (int col = 0; col < MS; ++col) {
      if (col >= n) break;
      int piv = col;
      double best = fabs(a[col][col]);
#pragma unroll
      for (int r = col + 1; r < MS; ++r)
        if (r < n && fabs(a[r][col]) > best) {
          best = fabs(a[r][col]);
          piv = r;
        }
#pragma unroll
      for (int r = col + 1; r < MS; ++r)
        if (r == piv) {
#pragma unroll
          for (int j = 0; j < MS; ++j) {
            const double t = a[col][j];
            a[col][j] = a[r][j];
            a[r][j] = t;
          }
          for (int j = 0; j < n; ++j) {
            const double t = inv[(col * n + j) * nt];
            inv[(col * n + j) * nt] = inv[(r * n + j) * nt];
            inv[(r * n + j) * nt] = t;
          }
        }
      const double p = a[col][col];
      ok = ok && (p != 0.0);
      const double ip = 1.0 / p;
#pragma unroll
      for (int j = 0; j < MS; ++j) a[col][j] *= ip;
      for (int j = 0; j < n; ++j) inv[(col * n + j) * nt] *= ip;
#pragma unroll
      for (int r = 0; r < MS; ++r) {
        if (r == col || r >= n) continue;
        const double f = a[r][col];
#pragma unroll
        for (int j = 0; j < MS; ++j) a[r][j] -= f * a[col][j];
        for (int j = 0; j < n; ++j) inv[(r * n + j) * nt] -= f * inv[(col * n + j) * nt];
      }
    }
  }
  return ok;
}

// One Metropolis move of electron e (box or Gaussian, the random streams of
// Walker::move); returns 1 when accepted.
template <class R, int MOVE, int MS>
__device__ __forceinline__ int batch_move(const SysParams<R>& sp, const BatchWalker<R>& wk, int e, R step,
                                          uint64_t seed, uint32_t wid, uint32_t t) {
  const int N = wk.nu + wk.nd;
  const int spin = e < wk.nu ? 0 : 1;
  const int n = spin ? wk.nd : wk.nu;
  const int i = spin ? e - wk.nu : e;
  const double* B = wk.B(spin);
  const int nt = wk.nt;

  constexpr bool F64 = sizeof(R) == sizeof(double);
  const uint4 ra = draw4(seed, wid, t, 2u * e, kTagMove);
  R dx[3];  // in the FP32 form the move is made on the FP32 copy; FP64 only on acceptance
  R uacc;
  uint32_t ubits;
  float z[3];
  double v64[3];  // FP64 form: the unit proposal (u - 1/2 exactly, or the FP32 normal)
  if constexpr (MOVE == kMoveBox && F64) {
    v64[0] = u01_centered(ra.x);
    v64[1] = u01_centered(ra.y);
    v64[2] = u01_centered(ra.z);
    ubits = ra.w;
  } else if constexpr (MOVE == kMoveBox) {
    dx[0] = step * (u01<R>(ra.x) - (R)0.5);
    dx[1] = step * (u01<R>(ra.y) - (R)0.5);
    dx[2] = step * (u01<R>(ra.z) - (R)0.5);
    uacc = u01<R>(ra.w);
    ubits = ra.w;
  } else {
    float z3;
    repro_box_muller(ra.x, ra.y, z[0], z[1]);
    repro_box_muller(ra.z, ra.w, z[2], z3);
    const uint4 rb = draw4(seed, wid, t, 2u * e + 1u, kTagMove);
    uacc = u01<R>(rb.x);
    ubits = rb.x;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if constexpr (F64) v64[c] = f2d(z[c]);
      else dx[c] = step * from_f<R>(z[c]);
    }
  }
  const R ro[3] = {wk.xr(e, 0), wk.xr(e, 1), wk.xr(e, 2)};
  R rn[3];
  double xn[3];
  if constexpr (F64) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      xn[c] = fma((double)step, v64[c], (double)ro[c]);  // x + step v rounded once
      rn[c] = xn[c];
    }
  } else {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      rn[c] = ro[c] + dx[c];
      xn[c] = wk.x(e, c);  // global load, consumed only if the move is accepted
    }
  }
  R phi[MS], jn;
  batch_orbitals<R, MS>(sp, spin, rn, phi, jn);
  const R jo = sp.en_on ? batch_jen<R>(sp, ro) : (R)0;
  double ratio = 0.0;
#pragma unroll
  for (int k = 0; k < MS; ++k)
    if (k < n) ratio += up_d<R>(phi[k]) * B[(k * n + i) * nt];
  R dJ = jn - jo;
  for (int j = 0; j < N; ++j) {
    if (j == e) continue;
    const bool same = (j < wk.nu) == (spin == 0);
    const R xj[3] = {wk.xr(j, 0), wk.xr(j, 1), wk.xr(j, 2)};
    dJ += batch_pair_u<R>(sp, same, rn[0] - xj[0], rn[1] - xj[1], rn[2] - xj[2]) -
          batch_pair_u<R>(sp, same, ro[0] - xj[0], ro[1] - xj[1], ro[2] - xj[2]);
  }
  if constexpr (F64) {
    if (!metropolis_accept(ratio, 2.0 * dJ, ubits)) return 0;
  } else {
    const float rf = d2f_rz(ratio);  // the acceptance test itself is a random comparison: FP32
    if (!(rf * rf * __expf(2.0f * dJ) > uacc)) return 0;
  }

  // commit: position and the FP64 Sherman-Morrison row update
  if constexpr (F64) {
#pragma unroll
    for (int c = 0; c < 3; ++c) wk.set_x(e, c, xn[c]);
  } else {
#pragma unroll
    for (int c = 0; c < 3; ++c) wk.set_x(e, c, xn[c] + up_d<R>(dx[c]));
  }
  double v[MS], col[MS];
  double* Bw = wk.B(spin);
#pragma unroll
  for (int j = 0; j < MS; ++j) {
    if (j >= n) break;
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < MS; ++k)
      if (k < n) s += up_d<R>(phi[k]) * Bw[(k * n + j) * nt];
    v[j] = s - (j == i ? 1.0 : 0.0);
  }
  const double ir = 1.0 / ratio;
#pragma unroll
  for (int k = 0; k < MS; ++k)
    if (k < n) col[k] = Bw[(k * n + i) * nt] * ir;
#pragma unroll
  for (int k = 0; k < MS; ++k) {
    if (k >= n) break;
#pragma unroll
    for (int j = 0; j < MS; ++j)
      if (j < n) Bw[(k * n + j) * nt] -= col[k] * v[j];
  }
  return 1;
}

// Local energy -1/2 sum_i lap_i psi / psi + V in log-derivative form: orbital
// gradients and Laplacians in R contracted with the FP64 inverse, Jastrow and
// potential terms re-evaluated per electron (each pair from both sides).
template <class R, int MS>
__device__ double batch_local_energy(const SysParams<R>& sp, const BatchWalker<R>& wk) {
  const int N = wk.nu + wk.nd;
  const int nt = wk.nt;
  double lap = 0.0, V = sp.vnn;
  for (int e = 0; e < N; ++e) {
    const int spin = e < wk.nu ? 0 : 1;
    const int n = spin ? wk.nd : wk.nu;
    const int i = spin ? e - wk.nu : e;
    const double* B = wk.B(spin);
    const R r[3] = {wk.xr(e, 0), wk.xr(e, 1), wk.xr(e, 2)};
    OneBody<R, MS, 0> o;
    one_body<R, MS, 0, true, false>(sp, spin, r, o);
    double gD[3] = {0.0, 0.0, 0.0}, lD = 0.0;
#pragma unroll
    for (int k = 0; k < MS; ++k)
      if (k < n) {
        const double b = B[(k * n + i) * nt];
        gD[0] += up_d<R>(o.grad[k][0]) * b;
        gD[1] += up_d<R>(o.grad[k][1]) * b;
        gD[2] += up_d<R>(o.grad[k][2]) * b;
        lD += up_d<R>(o.lap[k]) * b;
      }
    R gJ[3] = {o.gjen[0], o.gjen[1], o.gjen[2]};
    R lJ = o.ljen, Ve = o.ven;
    for (int j = 0; j < N; ++j) {
      if (j == e) continue;
      const R d0 = r[0] - wk.xr(j, 0), d1 = r[1] - wk.xr(j, 1), d2 = r[2] - wk.xr(j, 2);
      PairVals<R, 0> pv;
      pair_vals<R, 0, false>(sp, (j < wk.nu) == (spin == 0), d0, d1, d2, pv);
      gJ[0] += pv.f * d0;
      gJ[1] += pv.f * d1;
      gJ[2] += pv.f * d2;
      lJ += pv.l;
      if (j > e) Ve += pv.inv;
    }
    // the electron's Jastrow-only terms in R, the determinant terms in FP64
    const R jj = lJ + gJ[0] * gJ[0] + gJ[1] * gJ[1] + gJ[2] * gJ[2];
    const double dot = gD[0] * up_d<R>(gJ[0]) + gD[1] * up_d<R>(gJ[1]) + gD[2] * up_d<R>(gJ[2]);
    lap += lD + up_d<R>(jj) + 2.0 * dot;
    V += up_d<R>(Ve);
  }
  return -0.5 * lap + V;
}

// One work item: walkers [w0, w0 + blockDim.x) of one system, all sweeps of
// the call; writes the item's kNMom partial sums (deterministic CTA order).
// MS = max(nu, nd) bounds the unrolled orbital and inverse loops: a guarded
// iteration past a spin block's size would still issue its FP64
// instructions, each holding the FP64 pipe as long as a useful one.
template <class R, int MOVE, int MS>
__device__ void batch_item(const SysParams<R>& sp, const BatchSystem& bs, int id, int w0, double* st, double* red,
                           const BatchArgs& a, uint32_t t0) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int w = w0 + tid;
  const bool active = w < bs.W;
  const int N = bs.nu + bs.nd;
  constexpr bool F64 = sizeof(R) == sizeof(double);
  double* gp = a.pos + bs.pos_off;
  BatchWalker<R> wk;
  wk.nt = nt;
  wk.nu = bs.nu;
  wk.nd = bs.nd;
  if constexpr (F64) {
    wk.X = st + tid;
    wk.xs = nt;
    wk.Bu = wk.X + (size_t)3 * N * nt;
    wk.Xr = reinterpret_cast<R*>(wk.X);
  } else {
    wk.X = gp + (active ? w : 0);
    wk.xs = bs.W;
    wk.Bu = st + tid;
    wk.Xr = reinterpret_cast<R*>(st + (size_t)a.slots * nt + (size_t)kNMom * (nt / 32)) + tid;
  }
  wk.Bd = wk.Bu + (size_t)bs.nu * bs.nu * nt;
  double acc[kNMom] = {0, 0, 0, 0, 0, 0, 0};
  if (active) {
    for (int k = 0; k < 3 * N; ++k) {
      const double v = gp[(size_t)k * bs.W + w];
      if constexpr (F64) wk.X[k * nt] = v;
      else wk.Xr[k * nt] = (R)v;
    }
    bool ok = batch_refresh<R, MS>(sp, wk);
    const int total = a.n_eq + a.n_steps;
    const int refresh = a.refresh > 0 ? a.refresh : 100;
    const R step = (R)bs.step;
    double sE = 0.0, sE2 = 0.0, sB2 = 0.0, bsum = 0.0;
    int naccept = 0;
    for (int it = 0; it < total; ++it) {
      const uint32_t t = t0 + (uint32_t)it;
      for (int e = 0; e < N; ++e) naccept += batch_move<R, MOVE, MS>(sp, wk, e, step, bs.seed, (uint32_t)w, t);
      if ((it + 1) % refresh == 0) ok = batch_refresh<R, MS>(sp, wk) && ok;
      if (it < a.n_eq) continue;
      const double E = batch_local_energy<R, MS>(sp, wk);
      sE += E;
      sE2 += E * E;
      bsum += E;
      if ((it - a.n_eq + 1) % a.block_size == 0) {
        const double m = bsum / a.block_size;
        sB2 += m * m;
        bsum = 0.0;
      }
    }
    if constexpr (F64)
      for (int k = 0; k < 3 * N; ++k) gp[(size_t)k * bs.W + w] = wk.X[k * nt];
    if (!ok) atomicOr(a.status, 2);
    if (!(sE == sE) || !(sE2 < 1e300)) atomicOr(a.status, 1);
    acc[0] = (double)a.n_steps;
    acc[1] = sE;
    acc[2] = sE2;
    acc[3] = sB2;
    acc[4] = (double)(a.n_steps / a.block_size);
    acc[5] = (double)naccept;
    acc[6] = (double)total * N;
  }
  block_sum<kNMom>(acc, red);
  if (tid == 0)
#pragma unroll
    for (int k = 0; k < kNMom; ++k) a.partials[(size_t)id * kNMom + k] = acc[k];
}

}  // namespace mole
