// dispatch.cuh -- per-(NU, ND, precision) kernel launchers, instantiated in inst_*.cu.
#pragma once

#include "kernels.cuh"

namespace mole {

// SR accumulator widths compiled per family: slot 0 -> none, 1 -> 2, 2 -> 8.
constexpr int kPmSlots = 3;
constexpr int kPmWidth[kPmSlots] = {0, 2, 8};

template <class R>
struct KernelSetT {
  using Vmc = cudaError_t (*)(const SysParams<R>&, const VmcArgs&, int, cudaStream_t);
  using Eval = cudaError_t (*)(const SysParams<R>&, const EvalArgs&, int, cudaStream_t);
  using Dmc = cudaError_t (*)(const SysParams<R>&, const DmcArgs&, int, cudaStream_t);
  Vmc vmc[kPmSlots][2][2];  // [PM slot][drift][e-n Jastrow]; NULL where not compiled
  Eval eval[2];             // [e-n Jastrow]
  Dmc dmc[2];               // [e-n Jastrow]; NULL where not compiled
};

// Dynamic shared memory that keeps at most `ctas` CTAs of `kernel` resident
// per SM. The VMC grid is whole waves of (SMs x ctas); a kernel whose
// registers would admit one CTA more per SM can otherwise be placed unevenly
// (some SMs holding ctas + 1 CTAs, others fewer), stretching the launch by
// up to (ctas + 1) / ctas. Computed once per kernel on the current device.
template <class K>
size_t residency_pad(K kernel, int ctas, cudaError_t* err) {
  int dev = 0, per_sm = 0, reserved = 0;
  cudaFuncAttributes fa;
  if ((*err = cudaGetDevice(&dev)) != cudaSuccess) return 0;
  if ((*err = cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess) return 0;
  if ((*err = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess) return 0;
  if ((*err = cudaFuncGetAttributes(&fa, kernel)) != cudaSuccess) return 0;
  const long need = per_sm / (ctas + 1) + 1 - reserved - (long)fa.sharedSizeBytes;  // ctas + 1 do not fit
  if (need <= 0) return 0;
  if ((long)ctas * (need + reserved + (long)fa.sharedSizeBytes) > per_sm) return 0;  // keep ctas resident
  if (need > 48 * 1024 &&
      (*err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need)) != cudaSuccess)
    return 0;
  return (size_t)need;
}

template <int NU, int ND, class R, int PM, bool DRIFT, bool EN>
cudaError_t launch_vmc(const SysParams<R>& sp, const VmcArgs& a, int grid, cudaStream_t s) {
  auto k = vmc_kernel<NU, ND, R, PM, DRIFT, EN>;
  static cudaError_t pad_err = cudaSuccess;
  static const size_t pad = residency_pad(k, min_blocks<NU, ND>(), &pad_err);
  if (pad_err != cudaSuccess) return pad_err;
  k<<<grid, kBlock, pad, s>>>(sp, a);
  return cudaGetLastError();
}
template <int NU, int ND, class R, bool EN>
cudaError_t launch_eval(const SysParams<R>& sp, const EvalArgs& a, int grid, cudaStream_t s) {
  eval_kernel<NU, ND, R, 8, EN><<<grid, kBlock, 0, s>>>(sp, a);
  return cudaGetLastError();
}
template <int NU, int ND, class R, bool EN>
cudaError_t launch_dmc(const SysParams<R>& sp, const DmcArgs& a, int grid, cudaStream_t s) {
  dmc_step_kernel<NU, ND, R, EN><<<grid, kBlock, 0, s>>>(sp, a);
  return cudaGetLastError();
}

template <int NU, int ND, class R, int PM, bool DRIFT, bool EN, bool ON>
typename KernelSetT<R>::Vmc maybe_vmc() {
  if constexpr (ON) return launch_vmc<NU, ND, R, PM, DRIFT, EN>;
  else return nullptr;
}
template <int NU, int ND, class R, bool EN, bool ON>
typename KernelSetT<R>::Dmc maybe_dmc() {
  if constexpr (ON) return launch_dmc<NU, ND, R, EN>;
  else return nullptr;
}

// The VMC launchers of one SR width: [drift][e-n Jastrow]; ON = false leaves
// them NULL, DRIFT = false the drift-diffusion ones.
#define MOLE_VMC_EN(NU, ND, R, PM, ON, DRIFT)                                                             \
  {{maybe_vmc<NU, ND, R, PM, false, false, ON>(), maybe_vmc<NU, ND, R, PM, false, true, ON>()},          \
   {maybe_vmc<NU, ND, R, PM, true, false, (ON && DRIFT)>(), maybe_vmc<NU, ND, R, PM, true, true, (ON && DRIFT)>()}}
// Slices of a family's kernel set, one translation unit each so that the
// build compiles them in parallel; capi.cu merges them (kernel_set64/32).
// Slot SLOT holds the VMC launchers with PM SR accumulators (drift and
// non-drift, without and with the e-n term); the rest slice holds the
// evaluation and DMC launchers.
#define MOLE_PART_VMC(NU, ND, R, TAG, SLOT, PM)                                                     \
  KernelSetT<R> kparts_##TAG##_##NU##_##ND##_##SLOT() {                                            \
    KernelSetT<R> k{};                                                                             \
    const typename KernelSetT<R>::Vmc v[2][2] = MOLE_VMC_EN(NU, ND, R, PM, true, true);              \
    for (int d = 0; d < 2; ++d)                                                                    \
      for (int e = 0; e < 2; ++e) k.vmc[SLOT][d][e] = v[d][e];                                     \
    return k;                                                                                      \
  }
#define MOLE_PART_REST(NU, ND, R, TAG)                                                              \
  KernelSetT<R> kparts_##TAG##_##NU##_##ND##_r() {                                                 \
    KernelSetT<R> k{};                                                                             \
    k.eval[0] = launch_eval<NU, ND, R, false>;                                                     \
    k.eval[1] = launch_eval<NU, ND, R, true>;                                                      \
    k.dmc[0] = launch_dmc<NU, ND, R, false>;                                                       \
    k.dmc[1] = launch_dmc<NU, ND, R, true>;                                                        \
    return k;                                                                                      \
  }

// Double-float (FP64-accurate) kernels: box and Gaussian VMC and evaluation;
// drift-diffusion moves and DMC stay native FP64. Each family's launchers are
// compiled in three translation units (VMC without and with the e-n term,
// evaluation) so that the build runs them in parallel.
struct DfParts {
  KernelSetT<df64>::Vmc vmc[kPmSlots];  // [PM slot]; slot 2 (eight-wide SR) not compiled
  KernelSetT<df64>::Eval eval;
  KernelSetT<df64>::Dmc dmc;
};
#define MOLE_INSTANTIATE_DF_VMC(NU, ND, EN)                                                   \
  DfParts df_parts_vmc_##NU##_##ND##_##EN() {                                                \
    return DfParts{{launch_vmc<NU, ND, df64, 0, false, EN>, launch_vmc<NU, ND, df64, 2, false, EN>, nullptr}, \
                   nullptr, nullptr};                                                        \
  }
#define MOLE_INSTANTIATE_DF_EVAL(NU, ND)                                                      \
  DfParts df_parts_eval_##NU##_##ND##_0() { return DfParts{{}, launch_eval<NU, ND, df64, false>, nullptr}; } \
  DfParts df_parts_eval_##NU##_##ND##_1() { return DfParts{{}, launch_eval<NU, ND, df64, true>, nullptr}; }
#define MOLE_INSTANTIATE_DF_DMC(NU, ND)                                                       \
  DfParts df_parts_dmc_##NU##_##ND##_0() { return DfParts{{}, nullptr, launch_dmc<NU, ND, df64, false>}; } \
  DfParts df_parts_dmc_##NU##_##ND##_1() { return DfParts{{}, nullptr, launch_dmc<NU, ND, df64, true>}; }

const KernelSetT<double>* kernel_set64(int nu, int nd);
const KernelSetT<float>* kernel_set32(int nu, int nd);
const KernelSetT<df64>* kernel_set_df(int nu, int nd);

// Neural-Jastrow kernels (e-n terms on; the weights in dynamic shared memory).
template <class R>
struct NnKernelSetT {
  typename KernelSetT<R>::Vmc vmc[2];  // [drift]
  typename KernelSetT<R>::Eval eval;
  typename KernelSetT<R>::Dmc dmc;
};

template <class K>
cudaError_t nn_prepare(K kernel, size_t smem) {
  // opt in to more than 48 KB of dynamic shared memory (idempotent)
  return smem ? cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) : cudaSuccess;
}
// The FP64 form keeps both nets and the per-thread hidden-layer jets in
// shared memory; the FP32 form interpolates its tables and needs none.
template <class R>
constexpr size_t nn_launch_smem() {
  return std::is_same<R, float>::value ? 0 : nn_smem_bytes<R>(kBlock);
}
template <int NU, int ND, class R, bool DRIFT>
cudaError_t launch_vmc_nn(const SysParams<R>& sp, const VmcArgs& a, int grid, cudaStream_t s) {
  auto k = vmc_kernel<NU, ND, R, 0, DRIFT, true, true>;
  const size_t smem = nn_launch_smem<R>();
  cudaError_t e = nn_prepare(k, smem);
  if (e != cudaSuccess) return e;
  k<<<grid, kBlock, smem, s>>>(sp, a);
  return cudaGetLastError();
}
template <int NU, int ND, class R>
cudaError_t launch_eval_nn(const SysParams<R>& sp, const EvalArgs& a, int grid, cudaStream_t s) {
  auto k = eval_kernel<NU, ND, R, 8, true, true>;
  const size_t smem = nn_launch_smem<R>();
  cudaError_t e = nn_prepare(k, smem);
  if (e != cudaSuccess) return e;
  k<<<grid, kBlock, smem, s>>>(sp, a);
  return cudaGetLastError();
}
template <int NU, int ND, class R>
cudaError_t launch_dmc_nn(const SysParams<R>& sp, const DmcArgs& a, int grid, cudaStream_t s) {
  auto k = dmc_step_kernel<NU, ND, R, true, true>;
  const size_t smem = nn_launch_smem<R>();
  cudaError_t e = nn_prepare(k, smem);
  if (e != cudaSuccess) return e;
  k<<<grid, kBlock, smem, s>>>(sp, a);
  return cudaGetLastError();
}

#define MOLE_INSTANTIATE_NN(NU, ND, R, TAG)                                                               \
  const NnKernelSetT<R>* nn_kernels_##TAG##_##NU##_##ND() {                                              \
    static const NnKernelSetT<R> ks = {{launch_vmc_nn<NU, ND, R, false>, launch_vmc_nn<NU, ND, R, true>}, \
                                       launch_eval_nn<NU, ND, R>, launch_dmc_nn<NU, ND, R>};             \
    return &ks;                                                                                          \
  }

}  // namespace mole
