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
  Vmc vmc[kPmSlots][2];  // [PM slot][drift]; NULL where not compiled
  Eval eval;
  Dmc dmc;
};

template <int NU, int ND, class R, int PM, bool DRIFT>
cudaError_t launch_vmc(const SysParams<R>& sp, const VmcArgs& a, int grid, cudaStream_t s) {
  vmc_kernel<NU, ND, R, PM, DRIFT><<<grid, kBlock, 0, s>>>(sp, a);
  return cudaGetLastError();
}
template <int NU, int ND, class R>
cudaError_t launch_eval(const SysParams<R>& sp, const EvalArgs& a, int grid, cudaStream_t s) {
  eval_kernel<NU, ND, R, 8><<<grid, kBlock, 0, s>>>(sp, a);
  return cudaGetLastError();
}
template <int NU, int ND, class R>
cudaError_t launch_dmc(const SysParams<R>& sp, const DmcArgs& a, int grid, cudaStream_t s) {
  dmc_step_kernel<NU, ND, R><<<grid, kBlock, 0, s>>>(sp, a);
  return cudaGetLastError();
}

template <int NU, int ND, class R, int PM, bool DRIFT, bool ON>
typename KernelSetT<R>::Vmc maybe_vmc() {
  if constexpr (ON) return launch_vmc<NU, ND, R, PM, DRIFT>;
  else return nullptr;
}
template <int NU, int ND, class R, bool ON>
typename KernelSetT<R>::Dmc maybe_dmc() {
  if constexpr (ON) return launch_dmc<NU, ND, R>;
  else return nullptr;
}

// SR2: compile the exact two-parameter SR kernels (the H2 optimisation);
// SR8: the eight-wide SR kernels; DRIFT: drift-diffusion VMC and DMC
// kernels (compiled for up to four electrons).
#define MOLE_INSTANTIATE(NU, ND, R, TAG, SR2, SR8, DRIFT)                                                 \
  const KernelSetT<R>* kernels_##TAG##_##NU##_##ND() {                                                   \
    static const KernelSetT<R> ks = {                                                                    \
        {{maybe_vmc<NU, ND, R, 0, false, true>(), maybe_vmc<NU, ND, R, 0, true, DRIFT>()},               \
         {maybe_vmc<NU, ND, R, 2, false, SR2>(), maybe_vmc<NU, ND, R, 2, true, (SR2 && DRIFT)>()},        \
         {maybe_vmc<NU, ND, R, 8, false, SR8>(), maybe_vmc<NU, ND, R, 8, true, (SR8 && DRIFT)>()}},       \
        launch_eval<NU, ND, R>,                                                                          \
        maybe_dmc<NU, ND, R, DRIFT>()};                                                                  \
    return &ks;                                                                                          \
  }

const KernelSetT<double>* kernel_set64(int nu, int nd);
const KernelSetT<float>* kernel_set32(int nu, int nd);

}  // namespace mole
