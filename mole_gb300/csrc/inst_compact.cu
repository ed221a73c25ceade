// FP64 VMC launchers for spin blocks of 1 up and at most 1 down electron,
// without and with two-parameter SR sums: the packed FP64 moves (compact.cuh,
// large ensembles) and the four-warp teams (team.cuh, small ensembles; one
// or two nuclei).
#include "dispatch.cuh"

namespace mole {

// Two CTAs (2 x ~44 KB of static shared memory) must fit an SM: the kernel
// asks for the largest shared-memory carveout, which the default choice does
// need not give.
template <int NU, int ND, int PM>
cudaError_t launch_vmc_compact(const SysParams<double>& sp, const VmcArgs& a, int grid, cudaStream_t s) {
  static const cudaError_t attr = cudaFuncSetAttribute(vmc_compact_kernel<NU, ND, PM>,
                                                       cudaFuncAttributePreferredSharedMemoryCarveout,
                                                       (int)cudaSharedmemCarveoutMaxShared);
  if (attr != cudaSuccess) return attr;
  vmc_compact_kernel<NU, ND, PM><<<grid, kCompactBlock, 0, s>>>(sp, a);
  return cudaGetLastError();
}

template <int NU, int ND, int PM, int NB>
cudaError_t launch_vmc_team(const SysParams<double>& sp, const VmcArgs& a, int grid, cudaStream_t s) {
  vmc_team_kernel<NU, ND, PM, NB><<<grid, kTeamThreads, 0, s>>>(sp, a);
  return cudaGetLastError();
}

template <int NB>
static KernelSetT<double>::Vmc team_vmc64_nb(int nu, int nd, int slot) {
  if (nu == 1 && nd == 1)
    return slot == 0 ? launch_vmc_team<1, 1, 0, NB> : (slot == 1 ? launch_vmc_team<1, 1, 2, NB> : nullptr);
  if (nu == 1 && nd == 0)
    return slot == 0 ? launch_vmc_team<1, 0, 0, NB> : (slot == 1 ? launch_vmc_team<1, 0, 2, NB> : nullptr);
  return nullptr;
}

KernelSetT<double>::Vmc team_vmc64(int nu, int nd, int slot, int n_nuc) {
  if (n_nuc == 1) return team_vmc64_nb<1>(nu, nd, slot);
  if (n_nuc == 2) return team_vmc64_nb<2>(nu, nd, slot);
  return nullptr;
}

KernelSetT<double>::Vmc compact_vmc64(int nu, int nd, int slot) {
  if (nu == 1 && nd == 1) return slot == 0 ? launch_vmc_compact<1, 1, 0> : (slot == 1 ? launch_vmc_compact<1, 1, 2> : nullptr);
  if (nu == 1 && nd == 0) return slot == 0 ? launch_vmc_compact<1, 0, 0> : (slot == 1 ? launch_vmc_compact<1, 0, 2> : nullptr);
  return nullptr;
}

}  // namespace mole
