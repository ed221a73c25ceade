// handles.cuh -- the opaque handles of the C ABI (context, system, walker
// set) and helpers shared by the translation units that implement it.
#pragma once

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/mole_gpu.h"
#include "dispatch.cuh"
#include "ensemble.cuh"
#include "sr_large.cuh"

namespace mole {

// Records msg as the calling thread's last error and returns code.
int set_error(int code, const std::string& msg);

// Device buffer grown on demand (the context owns device memory).
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t reserve(size_t m) {
    if (m <= n) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(m, 1) * sizeof(T));
    if (e == cudaSuccess) n = m;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

cudaError_t launch_math_check(int fn, const double* x, int64_t n, double* y, cudaStream_t s);

// Kernel timing slots of a context (mole_ctx_kernel_time).
enum { kTimeVmc = 0, kTimeDmc = 1, kTimeEval = 2, kTimeSGemm = 3, kTimeBatch = 4, kTimeSlots = 5 };

}  // namespace mole

using namespace mole;  // the handle structs below are global (C ABI) types

struct mole_ctx {
  int device = 0;
  int n_sm = 0;
  int smem_optin = 0;  // shared memory a CTA may opt in to (bytes)
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  bool timing = false;
  double kernel_ms[mole::kTimeSlots] = {};  // VMC sweep, DMC step, evaluation, S-matrix GEMM, batch
  int64_t kernel_launches[mole::kTimeSlots] = {};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  DevBuf<double> partials, tb_partials, reduced, scratch;
  DevBuf<double> pos_backup;  // positions before a double-float launch (its native rerun starts there)
  int64_t df64_reruns = 0;    // double-float launches rerun in native FP64
  DevBuf<int> status;
  int refs = 1;
  bool closed = false;
};

struct mole_system {
  int version = 0;  // bumped by every parameter change (batches re-upload their copies)
  mole_ctx* ctx = nullptr;
  int n_nuc = 0, n_up = 0, n_dn = 0, n_basis = 0, n_exp = 0;
  std::vector<double> nuc_pos, en_coef, coef_up, coef_dn;
  std::vector<int> nuc_z, b_center, b_kind, b_exp;
  int ee_on = 0, ee_npoly = 0, en_on = 0, nn_on = 0, pot_kind = 0;
  double ee_kappa = 0, cusp_anti = 0.5, cusp_para = 0.25, omega = 0;
  int P = 0;
  std::vector<double> theta;
  SysParams<double> sp64;
  SysParams<float> sp32;
  SysParams<df64> spdf;
  const KernelSetT<double>* k64 = nullptr;
  const KernelSetT<float>* k32 = nullptr;
  const KernelSetT<df64>* kdf = nullptr;  // double-float kernels (NULL where not compiled)
  const NnKernelSetT<double>* nk64 = nullptr;  // neural systems
  const NnKernelSetT<float>* nk32 = nullptr;
  double* d_nn_theta = nullptr;  // device copy of the network parameters
  float* d_nn_tab = nullptr;      // quintic tables of the pair networks (FP32 form)
  double* d_nn_node = nullptr;    // FP64 node values the tables are built from
  int refs = 1;
  bool closed = false;
};

struct mole_walkers {
  mole_system* sys = nullptr;
  int W = 0;
  uint64_t seed = 0;
  uint64_t step = 0;
  double* pos = nullptr;  // SoA [3N][W]
  // DMC state (allocated on first DMC call)
  double *pos2 = nullptr, *eloc = nullptr, *eloc2 = nullptr, *weight = nullptr, *cum = nullptr, *btot = nullptr;
  double *e_ref = nullptr, *energies = nullptr;
  size_t energies_n = 0;
  uint64_t* dstep = nullptr;
  CombState* comb = nullptr;
  bool eloc_valid = false;
  double dmc_node_kills = 0.0;  // walkers given zero weight on a node of the guide, all DMC calls
  // many-parameter SR (allocated on first use)
  SrLargeState* srl = nullptr;
  CUtensorMap* srl_map = nullptr;
  double* srl_eval = nullptr;  // eval outputs: lnpsi, sign, lap, grad, O[W][8]
};


namespace mole {
// A batch keeps its systems alive like a walker set does.
void system_retain(mole_system* s);
void system_release(mole_system* s);
}  // namespace mole
