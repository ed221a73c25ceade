// ensemble.cuh -- declarations of the ensemble-wide kernels (ensemble.cu).
#pragma once

#include "common.cuh"

namespace mole {

constexpr int kScanBlock = 256;

struct CombState {
  double total;     // sum of weights this step
  double u;         // the comb's one uniform
  double accepted;  // running accepted moves
  double proposed;  // running proposed moves
  double killed;    // running count of walkers given zero weight on a node of the guide
};

cudaError_t launch_init_positions(double* pos, int W, int N, uint64_t seed, int kind, double width, cudaStream_t s);
cudaError_t launch_aos_to_soa(const double* aos, double* soa, int W, int NC, cudaStream_t s);
cudaError_t launch_soa_to_aos(const double* soa, double* aos, int W, int NC, cudaStream_t s);
cudaError_t launch_reduce_columns(const double* part, int rows, int cols, double* out, cudaStream_t s);
// Reduced VMC sums (7 moments, then PM O sums, PM E*O sums, upper triangle of
// O O^T) -> moments[7] and, if sr is not NULL, sr = [sum_O (P), sum_EO (P),
// sum_OO (P x P)].
cudaError_t launch_unpack_vmc_sums(const double* red, int PM, int P, double* moments, double* sr, cudaStream_t s);
cudaError_t launch_comb(const double* weight, double* cum, double* btot, int nb, const double* partials, int n_part,
                        CombState* cs, uint64_t* step, uint64_t seed, double* energies, int64_t e_index,
                        const double* pos_in, const double* eloc_in, double* pos_out, double* eloc_out, int W, int NC,
                        cudaStream_t s);
cudaError_t launch_fma_probe64(double* out, int blocks, int threads, int iters, cudaStream_t s);
cudaError_t launch_fma_probe32(float* out, int blocks, int threads, int iters, cudaStream_t s);

}  // namespace mole
