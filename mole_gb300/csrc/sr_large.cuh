// sr_large.cuh -- stochastic reconfiguration with many parameters (the
// neural Jastrow's 9,090 weights): O_k generation, the S = O^T O build on
// the tensor cores and the FP64 conjugate-gradient solve.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include "walker.cuh"

namespace mole {

// S-matrix tiles: 128 x 128 parameters, 64 samples per pipeline stage.
constexpr int kSBM = 128;
constexpr int kSBK = 64;
constexpr int kSStages = 3;  // 97 KB of stages: two CTAs per SM, one's epilogue under the other's MMAs
constexpr int kSBand = 16;  // tile rows per band of the tile order
constexpr uint32_t kSTileBytes = kSBM * kSBK * 2;  // one BF16 operand tile, 16 KB
constexpr size_t kSGemmSmem = 2 * kSStages * (size_t)kSTileBytes + 1024 + 256;

struct SrLargeState {
  int P;          // parameters
  int P_pad;      // rows of the BF16 operand, a multiple of 128
  int K_pad;      // samples per batch (walkers), a multiple of 64
  float* O;       // [W][P] FP32 log-derivatives of one batch
  __nv_bfloat16* Ot;  // [P_pad][K_pad] centred operand
  double* S;      // [P_pad][P_pad] accumulated (O-c)(O-c)^T (upper tiles)
  double* E;      // [W] local energies of the batch
  double* center; // [P] c
  double* sumO;   // [P] sum (O - c)
  double* sumEO;  // [P] sum E (O - c)
  double* work;   // CG vectors, 6 P + scalars
  int* status;
  double count;
  double sumE, sumE2;
  bool have_center;
  bool finalized;  // S holds the covariance (+ eps) rather than raw sums
  double eps;
};

// dst[w][c] = (float)src[w][c] for c < ncols
cudaError_t launch_copy_cols(const double* src, int lds, int ncols, float* dst, int ldd, int W, cudaStream_t s);
cudaError_t launch_nn_ogen64(const SysParams<float>& sp, const double* pos, int W, int n_up, int n_elec, double* O,
                             int ldO, int col0, int grid, cudaStream_t s);
cudaError_t launch_nn_ogen(const SysParams<float>& sp, const double* pos, int W, int n_up, int n_elec, float* O,
                           int ldO, int col0, int grid, cudaStream_t s);
cudaError_t launch_center_transpose(const float* O, int W, int P, int ldO, const double* E, double* center,
                                    bool set_center, __nv_bfloat16* Ot, int K_pad, double* sumO, double* sumEO,
                                    double* scratch, cudaStream_t s);
cudaError_t launch_s_gemm(const CUtensorMap* tmap, double* S, int P_pad, int K_pad, int* status, cudaStream_t s);
cudaError_t encode_ot_tensor_map(CUtensorMap* tmap, __nv_bfloat16* Ot, int P_pad, int K_pad);
// S_kl = (S_kl / n - m_k m_l) for k, l < P, symmetrised, with eps on the diagonal; m = sumO / n.
cudaError_t launch_finalize_s(double* S, int P, int P_pad, const double* sumO, double n, double eps, cudaStream_t s);
// Jacobi-preconditioned CG for S x = b (S symmetric positive definite, FP64).
cudaError_t sr_cg_solve(const double* S, int P, int ld, const double* b, double* x, double* work, int max_iter,
                        double tol, int* iters, double* rel_res, cudaStream_t s);

}  // namespace mole
