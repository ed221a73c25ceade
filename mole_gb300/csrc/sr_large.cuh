// sr_large.cuh -- stochastic reconfiguration with many parameters (the
// neural Jastrow's 9,090 weights): O_k generation straight into the centred
// BF16 operand, the S = Ob^T Ob build on the tensor cores and the FP64
// conjugate-gradient solve.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include "walker.cuh"

namespace mole {

// S-matrix tiles: 128 x 256 parameters, 64 samples per pipeline stage.
constexpr int kSBM = 128;  // rows of a tile (M)
constexpr int kSBN = 256;  // columns of a tile (N)
constexpr int kSBK = 64;
constexpr int kSStages = 4;  // 4 x 48 KB: one CTA per SM
constexpr int kSBand = 16;   // row tiles per band of the tile order
constexpr uint32_t kSBoxBytes = 64 * kSBK * 2;               // one TMA box, 8 KB
constexpr uint32_t kSATileBytes = kSBM * kSBK * 2;           // A: two boxes, 16 KB
constexpr uint32_t kSStageBytes = (kSBM + kSBN) * kSBK * 2;  // A + B (four boxes), 48 KB
constexpr size_t kSGemmSmem = kSStages * (size_t)kSStageBytes + 1024 + 256;

// Walkers of the first sample of an iteration whose mean O_k is the centre c.
constexpr int kCenterRows = 1024;
// Samples held in Ob before they go through the S-GEMM together (fewer when
// they would take more than kObBudget bytes).
constexpr int kObSamples = 4;
constexpr size_t kObBudget = (size_t)8 << 30;

struct SrLargeState {
  int P;          // parameters
  int P_pad;      // columns of Ob, a multiple of 256
  int K_cap;      // rows of Ob: whole samples, rounded up to a multiple of 64
  int rows;       // rows of Ob holding samples not yet added into S
  int n_cta;      // CTAs of the sample kernel (rows of `partial`)
  float* O;       // [kCenterRows][P] FP32 O_k of the walkers that set the centre
  float* center;  // [P] c
  __nv_bfloat16* Ob;  // [K_cap][P_pad] bf16(O - c), one row per walker and sample
  float* partial; // [n_cta][2 P] per-CTA sums of one sample
  double* S;      // [P_pad][P_pad] accumulated (O-c)(O-c)^T (upper tiles)
  double* E;      // [W] local energies of the sample
  double* x;      // [P] solution of the CG solve
  double* sumO;   // [P] sum (O - c)
  double* sumEO;  // [P] sum E (O - c)
  double* work;   // CG vectors, 6 P + scalars
  int* status;
  double count;
  double sumE, sumE2;
  bool have_center;
  bool s_stored;   // S holds the sums of earlier GEMM launches of this iteration
  bool finalized;  // S holds the covariance (+ eps) rather than raw sums
  double eps;
  int gemm_launches;  // S-GEMM launches and their rows since the SR state was made
  double gemm_rows;
};

// dst[w][c] = (float)src[w][c] for c < ncols, w < W
cudaError_t launch_copy_cols(const double* src, int lds, int ncols, float* dst, int ldd, int W, cudaStream_t s);
// The network's O_k of walkers w < nw (pos: coordinate-major with stride W)
// into O[w][col0 ..] in FP32 or FP64.
cudaError_t launch_nn_ogen64(const SysParams<float>& sp, const double* pos, int W, int n_up, int n_elec, double* O,
                             int ldO, int col0, int grid, cudaStream_t s);
cudaError_t launch_nn_ogen(const SysParams<float>& sp, const double* pos, int W, int nw, int n_up, int n_elec,
                           float* O, int ldO, int col0, int grid, cudaStream_t s);
// c[p] = mean of O[w][p] over w < n
cudaError_t launch_center_rows(const float* O, int n, int P, int ldO, float* c, cudaStream_t s);
// One SR sample's operand rows: Ob[w][p] = bf16(O_wp - c_p) for all W walkers
// (orbital/Pade columns 0 .. n_orb - 1 from Oorb, the networks' after them
// when `nets`), and sumO += sum_w (O - c), sumEO += sum_w E_w (O - c).
int sr_sample_ctas(int W, int n_sm);
size_t sr_sample_smem(int P);
cudaError_t launch_sr_sample(const SysParams<float>& sp, const double* pos, int W, int n_up, int n_elec, bool nets,
                             const double* Oorb, int ldorb, int n_orb, const float* center, const double* E,
                             __nv_bfloat16* Ob, int ldb, int P, float* partial, int n_cta, double* sumO,
                             double* sumEO, cudaStream_t s);
// S (+)= Ob[0:K_pad]^T Ob[0:K_pad] on the upper tiles.
cudaError_t launch_s_gemm(const CUtensorMap* tmap, double* S, int P_pad, int K_pad, bool accumulate, int* status,
                          cudaStream_t s);
cudaError_t encode_ob_tensor_map(CUtensorMap* tmap, __nv_bfloat16* Ob, int P_pad, int K_rows);
// S_kl = (S_kl / n - m_k m_l) for k, l < P, symmetrised, with eps on the diagonal; m = sumO / n.
cudaError_t launch_finalize_s(double* S, int P, int P_pad, const double* sumO, double n, double eps, cudaStream_t s);
// Jacobi-preconditioned CG for S x = b (S symmetric positive definite, FP64).
cudaError_t sr_cg_solve(const double* S, int P, int ld, const double* b, double* x, double* work, int max_iter,
                        double tol, int* iters, double* rel_res, cudaStream_t s);

}  // namespace mole
