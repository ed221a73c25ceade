/*
 * mole_gpu.h -- C ABI of the GB300 walker hot path for Jvanrhijn/mole.
 *
 * The reference exposes its hot path as Rust traits evaluated one walker at a
 * time: Function/Differentiate/WaveFunction (src/wavefunction_traits/src/lib.rs:7-24),
 * Optimize (src/optimize/src/traits.rs:8-16), LocalOperator (src/operator/src/traits.rs:262-265),
 * Metropolis (src/metropolis/src/traits.rs:10-38), MonteCarloSampler
 * (src/montecarlo/src/traits.rs:12-39), Optimizer (src/optimize/src/traits.rs:18-25)
 * and BranchingAlgorithm (src/dmc/src/traits.rs:4-7). A trait object cannot
 * cross into a kernel, so this ABI is ensemble-batched and selects the
 * wavefunction family by descriptor. Each entry point below names the
 * reference interface it replaces.
 *
 * Conventions
 *  - Every call returns a mole_status; MOLE_OK is 0. The first six codes map
 *    one-to-one to errors::Error (src/errors/src/lib.rs:8-15).
 *  - The caller owns host buffers; a context owns device memory.
 *  - Calls are ordered on the context's stream. Entry points that return
 *    results in host buffers synchronise that stream before returning.
 *  - One context per host thread; contexts are not shared across threads
 *    without external locking. mole_last_error_string is thread-local.
 *  - Positions cross the ABI as host float64 [W][N][3] (walker, electron,
 *    xyz), the layout of the reference's Array2<f64> configuration.
 */
#ifndef MOLE_GPU_H
#define MOLE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MOLE_ABI_VERSION 1

typedef enum {
  MOLE_OK = 0,
  MOLE_ERR_LINALG = 1,                 /* errors::Error::LinalgError (singular S or determinant) */
  MOLE_ERR_SHAPE = 2,                  /* errors::Error::ShapeError (inconsistent sizes) */
  MOLE_ERR_FUNC = 3,                   /* errors::Error::FuncError (NaN/Inf psi or E_L) */
  MOLE_ERR_OPERATOR_VALUE_ACCESS = 4,  /* errors::Error::OperatorValueAccessError */
  MOLE_ERR_DATA_ACCESS = 5,            /* errors::Error::DataAccessError (missing output) */
  MOLE_ERR_EMPTY_CACHE = 6,            /* errors::Error::EmptyCacheError */
  MOLE_ERR_CUDA = 100,                 /* a CUDA runtime call failed */
  MOLE_ERR_INVALID_ARG = 101,          /* NULL handle or out-of-range argument */
  MOLE_ERR_TIMEOUT = 102,              /* a bounded device wait gave up */
  MOLE_ERR_UNSUPPORTED = 103,          /* size outside the compiled kernel family */
  MOLE_ERR_IO = 104                    /* checkpoint file error */
} mole_status;

/* basis function kinds */
enum { MOLE_STO_1S = 0, MOLE_STO_2S = 1, MOLE_STO_2PX = 2, MOLE_STO_2PY = 3, MOLE_STO_2PZ = 4, MOLE_GTO_1S = 5 };
/* potentials: the electronic Hamiltonian of src/operator/src/operator.rs:150-184, or the
 * harmonic Hamiltonian of examples/custom_operator.rs:29-61 */
enum { MOLE_POT_COULOMB = 0, MOLE_POT_HARMONIC = 1 };
/* moves: MetropolisBox (src/metropolis/src/metrop.rs:22-101), a Gaussian single-electron
 * move with the same symmetric acceptance, MetropolisDiffuse (metrop.rs:104-217) */
enum { MOLE_MOVE_BOX = 0, MOLE_MOVE_GAUSS = 1, MOLE_MOVE_DIFFUSE = 2 };
/* arithmetic: all FP64, or FP32 orbital/Jastrow/MLP evaluation with FP64 inverse,
 * Sherman-Morrison ratio products, E_L and accumulation, or FP64-accurate
 * double-float: every term as a pair of FP32 numbers (48 significant bits) on
 * the FP32 pipe, results within about 1e-13 relative of FP64. MOLE_PREC_DF64
 * applies to box and Gaussian VMC sweeps (SR sums of at most 2 parameters),
 * mole_eval and mole_dmc_run of the non-neural fixed-size families; a call
 * whose values leave FP32's exponent range (or, in DMC, whose walkers meet a
 * node) is rerun in native FP64 on the device, and every other call treats
 * MOLE_PREC_DF64 as MOLE_PREC_FP64 */
enum { MOLE_PREC_FP64 = 0, MOLE_PREC_MIXED = 1, MOLE_PREC_DF64 = 2 };
/* initial positions: N(0, width^2) per coordinate, or U(-width, width) as
 * Sampler::new does (src/montecarlo/src/samplers.rs:44-55) */
enum { MOLE_INIT_NORMAL = 0, MOLE_INIT_UNIFORM = 1 };

#define MOLE_MAX_NUCLEI 8
#define MOLE_MAX_BASIS 32
#define MOLE_MAX_SPIN 5
#define MOLE_MAX_POLY 4
#define MOLE_NN_PARAMS 9090

typedef struct mole_ctx mole_ctx;
typedef struct mole_system mole_system;
typedef struct mole_walkers mole_walkers;

/* Wavefunction family descriptor: psi = det_up * det_dn * exp(J).
 * Orbital k of a spin block is sum_b coef[k][b] chi_b(r); chi_b is a basis
 * function of kind basis_kind[b] centred on nucleus basis_center[b] with
 * exponent theta[basis_exp[b]]. J = sum_{i<j} u(r_ij) + sum_{i,I} chi_I(r_iI)
 * (+ the pair MLP when nn_on), with the Pade form of theory/jastrow.tex:15-29
 * for u (b1 = cusp_anti or cusp_para, b2 = b, polynomial b_3.., scaled
 * distance with kappa) and chi_I(r) = en_coef[I] r / (1 + a r).
 * Parameter vector theta (the order of O_k):
 *   [n_exp exponents] [b, poly[ee_npoly]] if ee_on [a] if en_on [9090 MLP] if nn_on. */
typedef struct {
  int32_t n_nuclei;
  const double* nuc_pos;       /* [n_nuclei][3] */
  const int32_t* nuc_charge;   /* [n_nuclei] */
  int32_t n_up, n_dn;          /* 1 <= n_up <= 5, 0 <= n_dn <= n_up */
  int32_t n_basis;
  const int32_t* basis_center; /* [n_basis] */
  const int32_t* basis_kind;   /* [n_basis] */
  const int32_t* basis_exp;    /* [n_basis] index into the exponent parameters */
  int32_t n_exp;
  const double* coef_up;       /* [n_up][n_basis] */
  const double* coef_dn;       /* [n_dn][n_basis] */
  int32_t ee_on, ee_npoly;
  double ee_kappa, cusp_anti, cusp_para;
  int32_t en_on;
  const double* en_coef;       /* [n_nuclei] */
  int32_t nn_on;
  int32_t pot_kind;
  double omega;
} mole_system_desc;

typedef struct {
  int32_t move;        /* MOLE_MOVE_* */
  double step;         /* box side, Gaussian sigma, or diffusion time step */
  int32_t n_eq;        /* unsampled sweeps (the reference's block 0, montecarlo.rs:45-52) */
  int32_t n_steps;     /* sampled sweeps; a multiple of block_size */
  int32_t block_size;  /* sweeps per blocking block */
  int32_t sr;          /* accumulate sum O_k, sum E O_k, sum O_k O_l */
  int32_t precision;   /* MOLE_PREC_* */
  int32_t refresh;     /* Sherman-Morrison steps between FP64 inverse refreshes (0 = 100) */
} mole_vmc_opts;

/* moments returned by mole_vmc_run (length MOLE_NMOM) */
enum {
  MOLE_MOM_COUNT = 0,      /* samples */
  MOLE_MOM_SUM_E = 1,      /* sum E_L */
  MOLE_MOM_SUM_E2 = 2,     /* sum E_L^2 */
  MOLE_MOM_SUM_BLOCK2 = 3, /* sum over (walker, block) of block-mean^2 */
  MOLE_MOM_NBLOCKS = 4,    /* number of (walker, block) blocks */
  MOLE_MOM_ACCEPT = 5,     /* accepted single-electron moves (incl. equilibration) */
  MOLE_MOM_PROPOSED = 6,   /* proposed single-electron moves */
  MOLE_NMOM = 7
};

typedef struct {
  double tau;          /* time step */
  double e_ref;        /* reference energy in the weight factor */
  int32_t n_steps;     /* DMC steps, each a sweep + weight update + comb */
  int32_t precision;   /* MOLE_PREC_* */
  int32_t refresh;     /* steps between FP64 inverse refreshes (0 = 100) */
  double eloc_cutoff;  /* 0: the raw E_L in the weight, as DmcRunner::diffuse (src/dmc/src/dmc.rs:126-128);
                          > 0: E_L clipped to e_ref +- eloc_cutoff in the weight factor only (the
                          Umrigar-Nightingale-Runge 1993 remedy for trial functions that violate
                          the cusp conditions); the energy estimator keeps the raw E_L */
} mole_dmc_opts;

/* ---------------------------------------------------------------- context */
int32_t mole_abi_version(void);
const char* mole_last_error_string(void);
/* device: CUDA ordinal. Replaces the rayon worker pool of src/vmc/src/vmc.rs:63-76. */
int mole_ctx_create(int32_t device, mole_ctx** out);
int mole_ctx_destroy(mole_ctx* ctx);
/* Launch on an external cudaStream_t (NULL restores the context's own stream). */
int mole_ctx_set_stream(mole_ctx* ctx, void* cuda_stream);
int mole_sync(mole_ctx* ctx);
/* Per-kernel CUDA-event timing of the hot kernels (off by default). */
int mole_ctx_enable_timing(mole_ctx* ctx, int32_t on);
/* kernel: 0 = VMC sweep kernel, 1 = DMC step sequence, 2 = evaluation (and
 * O_k generation), 3 = tensor-core S-matrix GEMM, 4 = one batched VMC run
 * (the replayed graph). Returns the summed
 * milliseconds and launch count since timing was enabled. */
int mole_ctx_kernel_time(mole_ctx* ctx, int32_t kernel, double* total_ms, int64_t* launches);
/* SM count and compute capability of the context's device (the key of tuned tiles). */
int mole_ctx_device_info(mole_ctx* ctx, int32_t* n_sm, int32_t* cc_major, int32_t* cc_minor);
/* Double-float (MOLE_PREC_DF64) launches of this context that were rerun in
 * native FP64 because a value left FP32's exponent range (no reference
 * counterpart: the reference computes in f64 only). */
int mole_ctx_df64_reruns(mole_ctx* ctx, int64_t* reruns);
/* Evaluates the library's device arithmetic on n host values x (no reference
 * counterpart; for accuracy tests): fn 0 = the FP64 exponential of the native
 * FP64 kernels, 1 = double-float exp, 2 = double-float reciprocal square root,
 * 3 = double-float reciprocal, 4 = double-float x / (1 + x^2), 5 = x rounded
 * to float and widened by the integer-built conversion, 6 = x narrowed to
 * float toward zero by the integer-built conversion, 7 = the same for
 * magnitudes below FP32's largest (positions), 8 = the FP64 reciprocal and
 * 9 = the FP64 reciprocal square root of the native FP64 kernels. Results go
 * to the host array y. */
int mole_math_check(mole_ctx* ctx, int32_t fn, const double* x, int64_t n, double* y);
/* Device FP64 and FP32 FMA peaks measured by a microbenchmark (GFLOP/s). */
int mole_probe_peaks(mole_ctx* ctx, double* fp64_gflops, double* fp32_gflops);

/* ---------------------------------------------------------------- systems */
/* Replaces implementing Function + Differentiate + WaveFunction + Optimize for
 * a concrete psi (src/wavefunction_traits/src/lib.rs:7-24, src/optimize/src/traits.rs:8-16)
 * and constructing ElectronicHamiltonian::from_ions (src/operator/src/operator.rs:162-168). */
int mole_system_create(mole_ctx* ctx, const mole_system_desc* desc, const double* theta, int32_t n_theta,
                       mole_system** out);
int mole_system_destroy(mole_system* sys);
/* Optimize::num_parameters / parameters / update_parameters (optimize/src/traits.rs:8-16) */
int mole_num_params(const mole_system* sys, int32_t* out);
int mole_params_get(const mole_system* sys, double* theta, int32_t n);
int mole_params_set(mole_system* sys, const double* theta, int32_t n);
/* WaveFunction::num_electrons (wavefunction_traits/src/lib.rs:22-24) */
int mole_num_electrons(const mole_system* sys, int32_t* out);

/* ---------------------------------------------------------------- walkers */
/* A walker ensemble: replaces the per-chain Array2 configuration owned by
 * Sampler (src/montecarlo/src/samplers.rs:14-21) and DmcRunner's walker list
 * (src/dmc/src/dmc.rs:27-29). Positions stay resident on the device. */
int mole_walkers_create(mole_system* sys, int32_t n_walkers, uint64_t seed, mole_walkers** out);
int mole_walkers_destroy(mole_walkers* w);
int mole_walkers_count(const mole_walkers* w, int32_t* out);
/* Philox-seeded start (Sampler::new, samplers.rs:44-55; DmcRunner::new, dmc.rs:40-67) */
int mole_walkers_init(mole_walkers* w, int32_t kind, double width);
int mole_walkers_set_positions(mole_walkers* w, const double* pos, int64_t n_values);
int mole_walkers_get_positions(mole_walkers* w, double* pos, int64_t n_values);
/* Global sweep counter (the random stream position); persists across calls. */
int mole_walkers_get_step(const mole_walkers* w, uint64_t* step);
int mole_walkers_set_step(mole_walkers* w, uint64_t step);

/* -------------------------------------------------------------- evaluation */
/* Function::value + Differentiate::gradient/laplacian + Optimize::parameter_gradient and
 * ElectronicHamiltonian::act_on / psi (samplers.rs:89-90) at every walker's
 * current position, in log form. Host outputs, each may be NULL:
 *   lnpsi[W], sign[W], grad_lnpsi[W][N][3], lap_over_psi[W] (sum_i lap_i psi / psi),
 *   eloc[W], O[W][P] (d ln psi / d theta). */
int mole_eval(mole_walkers* w, int32_t precision, double* lnpsi, double* sign, double* grad_lnpsi,
              double* lap_over_psi, double* eloc, double* O);

/* ---------------------------------------------------------------------- VMC */
/* Runner::run + Sampler::move_state/sample + Metropolis::move_state for the
 * whole ensemble (src/montecarlo/src/montecarlo.rs:24-46, samplers.rs:81-117,
 * metrop.rs:60-198), with the "Energy", "Parameter gradient" and "Wavefunction value"
 * observables reduced on the device instead of stored per sample
 * (src/vmc/src/operators.rs:7-24, src/optimize/src/util.rs:6-46).
 * moments[MOLE_NMOM]; time_blocks[n_steps/block_size] (ensemble sum of E_L per
 * block, may be NULL); sum_O[P], sum_EO[P], sum_OO[P][P] when opts->sr (else may be NULL). */
int mole_vmc_run(mole_walkers* w, const mole_vmc_opts* opts, double* moments, double* time_blocks,
                 double* sum_O, double* sum_EO, double* sum_OO);

/* Allocation-free variant of mole_vmc_run (no counterpart in the reference).
 * For callers that cannot allocate device memory while they run: a host
 * framework that owns all device memory through its own pool, or code that
 * must not take cudaMalloc's implicit device synchronisation inside a timed or
 * latency-critical loop. The caller passes every input and output as device
 * memory: d_pos the positions as SoA float64 [3N][W] (updated in place),
 * d_moments[MOLE_NMOM], d_time_blocks[n_steps / block_size] (may be NULL when
 * n_steps is 0), d_sr = [sum_O (P), sum_EO (P), sum_OO (P x P)] when opts->sr
 * (else may be NULL); seed and step0 select the random streams (the same
 * streams mole_vmc_run uses for a walker set with that seed and step counter;
 * the caller advances step0 by n_eq + n_steps itself). The library's only
 * working memory is one fixed 2 MiB device array that every GPU loading the
 * library holds until the process exits; the call is rejected with
 * MOLE_ERR_SHAPE when (CTAs of the launch) x (accumulators + time blocks) does not
 * fit it. The first call on a device looks up that array's device address;
 * the address is kept for the life of the process and stays valid while the
 * device's primary context lives (a cudaDeviceReset by the caller invalidates
 * it). Every call shares the array:
 * calls that overlap on the GPU (other streams, other threads) race. The call
 * reads its status word back and synchronises `stream` (a cudaStream_t of the
 * system's device, NULL for the default stream; a stream of another device is
 * rejected with MOLE_ERR_INVALID_ARG) before returning, and leaves the
 * caller's current device as it found it. */
int mole_vmc_run_noalloc(const mole_system* sys, double* d_pos, int32_t n_walkers, uint64_t seed, uint64_t step0,
                         const mole_vmc_opts* opts, double* d_moments, double* d_time_blocks, double* d_sr,
                         void* stream);

/* StochasticReconfiguration::compute_parameter_update (src/optimize/src/optimizers.rs:236-252)
 * from the reduced sums of mole_vmc_run: S_kl = <O_k O_l> - <O_k><O_l>,
 * g_k = 2 (<E O_k> - <E><O_k>), S_kk += eps, delta = step * S^-1 (-g/2), FP64
 * Cholesky. Writes delta[P] and, if not NULL, g[P]. MOLE_ERR_LINALG when S is
 * not positive definite. */
int mole_sr_update(mole_ctx* ctx, int32_t P, double count, const double* sum_E, const double* sum_O,
                   const double* sum_EO, const double* sum_OO, double eps, double step, double* delta,
                   double* grad);

/* Stochastic reconfiguration for thousands of parameters (the neural Jastrow):
 * replaces StochasticReconfiguration::construct_sr_matrix and the solveh call
 * (src/optimize/src/optimizers.rs:191-252) when P is too large for per-walker
 * sums. Each sample takes O_k = d ln psi / d theta_k and E_L of every walker at
 * its current position (move the walkers with mole_vmc_run in between) and
 * writes each walker's row bf16(O - c) of the S-GEMM's operand, c being the
 * mean O_k of the first 1,024 walkers of the first sample after
 * mole_sr_collect_begin; the sums of O - c and E (O - c) are kept in FP32
 * within a CTA and FP64 across CTAs. S = sum (O-c)(O-c)^T is accumulated on
 * the tensor cores (BF16 operands, FP32 accumulation inside a 128 x 128 tile,
 * FP64 across launches) once per four samples (fewer when four would exceed
 * 8 GiB of operand rows): when a sample does not fit, and at
 * mole_sr_collect_solve / mole_sr_collect_matrix. S and g do not depend on c.
 * mole_sr_collect_solve forms
 * S_kl = <(O-c)_k (O-c)_l> - <O-c>_k <O-c>_l + eps delta_kl and
 * g_k = 2 (<E O_k> - <E><O_k>) and solves S x = -g/2 in FP64 by
 * Jacobi-preconditioned conjugate gradients (max_iter, relative residual tol;
 * 0 picks 500 and 1e-8); delta = step x. info[4] = {mean E, samples, CG
 * iterations, relative residual}. MOLE_ERR_LINALG when CG does not converge. */
int mole_sr_collect_begin(mole_walkers* w);
int mole_sr_collect_sample(mole_walkers* w, int32_t precision);
int mole_sr_collect_solve(mole_walkers* w, double eps, double step, int32_t max_iter, double tol, double* delta,
                          double* grad, double* info);
/* The finalised S matrix (P x P, row-major) of the collected samples. */
int mole_sr_collect_matrix(mole_walkers* w, double eps, double* S);

/* ------------------------------------------------------ batches of systems */
/* A ragged batch of independent systems -- different electron counts (up to
 * 5 + 5), parameters and walker counts -- advanced together by ONE persistent
 * launch whose CTAs pull (system, walker group) work items from a device
 * queue, most expensive first. It replaces running Runner::run /
 * VmcRunner::run_optimization once per (system, chain)
 * (src/montecarlo/src/montecarlo.rs:24-46, src/vmc/src/vmc.rs:43-106).
 * Systems keep their handles (a batch holds a reference to each and re-reads
 * parameters changed with mole_params_set before the next run). seeds[k] is
 * system k's random-stream key: the batch follows exactly the streams of a
 * mole_walkers set created with that seed and the same walker count. widths
 * (may be NULL = all 1) are the per-system proposal widths, multiplied by
 * opts->step at run time. Positions start N(0, 1) as in mole_walkers_create. */
typedef struct mole_batch mole_batch;
int mole_batch_create(mole_ctx* ctx, int32_t n_systems, mole_system* const* systems, const int32_t* n_walkers,
                      const uint64_t* seeds, const double* widths, mole_batch** out);
int mole_batch_destroy(mole_batch* b);
int mole_batch_info(const mole_batch* b, int32_t* n_systems, int64_t* n_walkers);
/* Philox-seeded start of every system (as mole_walkers_init) */
int mole_batch_init(mole_batch* b, int32_t kind, double width);
/* host float64 [W][N][3] of one system */
int mole_batch_set_positions(mole_batch* b, int32_t system, const double* pos, int64_t n_values);
int mole_batch_get_positions(mole_batch* b, int32_t system, double* pos, int64_t n_values);
/* shared sweep counter of the batch (the random-stream position) */
int mole_batch_get_step(const mole_batch* b, uint64_t* step);
int mole_batch_set_step(mole_batch* b, uint64_t step);
/* The sweep loop of Runner::run + Sampler::move_state/sample for every system
 * at once (box or Gaussian single-electron moves with Sherman-Morrison
 * updates, FP64 inverse refresh every opts->refresh sweeps, E_L every sampled
 * sweep). moments[n_systems][MOLE_NMOM] as for mole_vmc_run. A run is a
 * CUDA graph (counter resets, the persistent kernel, the per-system reduction
 * and the result copy) captured on the first call with given options and
 * replayed by later ones. opts->sr must be 0. */
int mole_batch_vmc_run(mole_batch* b, const mole_vmc_opts* opts, double* moments);
/* Tile autotuner: times the persistent kernel for every walkers-per-CTA tile
 * in {32, 64, 96, 128, 192, 256} that fits an SM (grid = SMs x resident CTAs)
 * on a copy of the positions (chains and streams are left untouched), keeps
 * the fastest and reports up to n_candidates (tile, ms) pairs. */
int mole_batch_autotune(mole_batch* b, const mole_vmc_opts* opts, int32_t n_candidates, int32_t* cand_wpb,
                        double* cand_ms, int32_t* n_timed);
int mole_batch_set_tile(mole_batch* b, int32_t walkers_per_cta);
/* the tile in use and the persistent grid it launches for `precision` */
int mole_batch_get_tile(const mole_batch* b, int32_t* walkers_per_cta, int32_t* ctas, int32_t precision);
/* number of graph replays run so far */
int mole_batch_graph_launches(const mole_batch* b, int64_t* n);

/* ---------------------------------------------------------------------- DMC */
/* DmcRunner::diffuse inner loop (src/dmc/src/dmc.rs:81-141) for opts->n_steps
 * steps: drift-diffusion sweep with Metropolis accept/reject, weight
 * exp(-tau((E_L + E_L')/2 - e_ref)), then a stochastic comb replacing
 * SRBrancher::branch (src/dmc/src/branching.rs:15-39): constant population,
 * equal weights. energies[n_steps] receives the per-step ensemble energy
 * sum_w w E_L(old) / sum_w w (dmc.rs:112-135); accept[2] = accepted, proposed. */
int mole_dmc_run(mole_walkers* w, const mole_dmc_opts* opts, double* energies, double* accept);
/* Walkers a DMC step found on a node of the guide (an exactly singular Slater
 * matrix at the precision of its orbital values, psi = 0 there) and gave zero
 * weight, so the comb removed them; summed over every mole_dmc_run call of
 * the walker set. The reference has no counterpart (its DMC would divide by
 * psi = 0). */
int mole_dmc_node_kills(const mole_walkers* w, double* killed);

/* ------------------------------------------------------------- checkpoints */
/* Versioned binary dump of positions, step counter, seed and parameters. */
int mole_checkpoint_save(mole_walkers* w, const char* path);
int mole_checkpoint_load(mole_walkers* w, const char* path);

#ifdef __cplusplus
}
#endif
#endif
