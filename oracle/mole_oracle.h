/*
 * mole_oracle.h -- CPU FP64 oracle for the mole walker hot path.
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the product (mole_gb300/, include/)
 * links or calls this code; only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py use it, and only as the reference the GPU results
 * are compared with.
 *
 * It restates the reference's algorithm (Jvanrhijn/mole, Rust) in plain C:
 *   - Metropolis box / diffuse moves        src/metropolis/src/metrop.rs:60-82, 150-198
 *   - sweep, acceptance, sampling order     src/montecarlo/src/samplers.rs:81-117,
 *                                           src/montecarlo/src/montecarlo.rs:24-46
 *   - local energy terms, n-n constant      src/operator/src/operator.rs:15-183
 *   - Pade Jastrow and its derivatives      theory/jastrow.tex:15-126
 *   - the example/test wavefunctions        the .rs files under examples/ and tests/
 * and writes the Slater-determinant x Jastrow evaluator (absent from the
 * reference) from its mathematics with dense LU determinants (no
 * Sherman-Morrison), so that it is an independent check of the GPU path.
 */
#ifndef MOLE_ORACLE_H
#define MOLE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_NUC 8
#define ORC_MAX_BASIS 32
#define ORC_MAX_SPIN 5
#define ORC_MAX_ELEC (2 * ORC_MAX_SPIN)
#define ORC_MAX_POLY 4
#define ORC_NN_H 64
#define ORC_NN_IN 4
#define ORC_NN_NET_P (ORC_NN_H * ORC_NN_IN + ORC_NN_H + ORC_NN_H * ORC_NN_H + ORC_NN_H + ORC_NN_H + 1)
#define ORC_NN_P (2 * ORC_NN_NET_P)

/* basis function kinds: Slater-type 1s, 2s, 2px, 2py, 2pz and a Gaussian 1s */
enum { ORC_STO_1S = 0, ORC_STO_2S = 1, ORC_STO_2PX = 2, ORC_STO_2PY = 3, ORC_STO_2PZ = 4, ORC_GTO_1S = 5 };
/* potential kinds: electronic Hamiltonian (Coulomb) or isotropic harmonic well */
enum { ORC_POT_COULOMB = 0, ORC_POT_HARMONIC = 1 };
/* move kinds */
enum { ORC_MOVE_BOX = 0, ORC_MOVE_GAUSS = 1, ORC_MOVE_DIFFUSE = 2 };

typedef struct {
  int32_t n_nuc;
  double nuc_pos[ORC_MAX_NUC * 3];
  int32_t nuc_z[ORC_MAX_NUC];
  int32_t n_up, n_dn;
  int32_t n_basis;
  int32_t b_center[ORC_MAX_BASIS];
  int32_t b_kind[ORC_MAX_BASIS];
  int32_t b_exp[ORC_MAX_BASIS];
  int32_t n_exp;
  double coef_up[ORC_MAX_SPIN * ORC_MAX_BASIS];
  double coef_dn[ORC_MAX_SPIN * ORC_MAX_BASIS];
  int32_t ee_on;
  int32_t ee_npoly;
  double ee_kappa;
  double cusp_anti, cusp_para;
  int32_t en_on;
  double en_coef[ORC_MAX_NUC];
  int32_t nn_on;
  int32_t pot_kind;
  double omega;
} orc_system;

typedef struct {
  double lnpsi;
  double sign;
  double grad[ORC_MAX_ELEC * 3]; /* grad ln psi, electron-major */
  double lap_over_psi;           /* sum_i lap_i psi / psi */
  double eloc;
  double vpot;
} orc_eval_out;

int orc_num_params(const orc_system* s);
/* The proposal normals: two N(0,1) floats from 2 x 32 random bits. */
void orc_normal_pair(uint32_t a, uint32_t b, float* z);
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* lnpsi, sign, grad ln psi, lap psi/psi, E_L and O_k = d ln psi / d theta_k
 * (O may be NULL) at one configuration pos[N][3]. Returns 0 or -1 on a
 * singular determinant. */
int orc_eval(const orc_system* s, const double* theta, const double* pos, orc_eval_out* out,
             double* O);

/* Reference example wavefunctions restated from the Rust (value, gradient,
 * laplacian of psi itself, not of ln psi). kind selects the function; par
 * holds its parameters. Returns psi. */
enum {
  ORC_REF_HELIUM = 0,     /* examples/helium_atom_singlet.rs:60-98, tests/helium_lcao.rs:48-87 */
  ORC_REF_STO_H = 1,      /* examples/dmc.rs:106-149 style 1-electron STO */
  ORC_REF_H2_HL = 2,      /* examples/hydrogen_molecule.rs:88-135 */
  ORC_REF_H2ION = 3,      /* tests/hydrogen_molecular_ion_lcao.rs:66-92 */
  ORC_REF_GAUSSIAN = 4    /* examples/custom_operator.rs:298-316, tests/sho_optimize.rs:52-75 */
};
double orc_ref_wf(int kind, const double* par, const double* pos, double* grad, double* lap,
                  double* dpsi_dpar);

/* E_L of a reference example via the reference's operator composition:
 * (T psi + V_ion psi + V_ee psi) / psi with T psi = -1/2 lap psi
 * (src/operator/src/operator.rs:103-183) or the harmonic Hamiltonian
 * (examples/custom_operator.rs:29-61). */
double orc_ref_eloc(int kind, const double* par, const double* pos, int n_nuc, const double* nuc_pos,
                    const int32_t* nuc_z, int harmonic, double omega);

typedef struct {
  int32_t move;        /* ORC_MOVE_* */
  double step;         /* box side L, Gaussian sigma or diffusion time step tau */
  int32_t n_eq;        /* unsampled steps */
  int32_t n_steps;     /* sampled steps */
  int32_t block_size;  /* steps per blocking block */
  int32_t sr;          /* accumulate O_k sums */
  uint64_t seed;
  uint32_t step0;      /* global step counter at entry */
  uint32_t walker0;    /* random-stream index of pos's first walker (a slice of a larger ensemble) */
} orc_vmc_opts;

/* moments layout (length ORC_NMOM) */
enum {
  ORC_MOM_COUNT = 0, ORC_MOM_SUM_E, ORC_MOM_SUM_E2, ORC_MOM_SUM_BLOCK2, ORC_MOM_NBLOCKS,
  ORC_MOM_ACCEPT, ORC_MOM_PROPOSED, ORC_NMOM
};

/* Runs W independent chains from pos (in/out, [W][N][3]) exactly as the GPU
 * path consumes its random numbers. time_block_sums has n_steps/block_size
 * entries; sr_* may be NULL when opts->sr is 0. Returns 0 or -1. */
int orc_vmc_run(const orc_system* s, const double* theta, int W, double* pos, const orc_vmc_opts* o,
                double* moments, double* time_block_sums, double* sr_O, double* sr_EO,
                double* sr_OO);

/* Initial positions for W walkers: kind 0 = N(0, width^2) per coordinate,
 * kind 1 = U(-width, width). Same random stream as the GPU path. */
void orc_init_positions(int W, int N, uint64_t seed, int kind, double width, double* pos);

/* One DMC step for W walkers (drift-diffusion sweep with Metropolis, weight
 * update) followed by a stochastic comb. pos, eloc are in/out; returns the
 * ensemble energy sum_w w E_L(old) / sum_w w, using the incoming weights
 * (all 1 after a comb). accepted/proposed are accumulated. */
double orc_dmc_step(const orc_system* s, const double* theta, int W, double* pos, double* eloc,
                    double tau, double e_ref, uint64_t seed, uint32_t step, double* accepted,
                    double* proposed, int* parent);

#ifdef __cplusplus
}
#endif
#endif
