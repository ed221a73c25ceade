// capi.cu -- implementation of the C ABI declared in include/mole_gpu.h.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mole_gpu.h"
#include "handles.cuh"

namespace mole {
// A family's kernel set from the slices its translation units compile.
template <class R>
KernelSetT<R> merge_parts(std::initializer_list<KernelSetT<R>> parts) {
  KernelSetT<R> k{};
  for (const KernelSetT<R>& p : parts) {
    for (int a = 0; a < kPmSlots; ++a)
      for (int d = 0; d < 2; ++d)
        for (int e = 0; e < 2; ++e)
          if (p.vmc[a][d][e]) k.vmc[a][d][e] = p.vmc[a][d][e];
    for (int e = 0; e < 2; ++e) {
      if (p.eval[e]) k.eval[e] = p.eval[e];
      if (p.dmc[e]) k.dmc[e] = p.dmc[e];
    }
  }
  return k;
}
#define MOLE_DECL_PARTS(NU, ND, R, TAG)                                                   \
  KernelSetT<R> kparts_##TAG##_##NU##_##ND##_0();                                         \
  KernelSetT<R> kparts_##TAG##_##NU##_##ND##_1();                                         \
  KernelSetT<R> kparts_##TAG##_##NU##_##ND##_2();                                         \
  KernelSetT<R> kparts_##TAG##_##NU##_##ND##_r();                                         \
  const KernelSetT<R>* kernels_##TAG##_##NU##_##ND() {                                    \
    static const KernelSetT<R> ks =                                                       \
        merge_parts<R>({kparts_##TAG##_##NU##_##ND##_0(), kparts_##TAG##_##NU##_##ND##_1(), \
                        kparts_##TAG##_##NU##_##ND##_2(), kparts_##TAG##_##NU##_##ND##_r()}); \
    return &ks;                                                                           \
  }
#define MOLE_DECL(NU, ND)               \
  MOLE_DECL_PARTS(NU, ND, double, f64) \
  MOLE_DECL_PARTS(NU, ND, float, f32)
MOLE_DECL(1, 0)
MOLE_DECL(1, 1)
MOLE_DECL(2, 1)
MOLE_DECL(2, 2)
#define MOLE_DECL_DF(NU, ND)                      \
  DfParts df_parts_vmc_##NU##_##ND##_0();         \
  DfParts df_parts_vmc_##NU##_##ND##_1();         \
  DfParts df_parts_eval_##NU##_##ND##_0();        \
  DfParts df_parts_eval_##NU##_##ND##_1();        \
  DfParts df_parts_dmc_##NU##_##ND##_0();         \
  DfParts df_parts_dmc_##NU##_##ND##_1();         \
  const KernelSetT<df64>* kernels_df_##NU##_##ND() { \
    static const KernelSetT<df64> ks = [] {       \
      KernelSetT<df64> k{};                       \
      const DfParts v0 = df_parts_vmc_##NU##_##ND##_0(), v1 = df_parts_vmc_##NU##_##ND##_1(); \
      for (int p = 0; p < kPmSlots; ++p) {        \
        k.vmc[p][0][0] = v0.vmc[p];               \
        k.vmc[p][0][1] = v1.vmc[p];               \
      }                                           \
      k.eval[0] = df_parts_eval_##NU##_##ND##_0().eval; \
      k.eval[1] = df_parts_eval_##NU##_##ND##_1().eval; \
      k.dmc[0] = df_parts_dmc_##NU##_##ND##_0().dmc; \
      k.dmc[1] = df_parts_dmc_##NU##_##ND##_1().dmc; \
      return k;                                   \
    }();                                          \
    return &ks;                                   \
  }
MOLE_DECL_DF(1, 0)
MOLE_DECL_DF(1, 1)
MOLE_DECL_DF(2, 1)
MOLE_DECL_DF(2, 2)
KernelSetT<double>::Vmc compact_vmc64(int nu, int nd, int slot);
KernelSetT<double>::Vmc team_vmc64(int nu, int nd, int slot, int n_nuc);
const NnKernelSetT<double>* nn_kernels_f64_2_2();
const NnKernelSetT<float>* nn_kernels_f32_2_2();

#define MOLE_CASE(NU, ND, TAG) \
  if (nu == NU && nd == ND) return kernels_##TAG##_##NU##_##ND();
const KernelSetT<double>* kernel_set64(int nu, int nd) {
  MOLE_CASE(1, 0, f64) MOLE_CASE(1, 1, f64) MOLE_CASE(2, 1, f64) MOLE_CASE(2, 2, f64)
  return nullptr;
}
const KernelSetT<float>* kernel_set32(int nu, int nd) {
  MOLE_CASE(1, 0, f32) MOLE_CASE(1, 1, f32) MOLE_CASE(2, 1, f32) MOLE_CASE(2, 2, f32)
  return nullptr;
}
const KernelSetT<df64>* kernel_set_df(int nu, int nd) {
  MOLE_CASE(1, 0, df) MOLE_CASE(1, 1, df) MOLE_CASE(2, 1, df) MOLE_CASE(2, 2, df)
  return nullptr;
}
}  // namespace mole

using namespace mole;

namespace {
thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
}  // namespace

int mole::set_error(int code, const std::string& msg) { return fail(code, msg); }

namespace {

#define CUDA_TRY(x)                                                                        \
  do {                                                                                     \
    cudaError_t e_ = (x);                                                                  \
    if (e_ != cudaSuccess) return fail(MOLE_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

}  // namespace

namespace {

template <class R>
void fill_params(const mole_system& s, SysParams<R>& sp) {
  std::memset(&sp, 0, sizeof(sp));
  sp.n_nuc = s.n_nuc;
  sp.n_basis = s.n_basis;
  // basis functions ordered by centre so each nucleus owns a contiguous range
  std::vector<int> order(s.n_basis);
  for (int b = 0; b < s.n_basis; ++b) order[b] = b;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return s.b_center[a] < s.b_center[b]; });
  int pos = 0;
  for (int I = 0; I < s.n_nuc; ++I) {
    sp.nuc_b0[I] = pos;
    while (pos < s.n_basis && s.b_center[order[pos]] == I) ++pos;
  }
  sp.nuc_b0[s.n_nuc] = pos;
  for (int I = 0; I < s.n_nuc; ++I) {
    for (int c = 0; c < 3; ++c) sp.nuc_pos[3 * I + c] = (R)s.nuc_pos[3 * I + c];
    sp.nuc_z[I] = (R)s.nuc_z[I];
    sp.en_coef[I] = (R)s.en_coef[I];
  }
  for (int j = 0; j < s.n_basis; ++j) {
    const int b = order[j];
    sp.b_kind[j] = s.b_kind[b];
    sp.b_exp[j] = s.b_exp[b];
    sp.b_zeta[j] = (R)s.theta[s.b_exp[b]];
    for (int k = 0; k < s.n_up; ++k) sp.coef[0][k][j] = (R)s.coef_up[(size_t)k * s.n_basis + b];
    for (int k = 0; k < s.n_dn; ++k) sp.coef[1][k][j] = (R)s.coef_dn[(size_t)k * s.n_basis + b];
  }
  sp.all_sto1s = 1;
  for (int j = 0; j < s.n_basis; ++j) sp.all_sto1s = sp.all_sto1s && sp.b_kind[j] == kSto1s;
  sp.n_exp = s.n_exp;
  sp.off_ee = s.n_exp;
  sp.off_en = sp.off_ee + (s.ee_on ? 1 + s.ee_npoly : 0);
  sp.off_nn = sp.off_en + (s.en_on ? 1 : 0);
  sp.P = s.P;
  sp.ee_on = s.ee_on;
  sp.ee_npoly = s.ee_npoly;
  sp.ee_kappa = (R)s.ee_kappa;
  sp.cusp_anti = (R)s.cusp_anti;
  sp.cusp_para = (R)s.cusp_para;
  sp.ee_scaled = s.ee_kappa > 0.0 ? 1 : 0;
  if (s.ee_on) {
    sp.ee_b = (R)s.theta[sp.off_ee];
    sp.ee_m2b = (R)(-2.0 * s.theta[sp.off_ee]);
    for (int p = 0; p < s.ee_npoly; ++p) sp.ee_poly[p] = (R)s.theta[sp.off_ee + 1 + p];
  }
  sp.en_on = s.en_on;
  if (s.en_on) sp.en_a = (R)s.theta[sp.off_en];
  sp.nn_on = s.nn_on;
  sp.pot_kind = s.pot_kind;
  sp.half_omega2 = (R)(0.5 * s.omega * s.omega);
  double vnn = 0.0;
  for (int I = 0; I < s.n_nuc; ++I)
    for (int K = I + 1; K < s.n_nuc; ++K) {
      double d2 = 0.0;
      for (int c = 0; c < 3; ++c) {
        const double d = s.nuc_pos[3 * I + c] - s.nuc_pos[3 * K + c];
        d2 += d * d;
      }
      vnn += (double)(s.nuc_z[I] * s.nuc_z[K]) / std::sqrt(d2);
    }
  sp.vnn = vnn;
  sp.vnn_r = (R)vnn;
  sp.nn_theta = s.d_nn_theta;
  sp.nn_tab = s.d_nn_tab;
  // the FP32 screen's mirror (basis in the kernel's centre order)
  sp.scr.rmax = 0.f;
  for (int k = 0; k < 3 * s.n_nuc; ++k) {
    sp.scr.nuc[k] = (float)s.nuc_pos[k];
    sp.scr.rmax = std::max(sp.scr.rmax, (float)std::fabs(s.nuc_pos[k]));
  }
  for (int j = 0; j < s.n_basis; ++j) {
    const int b = order[j];
    sp.scr.zeta[j] = (float)s.theta[s.b_exp[b]];
    sp.scr.coef[0][j] = s.n_up > 0 ? (float)s.coef_up[b] : 0.f;
    sp.scr.coef[1][j] = s.n_dn > 0 ? (float)s.coef_dn[b] : 0.f;
  }
  sp.scr.cusp_anti = s.ee_on ? (float)s.cusp_anti : 0.f;  // no e-e term: u = 0 in both forms
  sp.scr.cusp_para = s.ee_on ? (float)s.cusp_para : 0.f;
  sp.scr.ee_b = s.ee_on ? (float)s.theta[sp.off_ee] : 0.f;
}

// Re-derives both kernel-parameter images and, for neural systems, the
// device copy of the network parameters (a synchronous 72 KB copy) and the
// FP32 form's quintic tables (built on the context stream; the call waits for
// them and for any earlier work that may still read the old ones).
cudaError_t rebuild(mole_system& s) {
  fill_params(s, s.sp64);
  fill_params(s, s.sp32);
  fill_params(s, s.spdf);
  if (s.nn_on && s.d_nn_theta) {
    cudaStream_t st = s.ctx->stream;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    const int off = s.n_exp + (s.ee_on ? 1 + s.ee_npoly : 0) + (s.en_on ? 1 : 0);
    e = cudaMemcpy(s.d_nn_theta, s.theta.data() + off, sizeof(double) * kNnP, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    std::vector<double> z(s.n_nuc);
    for (int I = 0; I < s.n_nuc; ++I) z[I] = (double)s.nuc_z[I];
    e = launch_nn_tables(s.d_nn_theta, s.n_nuc, z.data(), s.d_nn_node, s.d_nn_tab, st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
  }
  return cudaSuccess;
}

int grid_for(int W) { return (W + kBlock - 1) / kBlock; }

constexpr const char* kNoSingleKernels =
    "no single-system kernels for this (n_up, n_dn) (compiled: 1+0, 1+1, 2+1, 2+2); run it in a mole_batch";

// Kernel selection: neural systems use the network kernels (no in-kernel SR
// sums), the others the family's kernels with or without the e-n term.
KernelSetT<double>::Vmc vmc64(const mole_system* s, int slot, int drift) {
  if (s->nn_on) return slot == 0 ? s->nk64->vmc[drift] : nullptr;
  return s->k64->vmc[slot][drift][s->en_on];
}
KernelSetT<float>::Vmc vmc32(const mole_system* s, int slot, int drift) {
  if (s->nn_on) return slot == 0 ? s->nk32->vmc[drift] : nullptr;
  return s->k32->vmc[slot][drift][s->en_on];
}
// Double-float kernels exist for the non-neural families, box and Gaussian
// moves and SR sums of at most two parameters; NULL means "run native FP64".
KernelSetT<df64>::Vmc vmc_df(const mole_system* s, int slot, int drift) {
  if (s->nn_on || !s->kdf || drift) return nullptr;
  return s->kdf->vmc[slot][0][s->en_on];
}
KernelSetT<df64>::Eval eval_df(const mole_system* s) { return s->nn_on || !s->kdf ? nullptr : s->kdf->eval[s->en_on]; }
// The packed FP64 VMC kernel (compact.cuh) covers FP64 box and Gaussian
// moves of 1s-STO systems with at most one electron per spin, the plain Pade
// e-e term (or none), no e-n Jastrow and the Coulomb potential, on ensembles
// of at least half a wave of its 224-thread CTAs; NULL otherwise.
bool one_electron_per_spin_1s(const mole_system* s, int drift) {
  if (drift || s->nn_on || s->en_on || s->n_up > 1 || s->n_dn > 1 || s->pot_kind != MOLE_POT_COULOMB) return false;
  if (s->ee_on && (s->ee_kappa > 0.0 || s->ee_npoly > 0)) return false;
  return s->sp64.all_sto1s;
}
KernelSetT<double>::Vmc vmc64_compact(const mole_system* s, int slot, int drift, int W, int n_sm) {
  if (!one_electron_per_spin_1s(s, drift) || n_sm <= 0 || W < n_sm * kCompactBlock) return nullptr;
  return compact_vmc64(s->n_up, s->n_dn, slot);
}
// The same systems on small ensembles (up to two 32-walker teams per SM),
// with one 1s function on each of at most two nuclei: the four-warp teams
// of team.cuh.
KernelSetT<double>::Vmc vmc64_team(const mole_system* s, int slot, int drift, int W, int n_sm) {
  if (!one_electron_per_spin_1s(s, drift) || n_sm <= 0 || W > 2 * 32 * n_sm) return nullptr;
  const SysParams<double>& sp = s->sp64;
  if (sp.n_nuc < 1 || sp.n_nuc > 2 || sp.n_basis != sp.n_nuc) return nullptr;
  for (int I = 0; I <= sp.n_nuc; ++I)
    if (sp.nuc_b0[I] != I) return nullptr;
  return team_vmc64(s->n_up, s->n_dn, slot, sp.n_nuc);
}
KernelSetT<double>::Eval eval64(const mole_system* s) { return s->nn_on ? s->nk64->eval : s->k64->eval[s->en_on]; }
KernelSetT<float>::Eval eval32(const mole_system* s) { return s->nn_on ? s->nk32->eval : s->k32->eval[s->en_on]; }
KernelSetT<double>::Dmc dmc64(const mole_system* s) { return s->nn_on ? s->nk64->dmc : s->k64->dmc[s->en_on]; }
KernelSetT<float>::Dmc dmc32(const mole_system* s) { return s->nn_on ? s->nk32->dmc : s->k32->dmc[s->en_on]; }

int check_status(mole_ctx* ctx) {
  int st = 0;
  CUDA_TRY(cudaMemcpyAsync(&st, ctx->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (st & 2) return fail(MOLE_ERR_LINALG, "singular Slater matrix encountered");
  if (st & 1) return fail(MOLE_ERR_FUNC, "non-finite local energy encountered");
  return MOLE_OK;
}

struct Timer {
  mole_ctx* ctx;
  int kind;
  Timer(mole_ctx* c, int k) : ctx(c), kind(k) {
    if (ctx->timing) cudaEventRecord(ctx->ev0, ctx->stream);
  }
  void stop() {
    if (!ctx->timing) return;
    cudaEventRecord(ctx->ev1, ctx->stream);
    cudaEventSynchronize(ctx->ev1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->kernel_ms[kind] += ms;
    ctx->kernel_launches[kind] += 1;
  }
};

}  // namespace

extern "C" {

int32_t mole_abi_version(void) { return MOLE_ABI_VERSION; }
const char* mole_last_error_string(void) { return g_err.c_str(); }

int mole_ctx_create(int32_t device, mole_ctx** out) {
  if (!out) return fail(MOLE_ERR_INVALID_ARG, "out is NULL");
  int n = 0;
  CUDA_TRY(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return fail(MOLE_ERR_INVALID_ARG, "no such CUDA device");
  CUDA_TRY(cudaSetDevice(device));
  mole_ctx* c = new mole_ctx();
  c->device = device;
  cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&c->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  cudaError_t e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  if (e == cudaSuccess) e = c->status.reserve(1);
  if (e != cudaSuccess) {
    delete c;
    return fail(MOLE_ERR_CUDA, std::string("context setup: ") + cudaGetErrorString(e));
  }
  c->stream = c->own;
  *out = c;
  return MOLE_OK;
}

// Handles are reference counted: a system keeps its context alive and a
// walker set its system, so destroying them in any order is safe; the
// memory goes when the last dependent handle is destroyed.
static void release_ctx(mole_ctx* c) {
  if (--c->refs > 0) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->own);
  c->partials.release();
  c->tb_partials.release();
  c->reduced.release();
  c->scratch.release();
  c->status.release();
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->own) cudaStreamDestroy(c->own);
  cudaGetLastError();  // teardown errors are not reported to later calls
  delete c;
}

static void release_sys(mole_system* s) {
  if (--s->refs > 0) return;
  if (s->d_nn_theta) {
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    for (void* p : {(void*)s->d_nn_theta, (void*)s->d_nn_tab, (void*)s->d_nn_node})
      if (p) cudaFree(p);
    cudaGetLastError();
  }
  mole_ctx* c = s->ctx;
  delete s;
  release_ctx(c);
}

}  // extern "C"

void mole::system_retain(mole_system* s) { s->refs += 1; }
void mole::system_release(mole_system* s) { release_sys(s); }

extern "C" {

int mole_ctx_destroy(mole_ctx* c) {
  if (!c || c->closed) return MOLE_OK;
  c->closed = true;
  if (c->stream != c->own) c->stream = c->own;
  release_ctx(c);
  return MOLE_OK;
}

int mole_ctx_set_stream(mole_ctx* c, void* s) {
  if (!c) return fail(MOLE_ERR_INVALID_ARG, "ctx is NULL");
  c->stream = s ? (cudaStream_t)s : c->own;
  return MOLE_OK;
}

int mole_sync(mole_ctx* c) {
  if (!c) return fail(MOLE_ERR_INVALID_ARG, "ctx is NULL");
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return MOLE_OK;
}

int mole_ctx_enable_timing(mole_ctx* c, int32_t on) {
  if (!c) return fail(MOLE_ERR_INVALID_ARG, "ctx is NULL");
  c->timing = on != 0;
  for (int k = 0; k < kTimeSlots; ++k) {
    c->kernel_ms[k] = 0;
    c->kernel_launches[k] = 0;
  }
  return MOLE_OK;
}

int mole_ctx_kernel_time(mole_ctx* c, int32_t kernel, double* total_ms, int64_t* launches) {
  if (!c || kernel < 0 || kernel >= kTimeSlots) return fail(MOLE_ERR_INVALID_ARG, "bad ctx or kernel id");
  if (total_ms) *total_ms = c->kernel_ms[kernel];
  if (launches) *launches = c->kernel_launches[kernel];
  return MOLE_OK;
}

int mole_math_check(mole_ctx* c, int32_t fn, const double* x, int64_t n, double* y) {
  cudaGetLastError();
  if (!c || !x || !y || n < 0 || fn < 0 || fn > 9) return fail(MOLE_ERR_INVALID_ARG, "bad argument");
  CUDA_TRY(c->scratch.reserve((size_t)2 * std::max<int64_t>(n, 1)));
  double* dx = c->scratch.p;
  double* dy = dx + n;
  CUDA_TRY(cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(launch_math_check(fn, dx, n, dy, c->stream));
  CUDA_TRY(cudaMemcpyAsync(y, dy, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return MOLE_OK;
}

int mole_ctx_df64_reruns(mole_ctx* c, int64_t* reruns) {
  if (!c || !reruns) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  *reruns = c->df64_reruns;
  return MOLE_OK;
}

int mole_ctx_device_info(mole_ctx* c, int32_t* n_sm, int32_t* cc_major, int32_t* cc_minor) {
  if (!c) return fail(MOLE_ERR_INVALID_ARG, "ctx is NULL");
  int ma = 0, mi = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&ma, cudaDevAttrComputeCapabilityMajor, c->device));
  CUDA_TRY(cudaDeviceGetAttribute(&mi, cudaDevAttrComputeCapabilityMinor, c->device));
  if (n_sm) *n_sm = c->n_sm;
  if (cc_major) *cc_major = ma;
  if (cc_minor) *cc_minor = mi;
  return MOLE_OK;
}

int mole_probe_peaks(mole_ctx* c, double* fp64, double* fp32) {
  cudaGetLastError();  // report only errors raised by this call
  if (!c) return fail(MOLE_ERR_INVALID_ARG, "ctx is NULL");
  CUDA_TRY(cudaSetDevice(c->device));
  const int blocks = c->n_sm * 8, threads = 256;
  CUDA_TRY(c->scratch.reserve((size_t)blocks * threads));
  cudaEvent_t a, b;
  CUDA_TRY(cudaEventCreate(&a));
  CUDA_TRY(cudaEventCreate(&b));
  double res[2] = {0, 0};
  for (int k = 0; k < 2; ++k) {
    const int iters = k == 0 ? 256 : 4096;
    for (int rep = 0; rep < 3; ++rep) {
      CUDA_TRY(cudaEventRecord(a, c->stream));
      if (k == 0) CUDA_TRY(launch_fma_probe64(c->scratch.p, blocks, threads, iters, c->stream));
      else CUDA_TRY(launch_fma_probe32((float*)c->scratch.p, blocks, threads, iters, c->stream));
      CUDA_TRY(cudaEventRecord(b, c->stream));
      CUDA_TRY(cudaEventSynchronize(b));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, b);
      const double flops = 2.0 * 64.0 * iters * (double)blocks * threads;
      res[k] = std::max(res[k], flops / (ms * 1e-3) / 1e9);
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (fp64) *fp64 = res[0];
  if (fp32) *fp32 = res[1];
  return MOLE_OK;
}

int mole_system_create(mole_ctx* ctx, const mole_system_desc* d, const double* theta, int32_t n_theta,
                       mole_system** out) {
  if (!ctx || !d || !out) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (d->n_nuclei < 1 || d->n_nuclei > MOLE_MAX_NUCLEI) return fail(MOLE_ERR_SHAPE, "n_nuclei out of range");
  if (d->n_up < 1 || d->n_up > MOLE_MAX_SPIN || d->n_dn < 0 || d->n_dn > d->n_up)
    return fail(MOLE_ERR_SHAPE, "need 1 <= n_up <= 5 and 0 <= n_dn <= n_up");
  if (d->n_basis < 1 || d->n_basis > MOLE_MAX_BASIS) return fail(MOLE_ERR_SHAPE, "n_basis out of range");
  if (d->n_exp < 1 || d->n_exp > MOLE_MAX_BASIS) return fail(MOLE_ERR_SHAPE, "n_exp out of range");
  if (d->ee_npoly < 0 || d->ee_npoly > MOLE_MAX_POLY) return fail(MOLE_ERR_SHAPE, "ee_npoly out of range");
  if (!d->nuc_pos || !d->nuc_charge || !d->basis_center || !d->basis_kind || !d->basis_exp || !d->coef_up ||
      (d->n_dn > 0 && !d->coef_dn) || (d->en_on && !d->en_coef))
    return fail(MOLE_ERR_INVALID_ARG, "NULL descriptor array");
  if (d->nn_on && !(d->n_up == 2 && d->n_dn == 2))
    return fail(MOLE_ERR_UNSUPPORTED, "neural-Jastrow kernels are compiled for 2 up + 2 down electrons");
  auto s = new mole_system();
  s->ctx = ctx;
  s->n_nuc = d->n_nuclei;
  s->n_up = d->n_up;
  s->n_dn = d->n_dn;
  s->n_basis = d->n_basis;
  s->n_exp = d->n_exp;
  s->nuc_pos.assign(d->nuc_pos, d->nuc_pos + 3 * d->n_nuclei);
  s->nuc_z.assign(d->nuc_charge, d->nuc_charge + d->n_nuclei);
  s->b_center.assign(d->basis_center, d->basis_center + d->n_basis);
  s->b_kind.assign(d->basis_kind, d->basis_kind + d->n_basis);
  s->b_exp.assign(d->basis_exp, d->basis_exp + d->n_basis);
  s->coef_up.assign(d->coef_up, d->coef_up + (size_t)d->n_up * d->n_basis);
  if (d->n_dn > 0) s->coef_dn.assign(d->coef_dn, d->coef_dn + (size_t)d->n_dn * d->n_basis);
  s->en_coef.assign(d->n_nuclei, 0.0);
  if (d->en_on) s->en_coef.assign(d->en_coef, d->en_coef + d->n_nuclei);
  for (int b = 0; b < d->n_basis; ++b) {
    if (s->b_center[b] < 0 || s->b_center[b] >= d->n_nuclei || s->b_exp[b] < 0 || s->b_exp[b] >= d->n_exp ||
        s->b_kind[b] < MOLE_STO_1S || s->b_kind[b] > MOLE_GTO_1S) {
      delete s;
      return fail(MOLE_ERR_SHAPE, "basis function index out of range");
    }
  }
  s->ee_on = d->ee_on != 0;
  s->ee_npoly = d->ee_on ? d->ee_npoly : 0;
  s->ee_kappa = d->ee_kappa;
  s->cusp_anti = d->cusp_anti;
  s->cusp_para = d->cusp_para;
  s->en_on = d->en_on != 0;
  s->nn_on = d->nn_on != 0;
  s->pot_kind = d->pot_kind;
  s->omega = d->omega;
  s->P = s->n_exp + (s->ee_on ? 1 + s->ee_npoly : 0) + (s->en_on ? 1 : 0) + (s->nn_on ? kNnP : 0);
  if (!theta || n_theta != s->P) {
    const int P = s->P;
    delete s;
    return fail(MOLE_ERR_SHAPE, "theta must hold " + std::to_string(P) + " parameters");
  }
  s->theta.assign(theta, theta + n_theta);
  // spin blocks without fixed-size kernels (up to 5 + 5) run in batches only
  s->k64 = kernel_set64(s->n_up, s->n_dn);
  s->k32 = kernel_set32(s->n_up, s->n_dn);
  s->kdf = kernel_set_df(s->n_up, s->n_dn);
  if (s->nn_on) {
    s->nk64 = nn_kernels_f64_2_2();
    s->nk32 = nn_kernels_f32_2_2();
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_nn_theta, sizeof(double) * kNnP);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_nn_tab, sizeof(float) * nn_tab_floats(s->n_nuc));
    if (e == cudaSuccess)
      e = cudaMalloc(&s->d_nn_node, sizeof(double) * 3 * (size_t)(2 + s->n_nuc) * kNnTabNodes);
    if (e != cudaSuccess) {
      for (void* p : {(void*)s->d_nn_theta, (void*)s->d_nn_tab, (void*)s->d_nn_node})
        if (p) cudaFree(p);
      delete s;
      return fail(MOLE_ERR_CUDA, std::string("network parameters: ") + cudaGetErrorString(e));
    }
  }
  if (rebuild(*s) != cudaSuccess) {
    for (void* p : {(void*)s->d_nn_theta, (void*)s->d_nn_tab, (void*)s->d_nn_node})
      if (p) cudaFree(p);
    delete s;
    return fail(MOLE_ERR_CUDA, "copying the network parameters or building their tables failed");
  }
  ctx->refs += 1;
  *out = s;
  return MOLE_OK;
}

int mole_system_destroy(mole_system* s) {
  if (!s || s->closed) return MOLE_OK;
  s->closed = true;
  release_sys(s);
  return MOLE_OK;
}

int mole_num_params(const mole_system* s, int32_t* out) {
  if (!s || !out) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  *out = s->P;
  return MOLE_OK;
}

int mole_num_electrons(const mole_system* s, int32_t* out) {
  if (!s || !out) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  *out = s->n_up + s->n_dn;
  return MOLE_OK;
}

int mole_params_get(const mole_system* s, double* theta, int32_t n) {
  if (!s || !theta) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (n != s->P) return fail(MOLE_ERR_SHAPE, "parameter count mismatch");
  std::memcpy(theta, s->theta.data(), sizeof(double) * n);
  return MOLE_OK;
}

int mole_params_set(mole_system* s, const double* theta, int32_t n) {
  if (!s || !theta) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (n != s->P) return fail(MOLE_ERR_SHAPE, "parameter count mismatch");
  s->theta.assign(theta, theta + n);
  s->version += 1;
  CUDA_TRY(rebuild(*s));
  return MOLE_OK;
}

int mole_walkers_create(mole_system* s, int32_t W, uint64_t seed, mole_walkers** out) {
  if (!s || !out) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (W < 1) return fail(MOLE_ERR_SHAPE, "need at least one walker");
  CUDA_TRY(cudaSetDevice(s->ctx->device));
  cudaGetLastError();  // a launch below reports its own error, not an earlier one
  auto w = new mole_walkers();
  w->sys = s;
  w->W = W;
  w->seed = seed;
  const size_t n = (size_t)W * 3 * (s->n_up + s->n_dn);
  cudaError_t e = cudaMalloc(&w->pos, n * sizeof(double));
  if (e != cudaSuccess) {
    delete w;
    return fail(MOLE_ERR_CUDA, std::string("walker positions: ") + cudaGetErrorString(e));
  }
  s->refs += 1;
  const int rc = mole_walkers_init(w, MOLE_INIT_NORMAL, 1.0);
  if (rc != MOLE_OK) {
    mole_walkers_destroy(w);
    return rc;
  }
  *out = w;
  return MOLE_OK;
}

static void free_dmc(mole_walkers* w) {
  for (double** p : {&w->pos2, &w->eloc, &w->eloc2, &w->weight, &w->cum, &w->btot, &w->e_ref, &w->energies}) {
    if (*p) cudaFree(*p);
    *p = nullptr;
  }
  if (w->dstep) cudaFree(w->dstep);
  if (w->comb) cudaFree(w->comb);
  w->dstep = nullptr;
  w->comb = nullptr;
  w->energies_n = 0;
  w->eloc_valid = false;
  if (w->srl) {
    SrLargeState* t = w->srl;
    for (void* p : {(void*)t->O, (void*)t->center, (void*)t->Ob, (void*)t->partial, (void*)t->S, (void*)t->E,
                    (void*)t->x, (void*)t->sumO, (void*)t->sumEO, (void*)t->work, (void*)t->status})
      if (p) cudaFree(p);
    delete t;
    w->srl = nullptr;
  }
  delete w->srl_map;
  w->srl_map = nullptr;
  if (w->srl_eval) cudaFree(w->srl_eval);
  w->srl_eval = nullptr;
}

int mole_walkers_destroy(mole_walkers* w) {
  if (!w) return MOLE_OK;
  mole_system* s = w->sys;
  cudaSetDevice(s->ctx->device);
  cudaStreamSynchronize(s->ctx->stream);
  if (w->pos) cudaFree(w->pos);
  free_dmc(w);
  cudaGetLastError();  // teardown errors are not reported to later calls
  delete w;
  release_sys(s);
  return MOLE_OK;
}

int mole_walkers_count(const mole_walkers* w, int32_t* out) {
  if (!w || !out) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  *out = w->W;
  return MOLE_OK;
}

int mole_walkers_init(mole_walkers* w, int32_t kind, double width) {
  cudaGetLastError();  // report only errors raised by this call
  if (!w) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (kind != MOLE_INIT_NORMAL && kind != MOLE_INIT_UNIFORM) return fail(MOLE_ERR_INVALID_ARG, "bad init kind");
  mole_ctx* c = w->sys->ctx;
  CUDA_TRY(launch_init_positions(w->pos, w->W, w->sys->n_up + w->sys->n_dn, w->seed, kind, width, c->stream));
  w->eloc_valid = false;
  return MOLE_OK;
}

int mole_walkers_set_positions(mole_walkers* w, const double* pos, int64_t n) {
  cudaGetLastError();  // report only errors raised by this call
  if (!w || !pos) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  const int NC = 3 * (w->sys->n_up + w->sys->n_dn);
  if (n != (int64_t)w->W * NC) return fail(MOLE_ERR_SHAPE, "positions must hold W * N * 3 values");
  mole_ctx* c = w->sys->ctx;
  CUDA_TRY(c->scratch.reserve((size_t)n));
  CUDA_TRY(cudaMemcpyAsync(c->scratch.p, pos, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(launch_aos_to_soa(c->scratch.p, w->pos, w->W, NC, c->stream));
  w->eloc_valid = false;
  return MOLE_OK;
}

int mole_walkers_get_positions(mole_walkers* w, double* pos, int64_t n) {
  cudaGetLastError();  // report only errors raised by this call
  if (!w || !pos) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  const int NC = 3 * (w->sys->n_up + w->sys->n_dn);
  if (n != (int64_t)w->W * NC) return fail(MOLE_ERR_SHAPE, "positions must hold W * N * 3 values");
  mole_ctx* c = w->sys->ctx;
  CUDA_TRY(c->scratch.reserve((size_t)n));
  CUDA_TRY(launch_soa_to_aos(w->pos, c->scratch.p, w->W, NC, c->stream));
  CUDA_TRY(cudaMemcpyAsync(pos, c->scratch.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return MOLE_OK;
}

int mole_walkers_get_step(const mole_walkers* w, uint64_t* step) {
  if (!w || !step) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  *step = w->step;
  return MOLE_OK;
}

int mole_walkers_set_step(mole_walkers* w, uint64_t step) {
  if (!w) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  w->step = step;
  return MOLE_OK;
}

int mole_eval(mole_walkers* w, int32_t precision, double* lnpsi, double* sign, double* grad, double* lap,
              double* eloc, double* O) {
  cudaGetLastError();  // report only errors raised by this call
  if (!w) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  mole_system* s = w->sys;
  mole_ctx* c = s->ctx;
  if (!s->nn_on && (!s->k64 || !s->k32)) return fail(MOLE_ERR_UNSUPPORTED, kNoSingleKernels);
  const int W = w->W, N = s->n_up + s->n_dn, P = s->P;
  const int nwalker_par = s->nn_on ? P - kNnP : P;
  if (nwalker_par > 8 && O) return fail(MOLE_ERR_UNSUPPORTED, "O_k output supports at most 8 orbital/Pade parameters");
  if (s->nn_on && O && (N * (N - 1) / 2 > 8 || N * s->n_nuc > 8))
    return fail(MOLE_ERR_UNSUPPORTED, "network O_k supports at most 8 pairs per network");
  const size_t per = 5 + 3 * (size_t)N + P;
  CUDA_TRY(c->reduced.reserve(per * W));
  double* base = c->reduced.p;
  EvalArgs a;
  a.pos = w->pos;
  a.W = W;
  a.lnpsi = base;
  a.sign = base + W;
  a.lap = base + 2 * (size_t)W;
  a.eloc = base + 3 * (size_t)W;
  a.grad = base + 4 * (size_t)W;
  a.O = a.grad + 3 * (size_t)N * W;
  a.ldO = P;
  CUDA_TRY(cudaMemsetAsync(c->status.p, 0, sizeof(int), c->stream));
  a.status = c->status.p;
  Timer tm(c, 2);
  auto edf = precision == MOLE_PREC_DF64 ? eval_df(s) : nullptr;
  if (precision == MOLE_PREC_MIXED) CUDA_TRY(eval32(s)(s->sp32, a, grid_for(W), c->stream));
  else if (edf) {
    CUDA_TRY(edf(s->spdf, a, grid_for(W), c->stream));
    int st = 0;
    CUDA_TRY(cudaMemcpyAsync(&st, c->status.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (st & 8) {  // a walker outside the double-float range: evaluate all of them in FP64
      ++c->df64_reruns;
      CUDA_TRY(cudaMemsetAsync(c->status.p, 0, sizeof(int), c->stream));
      CUDA_TRY(eval64(s)(s->sp64, a, grid_for(W), c->stream));
    }
  } else CUDA_TRY(eval64(s)(s->sp64, a, grid_for(W), c->stream));
  if (s->nn_on && O)  // the network's O_k (FP32 arithmetic) after the orbital/Pade ones
    CUDA_TRY(launch_nn_ogen64(s->sp32, w->pos, W, s->n_up, N, a.O, P, nwalker_par, std::min(W, 3 * c->n_sm),
                              c->stream));
  tm.stop();
  auto copy = [&](double* dst, const double* src, size_t n) -> int {
    if (dst) CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    return MOLE_OK;
  };
  int rc;
  if ((rc = copy(lnpsi, a.lnpsi, W)) || (rc = copy(sign, a.sign, W)) || (rc = copy(lap, a.lap, W)) ||
      (rc = copy(eloc, a.eloc, W)) || (rc = copy(grad, a.grad, (size_t)3 * N * W)) ||
      (rc = copy(O, a.O, (size_t)P * W)))
    return rc;
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  const int st = check_status(c);
  return st == MOLE_ERR_FUNC ? MOLE_OK : st;  // per-walker values are returned as computed
}

int mole_vmc_run(mole_walkers* w, const mole_vmc_opts* o, double* moments, double* time_blocks, double* sum_O,
                 double* sum_EO, double* sum_OO) {
  cudaGetLastError();  // report only errors raised by this call
  if (!w || !o || !moments) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  mole_system* s = w->sys;
  mole_ctx* c = s->ctx;
  if (!s->nn_on && (!s->k64 || !s->k32)) return fail(MOLE_ERR_UNSUPPORTED, kNoSingleKernels);
  if (o->block_size < 1 || o->n_steps < 0 || o->n_eq < 0 || o->n_steps % o->block_size != 0)
    return fail(MOLE_ERR_SHAPE, "n_steps must be a non-negative multiple of block_size >= 1");
  if (o->move < MOLE_MOVE_BOX || o->move > MOLE_MOVE_DIFFUSE || !(o->step > 0.0))
    return fail(MOLE_ERR_INVALID_ARG, "bad move kind or step");
  const int P = s->P;
  int slot = 0;
  if (o->sr) {
    if (!sum_O || !sum_EO || !sum_OO) return fail(MOLE_ERR_DATA_ACCESS, "SR outputs are NULL");
    const bool mixed = o->precision == MOLE_PREC_MIXED;
    // the two-parameter kernels cache one orbital-exponent derivative
    if (P <= 2 && s->n_exp <= 1 && (mixed ? s->k32->vmc[1][0][0] != nullptr : s->k64->vmc[1][0][0] != nullptr))
      slot = 1;
    else if (P <= 8) slot = 2;
    else return fail(MOLE_ERR_UNSUPPORTED, "SR accumulation supports at most 8 parameters on this path");
  }
  const int PM = kPmWidth[slot];
  const int drift = o->move == MOLE_MOVE_DIFFUSE ? 1 : 0;
  const bool mixed = o->precision == MOLE_PREC_MIXED;
  auto f64 = vmc64(s, slot, drift);
  auto f32 = vmc32(s, slot, drift);
  auto fdf = o->precision == MOLE_PREC_DF64 ? vmc_df(s, slot, drift) : nullptr;
  if (mixed ? !f32 : !f64) return fail(MOLE_ERR_UNSUPPORTED, "SR kernel not compiled for this family and precision");
  int wpc = kBlock;
  const int W = w->W;
  auto fcp = (!mixed && !fdf) ? vmc64_compact(s, slot, drift, W, c->n_sm) : nullptr;
  auto ftm = (!mixed && !fdf && !fcp) ? vmc64_team(s, slot, drift, W, c->n_sm) : nullptr;
  if (ftm) wpc = 32;
  const int grid = fcp ? compact_grid(W, c->n_sm, &wpc)
                       : (ftm ? (W + 31) / 32 : vmc_grid(W, s->n_up, s->n_dn, c->n_sm, &wpc));
  const int NA = n_acc(PM);
  const int n_tb = o->n_steps / o->block_size;
  CUDA_TRY(c->partials.reserve((size_t)grid * NA));
  CUDA_TRY(c->tb_partials.reserve((size_t)grid * std::max(n_tb, 1)));
  CUDA_TRY(c->reduced.reserve((size_t)NA + std::max(n_tb, 1)));
  CUDA_TRY(cudaMemsetAsync(c->status.p, 0, sizeof(int), c->stream));
  VmcArgs a;
  a.pos = w->pos;
  a.W = W;
  a.move = o->move;
  a.step = o->step;
  a.n_eq = o->n_eq;
  a.n_steps = o->n_steps;
  a.block_size = o->block_size;
  a.refresh = o->refresh;
  a.seed = w->seed;
  a.step0 = (uint32_t)w->step;
  a.wpc = wpc;
  a.partials = c->partials.p;
  a.tb_partials = c->tb_partials.p;
  a.status = c->status.p;
  const size_t pos_n = (size_t)3 * (s->n_up + s->n_dn) * W;
  if (fdf) {
    CUDA_TRY(c->pos_backup.reserve(pos_n));
    CUDA_TRY(cudaMemcpyAsync(c->pos_backup.p, w->pos, sizeof(double) * pos_n, cudaMemcpyDeviceToDevice, c->stream));
  }
  Timer tm(c, 0);
  if (mixed) CUDA_TRY(f32(s->sp32, a, grid, c->stream));
  else if (fdf) CUDA_TRY(fdf(s->spdf, a, grid, c->stream));
  else CUDA_TRY((fcp ? fcp : (ftm ? ftm : f64))(s->sp64, a, grid, c->stream));
  tm.stop();
  if (fdf) {
    int st = 0;
    CUDA_TRY(cudaMemcpyAsync(&st, c->status.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (st & 8) {
      // a value left FP32's exponent range: the same sweeps again in native
      // FP64 from the same positions and random streams
      ++c->df64_reruns;
      CUDA_TRY(cudaMemcpyAsync(w->pos, c->pos_backup.p, sizeof(double) * pos_n, cudaMemcpyDeviceToDevice, c->stream));
      CUDA_TRY(cudaMemsetAsync(c->status.p, 0, sizeof(int), c->stream));
      Timer tm2(c, 0);
      CUDA_TRY(f64(s->sp64, a, grid, c->stream));
      tm2.stop();
    }
  }
  CUDA_TRY(launch_reduce_columns(c->partials.p, grid, NA, c->reduced.p, c->stream));
  if (n_tb > 0) CUDA_TRY(launch_reduce_columns(c->tb_partials.p, grid, n_tb, c->reduced.p + NA, c->stream));
  std::vector<double> h((size_t)NA + std::max(n_tb, 0));
  CUDA_TRY(cudaMemcpyAsync(h.data(), c->reduced.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  w->step += (uint64_t)(o->n_eq + o->n_steps);
  w->eloc_valid = false;
  for (int k = 0; k < MOLE_NMOM; ++k) moments[k] = h[k];
  if (time_blocks)
    for (int k = 0; k < n_tb; ++k) time_blocks[k] = h[NA + k];
  if (o->sr) {
    for (int p = 0; p < P; ++p) {
      sum_O[p] = h[kNMom + p];
      sum_EO[p] = h[kNMom + PM + p];
    }
    int q = kNMom + 2 * PM;
    for (int p = 0; p < PM; ++p)
      for (int r = p; r < PM; ++r, ++q)
        if (p < P && r < P) sum_OO[p * P + r] = sum_OO[r * P + p] = h[q];
  }
  return check_status(c);
}

}  // extern "C"

// ------------------------------------------------- allocation-free VMC sweep
//
// Scratch of mole_vmc_run_noalloc: the per-CTA partial sums, the per-CTA
// time-block sums, the reduced sums and the status word. It is a fixed
// 2 MiB array that every GPU loading this library holds until the process
// exits. In host code g_noalloc_scratch is only a stand-in for the symbol; the
// device address comes from cudaGetSymbolAddress, once per device.
static constexpr size_t kNoAllocScratchDoubles = (size_t)1 << 18;  // 2 MiB
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_addr[256] = {nullptr};

// Restores the caller's current device when the entry point returns.
struct DeviceRestore {
  int prev = -1;
  DeviceRestore() {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
  }
  ~DeviceRestore() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// Device address of the scratch array on `device` (which must be current),
// looked up once per device: it stays valid while the device's primary
// context lives (for the whole process unless the caller resets the device).
cudaError_t noalloc_scratch(int device, double** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (device < 0 || device >= 256) return cudaErrorInvalidDevice;
  if (!g_noalloc_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[device] = (double*)p;
  }
  *out = g_noalloc_addr[device];
  return cudaSuccess;
}
}  // namespace

extern "C" {

int mole_vmc_run_noalloc(const mole_system* s, double* d_pos, int32_t W, uint64_t seed, uint64_t step0,
                         const mole_vmc_opts* o, double* d_moments, double* d_time_blocks, double* d_sr,
                         void* stream) {
  if (!s || !d_pos || !o || !d_moments) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (!s->nn_on && (!s->k64 || !s->k32)) return fail(MOLE_ERR_UNSUPPORTED, kNoSingleKernels);
  if (W < 1) return fail(MOLE_ERR_SHAPE, "need at least one walker");
  if (o->block_size < 1 || o->n_steps < 0 || o->n_eq < 0 || o->n_steps % o->block_size != 0)
    return fail(MOLE_ERR_SHAPE, "n_steps must be a non-negative multiple of block_size >= 1");
  if (o->move < MOLE_MOVE_BOX || o->move > MOLE_MOVE_DIFFUSE || !(o->step > 0.0))
    return fail(MOLE_ERR_INVALID_ARG, "bad move kind or step");
  const bool mixed = o->precision == MOLE_PREC_MIXED;
  const int P = s->P;
  int slot = 0;
  if (o->sr) {
    if (!d_sr) return fail(MOLE_ERR_DATA_ACCESS, "SR output is NULL");
    if (P <= 2 && s->n_exp <= 1 && (mixed ? s->k32->vmc[1][0][0] != nullptr : s->k64->vmc[1][0][0] != nullptr))
      slot = 1;
    else if (P <= 8) slot = 2;
    else return fail(MOLE_ERR_UNSUPPORTED, "SR accumulation supports at most 8 parameters on this path");
  }
  const int PM = kPmWidth[slot];
  const int drift = o->move == MOLE_MOVE_DIFFUSE ? 1 : 0;
  auto f64 = vmc64(s, slot, drift);
  auto f32 = vmc32(s, slot, drift);
  if (mixed ? !f32 : !f64) return fail(MOLE_ERR_UNSUPPORTED, "kernel not compiled for this family and precision");
  int wpc = kBlock;
  const int grid = vmc_grid(W, s->n_up, s->n_dn, s->ctx->n_sm, &wpc), NA = n_acc(PM), n_tb = o->n_steps / o->block_size;
  // scratch layout: partials [grid][NA] | time-block partials [grid][n_tb] | reduced [NA] | status
  const size_t need = (size_t)grid * NA + (size_t)grid * n_tb + NA + 1;
  if (need > kNoAllocScratchDoubles)
    return fail(MOLE_ERR_SHAPE, "walkers x (accumulators + time blocks) needs " + std::to_string(need * 8) +
                                    " bytes of scratch; the allocation-free entry point has " +
                                    std::to_string(kNoAllocScratchDoubles * 8));
  if (n_tb > 0 && !d_time_blocks) return fail(MOLE_ERR_DATA_ACCESS, "time_blocks output is NULL");
  DeviceRestore restore;  // the caller's current device is left as it was
  CUDA_TRY(cudaSetDevice(s->ctx->device));
  cudaGetLastError();  // report only errors raised by this call
  cudaStream_t st = (cudaStream_t)stream;
  int st_dev = -1;
  CUDA_TRY(cudaStreamGetDevice(st, &st_dev));
  if (st_dev != s->ctx->device)
    return fail(MOLE_ERR_INVALID_ARG, "the stream belongs to device " + std::to_string(st_dev) +
                                          ", the system to device " + std::to_string(s->ctx->device));
  double* scratch = nullptr;
  CUDA_TRY(noalloc_scratch(s->ctx->device, &scratch));
  double* partials = scratch;
  double* tb_partials = partials + (size_t)grid * NA;
  double* reduced = tb_partials + (size_t)grid * n_tb;
  int* status = (int*)(reduced + NA);
  CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
  VmcArgs a;
  a.pos = d_pos;
  a.W = W;
  a.move = o->move;
  a.step = o->step;
  a.n_eq = o->n_eq;
  a.n_steps = o->n_steps;
  a.block_size = o->block_size;
  a.refresh = o->refresh;
  a.seed = seed;
  a.step0 = (uint32_t)step0;
  a.wpc = wpc;
  a.partials = partials;
  a.tb_partials = tb_partials;
  a.status = status;
  if (mixed) CUDA_TRY(f32(s->sp32, a, grid, st));
  else CUDA_TRY(f64(s->sp64, a, grid, st));
  CUDA_TRY(launch_reduce_columns(partials, grid, NA, reduced, st));
  if (n_tb > 0) CUDA_TRY(launch_reduce_columns(tb_partials, grid, n_tb, d_time_blocks, st));
  CUDA_TRY(launch_unpack_vmc_sums(reduced, PM, P, d_moments, o->sr ? d_sr : nullptr, st));
  int h_status = 0;
  CUDA_TRY(cudaMemcpyAsync(&h_status, status, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (h_status & 2) return fail(MOLE_ERR_LINALG, "singular Slater matrix encountered");
  if (h_status & 1) return fail(MOLE_ERR_FUNC, "non-finite local energy encountered");
  return MOLE_OK;
}

int mole_sr_collect_begin(mole_walkers* w) {
  if (!w) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  cudaGetLastError();  // report only errors raised by this call
  mole_system* s = w->sys;
  mole_ctx* c = s->ctx;
  CUDA_TRY(cudaSetDevice(c->device));
  const int W = w->W, P = s->P;
  if (!w->srl) {
    auto t = new SrLargeState();
    std::memset(t, 0, sizeof(*t));
    t->P = P;
    t->P_pad = (P + kSBN - 1) / kSBN * kSBN;
    const size_t sample_bytes = sizeof(__nv_bfloat16) * (size_t)W * t->P_pad;
    const int n_samples = (int)std::max<size_t>(1, std::min<size_t>(kObSamples, kObBudget / sample_bytes));
    t->K_cap = (n_samples * W + kSBK - 1) / kSBK * kSBK;
    t->n_cta = sr_sample_ctas(W, c->n_sm);
    w->srl = t;  // freed by free_dmc on failure below
    if (sr_sample_smem(P) > (size_t)c->smem_optin)
      return fail(MOLE_ERR_UNSUPPORTED, "too many parameters for the SR sample kernel's shared-memory sums");
    CUDA_TRY(cudaMalloc(&t->O, sizeof(float) * (size_t)std::min(W, kCenterRows) * P));
    CUDA_TRY(cudaMalloc(&t->center, sizeof(float) * P));
    CUDA_TRY(cudaMalloc(&t->Ob, sizeof(__nv_bfloat16) * (size_t)t->K_cap * t->P_pad));
    // zero padding columns (never written); rows past a launch's last sample are zeroed before it
    CUDA_TRY(cudaMemset(t->Ob, 0, sizeof(__nv_bfloat16) * (size_t)t->K_cap * t->P_pad));
    CUDA_TRY(cudaMalloc(&t->partial, sizeof(float) * 2 * (size_t)t->n_cta * P));
    CUDA_TRY(cudaMalloc(&t->S, sizeof(double) * (size_t)t->P_pad * t->P_pad));
    CUDA_TRY(cudaMalloc(&t->E, sizeof(double) * W));
    CUDA_TRY(cudaMalloc(&t->x, sizeof(double) * P));
    CUDA_TRY(cudaMalloc(&t->sumO, sizeof(double) * P));
    CUDA_TRY(cudaMalloc(&t->sumEO, sizeof(double) * P));
    CUDA_TRY(cudaMalloc(&t->work, sizeof(double) * (6 * (size_t)P + 8)));
    CUDA_TRY(cudaMalloc(&t->status, sizeof(int)));
    CUDA_TRY(cudaMalloc(&w->srl_eval, sizeof(double) * (size_t)W * (3 + 3 * (s->n_up + s->n_dn) + 8)));
    w->srl_map = new CUtensorMap();
    CUDA_TRY(encode_ob_tensor_map(w->srl_map, t->Ob, t->P_pad, t->K_cap));
  }
  SrLargeState* t = w->srl;
  CUDA_TRY(cudaMemsetAsync(t->sumO, 0, sizeof(double) * P, c->stream));
  CUDA_TRY(cudaMemsetAsync(t->sumEO, 0, sizeof(double) * P, c->stream));
  CUDA_TRY(cudaMemsetAsync(t->status, 0, sizeof(int), c->stream));
  t->count = 0.0;
  t->sumE = t->sumE2 = 0.0;
  t->rows = 0;
  t->have_center = false;
  t->s_stored = false;
  t->finalized = false;
  return MOLE_OK;
}

// The samples held in Ob through the S-GEMM: S = their sum for the first
// launch of an iteration, S += it after.
static int srl_flush(mole_walkers* w) {
  SrLargeState* t = w->srl;
  mole_ctx* c = w->sys->ctx;
  if (t->rows == 0) return MOLE_OK;
  const int k_pad = (t->rows + kSBK - 1) / kSBK * kSBK;
  if (k_pad > t->rows)  // rows an earlier launch used
    CUDA_TRY(cudaMemsetAsync(t->Ob + (size_t)t->rows * t->P_pad, 0,
                             sizeof(__nv_bfloat16) * (size_t)(k_pad - t->rows) * t->P_pad, c->stream));
  Timer tg(c, 3);
  CUDA_TRY(launch_s_gemm(w->srl_map, t->S, t->P_pad, k_pad, t->s_stored, t->status, c->stream));
  tg.stop();
  int st = 0;
  CUDA_TRY(cudaMemcpyAsync(&st, t->status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (st & 4) return fail(MOLE_ERR_TIMEOUT, "S-matrix kernel wait timed out");
  t->s_stored = true;
  t->rows = 0;
  t->gemm_launches += 1;
  t->gemm_rows += k_pad;
  return MOLE_OK;
}

static int srl_finalize(mole_walkers* w, double eps) {
  SrLargeState* t = w->srl;
  mole_ctx* c = w->sys->ctx;
  if (t->finalized) {
    if (eps != t->eps) return fail(MOLE_ERR_INVALID_ARG, "S was already finalised with another shift");
    return MOLE_OK;
  }
  const int rc = srl_flush(w);
  if (rc) return rc;
  CUDA_TRY(launch_finalize_s(t->S, t->P, t->P_pad, t->sumO, t->count, eps, c->stream));
  t->finalized = true;
  t->eps = eps;
  return MOLE_OK;
}

int mole_sr_collect_matrix(mole_walkers* w, double eps, double* S_out) {
  if (!w || !S_out) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (!w->srl || !(w->srl->count > 0)) return fail(MOLE_ERR_EMPTY_CACHE, "no samples collected");
  cudaGetLastError();  // report only errors raised by this call
  SrLargeState* t = w->srl;
  mole_ctx* c = w->sys->ctx;
  const int rc = srl_finalize(w, eps);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpy2DAsync(S_out, sizeof(double) * t->P, t->S, sizeof(double) * t->P_pad, sizeof(double) * t->P,
                             t->P, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return MOLE_OK;
}

int mole_sr_collect_sample(mole_walkers* w, int32_t precision) {
  if (!w || !w->srl) return fail(MOLE_ERR_EMPTY_CACHE, "call mole_sr_collect_begin first");
  cudaGetLastError();  // report only errors raised by this call
  mole_system* s = w->sys;
  mole_ctx* c = s->ctx;
  SrLargeState* t = w->srl;
  if (t->finalized) return fail(MOLE_ERR_EMPTY_CACHE, "S was finalised; call mole_sr_collect_begin again");
  if (!s->nn_on && (!s->k64 || !s->k32)) return fail(MOLE_ERR_UNSUPPORTED, kNoSingleKernels);
  const int W = w->W, N = s->n_up + s->n_dn, P = s->P;
  const int nwalker_par = s->nn_on ? P - kNnP : P;
  if (nwalker_par > 8) return fail(MOLE_ERR_UNSUPPORTED, "more than 8 orbital/Pade parameters");
  if (s->nn_on && (N * (N - 1) / 2 > 8 || N * s->n_nuc > 8))
    return fail(MOLE_ERR_UNSUPPORTED, "network O_k supports at most 8 pairs per network");
  CUDA_TRY(cudaMemsetAsync(c->status.p, 0, sizeof(int), c->stream));
  // E_L and the orbital/Pade O_k at the current positions
  EvalArgs a;
  a.pos = w->pos;
  a.W = W;
  a.lnpsi = w->srl_eval;
  a.sign = a.lnpsi + W;
  a.lap = a.sign + W;
  a.grad = a.lap + W;
  a.O = a.grad + (size_t)3 * N * W;
  a.ldO = 8;
  a.eloc = t->E;
  a.status = c->status.p;
  Timer tm(c, 2);
  if (precision == MOLE_PREC_MIXED) CUDA_TRY(eval32(s)(s->sp32, a, grid_for(W), c->stream));
  else CUDA_TRY(eval64(s)(s->sp64, a, grid_for(W), c->stream));
  if (!t->have_center) {
    // c = the mean O_k of the first kCenterRows walkers of the iteration's
    // first sample: S and the gradient do not depend on c (finalize_s removes
    // the mean exactly), it only keeps the BF16 operand small
    const int nc = std::min(W, kCenterRows);
    CUDA_TRY(launch_copy_cols(a.O, 8, nwalker_par, t->O, P, nc, c->stream));
    if (s->nn_on)
      CUDA_TRY(launch_nn_ogen(s->sp32, w->pos, W, nc, s->n_up, N, t->O, P, nwalker_par, std::min(W, 3 * c->n_sm),
                              c->stream));
    CUDA_TRY(launch_center_rows(t->O, nc, P, P, t->center, c->stream));
    t->have_center = true;
  }
  if (t->rows + W > t->K_cap) {
    tm.stop();
    const int rc = srl_flush(w);
    if (rc) return rc;
    tm = Timer(c, 2);
  }
  CUDA_TRY(launch_sr_sample(s->sp32, w->pos, W, s->n_up, N, s->nn_on, a.O, 8, nwalker_par, t->center, t->E,
                            t->Ob + (size_t)t->rows * t->P_pad, t->P_pad, P, t->partial, t->n_cta, t->sumO,
                            t->sumEO, c->stream));
  tm.stop();
  t->rows += W;
  std::vector<double> e(W);
  CUDA_TRY(cudaMemcpyAsync(e.data(), t->E, sizeof(double) * W, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  for (double v : e) {
    t->sumE += v;
    t->sumE2 += v * v;
  }
  t->count += W;
  return check_status(c);
}

int mole_sr_collect_solve(mole_walkers* w, double eps, double step, int32_t max_iter, double tol, double* delta,
                          double* grad, double* info) {
  if (!w || !delta) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (!w->srl || !(w->srl->count > 0)) return fail(MOLE_ERR_EMPTY_CACHE, "no samples collected");
  cudaGetLastError();  // report only errors raised by this call
  mole_system* s = w->sys;
  mole_ctx* c = s->ctx;
  SrLargeState* t = w->srl;
  const int P = s->P;
  const double n = t->count, Eb = t->sumE / n;
  std::vector<double> sO(P), sEO(P), b(P), x(P);
  CUDA_TRY(cudaMemcpyAsync(sO.data(), t->sumO, sizeof(double) * P, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaMemcpyAsync(sEO.data(), t->sumEO, sizeof(double) * P, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  // g_k = 2 (<E O_k> - <E><O_k>), centring-invariant; b = -g / 2
  for (int k = 0; k < P; ++k) {
    const double g = 2.0 * (sEO[k] / n - Eb * sO[k] / n);
    if (grad) grad[k] = g;
    b[k] = -0.5 * g;
  }
  const int frc = srl_finalize(w, eps);
  if (frc) return frc;
  double* d_b = t->work + 5 * (size_t)P + 8;  // scratch after the CG vectors
  double* d_x = t->x;
  CUDA_TRY(cudaMemcpyAsync(d_b, b.data(), sizeof(double) * P, cudaMemcpyHostToDevice, c->stream));
  int iters = 0;
  double rel = 0.0;
  CUDA_TRY(sr_cg_solve(t->S, P, t->P_pad, d_b, d_x, t->work, max_iter > 0 ? max_iter : 500, tol > 0 ? tol : 1e-8,
                       &iters, &rel, c->stream));
  CUDA_TRY(cudaMemcpyAsync(x.data(), d_x, sizeof(double) * P, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < P; ++k) delta[k] = step * x[k];
  if (info) {
    info[0] = Eb;
    info[1] = n;
    info[2] = iters;
    info[3] = rel;
  }
  t->have_center = false;
  if (!(rel < 1e-3)) return fail(MOLE_ERR_LINALG, "CG did not converge on the SR system");
  return MOLE_OK;
}

int mole_sr_update(mole_ctx* ctx, int32_t P, double count, const double* sum_E, const double* sum_O,
                   const double* sum_EO, const double* sum_OO, double eps, double step, double* delta,
                   double* grad) {
  if (!ctx || !sum_E || !sum_O || !sum_EO || !sum_OO || !delta) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (P < 1 || !(count > 0)) return fail(MOLE_ERR_SHAPE, "need P >= 1 and count > 0");
  const double Eb = *sum_E / count;
  std::vector<double> S((size_t)P * P), f(P), ob(P);
  for (int k = 0; k < P; ++k) ob[k] = sum_O[k] / count;
  for (int k = 0; k < P; ++k) {
    const double g = 2.0 * (sum_EO[k] / count - Eb * ob[k]);
    if (grad) grad[k] = g;
    f[k] = -0.5 * g;
    for (int l = 0; l < P; ++l) S[(size_t)k * P + l] = sum_OO[(size_t)k * P + l] / count - ob[k] * ob[l];
    S[(size_t)k * P + k] += eps;
  }
  // Cholesky S = L L^T, then two triangular solves (FP64)
  for (int j = 0; j < P; ++j) {
    double d = S[(size_t)j * P + j];
    for (int k = 0; k < j; ++k) d -= S[(size_t)j * P + k] * S[(size_t)j * P + k];
    if (!(d > 0.0)) return fail(MOLE_ERR_LINALG, "SR matrix is not positive definite");
    const double l = std::sqrt(d);
    S[(size_t)j * P + j] = l;
    for (int i = j + 1; i < P; ++i) {
      double v = S[(size_t)i * P + j];
      for (int k = 0; k < j; ++k) v -= S[(size_t)i * P + k] * S[(size_t)j * P + k];
      S[(size_t)i * P + j] = v / l;
    }
  }
  for (int i = 0; i < P; ++i) {
    double v = f[i];
    for (int k = 0; k < i; ++k) v -= S[(size_t)i * P + k] * f[k];
    f[i] = v / S[(size_t)i * P + i];
  }
  for (int i = P - 1; i >= 0; --i) {
    double v = f[i];
    for (int k = i + 1; k < P; ++k) v -= S[(size_t)k * P + i] * f[k];
    f[i] = v / S[(size_t)i * P + i];
  }
  for (int k = 0; k < P; ++k) delta[k] = step * f[k];
  return MOLE_OK;
}

static int ensure_dmc(mole_walkers* w, int n_steps) {
  mole_ctx* c = w->sys->ctx;
  const int W = w->W, NC = 3 * (w->sys->n_up + w->sys->n_dn);
  const int nb = (W + kScanBlock - 1) / kScanBlock;
  if (!w->pos2) {
    CUDA_TRY(cudaMalloc(&w->pos2, sizeof(double) * (size_t)W * NC));
    CUDA_TRY(cudaMalloc(&w->eloc, sizeof(double) * W));
    CUDA_TRY(cudaMalloc(&w->eloc2, sizeof(double) * W));
    CUDA_TRY(cudaMalloc(&w->weight, sizeof(double) * W));
    CUDA_TRY(cudaMalloc(&w->cum, sizeof(double) * W));
    CUDA_TRY(cudaMalloc(&w->btot, sizeof(double) * nb));
    CUDA_TRY(cudaMalloc(&w->e_ref, sizeof(double)));
    CUDA_TRY(cudaMalloc(&w->dstep, sizeof(uint64_t)));
    CUDA_TRY(cudaMalloc(&w->comb, sizeof(CombState)));
  }
  if (w->energies_n < (size_t)n_steps) {
    if (w->energies) cudaFree(w->energies);
    CUDA_TRY(cudaMalloc(&w->energies, sizeof(double) * n_steps));
    w->energies_n = n_steps;
  }
  (void)c;
  return MOLE_OK;
}

int mole_dmc_run(mole_walkers* w, const mole_dmc_opts* o, double* energies, double* accept) {
  cudaGetLastError();  // report only errors raised by this call
  if (!w || !o) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (o->n_steps < 1 || !(o->tau > 0.0)) return fail(MOLE_ERR_SHAPE, "need n_steps >= 1 and tau > 0");
  mole_system* s = w->sys;
  mole_ctx* c = s->ctx;
  if (!s->nn_on && (!s->k64 || !s->k32)) return fail(MOLE_ERR_UNSUPPORTED, kNoSingleKernels);
  const bool mixed = o->precision == MOLE_PREC_MIXED;
  if (mixed ? !dmc32(s) : !dmc64(s))
    return fail(MOLE_ERR_UNSUPPORTED, "DMC kernels are compiled for up to four electrons");
  const int W = w->W, NC = 3 * (s->n_up + s->n_dn), grid = grid_for(W);
  const int nb = (W + kScanBlock - 1) / kScanBlock;
  int rc = ensure_dmc(w, o->n_steps);
  if (rc) return rc;
  CUDA_TRY(c->partials.reserve((size_t)grid * kDmcPart));
  CUDA_TRY(cudaMemsetAsync(c->status.p, 0, sizeof(int), c->stream));
  if (!w->eloc_valid) {
    // E_L at the current positions seeds E_L(old) of the first step
    CUDA_TRY(c->reduced.reserve((size_t)(5 + NC) * W));
    EvalArgs a;
    a.pos = w->pos;
    a.W = W;
    a.lnpsi = c->reduced.p;
    a.sign = a.lnpsi + W;
    a.lap = a.sign + W;
    a.eloc = w->eloc;
    a.grad = a.lap + W;
    a.O = nullptr;  // no parameter derivatives needed
    a.ldO = 0;
    a.status = c->status.p;
    if (mixed) CUDA_TRY(eval32(s)(s->sp32, a, grid, c->stream));
    else CUDA_TRY(eval64(s)(s->sp64, a, grid, c->stream));
    // walkers this evaluation finds singular are given zero weight by the
    // first step (which also flags a non-finite E_L of any other walker)
    CUDA_TRY(cudaMemsetAsync(c->status.p, 0, sizeof(int), c->stream));
    w->eloc_valid = true;
  }
  // the double-float steps keep the starting positions and E_L for a native rerun
  auto ddf = o->precision == MOLE_PREC_DF64 && !s->nn_on && s->kdf ? s->kdf->dmc[s->en_on] : nullptr;
  const size_t pos_n = (size_t)NC * W;
  if (ddf) {
    CUDA_TRY(c->pos_backup.reserve(pos_n + W));
    CUDA_TRY(cudaMemcpyAsync(c->pos_backup.p, w->pos, sizeof(double) * pos_n, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->pos_backup.p + pos_n, w->eloc, sizeof(double) * W, cudaMemcpyDeviceToDevice,
                             c->stream));
  }
  DmcArgs a;
  a.W = W;
  a.tau = o->tau;
  a.e_ref = w->e_ref;
  a.eloc_cut = o->eloc_cutoff;
  a.seed = w->seed;
  a.step = w->dstep;
  a.partials = c->partials.p;
  a.status = c->status.p;
  a.weight = w->weight;
  // n_steps steps of one kernel variant from the state at the call's start
  auto run_steps = [&](auto kernel, const auto& sp) -> int {
    const uint64_t step = w->step;
    CombState cs0 = {0.0, 0.0, 0.0, 0.0, 0.0};
    CUDA_TRY(cudaMemcpyAsync(w->dstep, &step, sizeof(uint64_t), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(w->e_ref, &o->e_ref, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(w->comb, &cs0, sizeof(CombState), cudaMemcpyHostToDevice, c->stream));
    for (int t = 0; t < o->n_steps; ++t) {
      a.pos = w->pos;
      a.eloc = w->eloc;
      CUDA_TRY(kernel(sp, a, grid, c->stream));
      CUDA_TRY(launch_comb(w->weight, w->cum, w->btot, nb, c->partials.p, grid, w->comb, w->dstep, w->seed,
                           w->energies, t, w->pos, w->eloc, w->pos2, w->eloc2, W, NC, c->stream));
      std::swap(w->pos, w->pos2);
      std::swap(w->eloc, w->eloc2);
    }
    return MOLE_OK;
  };
  Timer tm(c, 1);
  if (ddf) rc = run_steps(ddf, s->spdf);
  else if (mixed) rc = run_steps(dmc32(s), s->sp32);
  else rc = run_steps(dmc64(s), s->sp64);
  if (rc) return rc;
  if (ddf) {
    int st = 0;
    CUDA_TRY(cudaMemcpyAsync(&st, c->status.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (st & 8) {
      // a walker left FP32's range or met a node: the same steps in native FP64
      ++c->df64_reruns;
      CUDA_TRY(cudaMemcpyAsync(w->pos, c->pos_backup.p, sizeof(double) * pos_n, cudaMemcpyDeviceToDevice, c->stream));
      CUDA_TRY(cudaMemcpyAsync(w->eloc, c->pos_backup.p + pos_n, sizeof(double) * W, cudaMemcpyDeviceToDevice,
                               c->stream));
      CUDA_TRY(cudaMemsetAsync(c->status.p, 0, sizeof(int), c->stream));
      if ((rc = run_steps(dmc64(s), s->sp64))) return rc;
    }
  }
  tm.stop();
  CombState cs;
  if (energies)
    CUDA_TRY(cudaMemcpyAsync(energies, w->energies, sizeof(double) * o->n_steps, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaMemcpyAsync(&cs, w->comb, sizeof(CombState), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  w->step += (uint64_t)o->n_steps;
  w->dmc_node_kills += cs.killed;
  if (accept) {
    accept[0] = cs.accepted;
    accept[1] = cs.proposed;
  }
  return check_status(c);
}

int mole_dmc_node_kills(const mole_walkers* w, double* killed) {
  if (!w || !killed) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  *killed = w->dmc_node_kills;
  return MOLE_OK;
}

// checkpoint: "MOLECKP1", W, N, P, seed, step, theta[P], positions [W][N][3]
int mole_checkpoint_save(mole_walkers* w, const char* path) {
  if (!w || !path) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  mole_system* s = w->sys;
  const int N = s->n_up + s->n_dn;
  std::vector<double> pos((size_t)w->W * N * 3);
  int rc = mole_walkers_get_positions(w, pos.data(), (int64_t)pos.size());
  if (rc) return rc;
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(MOLE_ERR_IO, std::string("cannot open ") + path);
  const char magic[8] = {'M', 'O', 'L', 'E', 'C', 'K', 'P', '1'};
  const int64_t hdr[5] = {w->W, N, s->P, (int64_t)w->seed, (int64_t)w->step};
  bool ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(hdr, sizeof(int64_t), 5, f) == 5 &&
            std::fwrite(s->theta.data(), sizeof(double), s->P, f) == (size_t)s->P &&
            std::fwrite(pos.data(), sizeof(double), pos.size(), f) == pos.size();
  ok = (std::fclose(f) == 0) && ok;
  return ok ? MOLE_OK : fail(MOLE_ERR_IO, "short write");
}

int mole_checkpoint_load(mole_walkers* w, const char* path) {
  if (!w || !path) return fail(MOLE_ERR_INVALID_ARG, "NULL argument");
  mole_system* s = w->sys;
  const int N = s->n_up + s->n_dn;
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(MOLE_ERR_IO, std::string("cannot open ") + path);
  char magic[8];
  int64_t hdr[5];
  if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, "MOLECKP1", 8) != 0 ||
      std::fread(hdr, sizeof(int64_t), 5, f) != 5) {
    std::fclose(f);
    return fail(MOLE_ERR_IO, "not a mole checkpoint");
  }
  if (hdr[0] != w->W || hdr[1] != N || hdr[2] != s->P) {
    std::fclose(f);
    return fail(MOLE_ERR_SHAPE, "checkpoint sizes do not match this walker set");
  }
  std::vector<double> theta(s->P), pos((size_t)w->W * N * 3);
  const bool ok = std::fread(theta.data(), sizeof(double), s->P, f) == (size_t)s->P &&
                  std::fread(pos.data(), sizeof(double), pos.size(), f) == pos.size();
  std::fclose(f);
  if (!ok) return fail(MOLE_ERR_IO, "truncated checkpoint");
  int rc = mole_params_set(s, theta.data(), s->P);
  if (rc) return rc;
  w->seed = (uint64_t)hdr[3];
  w->step = (uint64_t)hdr[4];
  return mole_walkers_set_positions(w, pos.data(), (int64_t)pos.size());
}

}  // extern "C"
