// batch.cu -- the ragged-batch VMC path: the persistent kernel, its per-system
// reduction, the CUDA-graph replay of a run and the tile autotuner, behind
// the mole_batch_* entry points of include/mole_gpu.h.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "batch.cuh"
#include "handles.cuh"

namespace mole {

template <class R, int MOVE>
// 168 registers: shared memory holds about 12 warps per SM at N = 10 (520 B
// per walker), which 168 registers per thread also allow; below that the
// kernel spills.
__global__ void __maxnreg__(168) batch_vmc_kernel(const BatchArgs a) {
  auto* sp = reinterpret_cast<SysParams<R>*>(mole_dyn_smem);
  double* st = reinterpret_cast<double*>(mole_dyn_smem + batch_sp_bytes<R>());
  double* red = st + (size_t)a.slots * blockDim.x;
  __shared__ int s_item;
  const uint32_t t0 = (uint32_t)*a.step0;
  for (;;) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(a.queue, 1u);
    __syncthreads();
    const int q = s_item;
    if (q >= a.n_items) break;
    const int id = a.order[q];
    const int2 it = a.items[id];
    // the item's system image, 8 bytes per thread and step
    const unsigned long long* src =
        reinterpret_cast<const unsigned long long*>(static_cast<const SysParams<R>*>(a.sys) + it.x);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(sp);
    for (int k = threadIdx.x; k < (int)(sizeof(SysParams<R>) / 8); k += blockDim.x) dst[k] = src[k];
    __syncthreads();
    const BatchSystem& bs = a.info[it.x];
    switch (bs.nu > bs.nd ? bs.nu : bs.nd) {
      case 1: batch_item<R, MOVE, 1>(*sp, bs, id, it.y, st, red, a, t0); break;
      case 2: batch_item<R, MOVE, 2>(*sp, bs, id, it.y, st, red, a, t0); break;
      case 3: batch_item<R, MOVE, 3>(*sp, bs, id, it.y, st, red, a, t0); break;
      case 4: batch_item<R, MOVE, 4>(*sp, bs, id, it.y, st, red, a, t0); break;
      default: batch_item<R, MOVE, kMaxSpin>(*sp, bs, id, it.y, st, red, a, t0); break;
    }
    __syncthreads();  // the image and s_item are rewritten by the next item
  }
}

// Per-system sums of the item partials in item order (deterministic), the
// status word after them, and the sweep counter advanced for the next call.
__global__ void batch_reduce_kernel(const double* partials, const BatchSystem* info, int S, double* out,
                                    uint64_t* step0, uint64_t adv, const int* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < S * kNMom) {
    const int s = i / kNMom, k = i % kNMom;
    const BatchSystem b = info[s];
    double v = 0.0;
    for (int id = b.item0; id < b.item0 + b.n_items; ++id) v += partials[(size_t)id * kNMom + k];
    out[i] = v;
  }
  if (i == 0) {
    out[(size_t)S * kNMom] = (double)*status;
    *step0 += adv;
  }
}

// The kernel's dynamic shared-memory limit is raised by batch_occupancy,
// which every launch plan calls first (outside any stream capture).
template <class R, int MOVE>
cudaError_t launch_batch(const BatchArgs& a, int grid, int wpb, size_t smem, cudaStream_t s) {
  batch_vmc_kernel<R, MOVE><<<grid, wpb, smem, s>>>(a);
  return cudaGetLastError();
}

template <class R, int MOVE>
int batch_occupancy(int wpb, size_t smem) {
  auto k = batch_vmc_kernel<R, MOVE>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, wpb, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

}  // namespace mole

using namespace mole;

struct mole_batch {
  mole_ctx* ctx = nullptr;
  std::vector<mole_system*> sys;
  std::vector<int> versions;
  std::vector<BatchSystem> info;
  std::vector<double> widths;  // each system's own proposal width (scaled by opts->step)
  std::vector<SysParams<double>> h64;
  std::vector<SysParams<float>> h32;
  int S = 0;
  int64_t walkers = 0;
  long long pos_total = 0;
  int max_slots64 = 0, max_slots32 = 0;
  int max_elec = 0;
  double* pos = nullptr;
  SysParams<double>* d64 = nullptr;
  SysParams<float>* d32 = nullptr;
  BatchSystem* d_info = nullptr;
  DevBuf<int2> items;
  DevBuf<int> order;
  DevBuf<double> partials;
  int n_items = 0;
  double* d_out = nullptr;  // [S][kNMom] + status
  double* h_out = nullptr;  // pinned copy
  uint64_t* d_step = nullptr;
  unsigned* d_queue = nullptr;
  int* d_status = nullptr;
  uint64_t step = 0;
  int wpb = 64;
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<long long> graph_key;
  int64_t graph_launches = 0;
};

namespace {

#define BATCH_TRY(x)                                                                                   \
  do {                                                                                                 \
    cudaError_t e_ = (x);                                                                              \
    if (e_ != cudaSuccess) return set_error(MOLE_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Relative FP64 work of one walker-sweep of a system: N moves of O(n^2)
// Sherman-Morrison work plus the local energy's N^2 pair terms.
double walker_cost(const BatchSystem& b) {
  const int N = b.nu + b.nd;
  return (double)N * (b.nu * b.nu + b.nd * b.nd + 2 * N + 4);
}

// Work items for a tile of wpb walkers: ids in system order, dispatched most
// expensive first so that the last CTAs to finish carry the shortest items.
cudaError_t build_items(mole_batch* b, int wpb, cudaStream_t s) {
  std::vector<int2> items;
  std::vector<double> cost;
  for (int k = 0; k < b->S; ++k) {
    BatchSystem& in = b->info[k];
    in.item0 = (int)items.size();
    in.n_items = (in.W + wpb - 1) / wpb;
    for (int j = 0; j < in.n_items; ++j) {
      items.push_back(make_int2(k, j * wpb));
      cost.push_back(walker_cost(in) * std::min(wpb, in.W - j * wpb));
    }
  }
  std::vector<int> order(items.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
  b->n_items = (int)items.size();
  cudaError_t e;
  if ((e = b->items.reserve(items.size())) != cudaSuccess) return e;
  if ((e = b->order.reserve(order.size())) != cudaSuccess) return e;
  if ((e = b->partials.reserve((size_t)b->n_items * kNMom)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(b->items.p, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(b->order.p, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(b->d_info, b->info.data(), sizeof(BatchSystem) * b->S, cudaMemcpyHostToDevice, s)) !=
      cudaSuccess)
    return e;
  return cudaStreamSynchronize(s);
}

void drop_graph(mole_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->graph_key.clear();
}

// Re-uploads the system images when a system's parameters changed.
cudaError_t sync_params(mole_batch* b, bool force) {
  bool changed = force;
  for (int k = 0; k < b->S; ++k)
    if (b->versions[k] != b->sys[k]->version) changed = true;
  if (!changed) return cudaSuccess;
  for (int k = 0; k < b->S; ++k) {
    b->h64[k] = b->sys[k]->sp64;
    b->h32[k] = b->sys[k]->sp32;
    b->versions[k] = b->sys[k]->version;
  }
  cudaError_t e = cudaMemcpy(b->d64, b->h64.data(), sizeof(SysParams<double>) * b->S, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d32, b->h32.data(), sizeof(SysParams<float>) * b->S, cudaMemcpyHostToDevice);
  return e;
}

struct LaunchPlan {
  int grid = 0;
  size_t smem = 0;
};

int occupancy(bool mixed, int move, int wpb, size_t smem) {
  if (mixed) return move == kMoveBox ? batch_occupancy<float, kMoveBox>(wpb, smem) : batch_occupancy<float, kMoveGauss>(wpb, smem);
  return move == kMoveBox ? batch_occupancy<double, kMoveBox>(wpb, smem) : batch_occupancy<double, kMoveGauss>(wpb, smem);
}

LaunchPlan plan(const mole_batch* b, bool mixed, int move, int wpb) {
  LaunchPlan p;
  p.smem = mixed ? batch_smem_bytes<float>(wpb, b->max_slots32, b->max_elec)
                 : batch_smem_bytes<double>(wpb, b->max_slots64, b->max_elec);
  const int occ = occupancy(mixed, move, wpb, p.smem);
  p.grid = std::min(b->ctx->n_sm * occ, b->n_items);
  return p;
}

cudaError_t launch(const BatchArgs& a, bool mixed, int move, const LaunchPlan& p, int wpb, cudaStream_t s) {
  if (mixed)
    return move == kMoveBox ? launch_batch<float, kMoveBox>(a, p.grid, wpb, p.smem, s)
                            : launch_batch<float, kMoveGauss>(a, p.grid, wpb, p.smem, s);
  return move == kMoveBox ? launch_batch<double, kMoveBox>(a, p.grid, wpb, p.smem, s)
                          : launch_batch<double, kMoveGauss>(a, p.grid, wpb, p.smem, s);
}

BatchArgs make_args(const mole_batch* b, const mole_vmc_opts* o, double* pos, uint64_t* step0) {
  BatchArgs a;
  const bool mixed = o->precision == MOLE_PREC_MIXED;
  a.sys = mixed ? (const void*)b->d32 : (const void*)b->d64;
  a.info = b->d_info;
  a.items = b->items.p;
  a.order = b->order.p;
  a.n_items = b->n_items;
  a.n_systems = b->S;
  a.slots = mixed ? b->max_slots32 : b->max_slots64;
  a.rslots = mixed ? batch_rslots<float>(b->max_elec) : 0;
  a.pos = pos;
  a.move = o->move;
  a.n_eq = o->n_eq;
  a.n_steps = o->n_steps;
  a.block_size = o->block_size;
  a.refresh = o->refresh;
  a.step0 = step0;
  a.queue = b->d_queue;
  a.partials = b->partials.p;
  a.moments = b->d_out;
  a.status = b->d_status;
  return a;
}

int check_opts(const mole_vmc_opts* o) {
  if (o->block_size < 1 || o->n_steps < 0 || o->n_eq < 0 || o->n_steps % o->block_size != 0)
    return set_error(MOLE_ERR_SHAPE, "n_steps must be a non-negative multiple of block_size >= 1");
  if (o->move != MOLE_MOVE_BOX && o->move != MOLE_MOVE_GAUSS)
    return set_error(MOLE_ERR_UNSUPPORTED, "batched VMC supports box and Gaussian moves");
  if (!(o->step > 0.0)) return set_error(MOLE_ERR_INVALID_ARG, "step scale must be positive");
  if (o->sr) return set_error(MOLE_ERR_UNSUPPORTED, "batched VMC does not accumulate SR sums");
  return MOLE_OK;
}

// The per-system step is info.step = opts->step x the system's own width; the
// images are rewritten when the scale changes.
cudaError_t set_step_scale(mole_batch* b, double scale) {
  bool changed = false;
  for (int k = 0; k < b->S; ++k) {
    const double st = b->widths[k] * scale;
    if (b->info[k].step != st) {
      b->info[k].step = st;
      changed = true;
    }
  }
  if (!changed) return cudaSuccess;
  return cudaMemcpy(b->d_info, b->info.data(), sizeof(BatchSystem) * b->S, cudaMemcpyHostToDevice);
}

void free_batch(mole_batch* b) {
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  drop_graph(b);
  for (void* p : {(void*)b->pos, (void*)b->d64, (void*)b->d32, (void*)b->d_info, (void*)b->d_out, (void*)b->d_step,
                  (void*)b->d_queue, (void*)b->d_status})
    if (p) cudaFree(p);
  if (b->h_out) cudaFreeHost(b->h_out);
  b->items.release();
  b->order.release();
  b->partials.release();
  if (b->cap) cudaStreamDestroy(b->cap);
  cudaGetLastError();  // teardown errors are not reported to later calls
  for (mole_system* s : b->sys) system_release(s);
  delete b;
}

}  // namespace

extern "C" {

int mole_batch_create(mole_ctx* ctx, int32_t n, mole_system* const* systems, const int32_t* n_walkers,
                      const uint64_t* seeds, const double* widths, mole_batch** out) {
  cudaGetLastError();  // report only errors raised by this call
  if (!ctx || !systems || !n_walkers || !seeds || !out) return set_error(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (n < 1) return set_error(MOLE_ERR_SHAPE, "a batch needs at least one system");
  for (int k = 0; k < n; ++k) {
    const mole_system* s = systems[k];
    if (!s) return set_error(MOLE_ERR_INVALID_ARG, "NULL system in the batch");
    if (s->ctx != ctx) return set_error(MOLE_ERR_INVALID_ARG, "every system of a batch must belong to its context");
    if (s->nn_on) return set_error(MOLE_ERR_UNSUPPORTED, "batched VMC does not run neural-Jastrow systems");
    if (s->pot_kind != MOLE_POT_COULOMB) return set_error(MOLE_ERR_UNSUPPORTED, "batched VMC runs Coulomb systems");
    if (n_walkers[k] < 1) return set_error(MOLE_ERR_SHAPE, "every system needs at least one walker");
    if (widths && !(widths[k] > 0.0)) return set_error(MOLE_ERR_INVALID_ARG, "proposal widths must be positive");
  }
  BATCH_TRY(cudaSetDevice(ctx->device));
  auto b = new mole_batch();
  b->ctx = ctx;
  b->S = n;
  b->sys.assign(systems, systems + n);
  for (mole_system* s : b->sys) system_retain(s);
  b->versions.assign(n, -1);
  b->h64.resize(n);
  b->h32.resize(n);
  b->info.resize(n);
  b->widths.assign(n, 1.0);
  long long off = 0;
  for (int k = 0; k < n; ++k) {
    BatchSystem& in = b->info[k];
    in.pos_off = off;
    in.W = n_walkers[k];
    in.nu = systems[k]->n_up;
    in.nd = systems[k]->n_dn;
    in.seed = seeds[k];
    in.step = widths ? widths[k] : 1.0;
    b->widths[k] = in.step;
    off += (long long)3 * (in.nu + in.nd) * in.W;
    b->walkers += in.W;
    b->max_slots64 = std::max(b->max_slots64, batch_slots<double>(in.nu, in.nd));
    b->max_slots32 = std::max(b->max_slots32, batch_slots<float>(in.nu, in.nd));
    b->max_elec = std::max(b->max_elec, in.nu + in.nd);
  }
  b->pos_total = off;
  cudaError_t e = cudaMalloc(&b->pos, sizeof(double) * (size_t)off);
  if (e == cudaSuccess) e = cudaMalloc(&b->d64, sizeof(SysParams<double>) * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->d32, sizeof(SysParams<float>) * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_info, sizeof(BatchSystem) * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_out, sizeof(double) * ((size_t)n * kNMom + 1));
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_out, sizeof(double) * ((size_t)n * kNMom + 1));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_step, sizeof(uint64_t));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_queue, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_status, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(b->d_step, 0, sizeof(uint64_t));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = sync_params(b, true);
  if (e == cudaSuccess) e = build_items(b, b->wpb, ctx->stream);
  if (e != cudaSuccess) {
    free_batch(b);
    return set_error(MOLE_ERR_CUDA, std::string("batch setup: ") + cudaGetErrorString(e));
  }
  const int rc = mole_batch_init(b, MOLE_INIT_NORMAL, 1.0);
  if (rc != MOLE_OK) {
    free_batch(b);
    return rc;
  }
  *out = b;
  return MOLE_OK;
}

int mole_batch_destroy(mole_batch* b) {
  if (b) free_batch(b);
  return MOLE_OK;
}

int mole_batch_info(const mole_batch* b, int32_t* n_systems, int64_t* n_walkers) {
  if (!b) return set_error(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (n_systems) *n_systems = b->S;
  if (n_walkers) *n_walkers = b->walkers;
  return MOLE_OK;
}

int mole_batch_init(mole_batch* b, int32_t kind, double width) {
  cudaGetLastError();  // report only errors raised by this call
  if (!b) return set_error(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (kind != MOLE_INIT_NORMAL && kind != MOLE_INIT_UNIFORM) return set_error(MOLE_ERR_INVALID_ARG, "bad init kind");
  for (int k = 0; k < b->S; ++k) {
    const BatchSystem& in = b->info[k];
    BATCH_TRY(launch_init_positions(b->pos + in.pos_off, in.W, in.nu + in.nd, in.seed, kind, width, b->ctx->stream));
  }
  return MOLE_OK;
}

int mole_batch_set_positions(mole_batch* b, int32_t system, const double* pos, int64_t n) {
  cudaGetLastError();  // report only errors raised by this call
  if (!b || !pos) return set_error(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (system < 0 || system >= b->S) return set_error(MOLE_ERR_INVALID_ARG, "no such system in the batch");
  const BatchSystem& in = b->info[system];
  const int NC = 3 * (in.nu + in.nd);
  if (n != (int64_t)in.W * NC) return set_error(MOLE_ERR_SHAPE, "positions must hold W * N * 3 values");
  mole_ctx* c = b->ctx;
  BATCH_TRY(c->scratch.reserve((size_t)n));
  BATCH_TRY(cudaMemcpyAsync(c->scratch.p, pos, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  BATCH_TRY(launch_aos_to_soa(c->scratch.p, b->pos + in.pos_off, in.W, NC, c->stream));
  return MOLE_OK;
}

int mole_batch_get_positions(mole_batch* b, int32_t system, double* pos, int64_t n) {
  cudaGetLastError();  // report only errors raised by this call
  if (!b || !pos) return set_error(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (system < 0 || system >= b->S) return set_error(MOLE_ERR_INVALID_ARG, "no such system in the batch");
  const BatchSystem& in = b->info[system];
  const int NC = 3 * (in.nu + in.nd);
  if (n != (int64_t)in.W * NC) return set_error(MOLE_ERR_SHAPE, "positions must hold W * N * 3 values");
  mole_ctx* c = b->ctx;
  BATCH_TRY(c->scratch.reserve((size_t)n));
  BATCH_TRY(launch_soa_to_aos(b->pos + in.pos_off, c->scratch.p, in.W, NC, c->stream));
  BATCH_TRY(cudaMemcpyAsync(pos, c->scratch.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  BATCH_TRY(cudaStreamSynchronize(c->stream));
  return MOLE_OK;
}

int mole_batch_get_step(const mole_batch* b, uint64_t* step) {
  if (!b || !step) return set_error(MOLE_ERR_INVALID_ARG, "NULL argument");
  *step = b->step;
  return MOLE_OK;
}

int mole_batch_set_step(mole_batch* b, uint64_t step) {
  if (!b) return set_error(MOLE_ERR_INVALID_ARG, "NULL argument");
  BATCH_TRY(cudaMemcpyAsync(b->d_step, &step, sizeof(uint64_t), cudaMemcpyHostToDevice, b->ctx->stream));
  BATCH_TRY(cudaStreamSynchronize(b->ctx->stream));
  b->step = step;
  return MOLE_OK;
}

int mole_batch_get_tile(const mole_batch* b, int32_t* walkers_per_cta, int32_t* ctas, int32_t precision) {
  if (!b) return set_error(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (walkers_per_cta) *walkers_per_cta = b->wpb;
  if (ctas) *ctas = plan(b, precision == MOLE_PREC_MIXED, kMoveGauss, b->wpb).grid;
  return MOLE_OK;
}

int mole_batch_set_tile(mole_batch* b, int32_t wpb) {
  cudaGetLastError();  // report only errors raised by this call
  if (!b) return set_error(MOLE_ERR_INVALID_ARG, "NULL argument");
  if (wpb < 32 || wpb > kBatchMaxThreads || wpb % 32 != 0)
    return set_error(MOLE_ERR_INVALID_ARG, "walkers per CTA must be a multiple of 32 in [32, 256]");
  if (plan(b, false, kMoveGauss, wpb).grid < 1 || plan(b, true, kMoveGauss, wpb).grid < 1)
    return set_error(MOLE_ERR_UNSUPPORTED, "this tile does not fit the shared memory of one SM");
  if (wpb == b->wpb) return MOLE_OK;
  b->wpb = wpb;
  drop_graph(b);
  BATCH_TRY(build_items(b, wpb, b->ctx->stream));
  return MOLE_OK;
}

int mole_batch_vmc_run(mole_batch* b, const mole_vmc_opts* o, double* moments) {
  cudaGetLastError();  // report only errors raised by this call
  if (!b || !o || !moments) return set_error(MOLE_ERR_INVALID_ARG, "NULL argument");
  int rc = check_opts(o);
  if (rc != MOLE_OK) return rc;
  mole_ctx* c = b->ctx;
  BATCH_TRY(cudaSetDevice(c->device));
  const bool mixed = o->precision == MOLE_PREC_MIXED;
  BATCH_TRY(cudaStreamSynchronize(c->stream));  // earlier work on the context stream may still read the images
  BATCH_TRY(set_step_scale(b, o->step));
  BATCH_TRY(sync_params(b, false));
  const LaunchPlan p = plan(b, mixed, o->move, b->wpb);
  if (p.grid < 1) return set_error(MOLE_ERR_UNSUPPORTED, "the batch's tile does not fit one SM");
  const std::vector<long long> key = {o->precision, o->move, o->n_eq, o->n_steps, o->block_size, o->refresh, b->wpb};
  if (!b->exec || key != b->graph_key) {
    drop_graph(b);
    // one run = reset counters, the persistent sweep kernel, the per-system
    // reduction (which also advances the sweep counter) and the copy of the
    // results to pinned host memory, captured once and replayed
    const BatchArgs a = make_args(b, o, b->pos, b->d_step);
    BATCH_TRY(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned), b->cap);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_status, 0, sizeof(int), b->cap);
    if (e == cudaSuccess) e = launch(a, mixed, o->move, p, b->wpb, b->cap);
    if (e == cudaSuccess) {
      const int tot = b->S * kNMom;
      batch_reduce_kernel<<<(tot + 255) / 256, 256, 0, b->cap>>>(b->partials.p, b->d_info, b->S, b->d_out, b->d_step,
                                                                 (uint64_t)(o->n_eq + o->n_steps), b->d_status);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(b->h_out, b->d_out, sizeof(double) * ((size_t)b->S * kNMom + 1), cudaMemcpyDeviceToHost,
                          b->cap);
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(b->cap, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, g, 0);
    b->graph = g;
    if (e != cudaSuccess) {
      drop_graph(b);
      return set_error(MOLE_ERR_CUDA, std::string("capturing the batch graph: ") + cudaGetErrorString(e));
    }
    b->graph_key = key;
  }
  if (c->timing) BATCH_TRY(cudaEventRecord(c->ev0, c->stream));
  BATCH_TRY(cudaGraphLaunch(b->exec, c->stream));
  if (c->timing) {
    BATCH_TRY(cudaEventRecord(c->ev1, c->stream));
    BATCH_TRY(cudaEventSynchronize(c->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    c->kernel_ms[kTimeBatch] += ms;
    c->kernel_launches[kTimeBatch] += 1;
  }
  BATCH_TRY(cudaStreamSynchronize(c->stream));
  b->graph_launches += 1;
  b->step += (uint64_t)(o->n_eq + o->n_steps);
  std::memcpy(moments, b->h_out, sizeof(double) * (size_t)b->S * kNMom);
  const int st = (int)b->h_out[(size_t)b->S * kNMom];
  if (st & 2) return set_error(MOLE_ERR_LINALG, "singular Slater matrix encountered");
  if (st & 1) return set_error(MOLE_ERR_FUNC, "non-finite local energy encountered");
  return MOLE_OK;
}

int mole_batch_autotune(mole_batch* b, const mole_vmc_opts* o, int32_t n_candidates, int32_t* cand_wpb,
                        double* cand_ms, int32_t* n_timed) {
  cudaGetLastError();  // report only errors raised by this call
  if (!b || !o) return set_error(MOLE_ERR_INVALID_ARG, "NULL argument");
  int rc = check_opts(o);
  if (rc != MOLE_OK) return rc;
  mole_ctx* c = b->ctx;
  BATCH_TRY(cudaSetDevice(c->device));
  const bool mixed = o->precision == MOLE_PREC_MIXED;
  BATCH_TRY(cudaStreamSynchronize(c->stream));
  BATCH_TRY(set_step_scale(b, o->step));
  BATCH_TRY(sync_params(b, false));
  // The candidates run on a copy of the positions with their own sweep
  // counter, so tuning leaves the chains and the random streams untouched.
  double* tpos = nullptr;
  uint64_t* tstep = nullptr;
  BATCH_TRY(cudaMalloc(&tpos, sizeof(double) * (size_t)b->pos_total));
  cudaError_t e = cudaMalloc(&tstep, sizeof(uint64_t));
  const int wpbs[] = {32, 64, 96, 128, 192, 256};
  int best = b->wpb, timed = 0;
  double best_ms = 1e300;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (int wpb : wpbs) {
    if (e != cudaSuccess) break;
    const LaunchPlan p0 = plan(b, mixed, o->move, wpb);
    if (p0.grid < 1) continue;
    if ((e = build_items(b, wpb, c->stream)) != cudaSuccess) break;
    const LaunchPlan p = plan(b, mixed, o->move, wpb);
    const BatchArgs a = make_args(b, o, tpos, tstep);
    float ms = 0.f;
    for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {  // first run warms up
      e = cudaMemcpyAsync(tpos, b->pos, sizeof(double) * (size_t)b->pos_total, cudaMemcpyDeviceToDevice, c->stream);
      if (e == cudaSuccess) e = cudaMemsetAsync(tstep, 0, sizeof(uint64_t), c->stream);
      if (e == cudaSuccess) e = cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned), c->stream);
      if (e == cudaSuccess) e = cudaMemsetAsync(b->d_status, 0, sizeof(int), c->stream);
      if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
      if (e == cudaSuccess) e = launch(a, mixed, o->move, p, wpb, c->stream);
      if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    }
    if (e != cudaSuccess) break;
    if (cand_wpb && timed < n_candidates) cand_wpb[timed] = wpb;
    if (cand_ms && timed < n_candidates) cand_ms[timed] = ms;
    ++timed;
    if (ms < best_ms) {
      best_ms = ms;
      best = wpb;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(tpos);
  if (tstep) cudaFree(tstep);
  if (n_timed) *n_timed = timed;
  drop_graph(b);
  b->wpb = best;
  const cudaError_t e3 = build_items(b, best, c->stream);
  if (e != cudaSuccess) return set_error(MOLE_ERR_CUDA, std::string("autotuning: ") + cudaGetErrorString(e));
  if (e3 != cudaSuccess) return set_error(MOLE_ERR_CUDA, std::string("autotuning: ") + cudaGetErrorString(e3));
  return MOLE_OK;
}

int mole_batch_graph_launches(const mole_batch* b, int64_t* n) {
  if (!b || !n) return set_error(MOLE_ERR_INVALID_ARG, "NULL argument");
  *n = b->graph_launches;
  return MOLE_OK;
}

}  // extern "C"
