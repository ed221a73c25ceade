// ensemble.cu -- ensemble-wide kernels: initial positions, layout transposes,
// deterministic reductions, the DMC stochastic comb and FMA peak probes.
#include "ensemble.cuh"

namespace mole {

// Walker w, electron e: one Philox draw gives three N(0,1) (Box-Muller) or
// three U(-1,1) coordinates, scaled by width. Output SoA [3N][W].
__global__ void init_positions_kernel(double* pos, int W, int N, uint64_t seed, int kind, double width) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= W * N) return;
  const int w = id / N, e = id % N;
  const uint4 u = draw4(seed, (uint32_t)w, (uint32_t)e, 0u, kTagInit);
  double p[3];
  if (kind == 0) {
    double z0, z1, z2, z3;
    box_muller(u.x, u.y, z0, z1);
    box_muller(u.z, u.w, z2, z3);
    p[0] = width * z0; p[1] = width * z1; p[2] = width * z2;
  } else {
    p[0] = width * (2.0 * u01<double>(u.x) - 1.0);
    p[1] = width * (2.0 * u01<double>(u.y) - 1.0);
    p[2] = width * (2.0 * u01<double>(u.z) - 1.0);
  }
  for (int c = 0; c < 3; ++c) pos[(size_t)(3 * e + c) * W + w] = p[c];
}

__global__ void aos_to_soa_kernel(const double* aos, double* soa, int W, int NC) {
  const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (size_t)W * NC) return;
  const int k = (int)(id / W), w = (int)(id % W);
  soa[id] = aos[(size_t)w * NC + k];
}

__global__ void soa_to_aos_kernel(const double* soa, double* aos, int W, int NC) {
  const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (size_t)W * NC) return;
  const int w = (int)(id / NC), k = (int)(id % NC);
  aos[id] = soa[(size_t)k * W + w];
}

// out[c] = sum over rows of part[row][c], in row order (deterministic).
__global__ void reduce_columns_kernel(const double* part, int rows, int cols, double* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  double s = 0.0;
  for (int r = 0; r < rows; ++r) s += part[(size_t)r * cols + c];
  out[c] = s;
}

__global__ void unpack_vmc_sums_kernel(const double* red, int PM, int P, double* moments, double* sr) {
  const int t = threadIdx.x;
  if (t < 7) moments[t] = red[t];
  if (!sr) return;
  for (int p = t; p < P; p += blockDim.x) {
    sr[p] = red[7 + p];
    sr[P + p] = red[7 + PM + p];
  }
  int q = 7 + 2 * PM;
  for (int p = 0; p < PM; ++p)
    for (int r = p; r < PM; ++r, ++q)
      if (t == 0 && p < P && r < P) {
        sr[2 * P + p * P + r] = red[q];
        sr[2 * P + r * P + p] = red[q];
      }
}

// ---------------------------------------------------------------- DMC comb

// Per-CTA inclusive scan of the weights; CTA totals to btot.
__global__ void __launch_bounds__(kScanBlock) scan_blocks_kernel(const double* w, double* cum, double* btot, int W) {
  __shared__ double ws[kScanBlock / 32];
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double v = i < W ? w[i] : 0.0;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  if (lane == 31) ws[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double s = lane < kScanBlock / 32 ? ws[lane] : 0.0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += t;
    }
    if (lane < kScanBlock / 32) ws[lane] = s;
  }
  __syncthreads();
  if (warp > 0) v += ws[warp - 1];
  if (i < W) cum[i] = v;
  if (threadIdx.x == kScanBlock - 1) btot[blockIdx.x] = v;
}

// One CTA: exclusive offsets of the CTA totals (in place), the comb's
// uniform and total, this step's ensemble energy and acceptance, and the
// step counter increment.
// One block: the exclusive scan of the per-block weight totals (block
// offsets, in chunks of kTotThreads with a running carry), the step's sums
// of the step-kernel partials (one warp per column), the comb's uniform and
// the running counters.
constexpr int kTotThreads = 512;
__global__ void __launch_bounds__(kTotThreads) scan_totals_kernel(double* btot, int nb, const double* partials,
                                                                  int n_part, CombState* cs, uint64_t* step,
                                                                  uint64_t seed, double* energies, int64_t e_index,
                                                                  int W) {
  __shared__ double ws[kTotThreads / 32];
  __shared__ double sums[4];
  __shared__ double carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int nw = kTotThreads / 32;
  if (threadIdx.x == 0) carry = 0.0;
  __syncthreads();
  for (int base = 0; base < nb; base += kTotThreads) {
    const int i = base + threadIdx.x;
    const double x = i < nb ? btot[i] : 0.0;
    double v = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += t;
    }
    if (lane == 31) ws[warp] = v;
    __syncthreads();
    if (warp == 0) {
      double q = lane < nw ? ws[lane] : 0.0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double t = __shfl_up_sync(0xffffffffu, q, o);
        if (lane >= o) q += t;
      }
      if (lane < nw) ws[lane] = q;
    }
    __syncthreads();
    const double incl = v + (warp > 0 ? ws[warp - 1] : 0.0);
    const double c0 = carry;
    if (i < nb) btot[i] = c0 + incl - x;  // offset of block i
    __syncthreads();
    if (threadIdx.x == kTotThreads - 1) carry = c0 + incl;
    __syncthreads();
  }
  if (warp < 4) {  // partials rows: sum E_old, accepted, proposed, walkers on a node
    double q = 0.0;
    for (int r = lane; r < n_part; r += 32) q += partials[(size_t)r * 4 + warp];
    q = warp_sum(q);
    if (lane == 0) sums[warp] = q;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    cs->total = carry;
    const uint4 u = draw4(seed, 0u, (uint32_t)(*step), 0u, kTagComb);
    cs->u = u01<double>(u.x);
    energies[e_index] = sums[0] / ((double)W - sums[3]);  // over the walkers with weight
    cs->accepted += sums[1];
    cs->proposed += sums[2];
    cs->killed += sums[3];
    *step += 1;
  }
}

// New walker k copies parent j, the first index whose cumulative weight
// exceeds (k + u) * total / W.
__global__ void comb_gather_kernel(const double* pos_in, const double* eloc_in, double* pos_out, double* eloc_out,
                                   const double* cum, const double* boff, int nb, const CombState* cs, int W,
                                   int NC) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= W) return;
  const double target = ((double)k + cs->u) * (cs->total / (double)W);
  int lo = 0, hi = nb - 1;  // last block with boff <= target
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (boff[mid] <= target) lo = mid;
    else hi = mid - 1;
  }
  const int b = lo;
  const double off = boff[b];
  int a = b * kScanBlock, z = min(W, a + kScanBlock) - 1;  // first i with off + cum[i] > target
  while (a < z) {
    const int mid = (a + z) >> 1;
    if (off + cum[mid] > target) z = mid;
    else a = mid + 1;
  }
  const int j = a;
  for (int c = 0; c < NC; ++c) pos_out[(size_t)c * W + k] = pos_in[(size_t)c * W + j];
  eloc_out[k] = eloc_in[j];
}

// ------------------------------------------------------------- FMA probes

template <class T>
__global__ void fma_probe_kernel(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
template __global__ void fma_probe_kernel<double>(double*, int, double, double);
template __global__ void fma_probe_kernel<float>(float*, int, float, float);

cudaError_t launch_init_positions(double* pos, int W, int N, uint64_t seed, int kind, double width, cudaStream_t s) {
  const int n = W * N;
  init_positions_kernel<<<(n + 255) / 256, 256, 0, s>>>(pos, W, N, seed, kind, width);
  return cudaGetLastError();
}
cudaError_t launch_aos_to_soa(const double* aos, double* soa, int W, int NC, cudaStream_t s) {
  const size_t n = (size_t)W * NC;
  aos_to_soa_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(aos, soa, W, NC);
  return cudaGetLastError();
}
cudaError_t launch_soa_to_aos(const double* soa, double* aos, int W, int NC, cudaStream_t s) {
  const size_t n = (size_t)W * NC;
  soa_to_aos_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(soa, aos, W, NC);
  return cudaGetLastError();
}
cudaError_t launch_reduce_columns(const double* part, int rows, int cols, double* out, cudaStream_t s) {
  reduce_columns_kernel<<<(cols + 127) / 128, 128, 0, s>>>(part, rows, cols, out);
  return cudaGetLastError();
}
cudaError_t launch_unpack_vmc_sums(const double* red, int PM, int P, double* moments, double* sr, cudaStream_t s) {
  unpack_vmc_sums_kernel<<<1, 32, 0, s>>>(red, PM, P, moments, sr);
  return cudaGetLastError();
}
cudaError_t launch_comb(const double* weight, double* cum, double* btot, int nb, const double* partials, int n_part,
                        CombState* cs, uint64_t* step, uint64_t seed, double* energies, int64_t e_index,
                        const double* pos_in, const double* eloc_in, double* pos_out, double* eloc_out, int W, int NC,
                        cudaStream_t s) {
  scan_blocks_kernel<<<nb, kScanBlock, 0, s>>>(weight, cum, btot, W);
  scan_totals_kernel<<<1, kTotThreads, 0, s>>>(btot, nb, partials, n_part, cs, step, seed, energies, e_index, W);
  comb_gather_kernel<<<(W + 127) / 128, 128, 0, s>>>(pos_in, eloc_in, pos_out, eloc_out, cum, btot, nb, cs, W, NC);
  return cudaGetLastError();
}
cudaError_t launch_fma_probe64(double* out, int blocks, int threads, int iters, cudaStream_t s) {
  fma_probe_kernel<double><<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);
  return cudaGetLastError();
}
cudaError_t launch_fma_probe32(float* out, int blocks, int threads, int iters, cudaStream_t s) {
  fma_probe_kernel<float><<<blocks, threads, 0, s>>>(out, iters, 0.999999f, 1e-7f);
  return cudaGetLastError();
}

}  // namespace mole
