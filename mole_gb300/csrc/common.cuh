// common.cuh -- shared device helpers for the mole GB300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>
#include <utility>

namespace mole {

constexpr int kMaxNuc = 8;
constexpr int kMaxBasis = 32;
constexpr int kMaxSpin = 5;
constexpr int kMaxElec = 2 * kMaxSpin;
constexpr int kMaxPoly = 4;
constexpr int kNnH = 64;
constexpr int kNnIn = 4;
constexpr int kNnNetP = kNnH * kNnIn + kNnH + kNnH * kNnH + kNnH + kNnH + 1;  // 4545
constexpr int kNnP = 2 * kNnNetP;                                             // 9090

// Random-stream tags: the fourth Philox counter word separates the streams.
constexpr uint32_t kTagMove = 0x4d4f5645u;  // 'MOVE'
constexpr uint32_t kTagInit = 0x494e4954u;  // 'INIT'
constexpr uint32_t kTagComb = 0x434f4d42u;  // 'COMB'

enum { kMoveBox = 0, kMoveGauss = 1, kMoveDiffuse = 2 };
enum { kSto1s = 0, kSto2s = 1, kSto2px = 2, kSto2py = 3, kSto2pz = 4, kGto1s = 5 };

// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, SC'11):
// ten rounds of two 32x32->64 multiplies with Weyl-sequence key bumps.
__host__ __device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k.x += 0x9E3779B9u;
      k.y += 0xBB67AE85u;
    }
#ifdef __CUDA_ARCH__
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), hi1 = __umulhi(0xCD9E8D57u, c.z);
#else
    const uint32_t hi0 = (uint32_t)(((uint64_t)0xD2511F53u * c.x) >> 32);
    const uint32_t hi1 = (uint32_t)(((uint64_t)0xCD9E8D57u * c.z) >> 32);
#endif
    const uint32_t lo0 = 0xD2511F53u * c.x, lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
  }
  return c;
}

__host__ __device__ __forceinline__ uint4 draw4(uint64_t seed, uint32_t a, uint32_t b, uint32_t c, uint32_t tag) {
  return philox4x32_10(make_uint4(a, b, c, tag), make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
}

// Uniform in (0, 1) from 32 random bits.
template <class R>
__device__ __forceinline__ R u01(uint32_t x) {
  return ((R)x + (R)0.5) * (R)(1.0 / 4294967296.0);
}

// Box-Muller pair.
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, double& z0, double& z1) {
  const double r = sqrt(-2.0 * log(u01<double>(a)));
  double s, c;
  sincospi(2.0 * u01<double>(b), &s, &c);
  z0 = r * c;
  z1 = r * s;
}
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float& z0, float& z1) {
  const float r = sqrtf(-2.0f * __logf(u01<float>(a)));
  float s, c;
  __sincosf(6.283185307179586f * u01<float>(b), &s, &c);
  z0 = r * c;
  z1 = r * s;
}

template <int B, int E, class F>
__device__ __forceinline__ void static_for(F&& f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    static_for<B + 1, E>(f);
  }
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of K doubles per thread, deterministic order; the result is
// valid in thread 0. scratch holds K * (blockDim.x / 32) doubles.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) scratch[k * nw + warp] = v[k];
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double s = 0.0;
      for (int i = 0; i < nw; ++i) s += scratch[k * nw + i];
      v[k] = s;
    }
  __syncthreads();
}

}  // namespace mole
