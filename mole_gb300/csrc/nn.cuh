// nn.cuh -- the pairwise neural Jastrow on the device.
//
// J_nn = sum_{i<j} f_ee(r_ij, s_ij) + sum_{i,I} f_en(r_iI, Z_I), each f a
// 4 -> 64 -> 64 -> 1 tanh MLP of the features x = [r, e^-r, s r, s e^-r]
// (s = 1 for a same-spin pair, 0 otherwise; s = Z_I for e-n). The parameter
// layout of one net (4,545 values) is W1[64][4], b1[64], W2[64][64], b2[64],
// w3[64], b3; the e-e net precedes the e-n net.
//
// Shared-memory image of one net (NnNet<R>): W1, b1, W2 transposed to
// W2T[c][a] so that sixteen consecutive outputs a of input c are one aligned
// 64-byte run (four 16-byte broadcast loads in FP32), b2, w3, b3.
#pragma once

#include "common.cuh"

namespace mole {

constexpr int kNnOffW1 = 0;
constexpr int kNnOffB1 = kNnH * kNnIn;
constexpr int kNnOffW2 = kNnOffB1 + kNnH;
constexpr int kNnOffB2 = kNnOffW2 + kNnH * kNnH;
constexpr int kNnOffW3 = kNnOffB2 + kNnH;
constexpr int kNnOffB3 = kNnOffW3 + kNnH;

template <class R>
struct NnNet {
  R W2T[kNnH][kNnH];  // first: 16-byte aligned rows
  R W1[kNnH][kNnIn];
  R b1[kNnH];
  R b2[kNnH];
  R w3[kNnH];
  R b3;
  R pad[3];
};

// Both nets plus the per-thread scratch for the hidden-layer jets
// (value, d/dr, d2/dr2 of 64 units), laid out [unit][jet][thread].
template <class R>
struct NnShared {
  NnNet<R> net[2];
};

template <class R>
__host__ __device__ constexpr size_t nn_smem_bytes(int threads) {
  return sizeof(NnShared<R>) + sizeof(R) * 3 * kNnH * (size_t)threads;
}

template <class R>
__device__ __forceinline__ R exp_nn(R x);
template <>
__device__ __forceinline__ double exp_nn<double>(double x) {
  return exp(x);
}
template <>
__device__ __forceinline__ float exp_nn<float>(float x) {
  return __expf(x);
}

template <class R>
__device__ __forceinline__ R tanh_t(R z);
template <>
__device__ __forceinline__ double tanh_t<double>(double z) {
  return tanh(z);
}
template <>
__device__ __forceinline__ float tanh_t<float>(float z) {
  // 1 - 2 / (e^{2z} + 1), saturating correctly for large |z|
  const float e = __expf(2.0f * z);
  return 1.0f - __fdividef(2.0f, e + 1.0f);
}

// Loads the FP64 parameter image (two nets, 9,090 values) into shared memory
// as R, transposing W2. Cooperative over the CTA; ends with __syncthreads.
template <class R>
__device__ __forceinline__ void nn_load(NnShared<R>* sh, const double* theta) {
  for (int i = threadIdx.x; i < 2 * kNnNetP; i += blockDim.x) {
    const int n = i / kNnNetP, k = i % kNnNetP;
    NnNet<R>& net = sh->net[n];
    const R v = (R)theta[i];
    if (k < kNnOffB1) net.W1[k / kNnIn][k % kNnIn] = v;
    else if (k < kNnOffW2) net.b1[k - kNnOffB1] = v;
    else if (k < kNnOffB2) {
      const int j = k - kNnOffW2;
      net.W2T[j % kNnH][j / kNnH] = v;  // W2[a][c] -> W2T[c][a]
    } else if (k < kNnOffW3) net.b2[k - kNnOffB2] = v;
    else if (k < kNnOffB3) net.w3[k - kNnOffW3] = v;
    else net.b3 = v;
  }
  __syncthreads();
}

// y, dy/dr, d2y/dr2 of one net at distance r with feature flag s. `scr`
// points at this thread's jet scratch: element (unit c, jet j) at
// scr[(3 c + j) * stride].
template <class R>
__device__ __forceinline__ void nn_jet(const NnNet<R>& net, R r, R s, R* scr, int stride, R& y, R& dy, R& d2y) {
  const R er = exp_nn(-r);
  const R x0 = r, x1 = er, x2 = s * r, x3 = s * er;
  const R p1 = -er, p3 = -s * er;  // d x / dr = [1, -er, s, -s er]
  const R q1 = er, q3 = s * er;    // d2 x / dr2 = [0, er, 0, s er]
#pragma unroll 4
  for (int c = 0; c < kNnH; ++c) {
    const R w0 = net.W1[c][0], w1 = net.W1[c][1], w2 = net.W1[c][2], w3 = net.W1[c][3];
    const R z = net.b1[c] + w0 * x0 + w1 * x1 + w2 * x2 + w3 * x3;
    const R z1 = w0 + w1 * p1 + w2 * s + w3 * p3;
    const R z2 = w1 * q1 + w3 * q3;
    const R t = tanh_t<R>(z), sd = (R)1 - t * t;
    scr[(3 * c) * stride] = t;
    scr[(3 * c + 1) * stride] = sd * z1;
    scr[(3 * c + 2) * stride] = sd * z2 - (R)2 * t * sd * z1 * z1;
  }
  R out = net.b3, out1 = 0, out2 = 0;
  constexpr int G = 16;
  for (int a0 = 0; a0 < kNnH; a0 += G) {
    R acc0[G], acc1[G], acc2[G];
#pragma unroll
    for (int i = 0; i < G; ++i) {
      acc0[i] = net.b2[a0 + i];
      acc1[i] = 0;
      acc2[i] = 0;
    }
#pragma unroll 2
    for (int c = 0; c < kNnH; ++c) {
      const R h = scr[(3 * c) * stride], h1 = scr[(3 * c + 1) * stride], h2 = scr[(3 * c + 2) * stride];
      const R* w = &net.W2T[c][a0];
#pragma unroll
      for (int i = 0; i < G; ++i) {
        acc0[i] += w[i] * h;
        acc1[i] += w[i] * h1;
        acc2[i] += w[i] * h2;
      }
    }
#pragma unroll
    for (int i = 0; i < G; ++i) {
      const R t = tanh_t<R>(acc0[i]), sd = (R)1 - t * t, v = net.w3[a0 + i];
      out += v * t;
      out1 += v * sd * acc1[i];
      out2 += v * (sd * acc2[i] - (R)2 * t * sd * acc1[i] * acc1[i]);
    }
  }
  y = out;
  dy = out1;
  d2y = out2;
}

}  // namespace mole
