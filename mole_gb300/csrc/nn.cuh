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
//
// The features of a pair are functions of its distance r alone, so for a
// fixed pair type -- e-e same spin (s = 1), e-e opposite spin (s = 0), e-n
// on nucleus I (s = Z_I) -- the network output is a smooth function y(r).
// The FP32 form does not run the MLP in the sweep: after every parameter
// change nn_table_kernel evaluates y, dy/dr and d2y/dr2 in FP64 at the nodes
// nodes of [0, 340) bohr and stores, per interval, the coefficients of the
// quintic Hermite interpolant through (y, y', y'') at both ends; the sweep
// kernels evaluate that quintic (error O(h^6 y^(6)), below FP32 rounding for
// these networks at h = 1/64 bohr). The FP64 form evaluates the MLP directly
// (nn_jet).
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

// ------------------------------------------------------------ tabulated form

// Each pair type's table has two segments of quintic intervals: [0, 20) bohr
// at h = 1/64 and [20, 340) bohr at h = 1/4; beyond 340 bohr the term is
// frozen at its value there (no electron of a bound system gets there).
constexpr int kNnTabSeg = 1280;                          // intervals per segment
constexpr double kNnTabH = 1.0 / 64.0;                   // near spacing (bohr)
constexpr double kNnTabHFar = 1.0 / 4.0;                 // far spacing
constexpr double kNnTabRnear = kNnTabSeg * kNnTabH;      // 20 bohr
constexpr int kNnTabIntervals = 2 * kNnTabSeg;           // per pair type
constexpr int kNnTabNodes = 2 * (kNnTabSeg + 1);         // per pair type (both segments' ends)
constexpr int kNnTabMax = 2 + kMaxNuc;                   // e-e same, e-e opposite, e-n per nucleus
constexpr int kNnTabFloats = 8;                          // c0..c5 of the quintic, two pad
__host__ __device__ constexpr size_t nn_tab_floats(int n_nuc) {
  return (size_t)(2 + n_nuc) * kNnTabIntervals * kNnTabFloats;
}
__host__ __device__ inline double nn_tab_node_r(int n) {
  return n <= kNnTabSeg ? n * kNnTabH : kNnTabRnear + (n - kNnTabSeg - 1) * kNnTabHFar;
}

// y, y', y'' of one net at distance r, feature flag s, in FP64, reading the
// FP64 parameters of that net (4,545 values) straight from global memory.
__device__ inline void nn_jet_global(const double* th, double r, double s, double& y, double& dy,
                                           double& d2y) {
  const double er = exp(-r);
  const double x[kNnIn] = {r, er, s * r, s * er};
  const double p[kNnIn] = {1.0, -er, s, -s * er};
  const double q[kNnIn] = {0.0, er, 0.0, s * er};
  double h[kNnH], h1[kNnH], h2[kNnH];
  for (int c = 0; c < kNnH; ++c) {
    double z = th[kNnOffB1 + c], z1 = 0.0, z2 = 0.0;
#pragma unroll
    for (int k = 0; k < kNnIn; ++k) {
      const double w = th[kNnOffW1 + c * kNnIn + k];
      z += w * x[k];
      z1 += w * p[k];
      z2 += w * q[k];
    }
    const double t = tanh(z), sd = 1.0 - t * t;
    h[c] = t;
    h1[c] = sd * z1;
    h2[c] = sd * z2 - 2.0 * t * sd * z1 * z1;
  }
  double out = th[kNnOffB3], out1 = 0.0, out2 = 0.0;
  for (int a = 0; a < kNnH; ++a) {
    double z = th[kNnOffB2 + a], z1 = 0.0, z2 = 0.0;
    for (int c = 0; c < kNnH; ++c) {
      const double w = th[kNnOffW2 + a * kNnH + c];
      z += w * h[c];
      z1 += w * h1[c];
      z2 += w * h2[c];
    }
    const double t = tanh(z), sd = 1.0 - t * t, v = th[kNnOffW3 + a];
    out += v * t;
    out1 += v * sd * z1;
    out2 += v * (sd * z2 - 2.0 * t * sd * z1 * z1);
  }
  y = out;
  dy = out1;
  d2y = out2;
}

// Pair type of table k: the net (0 e-e, 1 e-n).
__host__ __device__ inline int nn_tab_net(int k) { return k < 2 ? 0 : 1; }

// Builds the 2 + n_nuc tables of a system from its FP64 network parameters:
// node values y, y', y'' in FP64 (node scratch: (2 + n_nuc) x kNnTabNodes x 3
// doubles), then the FP32 quintic coefficients of every interval.
// Table 0 is the e-e net at s = 1 (same spin), 1 at s = 0, 2 + I the e-n
// net at s = Z_I.
cudaError_t launch_nn_tables(const double* theta, int n_nuc, const double* nuc_z, double* node, float* tab,
                             cudaStream_t s);

// y, y', y'' of pair type k at distance r from its quintic table (FP32).
__device__ __forceinline__ void nn_tab_eval(const float* tab, int k, float r, float& y, float& dy, float& d2y) {
  const float u = r * (float)(1.0 / kNnTabH);
  int i;
  float t, ih;
  if (u < (float)kNnTabSeg) {
    i = (int)u;
    t = u - (float)i;
    ih = (float)(1.0 / kNnTabH);
  } else {
    const float v = (r - (float)kNnTabRnear) * (float)(1.0 / kNnTabHFar);
    ih = (float)(1.0 / kNnTabHFar);
    if (v < (float)kNnTabSeg) {
      i = (int)v;
      t = v - (float)i;
    } else {
      i = kNnTabSeg - 1;
      t = 1.f;
      ih = 0.f;  // frozen beyond the table
    }
    i += kNnTabSeg;
  }
  const float4* c = reinterpret_cast<const float4*>(tab + ((size_t)k * kNnTabIntervals + i) * kNnTabFloats);
  const float4 a = __ldg(c), b = __ldg(c + 1);  // c0 c1 c2 c3 | c4 c5 - -
  y = a.x + t * (a.y + t * (a.z + t * (a.w + t * (b.x + t * b.y))));
  dy = (a.y + t * (2.f * a.z + t * (3.f * a.w + t * (4.f * b.x + t * 5.f * b.y)))) * ih;
  d2y = (2.f * a.z + t * (6.f * a.w + t * (12.f * b.x + t * 20.f * b.y))) * (ih * ih);
}

// Builds the 2 + n_nuc tables of a system from its FP64 network parameters:
// node values y, y', y'' in FP64 (node scratch: (2 + n_nuc) x kNnTabNodes x 3
// doubles), then the FP32 quintic coefficients of every interval.
// Table 0 is the e-e net at s = 1 (same spin), 1 at s = 0, 2 + I the e-n
// net at s = Z_I.
cudaError_t launch_nn_tables(const double* theta, int n_nuc, const double* nuc_z, double* node, float* tab,
                             cudaStream_t s);

// y, y', y'' of pair type k at distance r from its quintic table (FP32),
// or from the direct FP64 MLP beyond the table.
__device__ __forceinline__ void nn_tab_eval(const float* tab, const double* theta, int k, float s, float r, float& y,
                                            float& dy, float& d2y) {
  const float u = r * (float)(1.0 / kNnTabH);
  if (u < (float)kNnTabIntervals) {
    const int i = (int)u;
    const float t = u - (float)i;
    const float4* c = reinterpret_cast<const float4*>(tab + ((size_t)k * kNnTabIntervals + i) * kNnTabFloats);
    const float4 a = __ldg(c), b = __ldg(c + 1);  // c0 c1 c2 c3 | c4 c5 - -
    y = a.x + t * (a.y + t * (a.z + t * (a.w + t * (b.x + t * b.y))));
    dy = (a.y + t * (2.f * a.z + t * (3.f * a.w + t * (4.f * b.x + t * 5.f * b.y)))) * (float)(1.0 / kNnTabH);
    d2y = (2.f * a.z + t * (6.f * a.w + t * (12.f * b.x + t * 20.f * b.y))) * (float)(1.0 / (kNnTabH * kNnTabH));
  } else {
    double yy, y1, y2;
    nn_jet_global(theta + nn_tab_net(k) * kNnNetP, (double)r, (double)s, yy, y1, y2);
    y = (float)yy;
    dy = (float)y1;
    d2y = (float)y2;
  }
}

}  // namespace mole
