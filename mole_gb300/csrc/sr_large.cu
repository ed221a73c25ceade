// sr_large.cu -- O_k of the neural Jastrow, the tensor-core S-matrix build
// and the FP64 CG solve for stochastic reconfiguration with many parameters.
#include <cuda_bf16.h>

#include <algorithm>

#include "sr_large.cuh"

namespace mole {

// --------------------------------------------------------------- O_k (network)

constexpr int kNnMaxPairs = 8;
constexpr int kOgenWarps = 8;    // walkers in flight per CTA of the plain form (one per warp)
constexpr int kOgenPB = 4;       // pairs per GEMV pass: each weight load feeds kOgenPB FMAs
constexpr int kW2Ld = kNnH + 1;  // padded row of the transposed W2: conflict-free both ways
constexpr int kNnSmall = kNnNetP - kNnH * kNnH;  // a net's parameters besides W2 (449)

struct NetWeights {
  float W2p[2][kNnH][kW2Ld];  // W2p[net][c][a] = W2[a][c]
  float W1[2][kNnH][kNnIn], b1[2][kNnH], b2[2][kNnH], w3[2][kNnH];
};

__device__ __forceinline__ void load_net_weights(NetWeights& sh, const SysParams<float>& sp) {
  for (int i = threadIdx.x; i < 2 * kNnH * kNnH; i += blockDim.x) {
    const int n = i / (kNnH * kNnH), j = i % (kNnH * kNnH);
    sh.W2p[n][j % kNnH][j / kNnH] = (float)sp.nn_theta[n * kNnNetP + kNnOffW2 + j];
  }
  for (int i = threadIdx.x; i < 2 * kNnH; i += blockDim.x) {
    const int n = i / kNnH, u = i % kNnH;
    const double* th = sp.nn_theta + n * kNnNetP;
#pragma unroll
    for (int k = 0; k < kNnIn; ++k) sh.W1[n][u][k] = (float)th[kNnOffW1 + u * kNnIn + k];
    sh.b1[n][u] = (float)th[kNnOffB1 + u];
    sh.b2[n][u] = (float)th[kNnOffB2 + u];
    sh.w3[n][u] = (float)th[kNnOffW3 + u];
  }
}

// The lane's gradients besides W2: units lane and lane + 32.
struct NetGrads {
  float W1[2][kNnIn], b1[2], b2[2], w3[2];
};

// Per-warp staging of a walker's pairs, unit-major with the pairs innermost:
// hs[u][p] = h1 of unit u for pair p, ds[u][p] = delta2. A GEMV reads four
// pairs' values of one unit with one broadcast 128-bit load; the h1 rows are
// padded to 12 floats so that lanes reading their own unit's row (32 lanes,
// 48-byte stride) hit distinct banks.
constexpr int kHsLd = 12;
typedef float HsRow[kHsLd];
typedef float DsRow[kNnMaxPairs];

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float a, float b, float c, float d) {
  *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}

// Forward and backward pass of net `net` over one walker's pairs, one warp:
// lane l owns hidden units l and l + 32, whose first-layer weights, biases
// and output weights sit in registers, W2 (transposed, rows padded to 65
// floats so that both the forward and the backward GEMV read it without bank
// conflicts) in shared memory. The pairs go through the two 64 x 64 GEMVs
// kOgenPB at a time: each weight load feeds kOgenPB FMAs, and the other
// units' activations arrive as one broadcast load of hs / ds per unit.
// Leaves h1 and delta2 of every pair in hs and ds (pairs np .. 7 of a group
// hold zeros; groups past np are not written) and the lane's other
// gradients in g. xv: lane t holds coordinate t of the walker.
__device__ __forceinline__ void net_pass(const NetWeights& sh, const SysParams<float>& sp, int net, int N, int n_up,
                                         float xv, int lane, HsRow* hs, DsRow* ds, NetGrads& g) {
  const int n_b = net == 0 ? N : sp.n_nuc;
  const int np = net == 0 ? N * (N - 1) / 2 : N * sp.n_nuc;
  float W1n[2][kNnIn], b1n[2], b2n[2], w3n[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int u = lane + 32 * h;
#pragma unroll
    for (int k = 0; k < kNnIn; ++k) W1n[h][k] = sh.W1[net][u][k];
    b1n[h] = sh.b1[net][u];
    b2n[h] = sh.b2[net][u];
    w3n[h] = sh.w3[net][u];
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
#pragma unroll
    for (int k = 0; k < kNnIn; ++k) g.W1[h][k] = 0.f;
    g.b1[h] = g.b2[h] = g.w3[h] = 0.f;
  }
#pragma unroll
  for (int p0 = 0; p0 < kNnMaxPairs; p0 += kOgenPB) {
    if (p0 >= np) break;
    float xf[kOgenPB][kNnIn], h1[kOgenPB][2];
    bool valid[kOgenPB];
#pragma unroll
    for (int q = 0; q < kOgenPB; ++q) {
      const int p = p0 + q;
      valid[q] = p < np;
      // pair p -> (i, j): e-e pairs i < j in order, e-n pairs (electron, nucleus)
      int i = 0, j = 0;
      if (net == 0) {
        int rem = valid[q] ? p : 0;
        while (rem >= N - 1 - i) {
          rem -= N - 1 - i;
          ++i;
        }
        j = i + 1 + rem;
      } else {
        i = valid[q] ? p / n_b : 0;
        j = valid[q] ? p % n_b : 0;
      }
      float d0 = __shfl_sync(0xffffffffu, xv, 3 * i), d1 = __shfl_sync(0xffffffffu, xv, 3 * i + 1),
            dd2 = __shfl_sync(0xffffffffu, xv, 3 * i + 2), s;
      if (net == 0) {
        d0 -= __shfl_sync(0xffffffffu, xv, 3 * j);
        d1 -= __shfl_sync(0xffffffffu, xv, 3 * j + 1);
        dd2 -= __shfl_sync(0xffffffffu, xv, 3 * j + 2);
        s = ((i < n_up) == (j < n_up)) ? 1.f : 0.f;
      } else {
        d0 -= sp.nuc_pos[3 * j];
        d1 -= sp.nuc_pos[3 * j + 1];
        dd2 -= sp.nuc_pos[3 * j + 2];
        s = sp.nuc_z[j];
      }
      const float r = sqrtf(d0 * d0 + d1 * d1 + dd2 * dd2);
      const float er = expf(-r);
      xf[q][0] = r;
      xf[q][1] = er;
      xf[q][2] = s * r;
      xf[q][3] = s * er;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float z = b1n[h];
#pragma unroll
        for (int k = 0; k < kNnIn; ++k) z += W1n[h][k] * xf[q][k];
        h1[q][h] = valid[q] ? tanhf(z) : 0.f;
      }
    }
    st4(&hs[lane][p0], h1[0][0], h1[1][0], h1[2][0], h1[3][0]);
    st4(&hs[lane + 32][p0], h1[0][1], h1[1][1], h1[2][1], h1[3][1]);
    __syncwarp();
    // layer 2: a2[a] = b2[a] + sum_c W2[a][c] h1[c], a = lane, lane + 32
    float a2[kOgenPB][2];
#pragma unroll
    for (int q = 0; q < kOgenPB; ++q) a2[q][0] = b2n[0], a2[q][1] = b2n[1];
#pragma unroll 8
    for (int c = 0; c < kNnH; ++c) {
      const float w0 = sh.W2p[net][c][lane], w1 = sh.W2p[net][c][lane + 32];
      const float4 hv = ld4(&hs[c][p0]);
      const float hq[4] = {hv.x, hv.y, hv.z, hv.w};
#pragma unroll
      for (int q = 0; q < kOgenPB; ++q) {
        a2[q][0] += w0 * hq[q];
        a2[q][1] += w1 * hq[q];
      }
    }
    float d2v[kOgenPB][2];
#pragma unroll
    for (int q = 0; q < kOgenPB; ++q)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float h2 = tanhf(a2[q][h]);
        const float dl2 = valid[q] ? w3n[h] * (1.f - h2 * h2) : 0.f;
        d2v[q][h] = dl2;
        g.b2[h] += dl2;
        g.w3[h] += valid[q] ? h2 : 0.f;
      }
    st4(&ds[lane][p0], d2v[0][0], d2v[1][0], d2v[2][0], d2v[3][0]);
    st4(&ds[lane + 32][p0], d2v[0][1], d2v[1][1], d2v[2][1], d2v[3][1]);
    __syncwarp();
    // back to layer 1: s1[c] = sum_a W2[a][c] delta2[a], c = lane, lane + 32
    float s1[kOgenPB][2] = {};
#pragma unroll 8
    for (int a = 0; a < kNnH; ++a) {
      const float w0 = sh.W2p[net][lane][a], w1 = sh.W2p[net][lane + 32][a];
      const float4 dv = ld4(&ds[a][p0]);
      const float dq[4] = {dv.x, dv.y, dv.z, dv.w};
#pragma unroll
      for (int q = 0; q < kOgenPB; ++q) {
        s1[q][0] += w0 * dq[q];
        s1[q][1] += w1 * dq[q];
      }
    }
#pragma unroll
    for (int q = 0; q < kOgenPB; ++q)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float dl1 = s1[q][h] * (1.f - h1[q][h] * h1[q][h]);  // zero for an invalid pair
        g.b1[h] += dl1;
#pragma unroll
        for (int k = 0; k < kNnIn; ++k) g.W1[h][k] += dl1 * xf[q][k];
      }
  }
}

struct OgenShared {
  NetWeights wt;
  HsRow hs[kOgenWarps][kNnH];
  DsRow ds[kOgenWarps][kNnH];
};

// d J_nn / d theta of one walker per warp, as rows of O (type T): walker w's
// row at O + w ldO, the network's columns from col0 on. J_nn = sum over pairs
// of y(pair), so every gradient is a sum over the walker's pairs (6 e-e, 8
// e-n for LiH). dJ/dW2[a][c] = sum_p delta2[p][a] h1[p][c] is formed with h1
// in registers and delta2 broadcast from shared memory, and written row by
// row in 128-byte segments. Walkers w < nw; W is the stride of pos.
template <class T>
__global__ void __launch_bounds__(kOgenWarps * 32, 2) nn_ogen_kernel(const __grid_constant__ SysParams<float> sp,
                                                                 const double* pos, int W, int nw, int n_up, int N,
                                                                 T* O, int ldO, int col0) {
  extern __shared__ __align__(16) unsigned char ogen_smem[];
  OgenShared& sh = *reinterpret_cast<OgenShared*>(ogen_smem);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  load_net_weights(sh.wt, sp);
  __syncthreads();
  const int n_warps = gridDim.x * kOgenWarps;
  for (int w = blockIdx.x * kOgenWarps + warp; w < nw; w += n_warps) {
    // the walker's coordinates, lane t holding coordinate t (FP32: these O_k are FP32 quantities)
    const float xv = lane < 3 * N ? (float)pos[(size_t)lane * W + w] : 0.f;
    T* out = O + (size_t)w * ldO + col0;
#pragma unroll 1
    for (int net = 0; net < 2; ++net) {
      const int np = net == 0 ? N * (N - 1) / 2 : N * sp.n_nuc;
      NetGrads g;
      net_pass(sh.wt, sp, net, N, n_up, xv, lane, sh.hs[warp], sh.ds[warp], g);
      __syncwarp();
      float h1k[2][kNnMaxPairs];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float4 x = ld4(&sh.hs[warp][lane + 32 * h][0]), y = ld4(&sh.hs[warp][lane + 32 * h][4]);
        h1k[h][0] = x.x, h1k[h][1] = x.y, h1k[h][2] = x.z, h1k[h][3] = x.w;
        h1k[h][4] = y.x, h1k[h][5] = y.y, h1k[h][6] = y.z, h1k[h][7] = y.w;
      }
      T* o = out + net * kNnNetP;
      // dJ/dW2[a][c] = sum_p delta2[p][a] h1[p][c]: lane writes columns lane and lane + 32 of each row a
#pragma unroll 4
      for (int a = 0; a < kNnH; ++a) {
        const float4 x = ld4(&sh.ds[warp][a][0]), y = ld4(&sh.ds[warp][a][4]);
        const float dv[kNnMaxPairs] = {x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
        float g0 = 0.f, g1 = 0.f;
#pragma unroll
        for (int p = 0; p < kNnMaxPairs; ++p)
          if (p < np) {
            g0 += dv[p] * h1k[0][p];
            g1 += dv[p] * h1k[1][p];
          }
        o[kNnOffW2 + a * kNnH + lane] = (T)g0;
        o[kNnOffW2 + a * kNnH + lane + 32] = (T)g1;
      }
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int u = lane + 32 * h;
#pragma unroll
        for (int k = 0; k < kNnIn; ++k) o[kNnOffW1 + u * kNnIn + k] = (T)g.W1[h][k];
        o[kNnOffB1 + u] = (T)g.b1[h];
        o[kNnOffB2 + u] = (T)g.b2[h];
        o[kNnOffW3 + u] = (T)g.w3[h];
      }
      if (lane == 0) o[kNnOffB3] = (T)np;
      __syncwarp();
    }
  }
}

static bool ogen_pairs_ok(const SysParams<float>& sp, int n_elec) {
  return n_elec * (n_elec - 1) / 2 <= kNnMaxPairs && n_elec * sp.n_nuc <= kNnMaxPairs && 3 * n_elec <= 32;
}

template <class T>
static cudaError_t launch_nn_ogen_t(const SysParams<float>& sp, const double* pos, int W, int nw, int n_up,
                                   int n_elec, T* O, int ldO, int col0, int grid, cudaStream_t s) {
  // `grid` bounds the walkers in flight (the callers pass about 3 per SM)
  if (!ogen_pairs_ok(sp, n_elec) || nw > W) return cudaErrorInvalidValue;
  if (nw <= 0) return cudaSuccess;
  const size_t smem = sizeof(OgenShared);
  cudaError_t e = cudaFuncSetAttribute(nn_ogen_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int ctas = std::max(1, std::min((nw + kOgenWarps - 1) / kOgenWarps, 2 * ((grid + 2) / 3)));
  nn_ogen_kernel<T><<<ctas, kOgenWarps * 32, smem, s>>>(sp, pos, W, nw, n_up, n_elec, O, ldO, col0);
  return cudaGetLastError();
}
cudaError_t launch_nn_ogen(const SysParams<float>& sp, const double* pos, int W, int nw, int n_up, int n_elec,
                           float* O, int ldO, int col0, int grid, cudaStream_t s) {
  return launch_nn_ogen_t<float>(sp, pos, W, nw, n_up, n_elec, O, ldO, col0, grid, s);
}
cudaError_t launch_nn_ogen64(const SysParams<float>& sp, const double* pos, int W, int n_up, int n_elec, double* O,
                             int ldO, int col0, int grid, cudaStream_t s) {
  return launch_nn_ogen_t<double>(sp, pos, W, W, n_up, n_elec, O, ldO, col0, grid, s);
}

// ------------------------------------------------ SR sample: O_k -> bf16 rows

// One SR sample's operand rows Ob[w][p] = bf16(O_wp - c_p) and the per-CTA
// sums of O - c and E (O - c), without the FP32 O leaving the SM. A CTA of
// kSampWarps warps takes walkers in batches of kSampWarps, per net in two
// phases:
//  A. each warp runs net_pass over its walker, leaving delta2 and h1 of every
//     pair (its hs / ds staging) and the 449 gradients besides W2 in shared
//     memory;
//  B. the CTA forms dJ/dW2[a][c] = sum_p delta2[p][a] h1[p][c] for the
//     batch's walkers, warp k for rows 4k .. 4k + 3 and lane l for columns l
//     and l + 32, thread t for gradient t besides W2.
// Every parameter thus belongs to one thread of the CTA, which writes it for
// all the CTA's walkers and keeps its two sums in a private shared-memory
// slot: no atomics, and the sums run in a fixed order. The orbital/Pade
// columns (from Oorb) belong to threads kNnSmall + j.
constexpr int kSampWarps = 16;  // 64 W2 rows = 16 warps x 4
constexpr int kSampThreads = kSampWarps * 32;
constexpr int kSampRows = kNnH / kSampWarps;
constexpr int kSampNetAcc = 2 * (2 * kSampRows + 1);  // per thread and net: 8 W2 + 1 other column, O and E O
constexpr int kSampAcc = 2 + 2 * kSampNetAcc;           // both nets after an orbital/Pade column's pair

struct SampleShared {
  NetWeights wt;
  HsRow hs[kSampWarps][kNnH];          // h1 of each warp's walker (current net)
  DsRow ds[kSampWarps][kNnH];          // delta2
  float sg[kSampWarps][kNnSmall + 3];  // the gradients besides W2
  float e[kSampWarps];                 // E of each warp's walker
  float acc[kSampAcc][kSampThreads];   // per-thread sums
};
static_assert(kSampThreads >= kNnSmall + 32, "threads for the small gradients and the orbital columns");

// net-relative offset of gradient i besides W2 (W1, b1, then b2, w3, b3)
__device__ __forceinline__ int small_offset(int i) { return i < kNnOffW2 ? i : i + kNnH * kNnH; }

__global__ void __launch_bounds__(kSampThreads, 1)
    sr_sample_kernel(const __grid_constant__ SysParams<float> sp, const double* pos, int W, int n_up, int N,
                     int n_nets, const double* Oorb, int ldorb, int n_orb, const float* center, const double* E,
                     __nv_bfloat16* Ob, int ldb, int P, float* partial) {
  extern __shared__ __align__(16) unsigned char samp_smem[];
  SampleShared& sh = *reinterpret_cast<SampleShared*>(samp_smem);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (n_nets > 0) load_net_weights(sh.wt, sp);
  for (int k = 0; k < kSampAcc; ++k) sh.acc[k][tid] = 0.f;
  __syncthreads();
  const int orb = tid - kNnSmall;  // this thread's orbital/Pade column, if 0 <= orb < n_orb
  for (int base = blockIdx.x * kSampWarps; base < W; base += gridDim.x * kSampWarps) {
    const int nb = min(kSampWarps, W - base);
    const int w = base + warp;
    float xv = 0.f;
    if (w < W) {
      xv = lane < 3 * N ? (float)pos[(size_t)lane * W + w] : 0.f;
      if (lane == 0) sh.e[warp] = (float)E[w];
    }
    if (orb >= 0 && orb < n_orb) {
      const float c = center[orb];
      float so = sh.acc[0][tid], se = sh.acc[1][tid];
      for (int j = 0; j < nb; ++j) {
        const float d = (float)Oorb[(size_t)(base + j) * ldorb + orb] - c;
        Ob[(size_t)(base + j) * ldb + orb] = __float2bfloat16_rn(d);
        so += d;
        se += (float)E[base + j] * d;
      }
      sh.acc[0][tid] = so;
      sh.acc[1][tid] = se;
    }
#pragma unroll 1
    for (int net = 0; net < n_nets; ++net) {
      const int np = net == 0 ? N * (N - 1) / 2 : N * sp.n_nuc;
      const int pbase = n_orb + net * kNnNetP;
      // phase A
      if (w < W) {
        NetGrads g;
        net_pass(sh.wt, sp, net, N, n_up, xv, lane, sh.hs[warp], sh.ds[warp], g);
        float* sg = sh.sg[warp];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int u = lane + 32 * h;
#pragma unroll
          for (int k = 0; k < kNnIn; ++k) sg[kNnOffW1 + u * kNnIn + k] = g.W1[h][k];
          sg[kNnOffB1 + u] = g.b1[h];
          sg[kNnOffW2 + u] = g.b2[h];         // small index of b2
          sg[kNnOffW2 + kNnH + u] = g.w3[h];  // w3
        }
        if (lane == 0) sg[kNnSmall - 1] = (float)np;  // b3
      }
      __syncthreads();
      // phase B: W2 rows 4 warp .. 4 warp + 3, columns lane and lane + 32
      {
        const int a0 = kSampRows * warp;
        const int ab = 2 + net * kSampNetAcc;  // this net's slots (after the orbital pair)
        float cen[kSampRows][2], so[kSampRows][2], se[kSampRows][2];
#pragma unroll
        for (int r = 0; r < kSampRows; ++r)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            cen[r][h] = center[pbase + kNnOffW2 + (a0 + r) * kNnH + lane + 32 * h];
            so[r][h] = sh.acc[ab + 2 * (2 * r + h)][tid];
            se[r][h] = sh.acc[ab + 2 * (2 * r + h) + 1][tid];
          }
#pragma unroll 1
        for (int j = 0; j < nb; ++j) {
          float hv[2][kNnMaxPairs];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const float4 x = ld4(&sh.hs[j][lane + 32 * h][0]), y = ld4(&sh.hs[j][lane + 32 * h][4]);
            hv[h][0] = x.x, hv[h][1] = x.y, hv[h][2] = x.z, hv[h][3] = x.w;
            hv[h][4] = y.x, hv[h][5] = y.y, hv[h][6] = y.z, hv[h][7] = y.w;
          }
          const float e = sh.e[j];
          __nv_bfloat16* row = Ob + (size_t)(base + j) * ldb + pbase + kNnOffW2;
#pragma unroll
          for (int r = 0; r < kSampRows; ++r) {
            const float4 x = ld4(&sh.ds[j][a0 + r][0]), y = ld4(&sh.ds[j][a0 + r][4]);
            const float dv[kNnMaxPairs] = {x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
            float g0 = 0.f, g1 = 0.f;
#pragma unroll
            for (int p = 0; p < kNnMaxPairs; ++p)
              if (p < np) {
                g0 += dv[p] * hv[0][p];
                g1 += dv[p] * hv[1][p];
              }
            const float d0 = g0 - cen[r][0], d1 = g1 - cen[r][1];
            row[(a0 + r) * kNnH + lane] = __float2bfloat16_rn(d0);
            row[(a0 + r) * kNnH + lane + 32] = __float2bfloat16_rn(d1);
            so[r][0] += d0;
            so[r][1] += d1;
            se[r][0] += e * d0;
            se[r][1] += e * d1;
          }
        }
#pragma unroll
        for (int r = 0; r < kSampRows; ++r)
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            sh.acc[ab + 2 * (2 * r + h)][tid] = so[r][h];
            sh.acc[ab + 2 * (2 * r + h) + 1][tid] = se[r][h];
          }
        // the gradient besides W2 that belongs to this thread
        if (tid < kNnSmall) {
          const int col = pbase + small_offset(tid);
          const float c = center[col];
          const int sb = ab + 2 * 2 * kSampRows;
          float s0 = sh.acc[sb][tid], s1 = sh.acc[sb + 1][tid];
          for (int j = 0; j < nb; ++j) {
            const float d = sh.sg[j][tid] - c;
            Ob[(size_t)(base + j) * ldb + col] = __float2bfloat16_rn(d);
            s0 += d;
            s1 += sh.e[j] * d;
          }
          sh.acc[sb][tid] = s0;
          sh.acc[sb + 1][tid] = s1;
        }
      }
      __syncthreads();  // the batch's shared rows are free for the next net / batch
    }
  }
  // the CTA's sums, each column written by the thread it belongs to
  __syncthreads();
  float* dst = partial + (size_t)blockIdx.x * 2 * P;
  if (orb >= 0 && orb < n_orb) {
    dst[orb] = sh.acc[0][tid];
    dst[P + orb] = sh.acc[1][tid];
  }
  for (int net = 0; net < n_nets; ++net) {
    const int pbase = n_orb + net * kNnNetP;
    const int ab = 2 + net * kSampNetAcc;
    for (int r = 0; r < kSampRows; ++r)
      for (int h = 0; h < 2; ++h) {
        const int col = pbase + kNnOffW2 + (kSampRows * warp + r) * kNnH + lane + 32 * h;
        dst[col] = sh.acc[ab + 2 * (2 * r + h)][tid];
        dst[P + col] = sh.acc[ab + 2 * (2 * r + h) + 1][tid];
      }
    if (tid < kNnSmall) {
      const int col = pbase + small_offset(tid);
      const int sb = ab + 2 * 2 * kSampRows;
      dst[col] = sh.acc[sb][tid];
      dst[P + col] = sh.acc[sb + 1][tid];
    }
  }
}

int sr_sample_ctas(int W, int n_sm) { return std::max(1, std::min((W + kSampWarps - 1) / kSampWarps, n_sm)); }

size_t sr_sample_smem(int P) {
  (void)P;
  return sizeof(SampleShared);
}

// out[j] += sum_b partial[b][j]: out = sumO for j < P, sumEO for P <= j < 2P.
// A block takes 32 columns; row group y (of 8) sums CTAs y, y + 8, ... in
// FP32, then thread y = 0 adds the 8 group sums in FP64, in order.
__global__ void sr_sums_kernel(const float* partial, int n_cta, int P, double* sumO, double* sumEO) {
  __shared__ float part[8][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + tx;
  float s = 0.f;
  if (j < 2 * P)
    for (int b = ty; b < n_cta; b += 8) s += partial[(size_t)b * 2 * P + j];
  part[ty][tx] = s;
  __syncthreads();
  if (ty == 0 && j < 2 * P) {
    double t = 0.0;
    for (int y = 0; y < 8; ++y) t += (double)part[y][tx];
    if (j < P) sumO[j] += t;
    else sumEO[j - P] += t;
  }
}

cudaError_t launch_sr_sample(const SysParams<float>& sp, const double* pos, int W, int n_up, int n_elec, bool nets,
                             const double* Oorb, int ldorb, int n_orb, const float* center, const double* E,
                             __nv_bfloat16* Ob, int ldb, int P, float* partial, int n_cta, double* sumO,
                             double* sumEO, cudaStream_t s) {
  if (nets && !ogen_pairs_ok(sp, n_elec)) return cudaErrorInvalidValue;
  if (n_orb < 0 || n_orb > 32 || (nets ? n_orb + kNnP : n_orb) != P || n_cta < 1 || W < 1)
    return cudaErrorInvalidValue;
  const size_t smem = sizeof(SampleShared);
  cudaError_t e = cudaFuncSetAttribute(sr_sample_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  sr_sample_kernel<<<n_cta, kSampThreads, smem, s>>>(sp, pos, W, n_up, n_elec, nets ? 2 : 0, Oorb, ldorb, n_orb,
                                                     center, E, Ob, ldb, P, partial);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  sr_sums_kernel<<<(2 * P + 31) / 32, 256, 0, s>>>(partial, n_cta, P, sumO, sumEO);
  return cudaGetLastError();
}

__global__ void copy_cols_kernel(const double* src, int lds, int ncols, float* dst, int ldd, int W) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W * ncols) return;
  const int w = i / ncols, c = i % ncols;
  dst[(size_t)w * ldd + c] = (float)src[(size_t)w * lds + c];
}

cudaError_t launch_copy_cols(const double* src, int lds, int ncols, float* dst, int ldd, int W, cudaStream_t s) {
  if (ncols <= 0 || W <= 0) return cudaSuccess;
  copy_cols_kernel<<<(W * ncols + 255) / 256, 256, 0, s>>>(src, lds, ncols, dst, ldd, W);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ centre

// c[p] = mean over rows w < n of O[w][p]. A block takes 32 columns; row
// group y (of 16) sums rows y, y + 16, ..., and thread y = 0 adds the groups
// in order.
__global__ void center_rows_kernel(const float* O, int n, int P, int ldO, float* c) {
  __shared__ float part[16][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int p = blockIdx.x * 32 + tx;
  float s = 0.f;
  if (p < P)
    for (int w = ty; w < n; w += 16) s += O[(size_t)w * ldO + p];
  part[ty][tx] = s;
  __syncthreads();
  if (ty == 0 && p < P) {
    float t = 0.f;
    for (int y = 0; y < 16; ++y) t += part[y][tx];
    c[p] = t / (float)n;
  }
}

cudaError_t launch_center_rows(const float* O, int n, int P, int ldO, float* c, cudaStream_t s) {
  if (n <= 0) return cudaErrorInvalidValue;
  center_rows_kernel<<<(P + 31) / 32, 512, 0, s>>>(O, n, P, ldO, c);
  return cudaGetLastError();
}

// ------------------------------------------------ S = Ob^T Ob on tcgen05

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after about a second of SM clock and reports false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, phase))
    if (clock64() - t0 > 2000000000LL) return false;
  return true;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor of an MN-major operand tile with 128-byte
// swizzle, as the TMA writes it from Ob (parameters contiguous): each
// 64-row x 64-parameter box is 64 rows of 128 bytes (one sample's 64
// parameters), 8-row swizzle atoms 1,024 bytes apart (the stride along K);
// the tile's two boxes (parameters 0-63 and 64-127) sit 8,192 bytes apart
// (the stride along M/N). Descriptor version 1.
__device__ __forceinline__ uint64_t umma_desc_mn_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(kSBoxBytes >> 4) << 16;  // leading byte offset: next 64 parameters
  d |= (uint64_t)(1024u >> 4) << 32;       // stride byte offset: next 8 samples
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor of kind::f16: BF16 A and B, FP32 accumulator,
// both MN-major (bits 15 and 16), M = 128, N = 256.
constexpr uint32_t kSIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
                             ((uint32_t)(kSBN >> 3) << 17) | ((uint32_t)(kSBM >> 4) << 24);

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// Tiles of S: row tile ti (128 parameters) against column block tb (256
// parameters), for the blocks that reach the upper triangle (tb >= ti / 2;
// an odd row tile's first block also covers the tile left of its diagonal,
// which finalize_s overwrites from the upper one).
__host__ __device__ inline int s_gemm_tiles(int P_pad) {
  const int T = P_pad / kSBM, TB = P_pad / kSBN;
  int n = 0;
  for (int ti = 0; ti < T; ++ti) n += TB - ti / 2;
  return n;
}

// S[ti][tb] (+)= sum_k Ob[k][ti tile]^T Ob[k][tb block] over K = K_pad rows
// of Ob; `accumulate` adds to S, else stores. One CTA per SM: four 48 KB
// pipeline stages (A 16 KB + B 32 KB), 256 TMEM columns.
__global__ void __launch_bounds__(128, 1) s_gemm_kernel(const __grid_constant__ CUtensorMap tmap, double* S, int P_pad,
                                                        int K_pad, int accumulate, int* status) {
  extern __shared__ __align__(1024) unsigned char gemm_smem[];
  const uintptr_t base = ((uintptr_t)gemm_smem + 1023) & ~(uintptr_t)1023;
  unsigned char* tiles = (unsigned char*)base;  // [stage][A | B]
  uint64_t* full = (uint64_t*)(tiles + kSStages * kSStageBytes);
  uint64_t* empty = full + kSStages;
  uint64_t* done = empty + kSStages;
  uint32_t* tmem_slot = (uint32_t*)(done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // this CTA's tile, in bands of kSBand row tiles walked column block by
  // column block: CTAs running together share the band's row panels and
  // each column panel
  const int T = P_pad / kSBM, TB = P_pad / kSBN;
  int ti = 0, tb = 0;
  {
    int rem = blockIdx.x;
    bool found = false;
    for (int r0 = 0; r0 < T && !found; r0 += kSBand) {
      const int r1 = min(r0 + kSBand, T);
      int band = 0;
      for (int r = r0; r < r1; ++r) band += TB - r / 2;
      if (rem >= band) {
        rem -= band;
        continue;
      }
      for (int c = r0 / 2; c < TB; ++c) {
        const int n = min(r1, 2 * c + 2) - r0;  // rows of the band that reach column block c
        if (rem < n) {
          ti = r0 + rem;
          tb = c;
          found = true;
          break;
        }
        rem -= n;
      }
    }
  }

  if (threadIdx.x == 0) {
    for (int s = 0; s < kSStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"((uint32_t)kSBN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  const int nk = K_pad / kSBK;
  bool ok = true;

  if (warp == 0 && lane == 0) {
    for (int kb = 0; kb < nk && ok; ++kb) {
      const int s = kb % kSStages;
      if (kb >= kSStages) ok = mbar_wait(&empty[s], ((kb / kSStages) - 1) & 1);
      if (!ok) break;
      mbar_expect_tx(&full[s], kSStageBytes);
      unsigned char* a = tiles + s * kSStageBytes;
      unsigned char* bt = a + kSATileBytes;
#pragma unroll
      for (int q = 0; q < kSBM / 64; ++q) tma_load_2d(a + q * kSBoxBytes, &tmap, ti * kSBM + 64 * q, kb * kSBK, &full[s]);
#pragma unroll
      for (int q = 0; q < kSBN / 64; ++q) tma_load_2d(bt + q * kSBoxBytes, &tmap, tb * kSBN + 64 * q, kb * kSBK, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {
    for (int kb = 0; kb < nk && ok; ++kb) {
      const int s = kb % kSStages;
      ok = mbar_wait(&full[s], (kb / kSStages) & 1);
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t a0 = smem_u32(tiles + s * kSStageBytes);
      const uint32_t b0 = a0 + kSATileBytes;
#pragma unroll
      for (int kk = 0; kk < kSBK / 16; ++kk)  // 16 samples = two swizzle atoms = 2,048 bytes
        umma_f16(tmem, umma_desc_mn_sw128(a0 + kk * 2048), umma_desc_mn_sw128(b0 + kk * 2048), kSIdesc,
                 (kb | kk) != 0 ? 1u : 0u);
      umma_commit(&empty[s]);
    }
    umma_commit(done);
  }
  __syncwarp();
  // epilogue: thread (warp, lane) reads row 32 warp + lane of the tile from
  // TMEM, 16 columns at a time, into a shared staging tile (the pipeline's
  // buffers, idle once `done` has fired); the warp then writes its 32 rows of
  // S two rows per instruction, 16 consecutive doubles per half-warp
  const bool got = mbar_wait(done, 0);
  if (!ok || !got) {
    if (lane == 0) atomicOr(status, 4);
  } else {
    asm volatile("tcgen05.fence::after_thread_sync;");
    constexpr int LD = 17;  // staging row stride (doubles), odd: conflict-free columns
    double* stage = reinterpret_cast<double*>(tiles) + (size_t)warp * 32 * LD;
    const int half = lane >> 4, col = lane & 15;
#pragma unroll 1
    for (int c0 = 0; c0 < kSBN; c0 += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
          "%14, %15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int i = 0; i < 16; ++i) stage[lane * LD + i] = (double)__uint_as_float(v[i]);
      __syncwarp();
      double* out0 = S + (size_t)(ti * kSBM + warp * 32 + half) * P_pad + tb * kSBN + c0 + col;
      if (accumulate) {
        // all 16 loads of the chunk in flight before the first store
        double old[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) old[k] = out0[(size_t)(2 * k) * P_pad];
#pragma unroll
        for (int k = 0; k < 16; ++k) out0[(size_t)(2 * k) * P_pad] = old[k] + stage[(2 * k + half) * LD + col];
      } else {
#pragma unroll
        for (int k = 0; k < 16; ++k) out0[(size_t)(2 * k) * P_pad] = stage[(2 * k + half) * LD + col];
      }
      __syncwarp();
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 2) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)kSBN));
}

cudaError_t launch_s_gemm(const CUtensorMap* tmap, double* S, int P_pad, int K_pad, bool accumulate, int* status,
                          cudaStream_t s) {
  if (P_pad % kSBN || K_pad % kSBK || K_pad <= 0) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(s_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSGemmSmem);
  if (e != cudaSuccess) return e;
  s_gemm_kernel<<<s_gemm_tiles(P_pad), 128, kSGemmSmem, s>>>(*tmap, S, P_pad, K_pad, accumulate ? 1 : 0, status);
  return cudaGetLastError();
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Ob as a 2-D tensor: x = parameter (P_pad, contiguous), y = sample row
// (K_rows); boxes of 64 x 64 with 128-byte swizzle.
cudaError_t encode_ob_tensor_map(CUtensorMap* tmap, __nv_bfloat16* Ob, int P_pad, int K_rows) {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) return cudaErrorNotSupported;
    fn = (EncodeTiledFn)p;
  }
  if (P_pad % kSBN || K_rows % kSBK) return cudaErrorInvalidValue;
  const cuuint64_t dims[2] = {(cuuint64_t)P_pad, (cuuint64_t)K_rows};
  const cuuint64_t strides[1] = {(cuuint64_t)P_pad * sizeof(__nv_bfloat16)};
  const cuuint32_t box[2] = {64u, (cuuint32_t)kSBK};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(tmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)Ob, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// ------------------------------------------------------------ finalize S

__global__ void finalize_s_kernel(double* S, int P, int P_pad, const double* sumO, double inv_n, double eps) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= P || j < i) return;
  const double mi = sumO[i] * inv_n, mj = sumO[j] * inv_n;
  double v = S[(size_t)i * P_pad + j] * inv_n - mi * mj;
  if (i == j) v += eps;
  S[(size_t)i * P_pad + j] = v;
  S[(size_t)j * P_pad + i] = v;
}

cudaError_t launch_finalize_s(double* S, int P, int P_pad, const double* sumO, double n, double eps, cudaStream_t s) {
  dim3 grid((P + 255) / 256, P);
  finalize_s_kernel<<<grid, 256, 0, s>>>(S, P, P_pad, sumO, 1.0 / n, eps);
  return cudaGetLastError();
}

// ------------------------------------------------------------------- CG

// y = S x, one warp per row
__global__ void gemv_rows_kernel(const double* S, int P, int ld, const double* x, double* y) {
  const int row = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= P) return;
  const double* r = S + (size_t)row * ld;
  double s = 0.0;
  for (int k = lane; k < P; k += 32) s += r[k] * x[k];
  s = warp_sum(s);
  if (lane == 0) y[row] = s;
}

// out = sum_i a_i b_i (one CTA, fixed order)
__global__ void dot_kernel(const double* a, const double* b, int n, double* out) {
  __shared__ double part[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += a[i] * b[i];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < blockDim.x / 32 ? part[threadIdx.x] : 0.0;
    v = warp_sum(v);
    if (threadIdx.x == 0) *out = v;
  }
}

// scal[0] = r.z, scal[1] = p.q; alpha = r.z / p.q; x += alpha p; r -= alpha q; z = r / diag
__global__ void cg_update_kernel(double* x, double* r, double* z, const double* p, const double* q, const double* dg,
                                 const double* scal, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double alpha = scal[0] / scal[1];
  x[i] += alpha * p[i];
  r[i] -= alpha * q[i];
  z[i] = r[i] / dg[i];
}
// p = z + beta p, beta = rz_new / rz_old (scal[2] / scal[0])
__global__ void cg_direction_kernel(double* p, const double* z, double* scal, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  p[i] = z[i] + (scal[2] / scal[0]) * p[i];
}
__global__ void cg_shift_kernel(double* scal) { scal[0] = scal[2]; }
__global__ void diag_kernel(const double* S, int P, int ld, double* dg, const double* b, double* r, double* z,
                            double* p, double* x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  dg[i] = S[(size_t)i * ld + i];
  x[i] = 0.0;
  r[i] = b[i];
  z[i] = b[i] / dg[i];
  p[i] = z[i];
}

cudaError_t sr_cg_solve(const double* S, int P, int ld, const double* b, double* x, double* work, int max_iter,
                        double tol, int* iters, double* rel_res, cudaStream_t s) {
  double* r = work;
  double* z = r + P;
  double* p = z + P;
  double* q = p + P;
  double* dg = q + P;
  double* scal = dg + P;  // [0] rz, [1] pq, [2] rz_new, [3] rr, [4] bb
  const int nb = (P + 255) / 256;
  diag_kernel<<<nb, 256, 0, s>>>(S, P, ld, dg, b, r, z, p, x);
  dot_kernel<<<1, 1024, 0, s>>>(r, z, P, scal);
  dot_kernel<<<1, 1024, 0, s>>>(b, b, P, scal + 4);
  double h[5];
  int it = 0;
  for (; it < max_iter; ++it) {
    gemv_rows_kernel<<<(P + 7) / 8, 256, 0, s>>>(S, P, ld, p, q);
    dot_kernel<<<1, 1024, 0, s>>>(p, q, P, scal + 1);
    cg_update_kernel<<<nb, 256, 0, s>>>(x, r, z, p, q, dg, scal, P);
    dot_kernel<<<1, 1024, 0, s>>>(r, z, P, scal + 2);
    cg_direction_kernel<<<nb, 256, 0, s>>>(p, z, scal, P);
    cg_shift_kernel<<<1, 1, 0, s>>>(scal);
    if ((it + 1) % 10 == 0 || it + 1 == max_iter) {
      dot_kernel<<<1, 1024, 0, s>>>(r, r, P, scal + 3);
      cudaError_t e = cudaMemcpyAsync(h, scal, sizeof(h), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return e;
      if (h[3] <= tol * tol * h[4]) {
        ++it;
        break;
      }
    }
  }
  cudaError_t e = cudaMemcpyAsync(h, scal, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (iters) *iters = it;
  if (rel_res) *rel_res = h[4] > 0 ? sqrt(h[3] / h[4]) : 0.0;
  return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace mole
