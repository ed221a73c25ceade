// nn_table.cu -- tabulation of the pair networks (see nn.cuh): the FP64
// network jets at the nodes, then the quintic Hermite coefficients.
#include "nn.cuh"

namespace mole {

struct NnTabArgs {
  const double* theta;
  double z[kMaxNuc];
  int n_tab;
  double* node;  // [n_tab][kNnTabNodes][3]
  float* tab;    // [n_tab][kNnTabIntervals][kNnTabFloats]
};

__global__ void nn_node_kernel(const NnTabArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n_tab * kNnTabNodes) return;
  const int k = i / kNnTabNodes, n = i % kNnTabNodes;
  const double s = k == 0 ? 1.0 : (k == 1 ? 0.0 : a.z[k - 2]);
  double y, y1, y2;
  nn_jet_global(a.theta + nn_tab_net(k) * kNnNetP, nn_tab_node_r(n), s, y, y1, y2);
  a.node[3 * (size_t)i] = y;
  a.node[3 * (size_t)i + 1] = y1;
  a.node[3 * (size_t)i + 2] = y2;
}

// Coefficients of p(t), t in [0, 1], with p, p', p'' (in t) matching the
// node values at both ends: c0 = p0, c1 = v0, c2 = a0 / 2 and
// c3..c5 from the three end conditions at t = 1.
__global__ void nn_coef_kernel(const NnTabArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n_tab * kNnTabIntervals) return;
  const int k = i / kNnTabIntervals, j = i % kNnTabIntervals;
  // interval j of the near segment joins nodes j, j + 1; of the far segment nodes j + 1, j + 2
  const int n = j < kNnTabSeg ? j : j + 1;
  const double* p = a.node + 3 * ((size_t)k * kNnTabNodes + n);
  const double h = j < kNnTabSeg ? kNnTabH : kNnTabHFar;
  const double p0 = p[0], v0 = h * p[1], a0 = h * h * p[2];
  const double p1 = p[3], v1 = h * p[4], a1 = h * h * p[5];
  const double d = p1 - p0;
  float* c = a.tab + (size_t)i * kNnTabFloats;
  c[0] = (float)p0;
  c[1] = (float)v0;
  c[2] = (float)(0.5 * a0);
  c[3] = (float)(10.0 * d - 6.0 * v0 - 4.0 * v1 - 1.5 * a0 + 0.5 * a1);
  c[4] = (float)(-15.0 * d + 8.0 * v0 + 7.0 * v1 + 1.5 * a0 - a1);
  c[5] = (float)(6.0 * d - 3.0 * v0 - 3.0 * v1 - 0.5 * a0 + 0.5 * a1);
  c[6] = 0.f;
  c[7] = 0.f;
}

cudaError_t launch_nn_tables(const double* theta, int n_nuc, const double* nuc_z, double* node, float* tab,
                             cudaStream_t s) {
  if (n_nuc < 0 || n_nuc > kMaxNuc) return cudaErrorInvalidValue;
  NnTabArgs a;
  a.theta = theta;
  for (int I = 0; I < kMaxNuc; ++I) a.z[I] = I < n_nuc ? nuc_z[I] : 0.0;
  a.n_tab = 2 + n_nuc;
  a.node = node;
  a.tab = tab;
  const int nn = a.n_tab * kNnTabNodes, nc = a.n_tab * kNnTabIntervals;
  nn_node_kernel<<<(nn + 127) / 128, 128, 0, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  nn_coef_kernel<<<(nc + 255) / 256, 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace mole
