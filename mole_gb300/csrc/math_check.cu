// math_check.cu -- evaluates the library's own device arithmetic on arrays so
// that tests can pin its accuracy: the FP64 exponential, reciprocal and
// reciprocal square root of the native FP64 kernels, the double-float exp,
// reciprocal square root and reciprocal of the double-float kernels, and the
// integer-built float <-> double conversions.
#include "fp64.cuh"

namespace mole {

__global__ void math_check_kernel(int fn, const double* x, int64_t n, double* y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = x[i];
  double r = 0.0;
  switch (fn) {
    case 0: r = exp64(v); break;
    case 1: r = (double)df_exp(df64(v)); break;
    case 2: r = (double)df_rsqrt(df64(v)); break;
    case 3: r = (double)df_rcp(df64(v)); break;
    case 4: r = (double)(df64(v) / df64(1.0 + v * v)); break;
    case 5: r = f2d(__double2float_rn(v)); break;
    case 6: r = (double)d2f_rz(v); break;
    case 7: r = (double)d2f_rz_small(v); break;
    case 8: r = rcp64(v); break;
    default: r = rsqrt64(v); break;
  }
  y[i] = r;
}

cudaError_t launch_math_check(int fn, const double* x, int64_t n, double* y, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int threads = 256;
  math_check_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(fn, x, n, y);
  return cudaGetLastError();
}

}  // namespace mole
