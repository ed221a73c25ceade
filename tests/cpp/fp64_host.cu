// Host entry points over the integer helpers of fp64.cuh, for the CPU tests
// (tests/test_fp64_helpers.py compares them with exact rational arithmetic).
#include "../../mole_gb300/csrc/fp64.cuh"

extern "C" {
void t_dbl_add_small(const float* h, const float* l, double* out, int n) {
  for (int i = 0; i < n; ++i) out[i] = mole::dbl_add_small(h[i], l[i]);
}
void t_split_double(const double* d, float* h, float* l, int n) {
  for (int i = 0; i < n; ++i) mole::split_double(d[i], h[i], l[i]);
}
void t_exp_nl1(const int* k, double* out, int n) {
  for (int i = 0; i < n; ++i) out[i] = mole::exp_nl1(k[i]);
}
void t_u01_centered(const unsigned* x, double* out, int n) {
  for (int i = 0; i < n; ++i) out[i] = mole::u01_centered(x[i]);
}
}
