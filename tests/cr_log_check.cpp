// Host build of the device logarithm (brownian_dynamics_cuda_gb300/csrc/cr_log.cuh)
// for tests/test_cr_log.py: the same source, compiled without FMA contraction
// (the device unit is compiled with -fmad=false), evaluated over an array.
#include "cr_log.cuh"

extern "C" void cr_log_many(const double* x, double* y, int n) {
  for (int i = 0; i < n; i++) y[i] = crlog::log_cr(x[i]);
}
