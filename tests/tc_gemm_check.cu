// Test shim for tests/test_gpu_tc_gemm.py: calls the library's tensor-core
// GEMM (bdk::tc_gemm_f32, csrc/k_tc_gemm.cu) on caller-owned device
// buffers and waits for it.
#include <cuda_runtime.h>
namespace bdk {
int tc_gemm_f32(cudaStream_t st, int M, int N, int K, float alpha, const float* A, int lda, const float* B, int ldb,
                float* C, int ldc, bool tb, int kmode, int batch, long zstride, int* err);
}
extern "C" int check_tc_gemm(int M, int N, int K, float alpha, const float* A, int lda, const float* B, int ldb,
                             float* C, int ldc, int tb, int kmode, int batch, long zs, int* err) {
  const int rc = bdk::tc_gemm_f32(0, M, N, K, alpha, A, lda, B, ldb, C, ldc, tb != 0, kmode, batch, zs, err);
  if (rc) return 100 + rc;
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : -1;
}
