// Allocation-free entry point: the noise displacement rd = s2dt * L p on
// caller-owned device buffers, with its split-K scratch held in a
// fixed-size array in the library's own device memory.
//
// Who needs it: a host application that has handed the GPU's memory to its
// own pool allocator, or that runs the step inside a latency-critical loop,
// cannot let a library call cudaMalloc/cudaFree (they take memory the pool
// owns and may synchronise the whole device).  This entry point therefore
// allocates nothing: the caller passes L, p and rd; the partial sums live in
// `g_scratch` below.
//
// Limits and rules:
//  * m <= kMaxM (16384, i.e. fibers of up to 5461 beads); larger m is
//    rejected with BD_ERR_ARG.  The scratch is kMaxChunks x kMaxM doubles
//    (4 MiB), resident on every device that loads the library until exit.
//  * Host code cannot use `g_scratch` as a device address (it names a host
//    stand-in).  The first call on each device looks the real address up
//    with cudaGetSymbolAddress, with that device current, and caches it
//    together with the device's current CUDA context; a call that finds a
//    different context (after cudaDeviceReset, say) looks it up again.
//    With lazy module loading (the CUDA default) that first look-up loads
//    this library's device code, and the 4 MiB array is committed at that
//    moment: the first call on a device (and the first after a reset)
//    allocates as any first use of a CUDA library does.  Make it once as a
//    warm-up, before the region that must not allocate and before any stream
//    capture on the device; every later call allocates nothing.
//  * All calls share the one scratch array and it keeps the last call's
//    contents.  Nothing in it has to start at zero: every partial sum a call
//    reads was written by the same call.  Calls whose kernels overlap on
//    the GPU (e.g. on two streams) race on the scratch and must be ordered
//    by the caller.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "bd_internal.h"

namespace {

constexpr int kRows = 256;          // rows per CTA
constexpr int kChunk = 512;         // columns per partial sum
constexpr int kMaxM = 16384;
constexpr int kMaxChunks = kMaxM / kChunk;

static __device__ __align__(256) double g_scratch[(size_t)kMaxChunks * kMaxM];

__global__ void __launch_bounds__(kRows) k_na_part(int m, const double* __restrict__ L, int lda,
                                                   const double* __restrict__ p, double s2dt,
                                                   double* __restrict__ part) {
  int i = blockIdx.x * kRows + threadIdx.x;
  int kc = blockIdx.y;
  int k0 = kc * kChunk, k1 = min(k0 + kChunk, m);
  if (i >= m) return;
  double s = 0.0;
  int kend = min(k1, i + 1);
#pragma unroll 8  // eight loads of the factor in flight per thread; the sum's order is unchanged
  for (int k = k0; k < kend; k++) s = s + (s2dt * L[(size_t)k * lda + i]) * p[k];
  part[(size_t)kc * m + i] = s;
}

__global__ void k_na_sum(int m, int nchunk, const double* __restrict__ part, double* __restrict__ rd) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double s = 0.0;
  for (int c = 0; c < nchunk; c++) s = s + part[(size_t)c * m + i];
  rd[i] = s;
}

std::mutex g_mu;
constexpr int kMaxDevices = 64;
struct ScratchAddr {
  CUcontext ctx = nullptr;  // context the address was looked up in
  double* addr = nullptr;
};
ScratchAddr g_addr[kMaxDevices];

// cuCtxGetCurrent through the runtime's driver entry point, so that the
// library does not link libcuda itself (it must load on hosts without a GPU).
using CtxGetCurrent = CUresult (*)(CUcontext*);
CtxGetCurrent ctx_get_current() {
  static CtxGetCurrent fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<CtxGetCurrent>(f);
  }();
  return fn;
}

CUcontext current_context() {
  CUcontext c = nullptr;
  CtxGetCurrent fn = ctx_get_current();
  if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
  return c;
}

}  // namespace

extern "C" int bd_noise_displacement_noalloc(int m, const double* d_L, int lda, const double* d_p, double s2dt,
                                             double* d_rd, void* stream) {
  if (!d_L || !d_p || !d_rd || m <= 0 || lda < m)
    return bdh::set_error(BD_ERR_ARG, "bd_noise_displacement_noalloc: bad pointer or size");
  if (m > kMaxM) {
    char b[160];
    snprintf(b, sizeof b, "bd_noise_displacement_noalloc: m = %d exceeds the fixed scratch limit of %d", m, kMaxM);
    return bdh::set_error(BD_ERR_ARG, b);
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return bdh::set_error(BD_ERR_CUDA, "bd_noise_displacement_noalloc: no current device");
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    ScratchAddr& a = g_addr[dev];
    CUcontext cur = current_context();
    if (!a.addr || !cur || cur != a.ctx) {
      // set-up, once per device and context, with that device current
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_scratch);
      if (e != cudaSuccess) {
        char b[200];
        snprintf(b, sizeof b, "bd_noise_displacement_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        return bdh::set_error(BD_ERR_CUDA, b);
      }
      a.addr = static_cast<double*>(ptr);
      a.ctx = current_context();  // current now, if it was not before the look-up
    }
    scratch = a.addr;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nchunk = (m + kChunk - 1) / kChunk;
  k_na_part<<<dim3((m + kRows - 1) / kRows, nchunk), kRows, 0, st>>>(m, d_L, lda, d_p, s2dt, scratch);
  k_na_sum<<<(m + 255) / 256, 256, 0, st>>>(m, nchunk, scratch, d_rd);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    char b[200];
    snprintf(b, sizeof b, "bd_noise_displacement_noalloc: launch failed: %s", cudaGetErrorString(e));
    return bdh::set_error(BD_ERR_CUDA, b);
  }
  return BD_OK;
}
