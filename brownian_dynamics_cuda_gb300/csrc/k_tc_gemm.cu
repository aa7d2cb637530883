// FP32 GEMM on the tensor cores for the adjoint's Cholesky backward:
// C = alpha A op(B), row-major FP32 operands split on the fly into three
// BF16 slices (hi, mid, lo: 24 significant bits), six slice products per K
// step (every product of weight >= 2^-16 of hi * hi) accumulated in tensor
// memory by tcgen05.mma - the FP32-class scheme of the mixed Cholesky's
// trailing updates, here on plain row-major matrices.
//
// CTA = one 128 x 128 output tile, 512 threads: all threads stream 64-wide
// K chunks of A and B from global memory into registers one chunk ahead
// (coalesced 32-byte reads; for op(B) = B, column reads coalesced across the
// tile's 128 columns), split them and store the slices in the
// 128-byte-swizzled K-major layout the MMA descriptors read,
// double-buffered; one thread issues the 24 MMAs of a chunk (4 K steps x 6
// products) and commits them to the chunk's stage barrier, so loads, splits
// and MMAs of consecutive chunks overlap.  Every wait is
// bounded: a timeout records an error code, waits (bounded) for the MMAs in
// flight, frees the tensor memory and leaves C unwritten.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "bd_internal.h"
#include "sm100_ptx.cuh"

namespace {

constexpr int kGT = 128;                      // output tile
constexpr int kGC = 64;                       // K chunk: one 128-byte swizzle row of BF16
constexpr int kSlice = kGT * kGC * 2;         // 16 KB: one BF16 slice of a 128 x 64 chunk
constexpr int kStage = 6 * kSlice;            // A and B, three slices each: 96 KB
constexpr size_t kGemmSmem = 2 * (size_t)kStage + 1024 + 64;
constexpr uint32_t kGemmWait = 1u << 24;
constexpr int kGemmThreads = 512;

// byte offset of (row r, column k < 64) in one swizzled 128 x 64 BF16 slice
__device__ __forceinline__ uint32_t chunk_off(int r, int k) {
  return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((((k >> 3) ^ (r & 7)) & 7) << 4) + (k & 7) * 2);
}

// eight FP32 values -> their hi, mid and lo BF16 slices (v = hi + mid + lo to
// 24 bits), each packed as 16 bytes; pairs converted together (bf16x2)
__device__ __forceinline__ void put3(unsigned char* s, uint32_t off, const float (&v)[8]) {
  uint32_t hw[4], mw[4], lw[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const float x0 = v[2 * j], x1 = v[2 * j + 1];
    const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
    const float2 hf = __bfloat1622float2(h);
    const float r0 = x0 - hf.x, r1 = x1 - hf.y;
    const __nv_bfloat162 md = __floats2bfloat162_rn(r0, r1);
    const float2 mf = __bfloat1622float2(md);
    const __nv_bfloat162 lo = __floats2bfloat162_rn(r0 - mf.x, r1 - mf.y);
    hw[j] = *reinterpret_cast<const uint32_t*>(&h);
    mw[j] = *reinterpret_cast<const uint32_t*>(&md);
    lw[j] = *reinterpret_cast<const uint32_t*>(&lo);
  }
  *reinterpret_cast<uint4*>(s + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
  *reinterpret_cast<uint4*>(s + kSlice + off) = make_uint4(mw[0], mw[1], mw[2], mw[3]);
  *reinterpret_cast<uint4*>(s + 2 * kSlice + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
}

// one thread's share of a K chunk: two 8-element groups of A and of B
struct ChunkRegs {
  float a[2][8], b[2][8];
};

template <bool TB>
__device__ __forceinline__ void load_chunk(ChunkRegs& R, const float* __restrict__ A, int lda,
                                           const float* __restrict__ B, int ldb, int r0, int c0, int k0, int tid) {
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int g = tid + kGemmThreads * q, row = g >> 3, k8 = g & 7;
    const float4* p = reinterpret_cast<const float4*>(A + (size_t)(r0 + row) * lda + k0 + 8 * k8);
    const float4 x = __ldg(p), y = __ldg(p + 1);
    R.a[q][0] = x.x, R.a[q][1] = x.y, R.a[q][2] = x.z, R.a[q][3] = x.w;
    R.a[q][4] = y.x, R.a[q][5] = y.y, R.a[q][6] = y.z, R.a[q][7] = y.w;
  }
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int g = tid + kGemmThreads * q;
    if (TB) {
      const int row = g >> 3, k8 = g & 7;
      const float4* p = reinterpret_cast<const float4*>(B + (size_t)(c0 + row) * ldb + k0 + 8 * k8);
      const float4 x = __ldg(p), y = __ldg(p + 1);
      R.b[q][0] = x.x, R.b[q][1] = x.y, R.b[q][2] = x.z, R.b[q][3] = x.w;
      R.b[q][4] = y.x, R.b[q][5] = y.y, R.b[q][6] = y.z, R.b[q][7] = y.w;
    } else {
      const int n = g & 127, k8 = g >> 7;
#pragma unroll
      for (int e = 0; e < 8; e++) R.b[q][e] = __ldg(B + (size_t)(k0 + 8 * k8 + e) * ldb + c0 + n);
    }
  }
}

template <bool TB>
__device__ __forceinline__ void store_chunk(const ChunkRegs& R, unsigned char* sa, unsigned char* sb, int tid) {
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int g = tid + kGemmThreads * q;
    put3(sa, chunk_off(g >> 3, 8 * (g & 7)), R.a[q]);
    if (TB) put3(sb, chunk_off(g >> 3, 8 * (g & 7)), R.b[q]);
    else put3(sb, chunk_off(g & 127, 8 * (g >> 7)), R.b[q]);
  }
}

// kmode restricts each tile's K range to the nonzero band of triangular
// operands: 1: k >= r0, 2: k >= c0, 4: k < c0 + 128 (tile granularity).
// gridDim.z independent products, every operand zstride elements apart.
// Chunk it + 1 is loaded into registers while chunk it is split and its
// MMAs issued; the slices are double-buffered, so the split of chunk it + 1
// overlaps the MMAs of chunk it.
template <bool TB>
__global__ void __launch_bounds__(kGemmThreads, 1)
    k_tc_gemm(int K, float alpha, const float* __restrict__ A, int lda, const float* __restrict__ B, int ldb,
              float* __restrict__ C, int ldc, int kmode, long zstride, int* err) {
  extern __shared__ unsigned char smraw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + 2 * kStage);  // [0], [1]: stage s read by its MMAs
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2);
  volatile int* abortf = reinterpret_cast<volatile int*>(tslot + 1);
  const int r0 = blockIdx.y * kGT, c0 = blockIdx.x * kGT;
  A += blockIdx.z * zstride;
  B += blockIdx.z * zstride;
  C += blockIdx.z * zstride;
  int kb = 0, ke = K;
  if (kmode & 1) kb = max(kb, r0);
  if (kmode & 2) kb = max(kb, c0);
  if (kmode & 4) ke = min(ke, c0 + kGT);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  ChunkRegs nxt;
  if (kb < ke) load_chunk<TB>(nxt, A, lda, B, ldb, r0, c0, kb, tid);
  if (tid == 0) {
    sm100::mbar_init(&bars[0], 1);
    sm100::mbar_init(&bars[1], 1);
    *abortf = 0;
    sm100::fence_mbar_init();
  }
  if (warp == 0) sm100::tmem_alloc(tslot, kGT);
  sm100::tc_fence_before();
  __syncthreads();
  sm100::tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = sm100::idesc_bf16_f32(kGT, kGT);
  const int pa[6] = {2, 1, 0, 1, 0, 0};  // (A slice, B slice) of each product, smallest first
  const int pb[6] = {0, 1, 2, 0, 1, 0};

  int it = 0;
  for (int k0 = kb; k0 < ke; k0 += kGC, it++) {
    const int s = it & 1;
    unsigned char* sa = sm + s * kStage;
    unsigned char* sb = sa + 3 * kSlice;
    const ChunkRegs cur = nxt;
    if (k0 + kGC < ke) load_chunk<TB>(nxt, A, lda, B, ldb, r0, c0, k0 + kGC, tid);
    // stage s free once the MMAs of chunk it - 2 are done: every thread
    // waits on the stage barrier itself; one that gives up writes nothing,
    // and the CTA leaves together after the barrier below
    bool ok = true;
    if (it >= 2) ok = sm100::mbar_wait(&bars[s], ((it >> 1) - 1) & 1, kGemmWait);
    if (ok) store_chunk<TB>(cur, sa, sb, tid);
    else *abortf = 1;
    sm100::fence_proxy_async();  // the slices, written by the threads, are read by the tensor cores
    __syncthreads();
    if (*abortf) break;
    if (tid == 0) {
      sm100::tc_fence_after();
#pragma unroll
      for (int p = 0; p < 6; p++) {
        const uint32_t aaddr = sm100::smem_u32(sa + pa[p] * kSlice);
        const uint32_t baddr = sm100::smem_u32(sb + pb[p] * kSlice);
#pragma unroll
        for (int kk = 0; kk < 4; kk++)
          sm100::mma_bf16(tmem, sm100::desc_kmajor_sw128(aaddr + kk * 32), sm100::desc_kmajor_sw128(baddr + kk * 32),
                          idesc, (it | p | kk) != 0);
      }
      sm100::mma_commit(&bars[s]);
    }
  }
  // the last chunk's commit covers every MMA issued before it
  if (tid == 0 && it > 0) {
    const int l = it - 1;
    if (!sm100::mbar_wait(&bars[l & 1], (l >> 1) & 1, kGemmWait)) *abortf = 2;
  }
  __syncthreads();
  const int bad = *abortf;
  if (bad) {
    if (tid == 0) {
      atomicExch(err, 20 + bad);
      if (it > 0) (void)sm100::mbar_wait(&bars[(it - 1) & 1], ((it - 1) >> 1) & 1, kGemmWait);  // MMAs in flight
    }
  } else if (warp < 16) {
    // 16 warps: lanes 32 (w % 4) .., columns 32 (w / 4) ..
    sm100::tc_fence_after();
    const int q = warp & 3, cq = warp >> 2, r = r0 + 32 * q + lane;
    float* crow = C + (size_t)r * ldc + c0 + 32 * cq;
    float v[32];
    if (it > 0) {
      sm100::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(32 * cq), v);
    } else {
#pragma unroll
      for (int j = 0; j < 32; j++) v[j] = 0.f;
    }
#pragma unroll
    for (int j = 0; j < 8; j++)
      reinterpret_cast<float4*>(crow)[j] =
          make_float4(alpha * v[4 * j], alpha * v[4 * j + 1], alpha * v[4 * j + 2], alpha * v[4 * j + 3]);
  }
  sm100::tc_fence_before();
  __syncthreads();
  if (warp == 0) sm100::tmem_dealloc(tmem, kGT);
}

bool g_gemm_attr = false;

}  // namespace

namespace bdk {

int tc_gemm_attributes() {
  if (g_gemm_attr) return 0;
  if (cudaFuncSetAttribute(k_tc_gemm<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem) !=
          cudaSuccess ||
      cudaFuncSetAttribute(k_tc_gemm<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem) !=
          cudaSuccess)
    return 1;
  g_gemm_attr = true;
  return 0;
}

int tc_gemm_f32(cudaStream_t st, int M, int N, int K, float alpha, const float* A, int lda, const float* B, int ldb,
                float* C, int ldc, bool tb, int kmode, int batch, long zstride, int* err) {
  if (M % kGT || N % kGT || K % kGC || lda % 4 || (tb && ldb % 4) || ldc % 4 || batch < 1) return 1;
  if (tc_gemm_attributes()) return 2;
  const dim3 grid(N / kGT, M / kGT, batch);
  if (tb) k_tc_gemm<true><<<grid, kGemmThreads, kGemmSmem, st>>>(K, alpha, A, lda, B, ldb, C, ldc, kmode, zstride, err);
  else k_tc_gemm<false><<<grid, kGemmThreads, kGemmSmem, st>>>(K, alpha, A, lda, B, ldb, C, ldc, kmode, zstride, err);
  return cudaGetLastError() == cudaSuccess ? 0 : 3;
}

}  // namespace bdk
