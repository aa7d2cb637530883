// Mixed-precision Cholesky of the RPY tensor on the sm_103a tensor cores.
//
// Right-looking blocked factorisation with 128-wide panels.  The matrix is
// stored in FP64 (column-major), so each trailing update is rounded at FP64
// however many panels precede it; the arithmetic is FP32-class:
//   k_diag32    Cholesky of the 128 x 128 diagonal block in shared memory,
//               left-looking (each element is one FP32 dot product and one
//               rounding of its FP64 value, not one rounding per column as a
//               right-looking FP32 update would do); a negative pivot is
//               replaced by its absolute value and counted (func.cpp:827-833).
//   k_panel32   L_ik = A_ik L_kk^-T by forward substitution for every 128-row
//               tile below the block (FP32), written back and split into three BF16 slices
//               (hi + mid + lo = the FP32 value exactly), stored pre-swizzled
//               in the 128-byte-swizzle K-major layout the MMA reads.
//   k_tc_syrk   trailing update A_IJ -= L_I L_J^T of one 128 x 128 tile per
//               CTA: both operands' slices are brought into shared memory by
//               bulk-async copies, six BF16 products (hi.hi, hi.mid, mid.hi,
//               hi.lo, mid.mid, lo.hi) accumulate in one FP32 tensor-memory
//               accumulator (tcgen05.mma, M = N = 128, K = 16 per
//               instruction), and the epilogue reads the accumulator with
//               tcgen05.ld and updates the FP64 tile.  The dropped products
//               are below 2^-24 of the kept ones: FP32-class products.
// Every mbarrier wait is bounded; on a timeout the kernel records an error
// code, frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "bd_internal.h"
#include "dev_physics.cuh"
#include "sm100_ptx.cuh"

namespace {

constexpr int kT = 128;                 // tile / panel width
constexpr int kSliceBytes = kT * kT * 2;  // one BF16 slice of a 128 x 128 tile (two 64-column halves)
constexpr int kHalfBytes = kSliceBytes / 2;
constexpr int kTileSlices = 3;
constexpr int kTileBytes = kTileSlices * kSliceBytes;  // 96 KB per 128-row panel tile
constexpr uint32_t kWaitLimit = 1u << 24;

inline int cdiv(int a, int b) { return (a + b - 1) / b; }

// byte offset of element (row r, column k) inside one pre-swizzled slice
__device__ __forceinline__ uint32_t swz_off(int r, int k) {
  int half = k >> 6, kk = k & 63;
  return half * kHalfBytes + (r >> 3) * 1024 + (r & 7) * 128 + ((((kk >> 3) ^ (r & 7)) & 7) << 4) + (kk & 7) * 2;
}

// ------------------------------------------------------------ diagonal block
__global__ void __launch_bounds__(256) k_diag32(double* A, int lda, int k0, int kb, int* negpiv) {
  extern __shared__ float sm32[];
  float (*S)[kT + 1] = reinterpret_cast<float (*)[kT + 1]>(sm32);   // [row][col]; lower part holds L as it forms
  __shared__ float diag_s[1];
  const int tid = threadIdx.x;
  for (int e = tid; e < kb * kb; e += blockDim.x) {
    int c = e / kb, rr = e - c * kb;
    S[rr][c] = (rr >= c) ? (float)A[(size_t)(k0 + c) * lda + k0 + rr] : 0.f;
  }
  __syncthreads();
  // column c: every row r >= c forms s = A[r][c] - sum_{q<c} L[r][q] L[c][q]
  // as one dot product (four partial sums), then L[c][c] = sqrt(|s_cc|) and
  // L[r][c] = s_rc / L[c][c]
  const int r = tid;
  for (int c = 0; c < kb; c++) {
    float sv = 0.f;
    if (r >= c && r < kb) {
      float s0 = S[r][c], s1 = 0.f, s2 = 0.f, s3 = 0.f;
      int q = 0;
      for (; q + 3 < c; q += 4) {
        s0 = fmaf(-S[r][q], S[c][q], s0);
        s1 = fmaf(-S[r][q + 1], S[c][q + 1], s1);
        s2 = fmaf(-S[r][q + 2], S[c][q + 2], s2);
        s3 = fmaf(-S[r][q + 3], S[c][q + 3], s3);
      }
      for (; q < c; q++) s0 = fmaf(-S[r][q], S[c][q], s0);
      sv = (s0 + s1) + (s2 + s3);
      if (r == c) {
        if (sv < 0.f) atomicAdd(negpiv, 1);
        diag_s[0] = sqrtf(fabsf(sv));
      }
    }
    __syncthreads();
    const float piv = diag_s[0];
    if (r == c) S[c][c] = piv;
    else if (r > c && r < kb) S[r][c] = sv / piv;
    __syncthreads();
  }
  for (int e = tid; e < kb * kb; e += blockDim.x) {
    int c = e / kb, rr = e - c * kb;
    if (rr >= c) A[(size_t)(k0 + c) * lda + k0 + rr] = (double)S[rr][c];
  }
}

// ------------------------------------------------------------ panel
// Rows of the 128-row tile `tile` (row0 = tile*128) solve X L_kk^T = A_ik by
// forward substitution (one thread per row, the factor in shared memory;
// backward stable, unlike multiplying by an explicit inverse); the result
// L_ik is written back (FP32) and split into three BF16 slices stored
// pre-swizzled at PS + tile*96KB.
__global__ void __launch_bounds__(128) k_panel32(double* A, int lda, int m, int k0, int kb, int tile0,
                                                 unsigned char* PS) {
  extern __shared__ float sm32[];
  float (*Lk)[kT + 1] = reinterpret_cast<float (*)[kT + 1]>(sm32);               // [c][q] factor
  float (*X)[kT + 1] = reinterpret_cast<float (*)[kT + 1]>(sm32 + kT * (kT + 1));  // [row][q]
  const int tile = tile0 + blockIdx.x;
  const int row0 = tile * kT;
  const int tid = threadIdx.x;
  for (int e = tid; e < kT * kT; e += blockDim.x) {
    int q = e / kT, rr = e - q * kT;  // column-major walk: coalesced
    int gr = row0 + rr;
    X[rr][q] = (gr < m && q < kb) ? (float)A[(size_t)(k0 + q) * lda + gr] : 0.f;
    Lk[rr][q] = (rr >= q && rr < kb && q < kb) ? (float)A[(size_t)(k0 + q) * lda + k0 + rr] : 0.f;
  }
  __syncthreads();
  {
    const int t = tid;
    for (int c = 0; c < kb; c++) {
      float s0 = X[t][c], s1 = 0.f, s2 = 0.f, s3 = 0.f;
      int q = 0;
      for (; q + 3 < c; q += 4) {
        s0 = fmaf(-X[t][q], Lk[c][q], s0);
        s1 = fmaf(-X[t][q + 1], Lk[c][q + 1], s1);
        s2 = fmaf(-X[t][q + 2], Lk[c][q + 2], s2);
        s3 = fmaf(-X[t][q + 3], Lk[c][q + 3], s3);
      }
      for (; q < c; q++) s0 = fmaf(-X[t][q], Lk[c][q], s0);
      X[t][c] = ((s0 + s1) + (s2 + s3)) / Lk[c][c];
    }
  }
  __syncthreads();
  unsigned char* ps = PS + (size_t)tile * kTileBytes;
  for (int e = tid; e < kT * kT; e += blockDim.x) {
    int c = e / kT, r = e - c * kT;
    int gr = row0 + r;
    bool in = gr < m && c < kb;
    float x = in ? X[r][c] : 0.f;
    if (in) A[(size_t)(k0 + c) * lda + gr] = (double)x;
    __nv_bfloat16 h = __float2bfloat16_rn(x);
    float r1 = x - __bfloat162float(h);
    __nv_bfloat16 md = __float2bfloat16_rn(r1);
    float r2 = r1 - __bfloat162float(md);
    __nv_bfloat16 lo = __float2bfloat16_rn(r2);
    uint32_t off = swz_off(r, c);
    *reinterpret_cast<__nv_bfloat16*>(ps + off) = h;
    *reinterpret_cast<__nv_bfloat16*>(ps + kSliceBytes + off) = md;
    *reinterpret_cast<__nv_bfloat16*>(ps + 2 * kSliceBytes + off) = lo;
  }
}

// ------------------------------------------------------------ tensor-core trailing update
constexpr int kSyrkThreads = 128;
constexpr size_t kSyrkSmem = 2 * (size_t)kTileBytes + 1024 + 64;

__global__ void __launch_bounds__(kSyrkThreads, 1) k_tc_syrk(double* A, int lda, int m, int kpanel, int nt,
                                                            const unsigned char* __restrict__ PS, int* err) {
  extern __shared__ unsigned char smraw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  unsigned char* sA = sm;
  unsigned char* sB = sm + kTileBytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + 2 * kTileBytes);  // [0] loads, [1] mma
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2);
  // tile (I, J), kpanel < J <= I < nt, from the linear block index
  const int rel = blockIdx.x;
  int Ip = (int)((sqrtf(8.f * (float)rel + 1.f) - 1.f) * 0.5f);
  while ((Ip + 1) * (Ip + 2) / 2 <= rel) Ip++;
  while (Ip * (Ip + 1) / 2 > rel) Ip--;
  const int Jp = rel - Ip * (Ip + 1) / 2;
  const int I = kpanel + 1 + Ip, J = kpanel + 1 + Jp;
  const bool diag = (I == J);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    sm100::mbar_init(&bars[0], 1);
    sm100::mbar_init(&bars[1], 1);
    sm100::fence_mbar_init();
  }
  if (warp == 0) sm100::tmem_alloc(tslot, 128);
  sm100::tc_fence_before();
  __syncthreads();
  sm100::tc_fence_after();
  const uint32_t tmem = *tslot;
  uint32_t* okflag = tslot + 1;
  if (threadIdx.x == 0) {
    const uint32_t bytes = diag ? kTileBytes : 2 * kTileBytes;
    sm100::mbar_arrive_expect_tx(&bars[0], bytes);
    const unsigned char* gA = PS + (size_t)I * kTileBytes;
    const unsigned char* gB = PS + (size_t)J * kTileBytes;
    for (int s = 0; s < kTileSlices; s++) sm100::bulk_g2s(sA + s * kSliceBytes, gA + s * kSliceBytes, kSliceBytes, &bars[0]);
    if (!diag)
      for (int s = 0; s < kTileSlices; s++) sm100::bulk_g2s(sB + s * kSliceBytes, gB + s * kSliceBytes, kSliceBytes, &bars[0]);
    bool ok = sm100::mbar_wait(&bars[0], 0, kWaitLimit);
    if (ok) {
      sm100::tc_fence_after();
      const unsigned char* bB = diag ? sA : sB;
      const uint32_t idesc = sm100::idesc_bf16_f32(128, 128);
      // (A slice, B slice) products, smallest first
      const int pa[6] = {2, 1, 0, 1, 0, 0};
      const int pb[6] = {0, 1, 2, 0, 1, 0};
      uint32_t accum = 0;
      for (int t = 0; t < 6; t++) {
        for (int h = 0; h < 2; h++) {
          for (int kk = 0; kk < 4; kk++) {
            uint32_t aaddr = sm100::smem_u32(sA + pa[t] * kSliceBytes + h * kHalfBytes) + kk * 32;
            uint32_t baddr = sm100::smem_u32(bB + pb[t] * kSliceBytes + h * kHalfBytes) + kk * 32;
            sm100::mma_bf16(tmem, sm100::desc_kmajor_sw128(aaddr), sm100::desc_kmajor_sw128(baddr), idesc, accum);
            accum = 1;
          }
        }
      }
      sm100::mma_commit(&bars[1]);
    } else {
      atomicExch(err, 1);
      // let the copies still in flight land before the CTA exits
      (void)sm100::mbar_wait(&bars[0], 0, kWaitLimit);
    }
    *okflag = ok ? 1u : 0u;
  }
  __syncthreads();
  const bool loaded = *okflag != 0;
  const bool mma_done = loaded && sm100::mbar_wait(&bars[1], 0, kWaitLimit);
  const int all_ok = __syncthreads_and(mma_done ? 1 : 0);
  if (all_ok) {
    sm100::tc_fence_after();
    const int i = 32 * warp + lane;
    const int gi = I * kT + i;
    const bool row_ok = gi < m;
    for (int c = 0; c < 4; c++) {
      double old[32];
      float v[32];
      const int gj0 = J * kT + 32 * c;
      // all loads of the chunk first (independent), then the subtracts and stores
#pragma unroll
      for (int j = 0; j < 32; j++) {
        const int gj = gj0 + j;
        const bool ok2 = row_ok && gj < m && (!diag || gi >= gj);
        old[j] = ok2 ? A[(size_t)gj * lda + gi] : 0.0;
      }
      sm100::tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + 32 * c, v);
#pragma unroll
      for (int j = 0; j < 32; j++) {
        const int gj = gj0 + j;
        if (row_ok && gj < m && (!diag || gi >= gj)) A[(size_t)gj * lda + gi] = old[j] - (double)v[j];
      }
    }
  } else if (threadIdx.x == 0 && loaded) {
    atomicExch(err, 2);
  }
  sm100::tc_fence_before();
  __syncthreads();
  if (warp == 0) sm100::tmem_dealloc(tmem, 128);
}

}  // namespace

namespace bdk {

size_t mixed_panel_bytes(int m) { return (size_t)cdiv(m, kT) * kTileBytes; }
int mixed_tiles(int m) { return cdiv(m, kT); }

static bool g_attr_done = false;

int set_mixed_attributes() {
  if (g_attr_done) return 0;
  cudaError_t e = cudaFuncSetAttribute(k_tc_syrk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSyrkSmem);
  if (e != cudaSuccess) return 1;
  size_t two = 2 * (size_t)kT * (kT + 1) * sizeof(float);
  e = cudaFuncSetAttribute(k_diag32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)two);
  if (e != cudaSuccess) return 1;
  e = cudaFuncSetAttribute(k_panel32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)two);
  if (e != cudaSuccess) return 1;
  g_attr_done = true;
  return 0;
}

// Returns the number of kernel launches.
int potrf_mixed(int m, double* A, int lda, unsigned char* PS, int* negpiv, int* err, cudaStream_t st,
                cudaEvent_t* syrk_ev, double* syrk_flop) {
  const int nt = cdiv(m, kT);
  const size_t two = 2 * (size_t)kT * (kT + 1) * sizeof(float);
  int L = 0;
  for (int k = 0; k < nt; k++) {
    const int k0 = k * kT, kb = (m - k0 < kT) ? m - k0 : kT;
    k_diag32<<<1, kT, two / 2, st>>>(A, lda, k0, kb, negpiv);
    L++;
    const int below = nt - k - 1;
    if (below <= 0) break;
    k_panel32<<<below, 128, two, st>>>(A, lda, m, k0, kb, k + 1, PS);
    const int pairs = below * (below + 1) / 2;
    if (syrk_ev) cudaEventRecord(syrk_ev[2 * k], st);
    k_tc_syrk<<<pairs, kSyrkThreads, kSyrkSmem, st>>>(A, lda, m, k, nt, PS, err);
    if (syrk_ev) cudaEventRecord(syrk_ev[2 * k + 1], st);
    if (syrk_flop) *syrk_flop += 6.0 * 2.0 * kT * kT * kT * pairs;  // BF16 tensor work issued
    L += 2;
  }
  return L;
}

}  // namespace bdk
