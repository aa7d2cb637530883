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

// ------------------------------------------------------------ diagonal block + panel
// One launch per panel k.  Every CTA loads the 128 x 128 diagonal block and
// factors it in shared memory (the factor is recomputed by each CTA instead
// of being passed between launches); CTA 0 writes L_kk back, CTA b >= 1
// solves the 128-row tile k + b:  X L_kk^T = A_ik.
//
// Both factorisations work on 32-column blocks, left-looking across blocks:
// block column j first takes  S[r][c] -= sum_{q < 32 j} S[r][q] L[c][q]  as
// one FP32 dot product per element (register-tiled 4 x 4 per thread), then
// the 32 x 32 diagonal block is factored by one warp in registers and the
// rows below it are solved by forward substitution, one row per thread.
// A negative pivot is replaced by its absolute value and counted
// (func.cpp:827-833), by CTA 0 only.
constexpr int kLd = 132;             // shared row stride (floats): 16-byte rows, conflict-free 4-wide loads
constexpr int kDpThreads = 256;
constexpr size_t kDpSmem = (2 * (size_t)kT * kLd + kT) * sizeof(float);

// Out[r][c] -= sum_{q < c0} In[r][q] * Lf[c][q] for r in [r0, r1), c in
// [c0, c0 + 32) (c < cend); lower-only (r >= c) when `lower`.
__device__ __forceinline__ void dp_block_update(float (*S)[kLd], const float (*Lf)[kLd], int r0, int r1, int c0,
                                                int cend, bool lower) {
  const int t = threadIdx.x;
  const int g = t & 7, rg = t >> 3;  // 8 column groups x 32 row groups
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.f;
  for (int q = 0; q < c0; q += 4) {
    float4 xv[4], lv[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int r = r0 + rg + 32 * i;
      xv[i] = (r < r1) ? *reinterpret_cast<const float4*>(&S[r][q]) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int j = 0; j < 4; j++) lv[j] = *reinterpret_cast<const float4*>(&Lf[c0 + g + 8 * j][q]);
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) {
        acc[i][j] = fmaf(xv[i].x, lv[j].x, acc[i][j]);
        acc[i][j] = fmaf(xv[i].y, lv[j].y, acc[i][j]);
        acc[i][j] = fmaf(xv[i].z, lv[j].z, acc[i][j]);
        acc[i][j] = fmaf(xv[i].w, lv[j].w, acc[i][j]);
      }
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int r = r0 + rg + 32 * i;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int c = c0 + g + 8 * j;
      if (r < r1 && c < cend && (!lower || r >= c)) S[r][c] -= acc[i][j];
    }
  }
}

// Forward substitution of one row against the 32 x 32 block of Lf at (c0, c0):
// x[c] = (b[c] - sum_{q < c} x[q] L[c0+c][c0+q]) / L[c0+c][c0+c], right-looking in registers.
__device__ __forceinline__ void dp_row_solve(float* row, const float (*Lf)[kLd], const float* invd, int c0, int w) {
  float x[32];
#pragma unroll
  for (int j = 0; j < 32; j++) x[j] = (j < w) ? row[j] : 0.f;
#pragma unroll
  for (int c = 0; c < 32; c++) {
    x[c] *= invd[c0 + c];
#pragma unroll
    for (int j = c + 1; j < 32; j++) x[j] = fmaf(-x[c], Lf[c0 + j][c0 + c], x[j]);
  }
#pragma unroll
  for (int j = 0; j < 32; j++)
    if (j < w) row[j] = x[j];
}

__global__ void __launch_bounds__(kDpThreads, 1) k_dpanel(double* A, int lda, int m, int k0, int kb, int tile0,
                                                         unsigned char* PS, int* negpiv) {
  extern __shared__ float4 sm4[];
  float (*Ls)[kLd] = reinterpret_cast<float (*)[kLd]>(sm4);
  float (*X)[kLd] = reinterpret_cast<float (*)[kLd]>(reinterpret_cast<float*>(sm4) + kT * kLd);
  float* invd = reinterpret_cast<float*>(sm4) + 2 * kT * kLd;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool is_diag = blockIdx.x == 0;
  const int tile = tile0 + (int)blockIdx.x - 1;
  const int row0 = tile * kT;
  const int nrows = is_diag ? 0 : min(kT, m - row0);
  for (int e = tid; e < kT * kT; e += kDpThreads) {
    const int c = e >> 7, r = e & (kT - 1);  // column-major walk: coalesced global reads
    Ls[r][c] = (r >= c && r < kb && c < kb) ? (float)A[(size_t)(k0 + c) * lda + k0 + r] : 0.f;
    if (!is_diag) X[r][c] = (r < nrows && c < kb) ? (float)A[(size_t)(k0 + c) * lda + row0 + r] : 0.f;
  }
  if (tid < kT) invd[tid] = 0.f;
  __syncthreads();
  const int nb = (kb + 31) >> 5;
  for (int jb = 0; jb < nb; jb++) {
    const int c0 = 32 * jb, w = min(32, kb - c0);
    if (jb > 0) {
      dp_block_update(Ls, Ls, c0, kb, c0, c0 + w, true);
      __syncthreads();
    }
    if (warp == 0) {
      float a[32];
#pragma unroll
      for (int j = 0; j < 32; j++) a[j] = (lane < w && j <= lane) ? Ls[c0 + lane][c0 + j] : 0.f;
#pragma unroll
      for (int c = 0; c < 32; c++) {
        if (c < w) {
          const float d = __shfl_sync(0xffffffffu, a[c], c);
          const float piv = sqrtf(fabsf(d));
          const float inv = 1.f / piv;
          if (lane == 0) {
            invd[c0 + c] = inv;
            if (is_diag && d < 0.f) atomicAdd(negpiv, 1);
          }
          if (lane == c) a[c] = piv;
          else if (lane > c) a[c] *= inv;
#pragma unroll
          for (int j = c + 1; j < 32; j++) {
            const float ljc = __shfl_sync(0xffffffffu, a[c], j);
            a[j] = fmaf(-a[c], ljc, a[j]);
          }
        }
      }
#pragma unroll
      for (int j = 0; j < 32; j++)
        if (lane < w && j <= lane) Ls[c0 + lane][c0 + j] = a[j];
    }
    __syncthreads();
    const int rb = c0 + 32;
    if (rb < kb && tid < kb - rb) dp_row_solve(&Ls[rb + tid][c0], Ls, invd, c0, w);
    __syncthreads();
  }
  if (is_diag) {
    for (int e = tid; e < kb * kb; e += kDpThreads) {
      const int c = e / kb, r = e - c * kb;
      if (r >= c) A[(size_t)(k0 + c) * lda + k0 + r] = (double)Ls[r][c];
    }
    return;
  }
  for (int jb = 0; jb < nb; jb++) {
    const int c0 = 32 * jb, w = min(32, kb - c0);
    if (jb > 0) {
      dp_block_update(X, Ls, 0, nrows, c0, c0 + w, false);
      __syncthreads();
    }
    if (tid < nrows) dp_row_solve(&X[tid][c0], Ls, invd, c0, w);
    __syncthreads();
  }
  // write L_ik back (FP64) and its three BF16 slices, pre-swizzled
  unsigned char* ps = PS + (size_t)tile * kTileBytes;
  for (int e = tid; e < kT * kT; e += kDpThreads) {
    const int c = e >> 7, r = e & (kT - 1);
    const bool in = r < nrows && c < kb;
    const float x = in ? X[r][c] : 0.f;
    if (in) A[(size_t)(k0 + c) * lda + row0 + r] = (double)x;
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h);
    const __nv_bfloat16 md = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(md);
    const __nv_bfloat16 lo = __float2bfloat16_rn(r2);
    const uint32_t off = swz_off(r, c);
    *reinterpret_cast<__nv_bfloat16*>(ps + off) = h;
    *reinterpret_cast<__nv_bfloat16*>(ps + kSliceBytes + off) = md;
    *reinterpret_cast<__nv_bfloat16*>(ps + 2 * kSliceBytes + off) = lo;
  }
}

// ------------------------------------------------------------ tensor-core trailing update
constexpr int kSyrkThreads = 128;
constexpr size_t kSyrkSmem = 2 * (size_t)kTileBytes + 1024 + 64;

// Tiles: col_only -> (jlo + blockIdx.x, jlo); otherwise the lower triangle
// of tiles (I, J) with jlo <= J <= I, from the linear block index.
__global__ void __launch_bounds__(kSyrkThreads, 1) k_tc_syrk(double* A, int lda, int m, int jlo, int col_only,
                                                            const unsigned char* __restrict__ PS, int* err) {
  extern __shared__ unsigned char smraw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  unsigned char* sA = sm;
  unsigned char* sB = sm + kTileBytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + 2 * kTileBytes);  // [0] loads, [1] mma
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2);
  const int rel = blockIdx.x;
  int Ip, Jp;
  if (col_only) {
    Ip = rel;
    Jp = 0;
  } else {
    Ip = (int)((sqrtf(8.f * (float)rel + 1.f) - 1.f) * 0.5f);
    while ((Ip + 1) * (Ip + 2) / 2 <= rel) Ip++;
    while (Ip * (Ip + 1) / 2 > rel) Ip--;
    Jp = rel - Ip * (Ip + 1) / 2;
  }
  const int I = jlo + Ip, J = jlo + Jp;
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

// two panel-slice buffers: panel k writes buffer k & 1 while the updates of
// panel k - 1 still read the other
size_t mixed_panel_bytes(int m) { return 2 * (size_t)cdiv(m, kT) * kTileBytes; }
int mixed_tiles(int m) { return cdiv(m, kT); }

static bool g_attr_done = false;

int set_mixed_attributes() {
  if (g_attr_done) return 0;
  cudaError_t e = cudaFuncSetAttribute(k_tc_syrk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSyrkSmem);
  if (e != cudaSuccess) return 1;
  e = cudaFuncSetAttribute(k_dpanel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDpSmem);
  if (e != cudaSuccess) return 1;
  g_attr_done = true;
  return 0;
}

int mixed_aux_create(MixedAux* x) {
  int lo = 0, hi = 0;
  if (cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess) return 1;
  x->prio_hi = hi;
  if (cudaStreamCreateWithPriority(&x->side, cudaStreamNonBlocking, lo) != cudaSuccess) return 1;
  for (cudaEvent_t* e : {&x->ev_fork, &x->ev_panel, &x->ev_rest})
    if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) return 1;
  return 0;
}

void mixed_aux_destroy(MixedAux* x) {
  for (cudaEvent_t* e : {&x->ev_fork, &x->ev_panel, &x->ev_rest})
    if (*e) cudaEventDestroy(*e), *e = nullptr;
  if (x->side) cudaStreamDestroy(x->side), x->side = nullptr;
}

template <typename... KArgs, typename... Args>
static void launch_prio(void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t st, int prio,
                        Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributePriority;
  at[0].val.priority = prio;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, args...);
}

// Right-looking with a lookahead of one panel, on two streams:
//   st   : panel k (k_dpanel), then panel k's update of column k+1 (the
//          next panel), at high priority;
//   side : panel k's update of the tiles right of column k+1.
// Panel k+1 is factored while the bulk of panel k's update runs.  Column
// k+1 is also updated by the side stream's update of panel k-1, so st waits
// for that one before updating the column; panel k+1's slices go to the
// other buffer, whose last reader (the side update of panel k-1) is done by
// then.  Returns the number of kernel launches.
int potrf_mixed(int m, double* A, int lda, unsigned char* PS, int* negpiv, int* err, cudaStream_t st,
                const MixedAux& aux, cudaEvent_t* kev, int* kev_pairs, double* kflop) {
  const int nt = cdiv(m, kT);
  const size_t buf = (size_t)nt * kTileBytes;
  int L = 0, pairs = 0;
  cudaEventRecord(aux.ev_fork, st);
  cudaStreamWaitEvent(aux.side, aux.ev_fork, 0);
  cudaEventRecord(aux.ev_rest, aux.side);
  for (int k = 0; k < nt; k++) {
    const int k0 = k * kT, kb = (m - k0 < kT) ? m - k0 : kT;
    const int below = nt - k - 1;
    unsigned char* psk = PS + (size_t)(k & 1) * buf;
    launch_prio(k_dpanel, below + 1, kDpThreads, kDpSmem, st, aux.prio_hi, A, lda, m, k0, kb, k + 1, psk, negpiv);
    L++;
    if (below <= 0) break;
    cudaEventRecord(aux.ev_panel, st);
    cudaStreamWaitEvent(st, aux.ev_rest, 0);
    launch_prio(k_tc_syrk, below, kSyrkThreads, kSyrkSmem, st, aux.prio_hi, A, lda, m, k + 1, 1,
                (const unsigned char*)psk, err);
    L++;
    const int rest = below - 1;
    cudaStreamWaitEvent(aux.side, aux.ev_panel, 0);
    if (rest > 0) {
      const int tiles = rest * (rest + 1) / 2;
      if (kev) cudaEventRecord(kev[2 * pairs], aux.side);
      k_tc_syrk<<<tiles, kSyrkThreads, kSyrkSmem, aux.side>>>(A, lda, m, k + 2, 0, psk, err);
      if (kev) cudaEventRecord(kev[2 * pairs + 1], aux.side);
      pairs++;
      if (kflop) *kflop += 6.0 * 2.0 * kT * kT * kT * tiles;  // BF16 tensor work issued
      L++;
    }
    cudaEventRecord(aux.ev_rest, aux.side);
  }
  cudaStreamWaitEvent(st, aux.ev_rest, 0);
  if (kev_pairs) *kev_pairs = pairs;
  return L;
}

}  // namespace bdk
