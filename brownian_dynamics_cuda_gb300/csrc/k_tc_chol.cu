// Mixed-precision Cholesky of the RPY tensor on the sm_103a tensor cores.
//
// Right-looking blocked factorisation with 128-wide panels.  The matrix is
// stored as double-float pairs (hi, lo) of FP32 (column-major, 8 bytes per
// element, ~48 significant bits), so the trailing updates accumulate without
// an FP32 rounding per panel and without FP64 arithmetic (GB300's FP64 rate
// is ~2 operations per clock per SM); the arithmetic is FP32-class.  One
// kernel, k_chol_step, runs two kinds of CTA side by side:
//   panel CTAs   factor the next panel: every one factors the 128 x 128
//                diagonal block in shared memory (FP32, 32-column blocks),
//                CTA 0 keeps it in a side buffer (copied into A after the
//                last panel) and the others solve one 128-row tile each,
//                L_ik = A_ik L_kk^-T, by forward substitution, write it back
//                and split it into three BF16 slices (hi + mid + lo = the
//                FP32 value exactly), stored pre-swizzled in the
//                128-byte-swizzle K-major layout the MMA reads; a negative
//                pivot is replaced by its absolute value and counted
//                (func.cpp:827-833).
//   update CTAs  trailing update A_IJ -= L_I L_J^T of one or two earlier
//                panels, a run of tiles per CTA, warp-specialised:
//                bulk-async operand copies, six BF16 products (hi.hi,
//                hi.mid, mid.hi, hi.lo, mid.mid, lo.hi) per panel into one of
//                two FP32 tensor-memory accumulators (tcgen05.mma,
//                M = N = 128, K = 16 per instruction), tcgen05.ld epilogue
//                subtracting into the double-float tile.  The dropped
//                products are below 2^-24 of the kept ones: FP32-class
//                products.
// The launches run on one stream, one at a time (the schedule is at
// potrf_mixed).  Every mbarrier wait is bounded; on a timeout the kernel
// records an error code, frees its tensor memory and returns.
#include <algorithm>
#include <utility>
#include <vector>

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
__device__ __forceinline__ int cdiv_d(int a, int b) { return (a + b - 1) / b; }

// byte offset of element (row r, column k) inside one pre-swizzled slice
__device__ __forceinline__ uint32_t swz_off(int r, int k) {
  int half = k >> 6, kk = k & 63;
  return half * kHalfBytes + (r >> 3) * 1024 + (r & 7) * 128 + ((((kk >> 3) ^ (r & 7)) & 7) << 4) + (kk & 7) * 2;
}

// (hi, lo) - v in double-float arithmetic: exact two-sums (Knuth), so the
// stored value keeps ~48 significant bits through every trailing update
// (no per-update FP32 rounding of the element) without any FP64 operation.
__device__ __forceinline__ float2 df_sub(float2 a, float v) {
  const float s = a.x - v;
  const float bb = s - a.x;
  float e = (a.x - (s - bb)) + (-v - bb);
  e += a.y;
  const float h = s + e;
  const float b2 = h - s;
  const float l = (s - (h - b2)) + (e - b2);
  return make_float2(h, l);
}

// ------------------------------------------------------------ diagonal block + panel
// Panel k runs in CTAs of the step launch: every panel CTA loads the
// 128 x 128 diagonal block and factors it in shared memory (the factor is
// recomputed by each CTA instead of being passed between CTAs); CTA 0 keeps
// L_kk, CTA b >= 1 also solves the 128-row tile k + b:  X L_kk^T = A_ik.
//
// The diagonal block and the tile are one tall 256-row panel in shared memory
// (rows 0..127 the diagonal block, 128..255 the tile), factored in 32-column
// blocks, left-looking across blocks: block column j first takes
//   S[r][c] -= sum_{q < 32 j} S[r][q] L[c][q]
// as one FP32 dot product per element (register-tiled, 7 rows x 4 columns per
// thread), then the 32 x 32 diagonal block is factored by one warp in
// registers and every row below it (diagonal-block rows and tile rows alike)
// is solved by forward substitution, one row per thread.  A negative pivot is
// replaced by its absolute value and counted (func.cpp:827-833), by CTA 0 only.
constexpr int kLd = 132;             // shared row stride (floats): 16-byte rows, conflict-free 4-wide loads
constexpr int kLt = 36;              // row stride of the transposed 32 x 32 factor
constexpr int kDpThreads = 256;
constexpr size_t kDpSmem = (2 * (size_t)kT * kLd + 32 * kLt) * sizeof(float);

#ifndef BD_DP_EVICT_FIRST
#define BD_DP_EVICT_FIRST 1  // L2 evict-first hint on the panel's tile loads and (L, 0) stores
#endif
#ifndef DP_MARK
#define DP_MARK(i)  // phase boundary of the panel CTAs (a timestamp hook for profiling builds)
#endif

// Row v of the block-column update: v < nd are diagonal-block rows c0 + v,
// the rest tile rows kT + (v - nd); -1 past the end.
__device__ __forceinline__ int dp_row(int v, int c0, int nd, int nv) {
  return v < nd ? c0 + v : (v < nv ? kT + v - nd : -1);
}

// S[r][c] -= sum_{qlo <= q < qhi} S[r][q] * S[c][q] for the nv rows of block
// column c0 (c in [c0, c0 + w)), lower part only inside the diagonal block;
// t in [0, 256) is the thread's index among the 256 taking part.  NI row
// groups of 32 (nv <= 32 NI); the operands of step q + 4 are loaded while
// step q's products are formed, and the products are issued component by
// component so that consecutive FMAs are independent.
template <int NI>
__device__ __forceinline__ void dp_block_update_n(float (*S)[kLd], int t, int c0, int w, int nd, int nv, int qlo,
                                                  int qhi) {
  const int g = t & 7, rg = t >> 3;  // 8 column groups x 32 row groups
  int rows[NI];
  const float* xr[NI];
  const float* lr[4];
  float acc[NI][4];
#pragma unroll
  for (int i = 0; i < NI; i++) {
    rows[i] = dp_row(rg + 32 * i, c0, nd, nv);
    xr[i] = S[rows[i] < 0 ? 0 : rows[i]];  // rows past the end read row 0; their sums are dropped
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.f;
  }
#pragma unroll
  for (int j = 0; j < 4; j++) lr[j] = S[c0 + g + 8 * j];
  float4 lv[4], xv[NI];
#pragma unroll
  for (int j = 0; j < 4; j++) lv[j] = *reinterpret_cast<const float4*>(lr[j] + qlo);
#pragma unroll
  for (int i = 0; i < NI; i++) xv[i] = *reinterpret_cast<const float4*>(xr[i] + qlo);
#pragma unroll 2
  for (int q = qlo; q < qhi; q += 4) {
    const int qn = (q + 4 < qhi) ? q + 4 : q;
    float4 ln[4], xn[NI];
#pragma unroll
    for (int j = 0; j < 4; j++) ln[j] = *reinterpret_cast<const float4*>(lr[j] + qn);
#pragma unroll
    for (int i = 0; i < NI; i++) xn[i] = *reinterpret_cast<const float4*>(xr[i] + qn);
#pragma unroll
    for (int i = 0; i < NI; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[i][j] = fmaf(xv[i].x, lv[j].x, acc[i][j]);
#pragma unroll
    for (int i = 0; i < NI; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[i][j] = fmaf(xv[i].y, lv[j].y, acc[i][j]);
#pragma unroll
    for (int i = 0; i < NI; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[i][j] = fmaf(xv[i].z, lv[j].z, acc[i][j]);
#pragma unroll
    for (int i = 0; i < NI; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[i][j] = fmaf(xv[i].w, lv[j].w, acc[i][j]);
#pragma unroll
    for (int j = 0; j < 4; j++) lv[j] = ln[j];
#pragma unroll
    for (int i = 0; i < NI; i++) xv[i] = xn[i];
  }
#pragma unroll
  for (int i = 0; i < NI; i++) {
    const int r = rows[i];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int c = c0 + g + 8 * j;
      if (r >= 0 && c < c0 + w && (r >= kT || r >= c)) S[r][c] -= acc[i][j];
    }
  }
}

// up to 96 diagonal-block rows + 128 tile rows: at most 7 row groups
__device__ __forceinline__ void dp_block_update(float (*S)[kLd], int t, int c0, int w, int nd, int nv, int qlo,
                                                int qhi) {
  switch ((nv + 31) >> 5) {
    case 1: dp_block_update_n<1>(S, t, c0, w, nd, nv, qlo, qhi); break;
    case 2: dp_block_update_n<2>(S, t, c0, w, nd, nv, qlo, qhi); break;
    case 3: dp_block_update_n<3>(S, t, c0, w, nd, nv, qlo, qhi); break;
    case 4: dp_block_update_n<4>(S, t, c0, w, nd, nv, qlo, qhi); break;
    case 5: dp_block_update_n<5>(S, t, c0, w, nd, nv, qlo, qhi); break;
    case 6: dp_block_update_n<6>(S, t, c0, w, nd, nv, qlo, qhi); break;
    default: dp_block_update_n<7>(S, t, c0, w, nd, nv, qlo, qhi); break;
  }
}

// Forward substitution of one row (32 entries at `row`, 16-byte aligned)
// against the factored 32 x 32 block, right-looking in registers:
//   x[c] = (b[c] - sum_{q < c} x[q] L[c][q]) / L[c][c].
// T is the block transposed, T[c][j] = L[j][c] (row stride kLt), with
// 1 / L[c][c] on its diagonal, so column c of L is one contiguous row.
__device__ __forceinline__ void dp_row_solve(float* row, const float* T, float (&x)[32]) {
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const float4 v = reinterpret_cast<const float4*>(row)[k];
    x[4 * k] = v.x, x[4 * k + 1] = v.y, x[4 * k + 2] = v.z, x[4 * k + 3] = v.w;
  }
#pragma unroll
  for (int c = 0; c < 32; c++) {
    float t[32];
#pragma unroll
    for (int k = c >> 2; k < 8; k++) {
      const float4 v = reinterpret_cast<const float4*>(T + c * kLt)[k];
      t[4 * k] = v.x, t[4 * k + 1] = v.y, t[4 * k + 2] = v.z, t[4 * k + 3] = v.w;
    }
    x[c] *= t[c];
#pragma unroll
    for (int j = c + 1; j < 32; j++) x[j] = fmaf(-x[c], t[j], x[j]);
  }
#pragma unroll
  for (int k = 0; k < 8; k++)
    reinterpret_cast<float4*>(row)[k] = make_float4(x[4 * k], x[4 * k + 1], x[4 * k + 2], x[4 * k + 3]);
}

// Cholesky of a 32 x 32 block held by one warp, lane i holding row i (a[j],
// j <= i), right-looking in registers.  Column c: 1/sqrt of the pivot once
// (rsqrt), the column scaled, then written as row c of T (T[c][j] = L[j][c],
// 1 / L[c][c] on the diagonal, zero above), from which every lane reads the
// column back with 16-byte broadcast loads for its rank-1 update.  The next
// pivot, A[c+1][c+1] - L[c+1][c]^2, is formed by lane c + 1 from its own
// entries and shuffled to all lanes at once, so only one shuffle per column
// is on the pivot chain.  FULL (w == 32) is branch-free; otherwise the rows
// of T past w are zeroed.  A negative pivot is replaced by its absolute
// value and flagged in `neg` (func.cpp:827-833).
template <bool FULL>
__device__ __forceinline__ void warp_chol32(float (&a)[32], int w, int lane, float* T, int& neg) {
  float d = __shfl_sync(0xffffffffu, a[0], 0);
#pragma unroll
  for (int c = 0; c < 32; c++) {
    if (!FULL && c >= w) break;
    const float ad = fabsf(d);
    const float inv = rsqrtf(ad);
    if (lane == c) neg |= d < 0.f;
    a[c] = (lane == c) ? ad * inv : ((lane > c) ? a[c] * inv : a[c]);
    if (c + 1 < 32) d = __shfl_sync(0xffffffffu, fmaf(-a[c], a[c], a[c + 1]), c + 1);
    T[c * kLt + lane] = (lane > c) ? a[c] : (lane == c ? inv : 0.f);
    __syncwarp();
#pragma unroll
    for (int k = (c + 1) >> 2; k < 8; k++) {
      const float4 tv = reinterpret_cast<const float4*>(T + c * kLt)[k];
      const float t4[4] = {tv.x, tv.y, tv.z, tv.w};
#pragma unroll
      for (int e = 0; e < 4; e++)
        if (4 * k + e > c) a[4 * k + e] = fmaf(-a[c], t4[e], a[4 * k + e]);
    }
  }
  if (!FULL)
    for (int c = w; c < 32; c++) T[c * kLt + lane] = 0.f;
  __syncwarp();
}

// Row r of the CTA's rows of L_ik (row rs of the 128-row tile), columns
// c0 .. c0 + 31 (x[j] = 0 past column w): (L, 0) pairs into A (`g` = A at
// column c0 of the CTA's first row) for rows inside the matrix, and the
// 16-byte chunks of the three BF16 slices (x = hi + mid + lo exactly,
// 8 + 8 + 8 significant bits) for every row of the tile.
__device__ __forceinline__ void dp_emit(const float (&x)[32], int r, int rs, int nrows, int c0, int w, float2* g,
                                        int lda, unsigned char* ps) {
  if (r < nrows) {  // read again only by the noise product after the factorisation (BD_DP_EVICT_FIRST)
    const uint64_t pol = sm100::policy_evict_first();
#pragma unroll
    for (int j = 0; j < 32; j++)
      if (j < w) {
        if (BD_DP_EVICT_FIRST) sm100::st_f2_hint(g + (size_t)j * lda + r, make_float2(x[j], 0.f), pol);
        else g[(size_t)j * lda + r] = make_float2(x[j], 0.f);
      }
  }
#pragma unroll
  for (int q8 = 0; q8 < 4; q8++) {
    uint32_t hw[4], mw[4], lw[4];
#pragma unroll
    for (int j2 = 0; j2 < 4; j2++) {
      uint32_t h2 = 0u, m2 = 0u, l2 = 0u;
#pragma unroll
      for (int e = 0; e < 2; e++) {
        const float v = x[8 * q8 + 2 * j2 + e];
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        const float r1 = v - __bfloat162float(h);
        const __nv_bfloat16 md = __float2bfloat16_rn(r1);
        const float r2 = r1 - __bfloat162float(md);
        const __nv_bfloat16 lo = __float2bfloat16_rn(r2);
        h2 |= (uint32_t)__bfloat16_as_ushort(h) << (16 * e);
        m2 |= (uint32_t)__bfloat16_as_ushort(md) << (16 * e);
        l2 |= (uint32_t)__bfloat16_as_ushort(lo) << (16 * e);
      }
      hw[j2] = h2, mw[j2] = m2, lw[j2] = l2;
    }
    const uint32_t off = swz_off(rs, c0 + 8 * q8);
    *reinterpret_cast<uint4*>(ps + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
    *reinterpret_cast<uint4*>(ps + kSliceBytes + off) = make_uint4(mw[0], mw[1], mw[2], mw[3]);
    *reinterpret_cast<uint4*>(ps + 2 * kSliceBytes + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
  }
}

// Runs in a CTA of kRestThreads (320) threads: 256 load, update and solve;
// while warp 0 factors a diagonal block, warps 2..9 update the next block
// column.  `b` is the CTA's index among the panel CTAs.
// The previous panel's update of this panel's column, applied in the panel
// CTA itself (so no separate launch precedes the panel): with panel p's
// slices PSpre, D0 = L_kp L_kp^T for the diagonal tile and (tile CTAs)
// D1 = L_ip L_kp^T for the CTA's tile, six BF16 products per K step on
// tcgen05 into two 128-column TMEM accumulators.  The operands are streamed
// in two K-halves into the memory the panel later uses for S, so the
// products are complete before S is loaded; they are subtracted from S
// after the load.  Every wait is bounded; a timeout records an error code.
struct PreBars {
  uint64_t full[2], done;
  uint32_t slot;
};
constexpr int kPreStage = 2 * kTileSlices * kHalfBytes;  // one K-half of the A and B slices (96 KB)

__device__ __forceinline__ void dpanel_body(float4* sm4, float2* A, float* Ldg, int lda, int m, int k0, int kb, int tile0,
                                            int b, unsigned char* PS, int* negpiv, const unsigned char* PSpre,
                                            int* err, int rpc) {
  float (*S)[kLd] = reinterpret_cast<float (*)[kLd]>(sm4);  // rows 0..127 diagonal block, 128..255 tile
  float* T = reinterpret_cast<float*>(sm4) + 2 * kT * kLd;  // the current 32 x 32 factor, transposed
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool work = tid < kDpThreads;
  const bool is_diag = b == 0;
  // tile CTAs take rpc (128 or 64) rows of a tile: b - 1 = (tile - tile0) (128 / rpc) + part
  const int parts = kT / rpc, part = is_diag ? 0 : (b - 1) % parts;
  const int tile = tile0 + (is_diag ? 0 : (b - 1) / parts);
  const int row0 = tile * kT + part * rpc;
  const int nrows = is_diag ? 0 : max(0, min(rpc, m - row0));
  DP_MARK(0);
  unsigned char* smA = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(sm4) + 1023) & ~uintptr_t(1023));
  PreBars* pbar = reinterpret_cast<PreBars*>(smA + 2 * kPreStage);
  uint32_t tmem = 0;
  bool pre_ok = true;
  if (PSpre) {
    if (tid == 0) {
      sm100::mbar_init(&pbar->full[0], 1);
      sm100::mbar_init(&pbar->full[1], 1);
      sm100::mbar_init(&pbar->done, 1);
      sm100::fence_mbar_init();
    }
    if (warp == 1) sm100::tmem_alloc(&pbar->slot, 2 * kT);
    sm100::tc_fence_before();
    __syncthreads();
    sm100::tc_fence_after();
    tmem = pbar->slot;
    if (tid == 0) {
      const unsigned char* gB = PSpre + (size_t)(tile0 - 1) * kTileBytes;  // this panel's tile row
      const unsigned char* gA = PSpre + (size_t)tile * kTileBytes;
      for (int h = 0; h < 2; h++) {  // stage h: [A: three 16 KB slice halves][B: three]
        unsigned char* st = smA + h * kPreStage;
        sm100::mbar_arrive_expect_tx(&pbar->full[h], (is_diag ? 1 : 2) * kTileSlices * kHalfBytes);
        for (int s2 = 0; s2 < kTileSlices; s2++)
          sm100::bulk_g2s(st + kTileSlices * kHalfBytes + s2 * kHalfBytes, gB + s2 * kSliceBytes + h * kHalfBytes,
                          kHalfBytes, &pbar->full[h]);
        if (!is_diag)
          for (int s2 = 0; s2 < kTileSlices; s2++)
            sm100::bulk_g2s(st + s2 * kHalfBytes, gA + s2 * kSliceBytes + h * kHalfBytes, kHalfBytes, &pbar->full[h]);
      }
      const uint32_t idesc = sm100::idesc_bf16_f32(128, 128);
      const int pa[6] = {2, 1, 0, 1, 0, 0};  // (A slice, B slice) products, smallest first
      const int pb[6] = {0, 1, 2, 0, 1, 0};
      bool ok = true;
      for (int h = 0; h < 2 && ok; h++) {
        ok = sm100::mbar_wait(&pbar->full[h], 0, kWaitLimit);
        if (!ok) break;
        sm100::tc_fence_after();
        const unsigned char* sa = smA + h * kPreStage;
        const unsigned char* sb = sa + kTileSlices * kHalfBytes;
#pragma unroll
        for (int p = 0; p < 6; p++) {
          const uint32_t b0 = sm100::smem_u32(sb + pa[p] * kHalfBytes), b1 = sm100::smem_u32(sb + pb[p] * kHalfBytes);
          const uint32_t a0 = sm100::smem_u32(sa + pa[p] * kHalfBytes);
#pragma unroll
          for (int kk = 0; kk < 4; kk++) {
            const uint32_t acc = (h | p | kk) != 0;
            sm100::mma_bf16(tmem, sm100::desc_kmajor_sw128(b0 + kk * 32), sm100::desc_kmajor_sw128(b1 + kk * 32), idesc,
                            acc);
            if (!is_diag)
              sm100::mma_bf16(tmem + kT, sm100::desc_kmajor_sw128(a0 + kk * 32), sm100::desc_kmajor_sw128(b1 + kk * 32),
                              idesc, acc);
          }
        }
      }
      sm100::mma_commit(&pbar->done);
      if (!ok) {
        atomicExch(err, 6);
        // copies still in flight land before their memory is reused
        (void)sm100::mbar_wait(&pbar->full[0], 0, kWaitLimit);
        (void)sm100::mbar_wait(&pbar->full[1], 0, kWaitLimit);
      }
    }
    // the products read the stage memory: complete before S overwrites it
    pre_ok = sm100::mbar_wait(&pbar->done, 0, kWaitLimit);
    sm100::tc_fence_after();
    pre_ok = __syncthreads_and(pre_ok);  // one decision for the whole CTA (it gates a named barrier below)
    if (!pre_ok && tid == 0) atomicExch(err, 7);
  }
  // Rows [0, nr) of a 128-row part of the panel (columns k0 .. k0 + kb) into
  // S[roff ..], FP32 (the nearest of each stored double-float; entries past
  // the part are zero), by 8 warps (w8 = 0 .. 7).  Two rows per 16-byte
  // load; lane l takes rows 2 (l & 3) + {0, 1} of an 8-row block and column
  // l >> 2 of an 8-column block, so a warp reads 64-byte runs of 8 columns
  // and its shared stores hit 32 distinct banks.  Row pairs start even and
  // lda is a multiple of 32: every load is aligned and stays inside its
  // column.  16 loads per thread in flight.
  const size_t ld4 = (size_t)lda / 2;
  const uint64_t pol = sm100::policy_evict_first();  // read once (BD_DP_EVICT_FIRST)
  auto load_part = [&](const float2* gbase, int roff, int nr, bool lower, int w8) {
    const int rr = 2 * (lane & 3), cc = lane >> 2;
    const float4* g4 = reinterpret_cast<const float4*>(gbase);
#pragma unroll 1
    for (int cb = w8; cb < kT / 8; cb += 8) {
      const int c = 8 * cb + cc;
      float4 v[16];
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const int r = 8 * i + rr;
        const bool in = (!lower || r + 1 >= c) && r < nr && c < kb;
        v[i] = in ? (BD_DP_EVICT_FIRST ? sm100::ld_f4_hint(g4 + c * ld4 + r / 2, pol) : g4[c * ld4 + r / 2])
                  : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const int r = 8 * i + rr;
        S[roff + r][c] = (r < nr && c < kb) ? v[i].x + v[i].y : 0.f;
        S[roff + r + 1][c] = (r + 1 < nr && c < kb) ? v[i].z + v[i].w : 0.f;
      }
    }
  };
  // the CTA's D accumulator rows into S: warp w reads TMEM lanes 32 (w % 4) ..
  auto subtract = [&](bool tile_part) {
    const int q = warp & 3, r = 32 * q + lane;
    const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16) + (tile_part ? (uint32_t)kT : 0u);
    float* row = tile_part ? S[kT + r - part * rpc] : S[r];
#pragma unroll 1
    for (int cc = 0; cc < kT; cc += 32) {
      float v[32];
      sm100::tmem_ld32(ta + cc, v);
#pragma unroll
      for (int k4 = 0; k4 < 8; k4++) {
        float4* p4 = reinterpret_cast<float4*>(row + cc + 4 * k4);
        float4 x = *p4;
        x.x -= v[4 * k4], x.y -= v[4 * k4 + 1], x.z -= v[4 * k4 + 2], x.w -= v[4 * k4 + 3];
        *p4 = x;
      }
    }
  };
  // the diagonal block first (and D0 off it); the tile rows load while the
  // first 32 x 32 block is factored (below)
  if (work) load_part(A + (size_t)k0 * lda + k0, 0, kb, true, warp);
  __syncthreads();
  if (PSpre && pre_ok && warp < 4) subtract(false);
  if (PSpre) sm100::tc_fence_before();
  __syncthreads();
  DP_MARK(1);
  const int nb = (kb + 31) >> 5;
  const int nrt = is_diag ? 0 : rpc;  // tile rows solved (rows past the matrix are zero and stay zero)
  for (int jb = 0; jb < nb; jb++) {
    const int c0 = 32 * jb, w = min(32, kb - c0);
    const int c1 = c0 + 32, w1 = kb - c1;  // the next block column (w1 <= 0: none)
    const int nd = max(0, w1);             // diagonal-block rows below this block
    // A: warp 0 factors the 32 x 32 diagonal block; warps 2..9 meanwhile
    // apply the finished block columns (q < c0) to the next block column
    if (warp == 0) {
      float a[32];
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const float4 v = lane < w ? reinterpret_cast<const float4*>(&S[c0 + lane][c0])[k] : make_float4(0.f, 0.f, 0.f, 0.f);
        a[4 * k] = v.x, a[4 * k + 1] = v.y, a[4 * k + 2] = v.z, a[4 * k + 3] = v.w;
      }
#pragma unroll
      for (int j = 0; j < 32; j++)
        if (j > lane) a[j] = 0.f;  // upper part: not referenced
      int neg = 0;
      if (w == 32) warp_chol32<true>(a, 32, lane, T, neg);
      else warp_chol32<false>(a, w, lane, T, neg);
      if (is_diag) {  // L_kk is kept by CTA 0 only; the others need T alone
        if (neg) atomicAdd(negpiv, 1);
#pragma unroll
        for (int j = 0; j < 32; j++)
          if (lane < w && j <= lane) S[c0 + lane][c0 + j] = a[j];
      }
    } else if (warp >= 2 && jb == 0) {
      // the tile rows (and the previous panel's update of them)
      if (!is_diag) {
        sm100::tc_fence_after();
        load_part(A + (size_t)k0 * lda + row0, kT, nrows, false, warp - 2);
        if (PSpre && pre_ok) {
          asm volatile("bar.sync 1, 256;" ::: "memory");  // warps 2..9: the tile rows loaded
          if (warp >= 4 && warp < 8 && (32 * (warp & 3)) / rpc == part) subtract(true);
        }
      }
    } else if (warp >= 2 && w1 > 0 && c0 > 0) {
      dp_block_update(S, tid - 64, c1, min(32, w1), nd, nd + nrows, 0, c0);
    }
    if (jb == 0 && PSpre) sm100::tc_fence_before();
    __syncthreads();
    if (jb == 0 && PSpre && warp == 1) sm100::tmem_dealloc(tmem, 2 * kT);
    DP_MARK(2 + 3 * jb);
    // B: the rows below the block, the rest of the diagonal block, then the
    // 128 tile rows; a tile row's 32 new entries of L_ik go out at once:
    // back into A as (L, 0) pairs and as three BF16 slices, pre-swizzled
    // (consecutive lanes take consecutive rows, so the pair stores are
    // coalesced)
    if (tid < nd + nrt) {
      float x[32];
      dp_row_solve(&S[tid < nd ? c1 + tid : kT + tid - nd][c0], T, x);
      if (tid >= nd) dp_emit(x, tid - nd, part * rpc + tid - nd, nrows, c0, w, A + (size_t)(k0 + c0) * lda + row0, lda,
                             PS + (size_t)tile * kTileBytes);
    }
    __syncthreads();
    DP_MARK(3 + 3 * jb);
    // C: this block column's contribution to the next one
    if (w1 > 0) {
      if (work) dp_block_update(S, tid, c1, min(32, w1), nd, nd + nrows, c0, c1);
      __syncthreads();
    }
    DP_MARK(4 + 3 * jb);
  }
  if (is_diag && work) {
    // L_kk goes to a side buffer, not into A: panel CTAs of this launch that
    // start after this one has finished (more CTAs than SMs) still read A_kk
    for (int e = tid; e < kT * kT; e += kDpThreads) {
      const int c = e >> 7, r = e & (kT - 1);
      Ldg[e] = (r >= c && r < kb && c < kb) ? S[r][c] : 0.f;  // column-major
    }
  }
  DP_MARK(15);
}

// ------------------------------------------------------------ tensor-core trailing update
// A_IJ -= L_I L_J^T for a run of up to `group` consecutive tiles per CTA
// (row-major order over the tile triangle, so consecutive tiles share I and
// the A operand stays in shared memory).  Warp-specialised, pipelined:
//   warp 0 (one lane)  bulk-async copies: the three A slices when I changes,
//                      the three B slices per tile in two K-halves (two
//                      48 KB stages), and an L2 prefetch of the FP64 tile;
//   warp 1 (one lane)  six BF16 products per K-half into one of two TMEM
//                      accumulators (128 columns each), tcgen05.commit to
//                      release stages, the accumulator and the A operand;
//   warps 2-9          epilogue: tcgen05.ld of the accumulator (warp w reads
//                      TMEM lanes 32 (w % 4) .. + 31, half of the columns),
//                      release it, then the FP64 read-modify-write.
// So the next tile's copies and MMAs run under the current tile's epilogue.
// Every wait is bounded; a timeout records an error code and raises a
// shared abort flag that ends every role's loop; copies still in flight
// are waited for (bounded) and TMEM is freed before the CTA exits.
#ifndef BD_REST_PREFETCH
#define BD_REST_PREFETCH 0  // L2 prefetch of the FP64 tile ahead of the epilogue (measured slower)
#endif
#ifndef BD_EPI_EVICT_FIRST
#define BD_EPI_EVICT_FIRST 1  // L2 evict-first hint on the epilogue's tile loads and stores
#endif
#ifndef BD_EPI_AHEAD
#define BD_EPI_AHEAD 8  // chunks of 8 columns whose old values are in flight per epilogue thread (4: 8 % slower bulk)
#endif
#ifndef BD_EPI_TMEM_COLS
#define BD_EPI_TMEM_COLS 8  // accumulator columns per TMEM read of the bulk epilogue (8, 16 or 32)
#endif
#ifndef BD_REST_GROUP
#define BD_REST_GROUP 0  // tiles per CTA; 0: from the tile count
#endif
#ifndef BD_REST_WAVES
#define BD_REST_WAVES 3  // from the tile count: about this many CTAs per SM ...
#endif
#ifndef BD_REST_GMIN
#define BD_REST_GMIN 1  // ... with at least / at most this many tiles each
#endif
#ifndef BD_REST_GMAX
#define BD_REST_GMAX 8
#endif
constexpr int kRestThreads = 320;
constexpr int kStageBytes = kTileSlices * kHalfBytes;  // one K-half of the three B slices
constexpr size_t kRestSmem = (size_t)kTileBytes + 2 * kStageBytes + 1024 + 256;
constexpr int kAccCols = 128;

struct RestBars {
  uint64_t fullA, emptyA, fullB[2], emptyB[2], accFull[2], accEmpty[2], done;
};

// Tile t of an update job's enumeration, from column jlo:
//   kRowTri  the triangle I >= J >= jlo row by row (consecutive tiles share I),
//   kCol     column jlo alone (I = jlo + t).
enum { kRowTri = 0, kCol = 1 };
__device__ __forceinline__ void rest_tile(int t, int jlo, int mode, int nt, int& I, int& J) {
  if (mode == kCol) {
    I = jlo + t;
    J = jlo;
    return;
  }
  int Ip = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
  while ((Ip + 1) * (Ip + 2) / 2 <= t) Ip++;
  while (Ip * (Ip + 1) / 2 > t) Ip--;
  I = jlo + Ip;
  J = jlo + (t - Ip * (Ip + 1) / 2);
}

// `cta` is the CTA's index among the update CTAs.
// NPAN = 1: one panel's update, the A operand resident per row of tiles.
// NPAN = 2, 3: two or three consecutive panels' updates (PS, PS2, PS3) in one
// read-modify-write of the tile (K = 256, 384): both operands streamed in
// 2 NPAN chunks of 96 KB per tile (panel, K-half) through the two stages.
template <int NPAN>
__device__ __forceinline__ void rest_body(unsigned char* smraw, float2* A, int lda, int m, int jlo, int mode,
                                          int tlo, int thi, int group, int cta, const unsigned char* __restrict__ PS,
                                          const unsigned char* __restrict__ PS2, const unsigned char* __restrict__ PS3,
                                          int* err) {
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  unsigned char* sA = sm;                 // 3 slices x 32 KB
  unsigned char* sB = sm + kTileBytes;    // 2 stages x (3 slices x 16 KB)
  RestBars* bars = reinterpret_cast<RestBars*>(sm + kTileBytes + 2 * kStageBytes);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t0 = tlo + cta * group, t1 = min(t0 + group, thi);
  const int nt = cdiv_d(m, kT);

  if (threadIdx.x == 0) {
    sm100::mbar_init(&bars->fullA, 1);
    sm100::mbar_init(&bars->emptyA, 1);
    for (int h = 0; h < 2; h++) {
      sm100::mbar_init(&bars->fullB[h], 1);
      sm100::mbar_init(&bars->emptyB[h], 1);
      sm100::mbar_init(&bars->accFull[h], 1);
      sm100::mbar_init(&bars->accEmpty[h], 8);
    }
    sm100::mbar_init(&bars->done, 1);
    *abort_flag = 0;
    sm100::fence_mbar_init();
  }
  if (warp == 1) sm100::tmem_alloc(tslot, 2 * kAccCols);
  sm100::tc_fence_before();
  __syncthreads();
  sm100::tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- producer
      if constexpr (NPAN == 1) {
      int curI = -1;
      uint32_t nA = 0, nfill[2] = {0, 0};
      bool ok = true;
      for (int t = t0; t < t1 && ok; t++) {
        int I, J;
        rest_tile(t, jlo, mode, nt, I, J);
        if (I != curI) {
          if (nA > 0) ok = sm100::mbar_wait(&bars->emptyA, (nA - 1) & 1, kWaitLimit);
          if (!ok || *abort_flag) break;
          sm100::mbar_arrive_expect_tx(&bars->fullA, kTileBytes);
          const unsigned char* g = PS + (size_t)I * kTileBytes;
          for (int s2 = 0; s2 < kTileSlices; s2++)
            sm100::bulk_g2s(sA + s2 * kSliceBytes, g + s2 * kSliceBytes, kSliceBytes, &bars->fullA);
          curI = I;
          nA++;
        }
        if (BD_REST_PREFETCH) {  // the FP64 tile's columns into L2 ahead of the epilogue
          const int rows = min(kT, lda - I * kT);
          const int jend = min(J * kT + kT, m);
          for (int gj = J * kT; gj < jend; gj++)
            sm100::prefetch_l2(A + (size_t)gj * lda + (size_t)I * kT, (uint32_t)rows * 8u);
        }
        for (int h = 0; h < 2 && ok; h++) {
          if (nfill[h] > 0) ok = sm100::mbar_wait(&bars->emptyB[h], (nfill[h] - 1) & 1, kWaitLimit);
          if (!ok || *abort_flag) {
            ok = false;
            break;
          }
          if (I == J) {
            sm100::mbar_arrive(&bars->fullB[h]);  // diagonal tile: B is the A operand
          } else {
            sm100::mbar_arrive_expect_tx(&bars->fullB[h], kStageBytes);
            const unsigned char* g = PS + (size_t)J * kTileBytes + h * kHalfBytes;
            for (int s2 = 0; s2 < kTileSlices; s2++)
              sm100::bulk_g2s(sB + h * kStageBytes + s2 * kHalfBytes, g + s2 * kSliceBytes, kHalfBytes,
                              &bars->fullB[h]);
          }
          nfill[h]++;
        }
      }
      if (!ok) {
        atomicExch(err, 3);
        *abort_flag = 1;
      }
      // copies still in flight land before the CTA exits
      for (int h = 0; h < 2; h++)
        if (nfill[h] > 0) (void)sm100::mbar_wait(&bars->fullB[h], (nfill[h] - 1) & 1, kWaitLimit);
      if (nA > 0) (void)sm100::mbar_wait(&bars->fullA, (nA - 1) & 1, kWaitLimit);
      } else {
        // NPAN panels: chunk q = (panel q >> 1, K-half q & 1) of both operands
        uint32_t nfill[2] = {0, 0};
        int ctot = 0;
        bool ok = true;
        for (int t = t0; t < t1 && ok; t++) {
          int I, J;
          rest_tile(t, jlo, mode, nt, I, J);
          const bool dg = I == J;
          for (int q = 0; q < 2 * NPAN; q++) {
            const int st = ctot & 1;
            if (nfill[st] > 0) ok = sm100::mbar_wait(&bars->emptyB[st], (nfill[st] - 1) & 1, kWaitLimit);
            if (!ok || *abort_flag) {
              ok = false;
              break;
            }
            const unsigned char* src = (q >> 1) == 0 ? PS : ((q >> 1) == 1 ? PS2 : PS3);
            const int h = q & 1;
            unsigned char* sa = sm + st * (2 * kStageBytes);
            sm100::mbar_arrive_expect_tx(&bars->fullB[st], dg ? kStageBytes : 2 * kStageBytes);
            for (int s2 = 0; s2 < kTileSlices; s2++)
              sm100::bulk_g2s(sa + s2 * kHalfBytes, src + (size_t)I * kTileBytes + s2 * kSliceBytes + h * kHalfBytes,
                              kHalfBytes, &bars->fullB[st]);
            if (!dg)
              for (int s2 = 0; s2 < kTileSlices; s2++)
                sm100::bulk_g2s(sa + kStageBytes + s2 * kHalfBytes,
                                src + (size_t)J * kTileBytes + s2 * kSliceBytes + h * kHalfBytes, kHalfBytes,
                                &bars->fullB[st]);
            nfill[st]++;
            ctot++;
          }
        }
        if (!ok) {
          atomicExch(err, 3);
          *abort_flag = 1;
        }
        for (int h = 0; h < 2; h++)
          if (nfill[h] > 0) (void)sm100::mbar_wait(&bars->fullB[h], (nfill[h] - 1) & 1, kWaitLimit);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer
      if constexpr (NPAN == 1) {
      const uint32_t idesc = sm100::idesc_bf16_f32(128, 128);
      const int pa[6] = {2, 1, 0, 1, 0, 0};  // (A slice, B slice) products, smallest first
      const int pb[6] = {0, 1, 2, 0, 1, 0};
      int curI = -1;
      uint32_t nA = 0;
      bool ok = true;
      int n = 0;
      for (int t = t0; t < t1; t++, n++) {
        int I, J;
        rest_tile(t, jlo, mode, nt, I, J);
        if (*abort_flag) break;
        if (I != curI) {
          ok = sm100::mbar_wait(&bars->fullA, nA & 1, kWaitLimit);
          if (!ok) break;
          curI = I;
          nA++;
        }
        const int acc = n & 1;
        if (n >= 2) {
          ok = sm100::mbar_wait(&bars->accEmpty[acc], ((n >> 1) - 1) & 1, kWaitLimit);
          if (!ok) break;
        }
        sm100::tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(acc * kAccCols);
        for (int h = 0; h < 2 && ok; h++) {
          ok = sm100::mbar_wait(&bars->fullB[h], n & 1, kWaitLimit);
          if (!ok) break;
          sm100::tc_fence_after();
#pragma unroll
          for (int p = 0; p < 6; p++) {
            const uint32_t aaddr = sm100::smem_u32(sA + pa[p] * kSliceBytes + h * kHalfBytes);
            const uint32_t baddr = (I == J) ? sm100::smem_u32(sA + pb[p] * kSliceBytes + h * kHalfBytes)
                                            : sm100::smem_u32(sB + h * kStageBytes + pb[p] * kHalfBytes);
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
              sm100::mma_bf16(d, sm100::desc_kmajor_sw128(aaddr + kk * 32), sm100::desc_kmajor_sw128(baddr + kk * 32),
                              idesc, (h | p | kk) != 0);
          }
          sm100::mma_commit(&bars->emptyB[h]);
        }
        if (!ok) break;
        sm100::mma_commit(&bars->accFull[acc]);
        int In = -1, Jn;
        if (t + 1 < t1) rest_tile(t + 1, jlo, mode, nt, In, Jn);
        if (In != I) sm100::mma_commit(&bars->emptyA);
      }
      if (!ok) {
        atomicExch(err, 4);
        *abort_flag = 1;
      }
      } else {
        const uint32_t idesc = sm100::idesc_bf16_f32(128, 128);
        const int pa[6] = {2, 1, 0, 1, 0, 0};
        const int pb[6] = {0, 1, 2, 0, 1, 0};
        uint32_t nuse[2] = {0, 0};
        int ctot = 0;
        bool ok = true;
        int n = 0;
        for (int t = t0; t < t1; t++, n++) {
          int I, J;
          rest_tile(t, jlo, mode, nt, I, J);
          if (*abort_flag) break;
          const bool dg = I == J;
          const int acc = n & 1;
          if (n >= 2) {
            ok = sm100::mbar_wait(&bars->accEmpty[acc], ((n >> 1) - 1) & 1, kWaitLimit);
            if (!ok) break;
          }
          sm100::tc_fence_after();
          const uint32_t d = tmem + (uint32_t)(acc * kAccCols);
          for (int q = 0; q < 2 * NPAN && ok; q++) {
            const int st = ctot & 1;
            ok = sm100::mbar_wait(&bars->fullB[st], nuse[st] & 1, kWaitLimit);
            if (!ok) break;
            sm100::tc_fence_after();
            const unsigned char* sa = sm + st * (2 * kStageBytes);
            const unsigned char* sb = dg ? sa : sa + kStageBytes;
#pragma unroll
            for (int p = 0; p < 6; p++) {
              const uint32_t aaddr = sm100::smem_u32(sa + pa[p] * kHalfBytes);
              const uint32_t baddr = sm100::smem_u32(sb + pb[p] * kHalfBytes);
#pragma unroll
              for (int kk = 0; kk < 4; kk++)
                sm100::mma_bf16(d, sm100::desc_kmajor_sw128(aaddr + kk * 32),
                                sm100::desc_kmajor_sw128(baddr + kk * 32), idesc, (q | p | kk) != 0);
            }
            sm100::mma_commit(&bars->emptyB[st]);
            nuse[st]++;
            ctot++;
          }
          if (!ok) break;
          sm100::mma_commit(&bars->accFull[acc]);
        }
        if (!ok) {
          atomicExch(err, 4);
          *abort_flag = 1;
        }
      }
      // every MMA issued has finished before TMEM is freed
      sm100::mma_commit(&bars->done);
      (void)sm100::mbar_wait(&bars->done, 0, kWaitLimit);
    }
  } else {
    // ---------------- epilogue
    // Each thread owns one row of the tile and the warp's 64-column half, in
    // chunks of kEpC columns.  The old double-float values of kEpS chunks are
    // in flight at all times: a chunk's slot is refilled as soon as it has
    // been written back, with a later chunk of this tile or the matching
    // chunk of the next one, so the loads run ahead of the accumulator and
    // across tile boundaries.
    constexpr int kEpC = 8, kEpN = 64 / kEpC, kEpS = BD_EPI_AHEAD;
    static_assert(kEpN % kEpS == 0, "slots must divide the chunks");
    const int q = warp & 3, ch = (warp - 2) >> 2;
    // the tiles stream through L2 once per launch: marked first for eviction
    // (BD_EPI_EVICT_FIRST), so the panel slices and the next launch's column
    // stay resident
    const uint64_t pol = sm100::policy_evict_first();
    auto ld_tile = [&](const float2* a) { return BD_EPI_EVICT_FIRST ? sm100::ld_f2_hint(a, pol) : *a; };
    auto st_tile = [&](float2* a, float2 v) {
      if (BD_EPI_EVICT_FIRST) sm100::st_f2_hint(a, v, pol);
      else *a = v;
    };
    // columns [0, jcnt) of this thread's row of tile t are inside the matrix
    // and the lower triangle, at colp + j lda
    auto row_of = [&](int t, float2*& colp, int& jcnt) {
      int I, J;
      rest_tile(t, jlo, mode, nt, I, J);
      const int gi = I * kT + 32 * q + lane;
      const int cbase = J * kT + 64 * ch;
      const int jlim0 = (I == J) ? max(0, gi - cbase + 1) : 64;  // diagonal tile: columns <= gi
      jcnt = gi < m ? min(min(jlim0, 64), m - cbase) : 0;
      colp = A + (size_t)cbase * lda + gi;
    };
    float2 old[kEpS][kEpC];
    auto load_chunk = [&](float2 (&o)[kEpC], const float2* colp, int jcnt, int c) {
#pragma unroll
      for (int j = 0; j < kEpC; j++)
        o[j] = (kEpC * c + j < jcnt) ? ld_tile(colp + (size_t)(kEpC * c + j) * lda) : make_float2(0.f, 0.f);
    };
    float2* colp = A;
    int jcnt = 0;
    if (t0 < t1) {
      row_of(t0, colp, jcnt);
#pragma unroll
      for (int s2 = 0; s2 < kEpS; s2++) load_chunk(old[s2], colp, jcnt, s2);
    }
    int n = 0;
    for (int t = t0; t < t1; t++, n++) {
      const bool more = t + 1 < t1;
      float2* ncolp = A;
      int njcnt = 0;
      if (more) row_of(t + 1, ncolp, njcnt);
      const int acc = n & 1;
      const bool ok = sm100::mbar_wait(&bars->accFull[acc], (n >> 1) & 1, kWaitLimit);
      if (!ok || *abort_flag) {
        if (!ok && lane == 0) {
          atomicExch(err, 5);
          *abort_flag = 1;
        }
        break;
      }
      sm100::tc_fence_after();
      const uint32_t ta = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(acc * kAccCols + 64 * ch);
      // the accumulator is read kEpT columns at a time (one wait per read)
      constexpr int kEpT = BD_EPI_TMEM_COLS, kEpR = kEpT / kEpC;
      static_assert(kEpT % kEpC == 0 && kEpN % kEpR == 0, "TMEM reads cover whole chunks");
      float vt[kEpT];
#pragma unroll
      for (int c = 0; c < kEpN; c++) {
        const int s2 = c % kEpS;
        if (c % kEpR == 0) {
          if (kEpT == 8) sm100::tmem_ld8(ta + kEpC * c, vt);
          else if (kEpT == 16) sm100::tmem_ld16(ta + kEpC * c, vt);
          else sm100::tmem_ld32(ta + kEpC * c, vt);
          if (c + kEpR == kEpN) {  // accumulator read out: hand it back to the MMA issuer
            sm100::tc_fence_before();
            __syncwarp();
            if (lane == 0) sm100::mbar_arrive(&bars->accEmpty[acc]);
          }
        }
        const float* v = vt + kEpC * (c % kEpR);
#pragma unroll
        for (int j = 0; j < kEpC; j++)
          if (kEpC * c + j < jcnt) st_tile(colp + (size_t)(kEpC * c + j) * lda, df_sub(old[s2][j], v[j]));
        if (c + kEpS < kEpN) load_chunk(old[s2], colp, jcnt, c + kEpS);
        else if (more) load_chunk(old[s2], ncolp, njcnt, c + kEpS - kEpN);
      }
      colp = ncolp;
      jcnt = njcnt;
    }
  }
  sm100::tc_fence_before();
  __syncthreads();
  if (warp == 1) sm100::tmem_dealloc(tmem, 2 * kAccCols);
}

// An update job: tiles [tlo, thi) of an enumeration (rest_tile) from column
// jlo, panel slices ps (and ps2: two panels, K = 256), `group` tiles per CTA.
struct UpdJob {
  const unsigned char* ps;
  const unsigned char* ps2;  // second panel (K = 256) or null
  const unsigned char* ps3;  // third panel (K = 384) or null
  int jlo, mode, tlo, thi, group, nctas;
};
struct StepArgs {
  float2* A;
  float* Ldg;           // this panel's diagonal factor
  unsigned char* PSp;   // this panel's slice buffer
  const unsigned char* PSpre;  // the previous panel's slices: its update of this panel's column, or null
  int* negpiv;
  int* err;
  int lda, m, ndp, pk0, pkb;
  int prows;  // tile rows per panel CTA (128, or 64 when the panel is split over twice the CTAs)
  UpdJob job[2];
};

// One launch per step: CTAs [0, ndp) factor panel pk (diagonal block and the
// tiles below it, writing its slices to PSp); then the CTAs of update job 0,
// then those of job 1.  The parts of one launch touch disjoint tiles and
// slice buffers.
__device__ __forceinline__ void chol_step_body(const StepArgs& a, int b, float4* smem4) {
  if (b < a.ndp) {
    dpanel_body(smem4, a.A, a.Ldg, a.lda, a.m, a.pk0, a.pkb, a.pk0 / kT + 1, b, a.PSp, a.negpiv, a.PSpre, a.err,
                a.prows);
    return;
  }
  b -= a.ndp;
  const int jn = b < a.job[0].nctas ? 0 : 1;
  if (jn) b -= a.job[0].nctas;
  const UpdJob& j = a.job[jn];
  if (j.ps3)
    rest_body<3>(reinterpret_cast<unsigned char*>(smem4), a.A, a.lda, a.m, j.jlo, j.mode, j.tlo, j.thi, j.group, b,
                 j.ps, j.ps2, j.ps3, a.err);
  else if (j.ps2)
    rest_body<2>(reinterpret_cast<unsigned char*>(smem4), a.A, a.lda, a.m, j.jlo, j.mode, j.tlo, j.thi, j.group, b,
                 j.ps, j.ps2, nullptr, a.err);
  else
    rest_body<1>(reinterpret_cast<unsigned char*>(smem4), a.A, a.lda, a.m, j.jlo, j.mode, j.tlo, j.thi, j.group, b,
                 j.ps, nullptr, nullptr, a.err);
}

__global__ void __launch_bounds__(kRestThreads, 1) k_chol_step(const __grid_constant__ StepArgs a) {
  extern __shared__ float4 smem4[];
  chol_step_body(a, (int)blockIdx.x, smem4);
}

// The same step for many independent factorisations in one launch (replicas
// of a batch): factorisation r owns CTAs [off[r], off[r + 1]) and runs its own
// schedule's step with args[r]; the factorisations share no memory.
__global__ void __launch_bounds__(kRestThreads, 1) k_chol_step_multi(const StepArgs* __restrict__ args,
                                                                      const int* __restrict__ off, int nrep) {
  extern __shared__ float4 smem4[];
  const int bid = (int)blockIdx.x;
  int lo = 0, hi = nrep;  // off[lo] <= bid < off[lo + 1]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= bid) lo = mid;
    else hi = mid;
  }
  chol_step_body(args[lo], bid - off[lo], smem4);
}

// After the last panel: the diagonal factors L_kk from the side buffer into
// the lower triangles of A's diagonal blocks, as (L, 0) pairs.
__device__ __forceinline__ void diag_scatter_body(float2* A, int lda, int m, const float* __restrict__ Ld, int k) {
  const int k0 = k * kT, kb = min(kT, m - k0);
  const float* src = Ld + (size_t)k * kT * kT;
  for (int e = threadIdx.x; e < kT * kT; e += blockDim.x) {
    const int c = e >> 7, r = e & (kT - 1);
    if (r >= c && r < kb && c < kb) A[(size_t)(k0 + c) * lda + k0 + r] = make_float2(src[e], 0.f);
  }
}
__global__ void __launch_bounds__(256) k_diag_scatter(float2* A, int lda, int m, const float* __restrict__ Ld) {
  diag_scatter_body(A, lda, m, Ld, blockIdx.x);
}
struct ScatterArgs {
  float2* A;
  int lda, m;
  const float* Ld;
};
// every factorisation of a batch (blockIdx.y), diagonal block blockIdx.x
__global__ void __launch_bounds__(256) k_diag_scatter_multi(const ScatterArgs* __restrict__ sc) {
  const ScatterArgs a = sc[blockIdx.y];
  if ((int)blockIdx.x * kT >= a.m) return;
  diag_scatter_body(a.A, a.lda, a.m, a.Ld, blockIdx.x);
}

}  // namespace

namespace bdk {

// kBufs panel-slice buffers, panel p in buffer p % kBufs: a triple's bulk
// update reads panels k .. k + 2 while panel k + 3 is written
constexpr int kBufs = 4;
size_t mixed_panel_bytes(int m) {  // the slice buffers, then the diagonal factors
  return kBufs * (size_t)cdiv(m, kT) * kTileBytes + (size_t)cdiv(m, kT) * kT * kT * sizeof(float);
}
int mixed_max_launches(int m) { return 2 * cdiv(m, kT) + 2; }
int mixed_tiles(int m) { return cdiv(m, kT); }

static bool g_attr_done = false;

int set_mixed_attributes() {
  if (g_attr_done) return 0;
  static_assert(kDpSmem <= kRestSmem, "panel CTAs run inside the update kernel's shared memory");
  cudaError_t e = cudaFuncSetAttribute(k_chol_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRestSmem);
  if (e != cudaSuccess) return 1;
  e = cudaFuncSetAttribute(k_chol_step_multi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRestSmem);
  if (e != cudaSuccess) return 1;
  g_attr_done = true;
  return 0;
}

// Tiles per CTA of the bulk update: enough CTAs to fill the GPU about three
// times over, at most 8 tiles each.
static int rest_group(int tiles) {
  if (BD_REST_GROUP > 0) return BD_REST_GROUP;
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  int g = tiles / (BD_REST_WAVES * sms);
  return g < BD_REST_GMIN ? BD_REST_GMIN : (g > BD_REST_GMAX ? BD_REST_GMAX : g);
}

// Right-looking with a lookahead of one panel, on one stream, no two kernels
// at a time; every launch is one k_chol_step: panel pn in its own CTAs (which
// first apply panel pn-1's update to column pn themselves) beside up to two
// update jobs.  Panel p's slices live in buffer p % kBufs, L_kk in a side
// buffer.  Invariant before the launch of panel k+1: panels <= k are
// factored and column k+1 holds the updates of panels < k.
// Single step: panel k+1 beside panel k's update of the tiles right of
// column k+1 (K = 128).
// Pair (k+1, k+2), while the trailing matrix is large: the bulk tiles get
// both panels in one read-modify-write (K = 256), half the HBM traffic:
//   1: panel k+1 beside panel k's update of column k+2;
//   2: panel k+2 beside panels k and k+1 on the tiles right of column k+2.
// Triple (k+1 .. k+3), while it is larger still (K = 384):
//   1: panel k+1 beside panel k's update of column k+2;
//   2: panel k+2 beside panels k and k+1 on column k+3 (K = 256);
//   3: panel k+3 beside panels k .. k+2 on the tiles right of column k+3.
// Returns the number of kernel launches.
#ifndef BD_PAIR_MIN
#define BD_PAIR_MIN 24  // pair while at least this many tile rows remain right of column k+2 (k: last factored)
#endif
#ifndef BD_SPLIT_CTAS
#define BD_SPLIT_CTAS 151  // panel CTAs allowed when the panel is split in 64-row parts
#endif
#ifndef BD_SPLIT_JOB_TILES
#define BD_SPLIT_JOB_TILES 400  // ... and at most this many update tiles in the launch
#endif
#ifndef BD_TRIPLE_MIN
#define BD_TRIPLE_MIN 40  // three panels per bulk pass while this many tile rows remain right of column k+3
#endif
namespace {
struct Job {
  const unsigned char* ps = nullptr;
  const unsigned char* ps2 = nullptr;
  const unsigned char* ps3 = nullptr;
  int jlo = 0, mode = kCol, tiles = 0, group = 1;
};
}  // namespace

// The launches of one factorisation: issued on st, or (plan != nullptr)
// only recorded with their grid sizes, without the final diagonal scatter.
// max_pass (1..3): most panels one bulk pass carries (K = 128 max_pass).
// Fewer panels per pass mean fewer FP32 tensor-memory accumulation steps per
// stored update and more read-modify-write passes: 3 is the fastest, 1 the
// most accurate.
static int potrf_mixed_impl(int m, double* A64, int lda, unsigned char* PS, int* negpiv, int* err, cudaStream_t st,
                            cudaEvent_t* kev, int* kev_pairs, double* kflop, double* kbytes,
                            std::vector<std::pair<StepArgs, int>>* plan, int max_pass) {
  float2* A = reinterpret_cast<float2*>(A64);  // double-float storage, 8 bytes per element
  const int nt = cdiv(m, kT);
  const size_t buf = (size_t)nt * kTileBytes;
  int L = 0, timed = 0;
  auto kb_of = [&](int k) { return (m - k * kT < kT) ? m - k * kT : kT; };
  auto psb = [&](int k) { return PS + (size_t)(k % kBufs) * buf; };
  float* Ld = reinterpret_cast<float*>(PS + kBufs * buf);  // [nt][128 x 128] diagonal factors
  // elements of the lower triangle in tile columns [j0, j1)
  auto elems = [&](int j0, int j1) {
    double e = 0.0;
    for (int J = j0; J < j1 && J < nt; J++) {
      const double cols = kb_of(J);
      e += cols * (double)(m - J * kT) - cols * (cols - 1) / 2;
    }
    return e;
  };
  auto col_job = [&](int p, int J, int npan = 1) {  // panels p .. p + npan - 1 on column J
    Job j;
    j.ps = psb(p), j.ps2 = npan > 1 ? psb(p + 1) : nullptr, j.jlo = J, j.mode = kCol, j.tiles = nt - J, j.group = 1;
    return j;
  };
  auto tri_job = [&](int p, int npan, int jlo) {  // panels p .. p + npan - 1 on the triangle from column jlo
    Job j;
    const int n = nt - jlo;
    j.ps = psb(p), j.ps2 = npan > 1 ? psb(p + 1) : nullptr, j.ps3 = npan > 2 ? psb(p + 2) : nullptr;
    j.jlo = jlo, j.mode = kRowTri;
    j.tiles = n > 0 ? n * (n + 1) / 2 : 0;
    j.group = rest_group(j.tiles);
    return j;
  };
  // pn: the panel factored by this launch (-1: none); pre: panel pn - 1's
  // update of column pn is applied by the panel CTAs themselves
  auto launch = [&](int pn, const Job& j0, const Job& j1, bool pre) {
    StepArgs a{};
    a.A = A, a.negpiv = negpiv, a.err = err, a.lda = lda, a.m = m;
    a.Ldg = Ld, a.PSp = PS, a.PSpre = nullptr, a.prows = kT;
    if (pn >= 0) {
      // the panel over twice the CTAs (64 tile rows each) when they fit on
      // the GPU beside small update jobs: the diagonal work is repeated,
      // the tile work halved
      const int jt = (j0.tiles > 0 ? j0.tiles : 0) + (j1.tiles > 0 ? j1.tiles : 0);
      if (2 * (nt - pn - 1) + 1 <= BD_SPLIT_CTAS && jt <= BD_SPLIT_JOB_TILES) a.prows = kT / 2;
      a.ndp = 1 + (nt - pn - 1) * (kT / a.prows), a.pk0 = pn * kT, a.pkb = kb_of(pn);
      a.Ldg = Ld + (size_t)pn * kT * kT, a.PSp = psb(pn);
      if (pre && pn > 0) a.PSpre = psb(pn - 1);
    }
    const Job* js[2] = {&j0, &j1};
    int grid = a.ndp;
    for (int q = 0; q < 2; q++) {
      const Job& j = *js[q];
      UpdJob& u = a.job[q];
      u.ps = j.ps, u.ps2 = j.ps2, u.ps3 = j.ps3, u.jlo = j.jlo, u.mode = j.mode, u.tlo = 0, u.thi = j.tiles,
      u.group = j.group;
      u.nctas = j.tiles > 0 ? cdiv(j.tiles, j.group) : 0;
      grid += u.nctas;
    }
    if (grid == 0) return;
    if (plan) {
      plan->emplace_back(a, grid);
      return;
    }
    if (kev) cudaEventRecord(kev[2 * timed], st);
    k_chol_step<<<grid, kRestThreads, kRestSmem, st>>>(a);
    if (kev) {
      cudaEventRecord(kev[2 * timed + 1], st);
      timed++;
    }
    L++;
    if (kbytes || kflop) {
      double by = pn >= 0 ? 16.0 * (double)(m - pn * kT) * kb_of(pn) : 0.0;  // panel read and written back
      double fl = a.PSpre ? 6.0 * 2.0 * kT * kT * kT * (2 * a.ndp - 1) : 0.0;  // the panel CTAs' own products
      for (int q = 0; q < 2; q++) {
        const Job& j = *js[q];
        if (j.tiles <= 0) continue;
        by += 16.0 * elems(j.jlo, j.mode == kCol ? j.jlo + 1 : nt);  // double-float tile read + write
        fl += 6.0 * 2.0 * kT * kT * kT * j.tiles * (j.ps3 ? 3 : (j.ps2 ? 2 : 1));  // BF16 tensor work issued
      }
      if (kbytes) *kbytes += by;
      if (kflop) *kflop += fl;
    }
  };
  const Job none;
  launch(0, none, none, false);  // panel 0 alone
  int k = 0;
  while (k + 1 < nt) {
    if (max_pass >= 3 && nt - (k + 4) >= BD_TRIPLE_MIN) {
      launch(k + 1, col_job(k, k + 2), none, true);
      launch(k + 2, col_job(k, k + 3, 2), none, true);
      launch(k + 3, tri_job(k, 3, k + 4), none, true);
      k += 3;
    } else if (max_pass >= 2 && nt - (k + 3) >= BD_PAIR_MIN) {
      launch(k + 1, col_job(k, k + 2), none, true);
      launch(k + 2, tri_job(k, 2, k + 3), none, true);
      k += 2;
    } else {
      launch(k + 1, tri_job(k, 1, k + 2), none, true);
      k += 1;
    }
  }
  if (plan) return L;
  k_diag_scatter<<<nt, 256, 0, st>>>(A, lda, m, Ld);
  L++;
  if (kev_pairs) *kev_pairs = timed;
  return L;
}

int potrf_mixed(int m, double* A64, int lda, unsigned char* PS, int* negpiv, int* err, cudaStream_t st,
                cudaEvent_t* kev, int* kev_pairs, double* kflop, double* kbytes, int max_pass) {
  return potrf_mixed_impl(m, A64, lda, PS, negpiv, err, st, kev, kev_pairs, kflop, kbytes, nullptr, max_pass);
}

// Factorisations of a batch advanced together: launch i of the batch runs
// step i of every factorisation whose schedule has one, each in its own CTA
// range; the step arguments and CTA offsets of every launch are uploaded
// once (the matrices and buffers do not move).
#ifndef BD_BATCH_ALIGN
#define BD_BATCH_ALIGN 0
#endif
struct MixedBatch {
  std::vector<int> nrep_at, grid_at;
  std::vector<size_t> args_at, off_at;
  StepArgs* d_args = nullptr;
  int* d_off = nullptr;
  ScatterArgs* d_sc = nullptr;
  int nrep = 0, max_nt = 0;
};

MixedBatch* mixed_batch_create(int nrep, const int* m, double* const* A, const int* lda, unsigned char* const* PS,
                               int* const* negpiv, int* const* err, int max_pass) {
  std::vector<std::vector<std::pair<StepArgs, int>>> plans(nrep);
  size_t steps = 0;
  MixedBatch* b = new MixedBatch();
  b->nrep = nrep;
  std::vector<ScatterArgs> sc(nrep);
  for (int r = 0; r < nrep; r++) {
    potrf_mixed_impl(m[r], A[r], lda[r], PS[r], negpiv[r], err[r], nullptr, nullptr, nullptr, nullptr, nullptr,
                     &plans[r], max_pass);
    steps = std::max(steps, plans[r].size());
    const int nt = cdiv(m[r], kT);
    b->max_nt = std::max(b->max_nt, nt);
    sc[r].A = reinterpret_cast<float2*>(A[r]);
    sc[r].lda = lda[r];
    sc[r].m = m[r];
    sc[r].Ld = reinterpret_cast<const float*>(PS[r] + kBufs * (size_t)nt * kTileBytes);
  }
  std::vector<StepArgs> args;
  std::vector<int> off;
  for (size_t i = 0; i < steps; i++) {
    b->args_at.push_back(args.size());
    b->off_at.push_back(off.size());
    int n = 0, total = 0;
    for (int r = 0; r < nrep; r++) {
      // replica r's schedule starts at launch `shift` (BD_BATCH_ALIGN 1: every
      // schedule ends with the last launch; 0: every one starts with the first)
      const size_t shift = BD_BATCH_ALIGN ? steps - plans[r].size() : 0;
      if (i < shift || i - shift >= plans[r].size()) continue;
      args.push_back(plans[r][i - shift].first);
      off.push_back(total);
      total += plans[r][i - shift].second;
      n++;
    }
    off.push_back(total);
    b->nrep_at.push_back(n);
    b->grid_at.push_back(total);
  }
  bool ok = cudaMalloc(&b->d_args, std::max<size_t>(1, args.size()) * sizeof(StepArgs)) == cudaSuccess &&
            cudaMalloc(&b->d_off, std::max<size_t>(1, off.size()) * sizeof(int)) == cudaSuccess &&
            cudaMalloc(&b->d_sc, nrep * sizeof(ScatterArgs)) == cudaSuccess &&
            cudaMemcpy(b->d_args, args.data(), args.size() * sizeof(StepArgs), cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(b->d_off, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(b->d_sc, sc.data(), nrep * sizeof(ScatterArgs), cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    mixed_batch_free(b);
    return nullptr;
  }
  return b;
}

int mixed_batch_run(const MixedBatch* b, cudaStream_t st) {
  int L = 0;
  for (size_t i = 0; i < b->grid_at.size(); i++) {
    k_chol_step_multi<<<b->grid_at[i], kRestThreads, kRestSmem, st>>>(b->d_args + b->args_at[i],
                                                                         b->d_off + b->off_at[i], b->nrep_at[i]);
    L++;
  }
  k_diag_scatter_multi<<<dim3(b->max_nt, b->nrep), 256, 0, st>>>(b->d_sc);
  return L + 1;
}

void mixed_batch_free(MixedBatch* b) {
  if (!b) return;
  if (b->d_args) cudaFree(b->d_args);
  if (b->d_off) cudaFree(b->d_off);
  if (b->d_sc) cudaFree(b->d_sc);
  delete b;
}

}  // namespace bdk


