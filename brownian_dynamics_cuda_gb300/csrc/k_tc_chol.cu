// Mixed-precision Cholesky of the RPY tensor on the sm_103a tensor cores.
//
// Right-looking blocked factorisation with 128-wide panels.  The matrix is
// stored as double-float pairs (hi, lo) of FP32 (column-major, 8 bytes per
// element, ~48 significant bits), so the trailing updates accumulate without
// an FP32 rounding per panel and without FP64 arithmetic (GB300's FP64 rate
// is ~2 operations per clock per SM); the arithmetic is FP32-class:
//   k_dpanel    one launch per panel: every CTA factors the 128 x 128
//               diagonal block in shared memory (FP32, 32-column blocks,
//               left-looking across blocks), CTA 0 keeps it in a side buffer
//               (copied into A after the last panel) and the
//               others solve one 128-row tile each, L_ik = A_ik L_kk^-T, by
//               forward substitution, write it back and split it into three
//               BF16 slices (hi + mid + lo = the FP32 value exactly), stored
//               pre-swizzled in the 128-byte-swizzle K-major layout the MMA
//               reads; a negative pivot is replaced by its absolute value and
//               counted (func.cpp:827-833).
//   k_tc_rest   trailing update A_IJ -= L_I L_J^T, a run of tiles per CTA,
//               warp-specialised: bulk-async operand copies, six BF16
//               products (hi.hi, hi.mid, mid.hi, hi.lo, mid.mid, lo.hi) into
//               one of two FP32 tensor-memory accumulators (tcgen05.mma,
//               M = N = 128, K = 16 per instruction), tcgen05.ld epilogue
//               subtracting into the double-float tile.  The dropped products are below 2^-24 of
//               the kept ones: FP32-class products.
// A one-panel lookahead runs the next panel on a second stream while the
// bulk update of the current one runs.  Every mbarrier wait is bounded; on
// a timeout the kernel records an error code, frees its tensor memory and
// returns.
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

// Runs in a CTA of kRestThreads threads; threads >= kDpThreads only take
// part in the barriers.  `b` is the CTA's index among the panel CTAs.
// Cholesky of a 32 x 32 block held by one warp, lane i holding row i (a[j],
// j <= i), right-looking in registers: pivot from lane c, 1/sqrt once
// (rsqrt), column c scaled, rank-1 update of the columns to its right with
// L[j][c] shuffled from lane j.  FULL (w == 32) is branch-free, so the
// compiler can start column c+1's pivot while column c's update is in
// flight.  Lane c keeps 1/L[c][c] in invv and flags a negative pivot
// (replaced by its absolute value, func.cpp:827-833).
template <bool FULL>
__device__ __forceinline__ void warp_chol32(float (&a)[32], int w, int lane, float& invv, int& neg) {
#pragma unroll
  for (int c = 0; c < 32; c++) {
    if (!FULL && c >= w) break;
    const float d = __shfl_sync(0xffffffffu, a[c], c);
    const float ad = fabsf(d);
    const float inv = rsqrtf(ad);
    if (lane == c) {
      invv = inv;
      neg = d < 0.f;
    }
    a[c] = (lane == c) ? ad * inv : ((lane > c) ? a[c] * inv : a[c]);
#pragma unroll
    for (int j = c + 1; j < 32; j++) a[j] = fmaf(-a[c], __shfl_sync(0xffffffffu, a[c], j), a[j]);
  }
}

__device__ __forceinline__ void dpanel_body(float4* sm4, float2* A, float* Ldg, int lda, int m, int k0, int kb, int tile0,
                                            int b, unsigned char* PS, int* negpiv) {
  float (*Ls)[kLd] = reinterpret_cast<float (*)[kLd]>(sm4);
  float (*X)[kLd] = reinterpret_cast<float (*)[kLd]>(reinterpret_cast<float*>(sm4) + kT * kLd);
  float* invd = reinterpret_cast<float*>(sm4) + 2 * kT * kLd;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool work = tid < kDpThreads;
  const bool is_diag = b == 0;
  const int tile = tile0 + b - 1;
  const int row0 = tile * kT;
  const int nrows = is_diag ? 0 : min(kT, m - row0);
  if (work) {
    // column-major walk (a warp reads 32 consecutive rows of one column),
    // 16 columns per batch so that 32 loads per thread are in flight
    const int r = tid & (kT - 1), cq = tid >> 7;
    const float2* ga = A + (size_t)k0 * lda + k0 + r;
    const float2* gx = A + (size_t)k0 * lda + row0 + r;
#pragma unroll 1
    for (int i0 = 0; i0 < kT / 2; i0 += 16) {
      float2 va[16], vx[16];
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const int c = cq + 2 * (i0 + i);
        va[i] = (r >= c && r < kb && c < kb) ? ga[(size_t)c * lda] : make_float2(0.f, 0.f);
        vx[i] = (!is_diag && r < nrows && c < kb) ? gx[(size_t)c * lda] : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const int c = cq + 2 * (i0 + i);
        Ls[r][c] = va[i].x + va[i].y;  // nearest FP32 of the stored double-float
        X[r][c] = vx[i].x + vx[i].y;
      }
    }
  }
  if (tid < kT) invd[tid] = 0.f;
  __syncthreads();
  const int nb = (kb + 31) >> 5;
  for (int jb = 0; jb < nb; jb++) {
    const int c0 = 32 * jb, w = min(32, kb - c0);
    if (jb > 0) {
      if (work) dp_block_update(Ls, Ls, c0, kb, c0, c0 + w, true);
      __syncthreads();
    }
    if (warp == 0) {
      float a[32];
#pragma unroll
      for (int j = 0; j < 32; j++) a[j] = (lane < w && j <= lane) ? Ls[c0 + lane][c0 + j] : 0.f;
      float invv = 0.f;
      int neg = 0;
      if (w == 32) warp_chol32<true>(a, 32, lane, invv, neg);
      else warp_chol32<false>(a, w, lane, invv, neg);
      if (lane < w) invd[c0 + lane] = invv;
      if (is_diag && neg) atomicAdd(negpiv, 1);
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
    // L_kk goes to a side buffer, not into A: panel CTAs of this launch that
    // start after this one has finished (more CTAs than SMs) still read A_kk
    if (work)
      for (int e = tid; e < kT * kT; e += kDpThreads) {
        const int c = e >> 7, r = e & (kT - 1);
        Ldg[e] = (r >= c && r < kb && c < kb) ? Ls[r][c] : 0.f;  // column-major
      }
    return;
  }
  for (int jb = 0; jb < nb; jb++) {
    const int c0 = 32 * jb, w = min(32, kb - c0);
    if (jb > 0) {
      if (work) dp_block_update(X, Ls, 0, nrows, c0, c0 + w, false);
      __syncthreads();
    }
    if (tid < nrows) dp_row_solve(&X[tid][c0], Ls, invd, c0, w);
    __syncthreads();
  }
  // write L_ik back (FP64) and its three BF16 slices, pre-swizzled: each
  // thread takes one row and 8 consecutive columns, i.e. one 16-byte chunk
  // of each slice (consecutive lanes: consecutive rows, coalesced FP64 stores)
  unsigned char* ps = PS + (size_t)tile * kTileBytes;
  float2* gout = A + (size_t)k0 * lda + row0;
#pragma unroll 1
  for (int e = tid; work && e < kT * (kT / 8); e += kDpThreads) {
    const int r = e & (kT - 1), c0 = (e >> 7) * 8;
    const float4 x0 = *reinterpret_cast<const float4*>(&X[r][c0]);
    const float4 x1 = *reinterpret_cast<const float4*>(&X[r][c0 + 4]);
    const float xs[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
    uint32_t hw[4], mw[4], lw[4];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const bool in = r < nrows && c0 + j < kb;
      const float x = in ? xs[j] : 0.f;
      if (in) gout[(size_t)(c0 + j) * lda + r] = make_float2(x, 0.f);
      // x = hi + mid + lo exactly (8 + 8 + 8 significant bits)
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      const float r1 = x - __bfloat162float(h);
      const __nv_bfloat16 md = __float2bfloat16_rn(r1);
      const float r2 = r1 - __bfloat162float(md);
      const __nv_bfloat16 lo = __float2bfloat16_rn(r2);
      const uint32_t sh = (j & 1) * 16;
      if ((j & 1) == 0) hw[j >> 1] = mw[j >> 1] = lw[j >> 1] = 0u;
      hw[j >> 1] |= (uint32_t)__bfloat16_as_ushort(h) << sh;
      mw[j >> 1] |= (uint32_t)__bfloat16_as_ushort(md) << sh;
      lw[j >> 1] |= (uint32_t)__bfloat16_as_ushort(lo) << sh;
    }
    const uint32_t off = swz_off(r, c0);
    *reinterpret_cast<uint4*>(ps + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
    *reinterpret_cast<uint4*>(ps + kSliceBytes + off) = make_uint4(mw[0], mw[1], mw[2], mw[3]);
    *reinterpret_cast<uint4*>(ps + 2 * kSliceBytes + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
  }
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
#ifndef BD_REST_GROUP
#define BD_REST_GROUP 0  // tiles per CTA; 0: from the tile count
#endif
constexpr int kRestThreads = 320;
constexpr int kStageBytes = kTileSlices * kHalfBytes;  // one K-half of the three B slices
constexpr size_t kRestSmem = (size_t)kTileBytes + 2 * kStageBytes + 1024 + 256;
constexpr int kAccCols = 128;

struct RestBars {
  uint64_t fullA, emptyA, fullB[2], emptyB[2], accFull[2], accEmpty[2], done;
};

__device__ __forceinline__ void rest_tile(int t, int jlo, int col_only, int& I, int& J) {
  if (col_only) {
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
// NPAN = 2: two consecutive panels' updates (PS, PS2) in one read-modify-write
// of the tile (K = 256): both operands streamed in four 96 KB chunks per
// tile (panel, K-half) through the two stages.
template <int NPAN>
__device__ __forceinline__ void rest_body(unsigned char* smraw, float2* A, int lda, int m, int jlo, int col_only,
                                          int ntiles, int group, int cta, const unsigned char* __restrict__ PS,
                                          const unsigned char* __restrict__ PS2, int* err) {
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
  unsigned char* sA = sm;                 // 3 slices x 32 KB
  unsigned char* sB = sm + kTileBytes;    // 2 stages x (3 slices x 16 KB)
  RestBars* bars = reinterpret_cast<RestBars*>(sm + kTileBytes + 2 * kStageBytes);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t0 = cta * group, t1 = min(t0 + group, ntiles);
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
        rest_tile(t, jlo, col_only, I, J);
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
        // two panels: chunk q = (panel q >> 1, K-half q & 1) of both operands
        uint32_t nfill[2] = {0, 0};
        int ctot = 0;
        bool ok = true;
        for (int t = t0; t < t1 && ok; t++) {
          int I, J;
          rest_tile(t, jlo, col_only, I, J);
          const bool dg = I == J;
          for (int q = 0; q < 4; q++) {
            const int st = ctot & 1;
            if (nfill[st] > 0) ok = sm100::mbar_wait(&bars->emptyB[st], (nfill[st] - 1) & 1, kWaitLimit);
            if (!ok || *abort_flag) {
              ok = false;
              break;
            }
            const unsigned char* src = (q >> 1) ? PS2 : PS;
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
        rest_tile(t, jlo, col_only, I, J);
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
        if (t + 1 < t1) rest_tile(t + 1, jlo, col_only, In, Jn);
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
          rest_tile(t, jlo, col_only, I, J);
          if (*abort_flag) break;
          const bool dg = I == J;
          const int acc = n & 1;
          if (n >= 2) {
            ok = sm100::mbar_wait(&bars->accEmpty[acc], ((n >> 1) - 1) & 1, kWaitLimit);
            if (!ok) break;
          }
          sm100::tc_fence_after();
          const uint32_t d = tmem + (uint32_t)(acc * kAccCols);
          for (int q = 0; q < 4 && ok; q++) {
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
    const int q = warp & 3, ch = (warp - 2) >> 2;
    int n = 0;
    for (int t = t0; t < t1; t++, n++) {
      int I, J;
      rest_tile(t, jlo, col_only, I, J);
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
      const int gi = I * kT + 32 * q + lane;
      const bool diag = I == J;
      const bool row_ok = gi < m;
      // columns [jlim0, jlim1) of this thread's row are inside the matrix and the lower triangle
      const int cbase = J * kT + 64 * ch;
      const int jlim0 = diag ? max(0, gi - cbase + 1) : 64;  // diagonal tile: columns <= gi
      const int jcnt = row_ok ? min(min(jlim0, 64), m - cbase) : 0;
      float2* colp = A + (size_t)cbase * lda + gi;
#pragma unroll
      for (int c = 0; c < 2; c++) {
        float2 old[32];
        float v[32];
#pragma unroll
        for (int j = 0; j < 32; j++)
          old[j] = (32 * c + j < jcnt) ? colp[(size_t)(32 * c + j) * lda] : make_float2(0.f, 0.f);
        sm100::tmem_ld32(ta + 32 * c, v);
        if (c == 1) {  // accumulator read out: hand it back to the MMA issuer
          sm100::tc_fence_before();
          __syncwarp();
          if (lane == 0) sm100::mbar_arrive(&bars->accEmpty[acc]);
        }
#pragma unroll
        for (int j = 0; j < 32; j++)
          if (32 * c + j < jcnt) colp[(size_t)(32 * c + j) * lda] = df_sub(old[j], v[j]);
      }
    }
  }
  sm100::tc_fence_before();
  __syncthreads();
  if (warp == 1) sm100::tmem_dealloc(tmem, 2 * kAccCols);
}

// One launch per panel step: CTAs [0, ndp) factor panel pk (diagonal block
// and the tiles below it, writing its slices to PSp); the remaining CTAs
// apply an earlier panel's trailing update (tiles from jlo, slices PSu).
// The two parts touch disjoint columns and slice buffers.
__global__ void __launch_bounds__(kRestThreads, 1) k_chol_step(float2* A, float* Ldg, int lda, int m, int ndp, int pk0, int pkb,
                                                              unsigned char* PSp, int* negpiv, int jlo, int col_only,
                                                              int ntiles, int group,
                                                              const unsigned char* __restrict__ PSu,
                                                              const unsigned char* __restrict__ PSu2, int* err) {
  extern __shared__ float4 smem4[];
  if ((int)blockIdx.x < ndp) {
    dpanel_body(smem4, A, Ldg, lda, m, pk0, pkb, pk0 / kT + 1, (int)blockIdx.x, PSp, negpiv);
    return;
  }
  if (PSu2)
    rest_body<2>(reinterpret_cast<unsigned char*>(smem4), A, lda, m, jlo, col_only, ntiles, group,
                 (int)blockIdx.x - ndp, PSu, PSu2, err);
  else
    rest_body<1>(reinterpret_cast<unsigned char*>(smem4), A, lda, m, jlo, col_only, ntiles, group,
                 (int)blockIdx.x - ndp, PSu, nullptr, err);
}

// After the last panel: the diagonal factors L_kk from the side buffer into
// the lower triangles of A's diagonal blocks, as (L, 0) pairs.
__global__ void __launch_bounds__(256) k_diag_scatter(float2* A, int lda, int m, const float* __restrict__ Ld) {
  const int k = blockIdx.x, k0 = k * kT, kb = min(kT, m - k0);
  const float* src = Ld + (size_t)k * kT * kT;
  for (int e = threadIdx.x; e < kT * kT; e += blockDim.x) {
    const int c = e >> 7, r = e & (kT - 1);
    if (r >= c && r < kb && c < kb) A[(size_t)(k0 + c) * lda + k0 + r] = make_float2(src[e], 0.f);
  }
}

}  // namespace

namespace bdk {

// two panel-slice buffers: panel k writes buffer k & 1 while the updates of
// panel k - 1 still read the other
size_t mixed_panel_bytes(int m) {  // three slice buffers, then the diagonal factors
  return 3 * (size_t)cdiv(m, kT) * kTileBytes + (size_t)cdiv(m, kT) * kT * kT * sizeof(float);
}
int mixed_tiles(int m) { return cdiv(m, kT); }

static bool g_attr_done = false;

int set_mixed_attributes() {
  if (g_attr_done) return 0;
  static_assert(kDpSmem <= kRestSmem, "panel CTAs run inside the update kernel's shared memory");
  cudaError_t e = cudaFuncSetAttribute(k_chol_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRestSmem);
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
  int g = tiles / (3 * sms);
  return g < 1 ? 1 : (g > 8 ? 8 : g);
}

// Right-looking with a lookahead of one panel, on one stream, no two kernels
// at a time.  Panel p's slices live in buffer p % 3; L_kk in a side buffer.
// Single step k (invariant: panel k factored, columns > k hold the updates
// of panels < k):
//   launch 1: panel k's update of column k+1;
//   launch 2: panel k+1 (extra CTAs) + panel k's update of the tiles right
//             of column k+1.
// Pair (k, k+1), used while the trailing matrix is large: the bulk tiles
// get both panels in one read-modify-write (K = 256), half the HBM traffic:
//   launch 1: panel k's update of column k+1;
//   launch 2: panel k+1 + panel k's update of column k+2;
//   launch 3: panel k+1's update of column k+2;
//   launch 4: panel k+2 + panels k and k+1 on the tiles right of column k+2.
// Returns the number of kernel launches.
#ifndef BD_PAIR_MIN
#define BD_PAIR_MIN 24  // pair while at least this many tile rows remain right of column k+2
#endif
int potrf_mixed(int m, double* A64, int lda, unsigned char* PS, int* negpiv, int* err, cudaStream_t st,
                cudaEvent_t* kev, int* kev_pairs, double* kflop, double* kbytes) {
  float2* A = reinterpret_cast<float2*>(A64);  // double-float storage, 8 bytes per element
  const int nt = cdiv(m, kT);
  const size_t buf = (size_t)nt * kTileBytes;
  int L = 0, pairs = 0;
  auto kb_of = [&](int k) { return (m - k * kT < kT) ? m - k * kT : kT; };
  auto psb = [&](int k) { return PS + (size_t)(k % 3) * buf; };
  float* Ld = reinterpret_cast<float*>(PS + 3 * buf);  // [nt][128 x 128] diagonal factors
  auto col = [&](int k) {  // panel k's update of column k+1
    const int below = nt - k - 1;
    k_chol_step<<<below, kRestThreads, kRestSmem, st>>>(A, Ld, lda, m, 0, 0, 0, nullptr, negpiv, k + 1, 1, below, 1,
                                                         psb(k), nullptr, err);
    L++;
  };
  // panel pn in extra CTAs + an update of the tiles from column jlo by panel
  // pu (and pu + 1 when two), triangle or (col_only) one column
  auto step = [&](int pn, int jlo, int pu, bool two, bool col_only, bool timed) {
    const int ndp = nt - pn;
    const int rows = nt - jlo;
    const int tiles = rows <= 0 ? 0 : (col_only ? rows : rows * (rows + 1) / 2);
    const int group = (tiles > 0 && !col_only) ? rest_group(tiles) : 1;
    if (timed && kev) cudaEventRecord(kev[2 * pairs], st);
    k_chol_step<<<ndp + cdiv(tiles, group), kRestThreads, kRestSmem, st>>>(
        A, Ld + (size_t)pn * kT * kT, lda, m, ndp, pn * kT, kb_of(pn), (unsigned char*)psb(pn), negpiv, jlo,
        col_only ? 1 : 0, tiles, group, psb(pu), two ? psb(pu + 1) : nullptr, err);
    if (timed && kev) {
      cudaEventRecord(kev[2 * pairs + 1], st);
      pairs++;
    }
    if (timed) {
      const double n2 = (double)(m - jlo * kT);
      if (kflop) *kflop += 6.0 * 2.0 * kT * kT * kT * tiles * (two ? 2 : 1);  // BF16 tensor work issued
      if (kbytes && n2 > 0) *kbytes += 16.0 * n2 * (n2 + 1) / 2;           // double-float read + write
    }
    L++;
  };
  // panel 0 alone
  k_chol_step<<<nt, kRestThreads, kRestSmem, st>>>(A, Ld, lda, m, nt, 0, kb_of(0), PS, negpiv, 0, 0, 0, 1, PS,
                                                   nullptr, err);
  L++;
  int k = 0;
  while (k + 1 < nt) {
    if (nt - (k + 3) >= BD_PAIR_MIN) {
      col(k);
      step(k + 1, k + 2, k, false, true, false);
      col(k + 1);
      step(k + 2, k + 3, k, true, false, true);
      k += 2;
    } else {
      col(k);
      step(k + 1, k + 2, k, false, false, true);
      k += 1;
    }
  }
  k_diag_scatter<<<nt, 256, 0, st>>>(A, lda, m, Ld);
  L++;
  if (kev_pairs) *kev_pairs = pairs;
  return L;
}

}  // namespace bdk


