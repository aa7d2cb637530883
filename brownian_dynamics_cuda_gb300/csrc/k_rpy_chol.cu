// Diffusion tensor and its Cholesky factor (FP64 parity path).
//
//   rpy_assemble   Diffusion_Tensor (func.cpp:728-804): lower triangle of
//                  the 3N x 3N RPY tensor, column-major with leading dim
//                  lda, written once (the reference writes the full matrix
//                  twice, func_cuda.cu:500-559).
//   potrf_fp64     blocked right-looking Cholesky, in place, lower: a
//                  one-CTA diagonal factor, a row-parallel triangular
//                  solve of the panel and a register-tiled FP64 SYRK/GEMM
//                  trailing update.  A negative pivot is replaced by its
//                  absolute value and counted (func.cpp:827-833).
//   trmv_lower     rd = s2dt * L p (rd_cal, func_cuda.cu:634-647), split
//                  over column chunks with a fixed-order final sum.
#include <cuda_runtime.h>

#include "bd_internal.h"
#include "dev_physics.cuh"

using namespace bdp;

namespace {

inline int cdiv(int a, int b) { return (a + b - 1) / b; }

// ------------------------------------------------------------ RPY
constexpr int kRpyTile = 32;

__global__ void __launch_bounds__(256) k_rpy(int nD, const double* __restrict__ r, const double* __restrict__ rad,
                                             double a1, double a2, double* __restrict__ A, int lda) {
  int bi = blockIdx.y, bj = blockIdx.x;
  if (bj > bi) return;
  int i = bi * kRpyTile + threadIdx.x;
  if (i >= nD) return;
  V3 ri = ld3(r + 3 * i);
  double radi = rad[i];
  for (int jj = threadIdx.y; jj < kRpyTile; jj += blockDim.y) {
    int j = bj * kRpyTile + jj;
    if (j >= nD || j > i) continue;
    if (j == i) {
      for (int l = 0; l < 3; l++)
        for (int k = l; k < 3; k++) A[(size_t)(3 * j + l) * lda + 3 * i + k] = (k == l) ? a1 / radi : 0.0;
      continue;
    }
    V3 rj = ld3(r + 3 * j);
    V3 sij{ri.x - rj.x, ri.y - rj.y, ri.z - rj.z};
    double ssq = sij.x * sij.x + sij.y * sij.y + sij.z * sij.z;
    double s = sqrt(ssq);
    double radj = rad[j];
    double Db[3][3];
    rpy_block(sij, ssq, s, radi, radj, a1, a2, Db);
    for (int l = 0; l < 3; l++) {
      double* col = A + (size_t)(3 * j + l) * lda + 3 * i;
      for (int k = 0; k < 3; k++) col[k] = Db[k][l];
    }
  }
}

// Mixed path: the same lower triangle from the FP32 form of the RPY block
// (separations formed in FP64, then FP32), stored as the double-float pair
// (value, 0).  No FP64 arithmetic beyond the separation.
// Mixed path: FP32 blocks from the double-float positions (hi differences
// plus lo differences; radius in qh.w), no FP64 per pair; stored as (D, 0)
// pairs.  The same separations and block formula as the mixed drift.
__global__ void __launch_bounds__(256) k_rpy_mx(int nD, const float4* __restrict__ qh, const float4* __restrict__ ql,
                                                float a1f, float a2f, float2* __restrict__ A, int lda) {
  int bi = blockIdx.y, bj = blockIdx.x;
  if (bj > bi) return;
  int i = bi * kRpyTile + threadIdx.x;
  if (i >= nD) return;
  const float4 hi = qh[i], lo = ql[i];
  for (int jj = threadIdx.y; jj < kRpyTile; jj += blockDim.y) {
    int j = bj * kRpyTile + jj;
    if (j >= nD || j > i) continue;
    if (j == i) {
      for (int l = 0; l < 3; l++)
        for (int k = l; k < 3; k++)
          A[(size_t)(3 * j + l) * lda + 3 * i + k] = make_float2((k == l) ? a1f / hi.w : 0.f, 0.f);
      continue;
    }
    const float4 hj = qh[j], lj = ql[j];
    float Db[3][3];
    rpy_block_f((hi.x - hj.x) + (lo.x - lj.x), (hi.y - hj.y) + (lo.y - lj.y), (hi.z - hj.z) + (lo.z - lj.z), hi.w, hj.w,
                a1f, a2f, Db);
    for (int l = 0; l < 3; l++) {
      float2* col = A + (size_t)(3 * j + l) * lda + 3 * i;
      for (int k = 0; k < 3; k++) col[k] = make_float2(Db[k][l], 0.f);
    }
  }
}

// ------------------------------------------------------------ Cholesky
constexpr int kNB = 64;

// Factor the kb x kb diagonal block at (k0,k0) in shared memory.
__global__ void __launch_bounds__(256) k_potrf_diag(double* A, int lda, int k0, int kb, int* negpiv) {
  __shared__ double S[kNB][kNB + 1];
  const int tid = threadIdx.x;
  for (int e = tid; e < kb * kb; e += blockDim.x) {
    int c = e / kb, rr = e - c * kb;  // column-major walk
    S[rr][c] = (rr >= c) ? A[(size_t)(k0 + c) * lda + k0 + rr] : 0.0;
  }
  __syncthreads();
  // the pivot's reciprocal, formed once per column by thread 0 beside its
  // square root, scales the column (one FP64 division per column instead of
  // one per element on the column's critical path)
  __shared__ double rpiv;
  for (int c = 0; c < kb; c++) {
    if (tid == 0) {
      double f = S[c][c];
      if (f < 0) {
        f = -f;
        atomicAdd(negpiv, 1);
      }
      const double d = sqrt(f);
      S[c][c] = d;
      rpiv = 1.0 / d;
    }
    __syncthreads();
    const double rp = rpiv;
    for (int rr = c + 1 + tid; rr < kb; rr += blockDim.x) S[rr][c] = S[rr][c] * rp;
    __syncthreads();
    // rank-1 update of the remaining lower triangle
    int rem = kb - c - 1;
    for (int e = tid; e < rem * rem; e += blockDim.x) {
      int q = e / rem, rr = e - q * rem;
      int col = c + 1 + q, row = c + 1 + rr;
      if (row >= col) S[row][col] = S[row][col] - S[row][c] * S[col][c];
    }
    __syncthreads();
  }
  for (int e = tid; e < kb * kb; e += blockDim.x) {
    int c = e / kb, rr = e - c * kb;
    if (rr >= c) A[(size_t)(k0 + c) * lda + k0 + rr] = S[rr][c];
  }
}

// Panel solve: rows [k0+kb, m) of columns [k0, k0+kb): X L_kk^T = A, a
// row per thread (64 dependent column steps on the FP64 pipe), 128 rows per
// CTA (32 per CTA spread the rows over more SMs but staged L_kk four times
// longer per thread: 229 vs 210 us per panel at 3N = 1,944)
constexpr int kTrsmThreads = 128;
__global__ void __launch_bounds__(kTrsmThreads) k_trsm_panel(double* A, int lda, int m, int k0, int kb) {
  __shared__ double Lkk[kNB][kNB + 1];
  __shared__ double rdiag[kNB];  // 1 / L_cc: the row solves multiply instead of dividing
  for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
    int c = e / kb, rr = e - c * kb;
    Lkk[rr][c] = (rr >= c) ? A[(size_t)(k0 + c) * lda + k0 + rr] : 0.0;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < kb; c += blockDim.x) rdiag[c] = 1.0 / Lkk[c][c];
  __syncthreads();
  int r = k0 + kb + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  double x[kNB];
#pragma unroll
  for (int c = 0; c < kNB; c++) {
    if (c < kb) x[c] = A[(size_t)(k0 + c) * lda + r];
  }
#pragma unroll
  for (int c = 0; c < kNB; c++) {
    if (c < kb) {
      double v = x[c];
#pragma unroll
      for (int q = 0; q < kNB; q++)
        if (q < c) v = v - x[q] * Lkk[c][q];
      x[c] = v * rdiag[c];
    }
  }
#pragma unroll
  for (int c = 0; c < kNB; c++)
    if (c < kb) A[(size_t)(k0 + c) * lda + r] = x[c];
}

// Trailing update of the lower triangle of A[t0:, t0:] (t0 = k0 + kb):
// A_ij -= P_i P_j^T with P = A[:, k0:k0+kb].  64 x 64 output tile per CTA,
// 256 threads each owning a 4 x 4 register block.
constexpr int kTM = 64;
constexpr int kKC = 16;  // panel columns staged per pass

__global__ void __launch_bounds__(256) k_syrk_update(double* A, int lda, int m, int k0, int kb) {
  const int t0 = k0 + kb;
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (bj > bi) return;
  const int row0 = t0 + bi * kTM, col0 = t0 + bj * kTM;
  __shared__ double Pr[kKC][kTM + 1];  // [k][row]
  __shared__ double Pc[kKC][kTM + 1];  // [k][col]
  const int tid = threadIdx.x;
  const int tr = (tid & 15) * 4, tc = (tid >> 4) * 4;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = 0.0;
  for (int kc = 0; kc < kb; kc += kKC) {
    const int kn = kb - kc < kKC ? kb - kc : kKC;
    for (int e = tid; e < kKC * kTM; e += blockDim.x) {
      int k = e / kTM, q = e - k * kTM;
      int rr = row0 + q, cc = col0 + q;
      bool in = k < kn;
      Pr[k][q] = (in && rr < m) ? A[(size_t)(k0 + kc + k) * lda + rr] : 0.0;
      Pc[k][q] = (in && cc < m) ? A[(size_t)(k0 + kc + k) * lda + cc] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < kKC; k++) {
      double pr[4], pc[4];
#pragma unroll
      for (int a = 0; a < 4; a++) { pr[a] = Pr[k][tr + a]; pc[a] = Pc[k][tc + a]; }
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = fma(pr[a], pc[b], acc[a][b]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int b = 0; b < 4; b++) {
    int cc = col0 + tc + b;
    if (cc >= m) continue;
#pragma unroll
    for (int a = 0; a < 4; a++) {
      int rr = row0 + tr + a;
      if (rr >= m || rr < cc) continue;
      double* p = A + (size_t)cc * lda + rr;
      *p = *p - acc[a][b];
    }
  }
}

// ------------------------------------------------------------ L p
constexpr int kRdRows = 256;
constexpr int kRdChunk = 512;

__global__ void __launch_bounds__(kRdRows) k_trmv_part(int m, const double* __restrict__ A, int lda,
                                                       const double* __restrict__ p, double s2dt,
                                                       double* __restrict__ part) {
  int i = blockIdx.x * kRdRows + threadIdx.x;
  int kc = blockIdx.y;
  int k0 = kc * kRdChunk, k1 = min(k0 + kRdChunk, m);
  double s = 0.0;
  if (i < m) {
    int kend = min(k1, i + 1);
#pragma unroll 8
    for (int k = k0; k < kend; k++) s = s + (s2dt * A[(size_t)k * lda + i]) * p[k];
  }
  if (i < m) part[(size_t)kc * m + i] = s;
}

// The same over the double-float factor of the mixed path, in FP32
// arithmetic: each product L_ik p_k is formed exactly as x + ex (p split into
// FP32 hi + lo once per CTA, FMA for the rounding error of L_ik p_hi) and
// summed with a two-sum into (s, c); ~40 significant bits per partial sum.
__global__ void __launch_bounds__(kRdRows) k_trmv_part_df(int m, const float2* __restrict__ A, int lda,
                                                          const double* __restrict__ p, double s2dt,
                                                          double* __restrict__ part) {
  __shared__ float2 ps[kRdChunk];
  int i = blockIdx.x * kRdRows + threadIdx.x;
  int kc = blockIdx.y;
  int k0 = kc * kRdChunk, k1 = min(k0 + kRdChunk, m);
  for (int k = k0 + threadIdx.x; k < k1; k += kRdRows) {
    const double pk = p[k];
    const float h = (float)pk;
    ps[k - k0] = make_float2(h, (float)(pk - (double)h));
  }
  __syncthreads();
  if (i >= m) return;
  float sh = 0.f, sc = 0.f;
  int kend = min(k1, i + 1);
  // unrolled so that eight loads of the factor are in flight per thread (the
  // sum's order is unchanged)
#pragma unroll 8
  for (int k = k0; k < kend; k++) {
    const float2 a = A[(size_t)k * lda + i];
    const float2 q = ps[k - k0];
    const float x = a.x * q.x;
    const float ex = fmaf(a.x, q.x, -x) + fmaf(a.x, q.y, a.y * q.x);
    const float t = sh + x;
    const float bp = t - sh;
    sc += ((sh - (t - bp)) + (x - bp)) + ex;
    sh = t;
  }
  part[(size_t)kc * m + i] = s2dt * ((double)sh + (double)sc);
}

__global__ void k_trmv_sum(int m, int nchunk, const double* __restrict__ part, double* __restrict__ rd) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double s = 0.0;
  for (int c = 0; c < nchunk; c++) s = s + part[(size_t)c * m + i];
  rd[i] = s;
}

}  // namespace

namespace bdk {

void rpy_assemble(int nD, const double* r_all, const double* rad, double a1, double a2, double* A, int lda,
                  cudaStream_t st, const float4* qh, const float4* ql) {
  int nt = cdiv(nD, kRpyTile);
  if (qh)
    k_rpy_mx<<<dim3(nt, nt), dim3(kRpyTile, 8), 0, st>>>(nD, qh, ql, (float)a1, (float)a2,
                                                         reinterpret_cast<float2*>(A), lda);
  else
    k_rpy<<<dim3(nt, nt), dim3(kRpyTile, 8), 0, st>>>(nD, r_all, rad, a1, a2, A, lda);
}

int potrf_fp64(int m, double* A, int lda, double* /*rd_acc*/, const double* /*p*/, double /*s2dt*/, int* d_negpiv,
               cudaStream_t st) {
  int launches = 0;
  for (int k0 = 0; k0 < m; k0 += kNB) {
    int kb = m - k0 < kNB ? m - k0 : kNB;
    k_potrf_diag<<<1, 256, 0, st>>>(A, lda, k0, kb, d_negpiv);
    launches++;
    int rest = m - k0 - kb;
    if (rest <= 0) break;
    k_trsm_panel<<<cdiv(rest, kTrsmThreads), kTrsmThreads, 0, st>>>(A, lda, m, k0, kb);
    int nt = cdiv(rest, kTM);
    k_syrk_update<<<dim3(nt, nt), 256, 0, st>>>(A, lda, m, k0, kb);
    launches += 2;
  }
  return launches;
}

size_t trmv_scratch_doubles(int m) { return (size_t)cdiv(m, kRdChunk) * m; }

void trmv_lower_ws(int m, const double* A, int lda, const double* p, double s2dt, double* rd, double* part,
                   cudaStream_t st, bool df) {
  int nchunk = cdiv(m, kRdChunk);
  if (df)
    k_trmv_part_df<<<dim3(cdiv(m, kRdRows), nchunk), kRdRows, 0, st>>>(m, reinterpret_cast<const float2*>(A), lda, p,
                                                                       s2dt, part);
  else
    k_trmv_part<<<dim3(cdiv(m, kRdRows), nchunk), kRdRows, 0, st>>>(m, A, lda, p, s2dt, part);
  k_trmv_sum<<<cdiv(m, 256), 256, 0, st>>>(m, nchunk, part, rd);
}

}  // namespace bdk
