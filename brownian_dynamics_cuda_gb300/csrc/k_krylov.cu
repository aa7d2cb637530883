// Krylov noise displacement: rd = s2dt D^{1/2} p by the Lanczos process on the
// RPY tensor, without a factorisation (Ando, Chow, Saad and Skolnick, J.
// Chem. Phys. 137, 064106 (2012): the symmetric square root of D applied to
// the Gaussian vector through a Krylov subspace).  D^{1/2} p has the
// covariance 2 dt D that the Ermak-McCammon step needs, as L p does, but it is
// a different vector from the reference's L p (func_cuda.cu:634-647): a
// non-parity mode.  Its cost is one tensor-vector product per iteration
// (HBM-bound, D read once) instead of an O((3N)^3) factorisation.
//
// Lanczos with full re-orthogonalisation: v_0 = p / |p|; w = D v_k;
// alpha_k = v_k . w; w -= V (V^T w) twice (classical Gram-Schmidt against the
// whole stored basis, which removes alpha_k v_k and beta_k v_{k-1} with the
// rest); beta_{k+1} = |w|; v_{k+1} = w / beta_{k+1}.
// The coefficients stay on the device; every 8 iterations the host reads
// them back, diagonalises the tridiagonals T_{k-1} and T_k (implicit QL) and
// forms c = |p| T^{1/2} e_1 of both; the process stops at the first check with
// |c_k - c_{k-1}| <= tol |c_k| (the relative change of the approximation,
// since V is orthonormal) or at kmax iterations; then y = V c_k.
//
// FP64 contexts: the tensor product reads the stored lower triangle once: a CTA per 64 x 64 tile
// (I >= J) forms D_IJ x_J and D_IJ^T x_I and writes both into their own slots
// of a partial array, which a second kernel sums in a fixed order: the result
// does not depend on scheduling, in FP64 arithmetic.  Mixed contexts: the
// product is matrix-free (k_rpy_mv: the FP32 RPY block of every bead pair,
// compensated sums), so neither the tensor nor its assembly is needed.
#include <cmath>
#include <vector>

#include "bd_internal.h"
#include "dev_physics.cuh"

using bdp::rpy_block_f;

namespace {

constexpr int kKT = 64;   // tile of the tensor product
constexpr int kKB = 256;  // threads per CTA

inline int cdivk(int a, int b) { return (a + b - 1) / b; }

__device__ __forceinline__ void tile_of(long t, int& I, int& J) {
  int Ip = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
  while ((long)(Ip + 1) * (Ip + 2) / 2 <= t) Ip++;
  while ((long)Ip * (Ip + 1) / 2 > t) Ip--;
  I = Ip;
  J = (int)(t - (long)Ip * (Ip + 1) / 2);
}

// P[(I nt + J) 64 + i]: tile (I, J >= ...) contribution to y_I (J <= I: D_IJ x_J;
// J > I: (D_JI)^T x_J).  Diagonal tiles: the lower part and its mirror.
template <bool DF>
__global__ void __launch_bounds__(kKB) k_symv_tiles(int m, int nt, const double* __restrict__ A, int lda,
                                                    const double* __restrict__ x, double* __restrict__ P) {
  __shared__ double xJ[kKT], xI[kKT];
  __shared__ double rpart[4][kKT], cpart[2][kKT];
  int I, J;
  tile_of(blockIdx.x, I, J);
  const int tid = threadIdx.x, i = tid & (kKT - 1), g = tid >> 6, half = i >> 5, lane = tid & 31;
  if (tid < kKT) {
    const int cj = J * kKT + tid, ri = I * kKT + tid;
    xJ[tid] = cj < m ? x[cj] : 0.0;
    xI[tid] = ri < m ? x[ri] : 0.0;
  }
  __syncthreads();
  const int row = I * kKT + i;
  const bool diag = I == J;
  const double xi = xI[i];
  double rs = 0.0;
  float rsf = 0.f;
#pragma unroll 4
  for (int jj = 0; jj < 16; jj++) {
    const int j = g * 16 + jj, col = J * kKT + j;
    const bool in = row < m && col < m && (!diag || i >= j);
    double cs = 0.0;
    if (DF) {
      float d = 0.f;
      if (in) {
        const float2 e = reinterpret_cast<const float2*>(A)[(size_t)col * lda + row];
        d = e.x + e.y;
      }
      rsf = fmaf(d, (float)xJ[j], rsf);
      cs = (!diag || i > j) ? (double)(d * (float)xi) : 0.0;
    } else {
      const double d = in ? A[(size_t)col * lda + row] : 0.0;
      rs = fma(d, xJ[j], rs);
      cs = (!diag || i > j) ? d * xi : 0.0;
    }
    for (int o = 16; o > 0; o >>= 1) cs += __shfl_xor_sync(0xffffffffu, cs, o);
    if (lane == 0) cpart[half][j] = cs;
  }
  rpart[g][i] = DF ? (double)rsf : rs;
  __syncthreads();
  if (tid < kKT) {
    const double yr = ((rpart[0][tid] + rpart[1][tid]) + rpart[2][tid]) + rpart[3][tid];
    const double yc = cpart[0][tid] + cpart[1][tid];
    if (diag) {
      P[((size_t)I * nt + I) * kKT + tid] = yr + yc;
    } else {
      P[((size_t)I * nt + J) * kKT + tid] = yr;
      P[((size_t)J * nt + I) * kKT + tid] = yc;
    }
  }
}

// y[I 64 + i] = sum_J P[(I nt + J) 64 + i], J in increasing order
__global__ void k_symv_sum(int m, int nt, const double* __restrict__ P, double* __restrict__ y) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  const int I = r / kKT, i = r % kKT;
  double s = 0.0;
  for (int J = 0; J < nt; J++) s += P[((size_t)I * nt + J) * kKT + i];
  y[r] = s;
}

// Matrix-free product y = D x for mixed contexts: no tensor in memory.  A
// warp per bead i; the other beads (double-float positions qh/ql with the
// radius in w, and x as float4) staged through shared memory; the FP32 RPY
// block of every pair (rpy_block_f, the mixed tensor's own formula) applied
// to x_j; runs of 32 terms in FP32, the runs added with Kahan compensation;
// lanes summed in FP64 in a fixed order.
constexpr int kMvTile = 256;
constexpr int kMvB = 2;   // beads per warp: each staged bead j serves both
constexpr int kMvW = 8;   // warps per CTA (4 measured slower: the staging is per CTA)
__global__ void __launch_bounds__(32 * kMvW) k_rpy_mv(int nD, const float4* __restrict__ qh, const float4* __restrict__ ql,
                                                const float4* __restrict__ xf, float a1f, float a2f,
                                                double* __restrict__ y) {
  __shared__ float4 sh[kMvTile], sl[kMvTile], sx[kMvTile];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i0 = (blockIdx.x * kMvW + warp) * kMvB;
  float4 hi[kMvB], lo[kMvB];
  bool act[kMvB];
#pragma unroll
  for (int b = 0; b < kMvB; b++) {
    const int i = i0 + b;
    act[b] = i < nD;
    hi[b] = act[b] ? qh[i] : make_float4(0.f, 0.f, 0.f, 1.f);
    lo[b] = act[b] ? ql[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  float run[kMvB][3], ks[kMvB][3], kc[kMvB][3];
#pragma unroll
  for (int b = 0; b < kMvB; b++)
#pragma unroll
    for (int q = 0; q < 3; q++) run[b][q] = ks[b][q] = kc[b][q] = 0.f;
  int cnt = 0;
  for (int base = 0; base < nD; base += kMvTile) {
    __syncthreads();
    for (int t = threadIdx.x; t < kMvTile && base + t < nD; t += blockDim.x) {
      sh[t] = qh[base + t];
      sl[t] = ql[base + t];
      sx[t] = xf[base + t];
    }
    __syncthreads();
    if (!act[0]) continue;  // warp-uniform: the warp's first bead is past the end
    const int je = min(nD, base + kMvTile);
    for (int j = base + lane; j < je; j += 32) {
      const int t = j - base;
      const float4 v = sx[t], hj = sh[t], lj = sl[t];
#pragma unroll
      for (int b = 0; b < kMvB; b++) {
        if (j == i0 + b) {
          const float d = a1f / hi[b].w;
          run[b][0] += d * v.x;
          run[b][1] += d * v.y;
          run[b][2] += d * v.z;
          continue;
        }
        // the RPY block of the pair applied to v without forming it:
        // D v = c_d v + w s (s . v)
        const float sxv = (hi[b].x - hj.x) + (lo[b].x - lj.x), syv = (hi[b].y - hj.y) + (lo[b].y - lj.y),
                    szv = (hi[b].z - hj.z) + (lo[b].z - lj.z);
        const float ssq = sxv * sxv + syv * syv + szv * szv;
        const float inv_s = rsqrtf(ssq);
        const float sd = ssq * inv_s;
        const float ri = hi[b].w, rj = hj.w;
        float cd, w;
        if (sd >= ri + rj) {
          const float inv_ssq = inv_s * inv_s;
          const float f = (ri * ri + rj * rj) * inv_ssq;
          const float as = a2f * inv_s;
          cd = as * (1.f + f * (1.f / 3.f));
          w = as * (1.f - f) * inv_ssq;
        } else {
          const float se = cbrtf((ri * ri * ri + rj * rj * rj) / 2.f);
          const float as = a1f / se;
          cd = as * (1.f - 9.f * sd / (32.f * se));
          w = as * 3.f / (32.f * se * sd);
        }
        const float sv = w * (sxv * v.x + syv * v.y + szv * v.z);
        run[b][0] += cd * v.x + sxv * sv;
        run[b][1] += cd * v.y + syv * sv;
        run[b][2] += cd * v.z + szv * sv;
      }
      if (++cnt == 32) {
#pragma unroll
        for (int b = 0; b < kMvB; b++)
#pragma unroll
          for (int q = 0; q < 3; q++) {
            const float u = run[b][q] - kc[b][q], t2 = ks[b][q] + u;
            kc[b][q] = (t2 - ks[b][q]) - u;
            ks[b][q] = t2;
            run[b][q] = 0.f;
          }
        cnt = 0;
      }
    }
  }
#pragma unroll
  for (int b = 0; b < kMvB; b++) {
    double sum[3];
#pragma unroll
    for (int q = 0; q < 3; q++) {
      const float u = run[b][q] - kc[b][q], t2 = ks[b][q] + u;
      sum[q] = (double)t2 - (double)((t2 - ks[b][q]) - u);
    }
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int q = 0; q < 3; q++) sum[q] = sum[q] + __shfl_xor_sync(0xffffffffu, sum[q], o);
    }
    if (act[b] && lane == 0) {
      const int i = i0 + b;
      y[3 * i] = sum[0];
      y[3 * i + 1] = sum[1];
      y[3 * i + 2] = sum[2];
    }
  }
}

// partial dot products of the first ncol basis vectors with w, per block;
// out[col * nb + block]
constexpr int kDotB = 256;
__global__ void __launch_bounds__(kDotB) k_dots(int m, const double* __restrict__ V, int ncol,
                                                const double* __restrict__ w, double* __restrict__ out) {
  __shared__ double red[kDotB / 32];
  const int col = blockIdx.y;
  const double* v = V + (size_t)col * m;
  double s = 0.0;
  for (int r = blockIdx.x * kDotB + threadIdx.x; r < m; r += gridDim.x * kDotB) s = fma(v[r], w[r], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < kDotB / 32; k++) t += red[k];
    out[(size_t)col * gridDim.x + blockIdx.x] = t;
  }
}

// y = s sum_l c[l] V_l
__global__ void k_combine(int m, const double* __restrict__ V, int ncol, const double* __restrict__ c, double s,
                          double* __restrict__ y) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  double t = 0.0;
  for (int l = 0; l < ncol; l++) t = fma(c[l], V[(size_t)l * m + r], t);
  y[r] = s * t;
}

// w -= sum_{l < ncol} h_l V_l with h_l the fixed-order sums of k_dots'
// partials (block 0, 1, ...), formed by every block into shared memory;
// block 0 also stores h_{ncol-1} in *alpha when alpha is given
constexpr int kProjMax = 520;
__global__ void __launch_bounds__(128) k_sub_proj_sum(int m, const double* __restrict__ V, int ncol, int nb,
                                                      const double* __restrict__ part, double* __restrict__ w,
                                                      double* __restrict__ alpha) {
  __shared__ double hs[kProjMax];
  for (int col = threadIdx.x; col < ncol; col += blockDim.x) {
    double t = 0.0;
    for (int b = 0; b < nb; b++) t += part[(size_t)col * nb + b];
    hs[col] = t;
  }
  __syncthreads();
  if (alpha && blockIdx.x == 0 && threadIdx.x == 0) alpha[0] = hs[ncol - 1];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  double s = w[r];
  for (int l = 0; l < ncol; l++) s -= hs[l] * V[(size_t)l * m + r];
  w[r] = s;
}

// |w| from k_dots' partials (fixed order, in every block), kept in *nrm
// and *beta; then, unless v is null, v = w / |w| and, for matrix-free
// products, its float4 copy per bead (three rows per thread)
__global__ void __launch_bounds__(256) k_norm_scale(int nD, int nb, const double* __restrict__ part,
                                                    const double* __restrict__ w, double* __restrict__ nrm,
                                                    double* __restrict__ beta, double* __restrict__ v,
                                                    float4* __restrict__ xf) {
  __shared__ double sn;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int b = 0; b < nb; b++) t += part[b];
    sn = sqrt(t);
    if (blockIdx.x == 0) {
      nrm[0] = sn;
      if (beta) beta[0] = sn;
    }
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (!v || i >= nD) return;
  const double n = sn;
  const double x = w[3 * i] / n, yv = w[3 * i + 1] / n, z = w[3 * i + 2] / n;
  v[3 * i] = x;
  v[3 * i + 1] = yv;
  v[3 * i + 2] = z;
  if (xf) xf[i] = make_float4((float)x, (float)yv, (float)z, 0.f);
}

// Eigenvalues and eigenvectors of a symmetric tridiagonal matrix (diagonal d,
// sub-diagonal e[1..k)) by the implicit QL method with Wilkinson-type
// shifts (the method of the EISPACK routine tql2); z (row-major k x k) holds
// the eigenvectors in its columns.
bool tridiag_eig(int k, std::vector<double>& d, std::vector<double> e, std::vector<double>& z) {
  z.assign((size_t)k * k, 0.0);
  for (int i = 0; i < k; i++) z[(size_t)i * k + i] = 1.0;
  for (int i = 1; i < k; i++) e[i - 1] = e[i];
  e[k - 1] = 0.0;
  for (int l = 0; l < k; l++) {
    int iter = 0, m;
    do {
      for (m = l; m < k - 1; m++) {
        const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= 1e-16 * dd) break;
      }
      if (m != l) {
        if (iter++ == 100) return false;
        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        double r = std::hypot(g, 1.0);
        g = d[m] - d[l] + e[l] / (g + (g >= 0 ? std::fabs(r) : -std::fabs(r)));
        double sn = 1.0, cs = 1.0, p = 0.0;
        int i;
        for (i = m - 1; i >= l; i--) {
          double f = sn * e[i], b = cs * e[i];
          e[i + 1] = (r = std::hypot(f, g));
          if (r == 0.0) {
            d[i + 1] -= p;
            e[m] = 0.0;
            break;
          }
          sn = f / r;
          cs = g / r;
          g = d[i + 1] - p;
          r = (d[i] - g) * sn + 2.0 * cs * b;
          d[i + 1] = g + (p = sn * r);
          g = cs * r - b;
          for (int q = 0; q < k; q++) {
            f = z[(size_t)q * k + i + 1];
            z[(size_t)q * k + i + 1] = sn * z[(size_t)q * k + i] + cs * f;
            z[(size_t)q * k + i] = cs * z[(size_t)q * k + i] - sn * f;
          }
        }
        if (r == 0.0 && i >= l) continue;
        d[l] -= p;
        e[l] = g;
        e[m] = 0.0;
      }
    } while (m != l);
  }
  return true;
}

// c = |p| T^{1/2} e_1 for the tridiagonal (alpha[0..k), beta[1..k))
bool sqrt_e1(int k, const std::vector<double>& al, const std::vector<double>& be, double pn, std::vector<double>& c) {
  std::vector<double> d(al.begin(), al.begin() + k), e(k, 0.0), z;
  for (int i = 1; i < k; i++) e[i] = be[i];
  if (!tridiag_eig(k, d, e, z)) return false;
  c.assign(k, 0.0);
  for (int l = 0; l < k; l++) {
    const double w = std::sqrt(std::fmax(d[l], 0.0)) * z[l];  // z[0][l]
    for (int j = 0; j < k; j++) c[j] += z[(size_t)j * k + l] * w;
  }
  for (auto& x : c) x *= pn;
  return true;
}

}  // namespace

namespace bdk {

size_t krylov_scratch_doubles(int m, int kmax) {
  const int nt = cdivk(m, kKT);
  const int nb = std::min(cdivk(m, kDotB), 64);
  return (size_t)(kmax + 1) * m + (size_t)m + (size_t)nt * nt * kKT + (size_t)(kmax + 1) * nb +
         3 * (size_t)(kmax + 2) + 8 + 2 * (size_t)cdivk(m, 3) + 2;
}

// rd = s2dt D^{1/2} p.  The tensor products: with A != nullptr from the
// lower-stored tensor (double-float pairs when df); with A == nullptr
// matrix-free from the bead positions (qh, ql: double-float mirror with the
// radius in w).  p is a device vector.  The coefficients stay on the device;
// the host reads them back every kCheck iterations (and at kmax) to test
// convergence, and takes the first iteration that met the tolerance.
// *iters and *change describe the run.
constexpr int kCheck = 8;
int krylov_sqrt(int m, const double* A, int lda, bool df, const float4* qh, const float4* ql, double a1, double a2,
                const double* p, double s2dt, double tol, int kmax, double* rd, double* scratch, cudaStream_t st,
                int* iters, double* change, KrylovGraphs* graphs) {
  const int nt = cdivk(m, kKT), nD = m / 3;
  const int nb = std::min(cdivk(m, kDotB), 64);
  double* V = scratch;
  double* w = V + (size_t)(kmax + 1) * m;
  double* P = w + m;
  double* part = P + (size_t)nt * nt * kKT;
  double* h = part + (size_t)(kmax + 1) * nb;  // kmax + 2
  double* alpha = h + (kmax + 2);              // kmax + 2
  double* beta = alpha + (kmax + 2);           // kmax + 2
  double* nrm = beta + (kmax + 2);             // 8
  // float4 needs 16-byte alignment: start on an even double offset from the (256-aligned) base
  const size_t xoff = ((size_t)(nrm + 8 - scratch) + 1) & ~(size_t)1;
  float4* xf = reinterpret_cast<float4*>(scratch + xoff);
  const int tb = 256, gm = cdivk(m, tb);
  const long tiles = (long)nt * (nt + 1) / 2;
  if (kmax + 1 > kProjMax) return BD_ERR_ARG;
  float4* xfm = A ? nullptr : xf;  // the float4 copy of v_k that matrix-free products read
  const int gb = cdivk(nD, tb);
  // x = V_k: its float4 copy (matrix-free) was written with it by k_norm_scale
  auto product = [&](const double* x, double* y) {
    if (A) {
      if (df) k_symv_tiles<true><<<(unsigned)tiles, kKB, 0, st>>>(m, nt, A, lda, x, P);
      else k_symv_tiles<false><<<(unsigned)tiles, kKB, 0, st>>>(m, nt, A, lda, x, P);
      k_symv_sum<<<gm, tb, 0, st>>>(m, nt, P, y);
    } else {
      k_rpy_mv<<<cdivk(nD, kMvW * kMvB), 32 * kMvW, 0, st>>>(nD, qh, ql, xf, (float)a1, (float)a2, y);
    }
  };
  // v_0 = p / |p|
  k_dots<<<dim3(nb, 1), kDotB, 0, st>>>(m, p, 1, p, part);
  k_norm_scale<<<gb, tb, 0, st>>>(nD, nb, part, p, nrm, nullptr, V, xfm);
  double pn = 0.0;
  if (cudaMemcpyAsync(&pn, nrm, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return BD_ERR_CUDA;
  *iters = 0;
  *change = 1.0;
  if (pn == 0.0) {
    cudaMemsetAsync(rd, 0, (size_t)m * sizeof(double), st);
    return BD_OK;
  }
  std::vector<double> al, be, c, cprev, hal(kmax + 2), hbe(kmax + 2);
  // one Lanczos iteration in seven launches: the product, twice the
  // projections on the basis so far (alpha_k from the first), the norm with
  // v_{k+1} = w / |w| (and its float4 copy)
  auto iteration = [&](int k) {
    product(V + (size_t)k * m, w);
    for (int pass = 0; pass < 2; pass++) {
      k_dots<<<dim3(nb, k + 1), kDotB, 0, st>>>(m, V, k + 1, w, part);
      k_sub_proj_sum<<<cdivk(m, 128), 128, 0, st>>>(m, V, k + 1, nb, part, w, pass == 0 ? alpha + k : nullptr);
    }
    k_dots<<<dim3(nb, 1), kDotB, 0, st>>>(m, w, 1, w, part);
    k_norm_scale<<<gb, tb, 0, st>>>(nD, nb, part, w, nrm, beta + k + 1, k + 1 < kmax ? V + (size_t)(k + 1) * m : nullptr,
                                    xfm);
  };
  // a block of kCheck iterations is ~100 small launches: captured once per
  // context as a CUDA graph (its pointers and sizes are the context's) and
  // replayed; the legacy stream cannot be captured, so it runs them eagerly
  if (graphs && (graphs->m != m || graphs->kmax != kmax || graphs->scratch != scratch || graphs->A != A ||
                 graphs->df != df || graphs->a1 != a1 || graphs->a2 != a2)) {
    graphs->clear();
    graphs->m = m, graphs->kmax = kmax, graphs->scratch = scratch, graphs->A = A, graphs->df = df;
    graphs->a1 = a1, graphs->a2 = a2;
  }
  const bool use_graphs = graphs && st != nullptr;
  int done = -1;
  for (int k0 = 0; k0 < kmax && done < 0; k0 += kCheck) {
    const int k1 = std::min(k0 + kCheck, kmax);
    bool ran = false;
    if (use_graphs && k1 - k0 == kCheck) {
      const size_t b = (size_t)(k0 / kCheck);
      if (graphs->blocks.size() <= b) graphs->blocks.resize(b + 1, nullptr);
      if (!graphs->blocks[b]) {
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
          for (int k = k0; k < k1; k++) iteration(k);
          if (cudaStreamEndCapture(st, &g) == cudaSuccess && g) {
            if (cudaGraphInstantiate(&graphs->blocks[b], g, 0) != cudaSuccess) graphs->blocks[b] = nullptr;
            cudaGraphDestroy(g);
          }
        }
        if (cudaGetLastError() != cudaSuccess) return BD_ERR_CUDA;
      }
      if (graphs->blocks[b]) {
        if (cudaGraphLaunch(graphs->blocks[b], st) != cudaSuccess) return BD_ERR_CUDA;
        ran = true;
      }
    }
    if (!ran)
      for (int k = k0; k < k1; k++) iteration(k);
    int k = k1 - 1;
    if (cudaMemcpyAsync(hal.data(), alpha, (k + 1) * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(hbe.data(), beta, (k + 2) * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return BD_ERR_CUDA;
    // an invariant subspace reached inside the batch (beta_{q+1} ~ 0): stop at q
    for (int q = 0; q < k; q++)
      if (hbe[q + 1] <= 1e-14 * std::fabs(hal[0])) {
        k = q;
        break;
      }
    // the approximations after iterations k - 1 and k; their relative change
    al.assign(hal.begin(), hal.begin() + k + 1);
    be.assign(hbe.begin(), hbe.begin() + k + 2);
    if (!sqrt_e1(k + 1, al, be, pn, c)) return BD_ERR_NONFINITE;
    if (k > 0) {
      if (!sqrt_e1(k, al, be, pn, cprev)) return BD_ERR_NONFINITE;
      double num = 0.0, den = 0.0;
      for (int j2 = 0; j2 <= k; j2++) {
        const double d = c[j2] - (j2 < k ? cprev[j2] : 0.0);
        num += d * d;
        den += c[j2] * c[j2];
      }
      *change = std::sqrt(num / den);
    }
    *iters = k + 1;
    if ((k > 0 && *change <= tol) || be[k + 1] <= 1e-14 * std::fabs(al[0]) || k + 1 == kmax) done = k;
  }
  const int ncol = (int)c.size();
  if (cudaMemcpyAsync(h, c.data(), ncol * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return BD_ERR_CUDA;
  k_combine<<<gm, tb, 0, st>>>(m, V, ncol, h, s2dt, rd);
  if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) return BD_ERR_CUDA;
  return BD_OK;
}

}  // namespace bdk
