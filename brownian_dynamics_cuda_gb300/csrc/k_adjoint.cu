// Gradient of a rollout observable with respect to the fiber's stretch,
// bend and twist moduli and its Debye length: the reverse-mode (adjoint)
// pass of the Ermak-McCammon step, with recomputation checkpointing.
//
// Forward: the production step (bdh::step_device, FP32-class arithmetic on
// a mixed-precision context, FP64 on an FP64 one) advances the fiber
// n_steps times from the context's state with the caller's noise; the full
// state is kept every `checkpoint` steps.  Observable: the mean over the
// final `window` states of |r_{n-1} - r_0|^2 + Rg (chain beads).
//
// Reverse: per segment (last first) the segment's steps are recomputed from
// its checkpoint, each keeping its intermediates (the factor L, the forces,
// the predictor and corrector states); per step (last first) the adjoint of
// the state is carried back through
//   corrector frame refresh -> rotation + translation (drift del D F and
//   noise rd) -> averaged forces -> forces at the refreshed predictor ->
//   predictor refresh -> rotation + translation -> forces at the state ->
//   rd = s2dt L p (Cholesky backward: D_bar = L^-T Phi(L^T rd_bar p^T) L^-1,
//   Phi = lower triangle with the diagonal halved) -> the RPY tensor D(r).
// The moduli adjoints accumulate in the force kernels.  Local Jacobians come
// from forward-mode dual numbers over each interaction's inputs
// (adj_dual.cuh, adj_terms.cuh); the O(m^3) Cholesky backward runs as a
// blocked triangular inverse and a triangle-aware GEMM.
#include <cuda_runtime.h>
#include <type_traits>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "adj_terms.cuh"
#include "bd_internal.h"

using bdh::set_error;

#define CK(call)                                                                                 \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) {                                                                     \
      char b_[256];                                                                              \
      snprintf(b_, sizeof b_, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
      return set_error(e_ == cudaErrorMemoryAllocation ? BD_ERR_NOMEM : BD_ERR_CUDA, b_);        \
    }                                                                                            \
  } while (0)

namespace {
using namespace adj;

inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

// index of component q (0..11: r, a, b, c) of chain bead i in a state vector
// [r | a | b | c | r_t] (n3 = 3n)
__device__ __forceinline__ int sidx(int n3, int i, int q) { return (q / 3) * n3 + 3 * i + q % 3; }

template <class R>
__device__ __forceinline__ void ld_bead(const double* x, int n3, int i, R* o) {
  for (int q = 0; q < 12; q++) o[q] = R(x[sidx(n3, i, q)]);
}

template <class R>
__device__ __forceinline__ R warp_sum(R v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// DNA/core pair selection of the electrostatics loop (func.cpp:1320-1330)
__device__ __forceinline__ bool pair_ok(const DevModel& M, int i, int j) {
  if (M.type[i + 1] != 0) return false;
  if (i > 0 && M.type[i - 1] != 0) return false;
  if (j < M.n - 1 && M.type[j + 1] != 0) return false;
  if (M.type[j - 1] != 0) return false;
  return true;
}

// ------------------------------------------------------------ chain bonds
constexpr int kBW = 8;         // inputs seeded per thread (frame refresh, anchors)
constexpr int kBondIn = 39;
// inputs seeded per thread of the bond term (many short threads: the
// term's FP64 chain is latency-bound), with FP64 derivatives or, on mixed
// contexts, FP32 derivatives of the FP64 values
#ifndef BD_BOND_WM
#define BD_BOND_WM 2
#endif
constexpr int kBondW = 2;
constexpr int kBondWm = BD_BOND_WM;
__host__ __device__ constexpr int bond_chunks(int w) { return (kBondIn + w - 1) / w; }

template <class R, class G, int BW>
__global__ void __launch_bounds__(64) k_adj_bonds(DevModel M, const double* __restrict__ x,
                                                  const double* __restrict__ fb, double* lam, double* th) {
  constexpr int kBondChunks = bond_chunks(BW);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / kBondChunks, ch = t % kBondChunks;
  if (i >= M.n - 1) return;
  const int n3 = 3 * M.n;
  BondInfo k;
  k.ti = M.type[i];
  k.tn = M.type[i + 1];
  k.has_prev = i > 0;
  k.tp = i > 0 ? M.type[i - 1] : 1;
  k.last = (i == M.n - 2);
  k.phi_i = M.phi_o[i];
  k.phi_p = i > 0 ? M.phi_o[i - 1] : 0.0;
  R xin[kBondIn];
  for (int q = 0; q < 12; q++) xin[q] = i > 0 ? R(x[sidx(n3, i - 1, q)]) : R(0);
  ld_bead(x, n3, i, xin + 12);
  ld_bead(x, n3, i + 1, xin + 24);
  xin[36] = R(M.h);
  xin[37] = R(M.g);
  xin[38] = R(M.s);
  R yb[12];
  for (int q = 0; q < 3; q++) {
    yb[q] = R(fb[3 * i + q]);
    yb[3 + q] = R(fb[3 * (i + 1) + q]);
    yb[6 + q] = R(fb[n3 + 3 * i + q]);
    yb[9 + q] = R(fb[n3 + 3 * (i + 1) + q]);
  }
  R xb[BW];
  vjp_chunk_g<BW, kBondIn, 12, G>(
      [&](const auto* xd, auto* yd) { bond_term(k, xd, xd + 12, xd + 24, xd[36], xd[37], xd[38], yd); }, xin, yb,
      ch, xb);
  for (int j = 0; j < BW; j++) {
    const int q = ch * BW + j;
    if (q >= kBondIn) break;
    const double v = (double)xb[j];
    if (q < 12) {
      if (i > 0) atomicAdd(lam + sidx(n3, i - 1, q), v);
    } else if (q < 24) {
      atomicAdd(lam + sidx(n3, i, q - 12), v);
    } else if (q < 36) {
      atomicAdd(lam + sidx(n3, i + 1, q - 24), v);
    } else {
      atomicAdd(th + (q - 36), v);
    }
  }
}

// ------------------------------------------------------------ DNA-DNA
template <class R>
__global__ void k_adj_dnadna(DevModel M, const double* __restrict__ x, const double* __restrict__ fb, double* lam,
                             double* th) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = M.n;
  const int i = t / n, j = t % n;
  R kb = R(0);
  if (t < n * n && i < j && j - i > 1 && M.type[i] == 0 && M.type[j] == 0 && pair_ok(M, i, j)) {
    R z[3], v[3];
    for (int q = 0; q < 3; q++) {
      z[q] = R(x[3 * i + q] - x[3 * j + q]);
      v[q] = R(fb[3 * i + q] - fb[3 * j + q]);
    }
    if (!(val(norm3(z)) > 25.0)) {
      using D = Dual<R, 4>;
      D zd[3], f[3];
      for (int q = 0; q < 3; q++) {
        zd[q] = D(z[q]);
        zd[q].d[q] = R(1);
      }
      D kd(M.debyell);
      kd.d[3] = R(1);
      pair_dna_dna(R(M.k_e * M.q_l * M.q_l), R(M.k_ex), R(M.sDD), zd, kd, f);
      for (int g = 0; g < 3; g++) {
        R zb = v[0] * f[0].d[g] + v[1] * f[1].d[g] + v[2] * f[2].d[g];
        atomicAdd(lam + 3 * i + g, (double)zb);
        atomicAdd(lam + 3 * j + g, -(double)zb);
      }
      kb = v[0] * f[0].d[3] + v[1] * f[1].d[3] + v[2] * f[2].d[3];
    }
  }
  kb = warp_sum(kb);
  if ((threadIdx.x & 31) == 0 && kb != R(0)) atomicAdd(th + 4, (double)kb);
}

// ------------------------------------------------------------ DNA-core
// one CTA per (linker bead, core); threads over the core's charges
template <class R>
__global__ void __launch_bounds__(128) k_adj_dnacore(DevModel M, const double* __restrict__ x,
                                                     const double* __restrict__ fb, double* lam, double* th) {
  const int kd = blockIdx.x / M.n_c, kc = blockIdx.x % M.n_c;
  const int dn = M.dna_bead[kd], cr = M.core_bead[kc];
  const int i = min(dn, cr), j = max(dn, cr), n3 = 3 * M.n;
  if (!pair_ok(M, i, j)) return;
  R rd[3], xc[12];
  for (int q = 0; q < 3; q++) rd[q] = R(x[3 * dn + q]);
  ld_bead(x, n3, cr, xc);
  {
    R dd[3] = {rd[0] - xc[0], rd[1] - xc[1], rd[2] - xc[2]};
    if (val(norm3(dd)) > 25.0) return;
  }
  const bool adj = (j - i) > 1;
  const R *a = xc + 3, *b = xc + 6, *c = xc + 9;
  R Fdn[3], Fc[3], Tc[3];
  for (int q = 0; q < 3; q++) {
    Fdn[q] = R(fb[3 * dn + q]);
    Fc[q] = R(fb[3 * cr + q]);
    Tc[q] = R(fb[n3 + 3 * cr + q]);
  }
  R acc[16];
  for (int q = 0; q < 16; q++) acc[q] = R(0);  // r_dn(3) r_c(3) a(3) b(3) c(3) kappa
  const R ke = R(M.k_e * M.q_l), kex = R(M.k_ex), sg = R(M.sDC);
  for (int s = threadIdx.x; s < M.Nq; s += blockDim.x) {
    const R cp[3] = {R(M.core_pos[3 * s]), R(M.core_pos[3 * s + 1]), R(M.core_pos[3 * s + 2])};
    const R cq = R(M.core_q[s]);
    using D = Dual<R, 4>;
    D zd[3], f[3];
    for (int q = 0; q < 3; q++) {
      zd[q] = D(rd[q] - (xc[q] + a[q] * cp[0] + b[q] * cp[1] + c[q] * cp[2]));
      zd[q].d[q] = R(1);
    }
    D kk(M.debye);
    kk.d[3] = R(1);
    pair_site(ke * cq, adj, M.core_q[s] > 0, kex, sg, zd, kk, f);
    R Q[3];
    cross3(Tc, cp, Q);  // adjoint of the body-frame force on the core
    R fbar[3];
    for (int q = 0; q < 3; q++) fbar[q] = Fdn[q] - Fc[q] - (Q[0] * a[q] + Q[1] * b[q] + Q[2] * c[q]);
    R zb[3];
    for (int g = 0; g < 3; g++) zb[g] = fbar[0] * f[0].d[g] + fbar[1] * f[1].d[g] + fbar[2] * f[2].d[g];
    acc[15] += fbar[0] * f[0].d[3] + fbar[1] * f[1].d[3] + fbar[2] * f[2].d[3];
    for (int q = 0; q < 3; q++) {
      acc[q] += zb[q];
      acc[3 + q] -= zb[q];
      acc[6 + q] += -Q[0] * f[q].v - cp[0] * zb[q];
      acc[9 + q] += -Q[1] * f[q].v - cp[1] * zb[q];
      acc[12 + q] += -Q[2] * f[q].v - cp[2] * zb[q];
    }
  }
  for (int q = 0; q < 16; q++) {
    R v = warp_sum(acc[q]);
    if ((threadIdx.x & 31) == 0 && v != R(0)) {
      double* dst;
      if (q < 3) dst = lam + 3 * dn + q;
      else if (q < 15) dst = lam + sidx(n3, cr, q - 3);
      else dst = th + 3;
      atomicAdd(dst, (double)v);
    }
  }
}

// ------------------------------------------------------------ core-core
// one CTA per core pair; threads over the first core's charges, the second
// core's sites (position, torque-adjoint terms) staged in shared memory
constexpr int kCcThreads = 64;  // core i's sites per CTA of a core pair

template <class R>
__global__ void __launch_bounds__(kCcThreads) k_adj_corecore(DevModel M, const double* __restrict__ x,
                                                      const double* __restrict__ fb, double* lam, double* th) {
  extern __shared__ unsigned char smem_raw[];
  R* sl = reinterpret_cast<R*>(smem_raw);  // per site l: p_l(3), Qj(3), Kj(3), cp_l(3), q_l
  const int ci = blockIdx.x / M.n_c, cj = blockIdx.x % M.n_c;
  if (ci >= cj) return;
  const int i = M.core_bead[ci], j = M.core_bead[cj], n3 = 3 * M.n;
  if (!pair_ok(M, i, j)) return;
  R xi[12], xj[12];
  ld_bead(x, n3, i, xi);
  ld_bead(x, n3, j, xj);
  {
    R dd[3] = {xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2]};
    if (val(norm3(dd)) > 25.0) return;
  }
  R Fi[3], Fj[3], Ti[3], Tj[3];
  for (int q = 0; q < 3; q++) {
    Fi[q] = R(fb[3 * i + q]);
    Fj[q] = R(fb[3 * j + q]);
    Ti[q] = R(fb[n3 + 3 * i + q]);
    Tj[q] = R(fb[n3 + 3 * j + q]);
  }
  const int Nq = M.Nq;
  for (int l = threadIdx.x; l < Nq; l += blockDim.x) {
    R cp[3] = {R(M.core_pos[3 * l]), R(M.core_pos[3 * l + 1]), R(M.core_pos[3 * l + 2])};
    R* e = sl + 13 * l;  // core j's sites, staged by every CTA of the pair
    for (int q = 0; q < 3; q++) e[q] = xj[q] + xj[3 + q] * cp[0] + xj[6 + q] * cp[1] + xj[9 + q] * cp[2];
    R Q[3];
    cross3(Tj, cp, Q);
    for (int q = 0; q < 3; q++) {
      e[3 + q] = Q[q];
      e[6 + q] = Q[0] * xj[3 + q] + Q[1] * xj[6 + q] + Q[2] * xj[9 + q];
      e[9 + q] = cp[q];
    }
    e[12] = R(M.core_q[l]);
  }
  __syncthreads();
  R acc[25];
  for (int q = 0; q < 25; q++) acc[q] = R(0);  // bead i: r a b c (12), bead j: r a b c (12), kappa
  const R ke = R(M.k_e), kex = R(M.k_ex), sg = R(M.sCC);
  // this CTA's slice of core i's sites: one per thread (the pair spread over
  // gridDim.y small CTAs, so the pairs of a step balance across the SMs)
  const int kend = min(Nq, (int)(blockIdx.y + 1) * (int)blockDim.x);
  for (int k = blockIdx.y * blockDim.x + threadIdx.x; k < kend; k += blockDim.x) {
    const R cp[3] = {R(M.core_pos[3 * k]), R(M.core_pos[3 * k + 1]), R(M.core_pos[3 * k + 2])};
    const R qk = R(M.core_q[k]);
    R pk[3], Qi[3], Ki[3];
    for (int q = 0; q < 3; q++) pk[q] = xi[q] + xi[3 + q] * cp[0] + xi[6 + q] * cp[1] + xi[9 + q] * cp[2];
    cross3(Ti, cp, Qi);
    for (int q = 0; q < 3; q++) Ki[q] = Qi[0] * xi[3 + q] + Qi[1] * xi[6 + q] + Qi[2] * xi[9 + q];
    R sumf[3] = {R(0), R(0), R(0)}, sumz[3] = {R(0), R(0), R(0)}, kap = R(0);
    R rj[3] = {R(0), R(0), R(0)}, aj[3] = {R(0), R(0), R(0)}, bj[3] = {R(0), R(0), R(0)}, cj3[3] = {R(0), R(0), R(0)};
    for (int l = 0; l < Nq; l++) {
      const R* e = sl + 13 * l;
      using D = Dual<R, 4>;
      D zd[3], f[3];
      for (int q = 0; q < 3; q++) {
        zd[q] = D(pk[q] - e[q]);
        zd[q].d[q] = R(1);
      }
      D kk(M.debye);
      kk.d[3] = R(1);
      pair_site(ke * qk * e[12], true, true, kex, sg, zd, kk, f);
      R fbar[3];
      for (int q = 0; q < 3; q++) fbar[q] = Fi[q] - Fj[q] + Ki[q] - e[6 + q];
      R zb[3];
      for (int g = 0; g < 3; g++) zb[g] = fbar[0] * f[0].d[g] + fbar[1] * f[1].d[g] + fbar[2] * f[2].d[g];
      kap += fbar[0] * f[0].d[3] + fbar[1] * f[1].d[3] + fbar[2] * f[2].d[3];
      for (int q = 0; q < 3; q++) {
        sumf[q] += f[q].v;
        sumz[q] += zb[q];
        rj[q] -= zb[q];
        aj[q] += -e[3] * f[q].v - e[9] * zb[q];
        bj[q] += -e[4] * f[q].v - e[10] * zb[q];
        cj3[q] += -e[5] * f[q].v - e[11] * zb[q];
      }
    }
    for (int q = 0; q < 3; q++) {
      acc[q] += sumz[q];
      acc[3 + q] += Qi[0] * sumf[q] + cp[0] * sumz[q];
      acc[6 + q] += Qi[1] * sumf[q] + cp[1] * sumz[q];
      acc[9 + q] += Qi[2] * sumf[q] + cp[2] * sumz[q];
      acc[12 + q] += rj[q];
      acc[15 + q] += aj[q];
      acc[18 + q] += bj[q];
      acc[21 + q] += cj3[q];
    }
    acc[24] += kap;
  }
  for (int q = 0; q < 25; q++) {
    R v = warp_sum(acc[q]);
    if ((threadIdx.x & 31) == 0 && v != R(0)) {
      double* dst;
      if (q < 12) dst = lam + sidx(n3, i, q);
      else if (q < 24) dst = lam + sidx(n3, j, q - 12);
      else dst = th + 3;
      atomicAdd(dst, (double)v);
    }
  }
}

// ------------------------------------------------------------ tails
template <class R, class G = R>
__global__ void k_adj_tail_bonded(DevModel M, const double* __restrict__ x, const double* __restrict__ fb,
                                  double* lam) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = M.n_tail;
  if (i >= nt) return;
  const int ot = 12 * M.n, of = 6 * M.n;
  if (i < nt - 1 && M.t_grp[i] == M.t_grp[i + 1]) {  // func.cpp:1796-1802
    R xin[6], yb[3], xb[6];
    for (int q = 0; q < 6; q++) xin[q] = R(x[ot + 3 * i + q]);
    for (int q = 0; q < 3; q++) yb[q] = R(fb[of + 3 * i + q] - fb[of + 3 * i + 3 + q]);
    const R ht = R(M.h_t[i]), lo = R(M.lo_t[i]);
    vjp_chunk_g<6, 6, 3, G>([&](const auto* xd, auto* yd) { stretch_f(ht, lo, xd, xd + 3, yd); }, xin, yb, 0, xb);
    for (int q = 0; q < 6; q++) atomicAdd(lam + ot + 3 * i + q, (double)xb[q]);
  }
  if (i < nt - 2 && M.t_grp[i] == M.t_grp[i + 1] && M.t_grp[i] == M.t_grp[i + 2]) {  // func.cpp:1803-1810
    R xin[9], yb[9], xb[9];
    for (int q = 0; q < 9; q++) {
      xin[q] = R(x[ot + 3 * i + q]);
      yb[q] = -R(fb[of + 3 * i + q]);
    }
    const R gt = R(M.g_t[i]), b0 = R(M.beta_o_t[i]);
    vjp_chunk_g<9, 9, 9, G>([&](const auto* xd, auto* yd) { bend3_f(gt, b0, xd, xd + 3, xd + 6, yd); }, xin, yb, 0, xb);
    for (int q = 0; q < 9; q++) atomicAdd(lam + ot + 3 * i + q, (double)xb[q]);
  }
}

// tail-tail (clamped DH) and tail-linker (clamped DH + LJ) pairs
// (func.cpp:1811-1830); one thread per (tail, tail or chain bead)
template <class R>
__global__ void k_adj_tail_pairs(DevModel M, const double* __restrict__ x, const double* __restrict__ fb, double* lam,
                                 double* th) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int nt = M.n_tail, n = M.n, w = nt + n;
  const int i = (int)(t / w), j = (int)(t % w);
  const int ot = 12 * n, of = 6 * n;
  R kb = R(0);
  if (t < (long)nt * w) {
    bool tt = j < nt;
    bool ok = tt ? (i < j && (M.t_grp[i] != M.t_grp[j] || j > i + 2)) : (M.type[j - nt] == 0);
    if (ok) {
      const int jj = tt ? j : j - nt;
      const double* xj = tt ? x + ot + 3 * jj : x + 3 * jj;
      const double* fj = tt ? fb + of + 3 * jj : fb + 3 * jj;
      R v[3];
      using D = Dual<R, 4>;
      D zd[3], f[3];
      for (int q = 0; q < 3; q++) {
        zd[q] = D(x[ot + 3 * i + q] - xj[q]);
        zd[q].d[q] = R(1);
        v[q] = R(fb[of + 3 * i + q] - fj[q]);
      }
      D kk(M.debye);
      kk.d[3] = R(1);
      const R eps = R(1.0 / (4 * kPi * M.k_e));
      if (tt) pair_clamped(R(M.t_q[i] * M.t_q[jj]), eps, false, R(0), R(1), zd, kk, f);
      else pair_clamped(R(M.t_q[i] * M.q_l), eps, true, R(M.k_ex), R(M.sTL), zd, kk, f);
      double* lj = tt ? lam + ot + 3 * jj : lam + 3 * jj;
      for (int g = 0; g < 3; g++) {
        R zb = v[0] * f[0].d[g] + v[1] * f[1].d[g] + v[2] * f[2].d[g];
        if (zb != R(0)) {
          atomicAdd(lam + ot + 3 * i + g, (double)zb);
          atomicAdd(lj + g, -(double)zb);
        }
      }
      kb = v[0] * f[0].d[3] + v[1] * f[1].d[3] + v[2] * f[2].d[3];
    }
  }
  kb = warp_sum(kb);
  if ((threadIdx.x & 31) == 0 && kb != R(0)) atomicAdd(th + 3, (double)kb);
}

// anchors of the template tail beads to their cores (func.cpp:1831-1856)
template <class R, class G = R>
__global__ void k_adj_anchor(DevModel M, const double* __restrict__ x, const double* __restrict__ fb, double* lam,
                             double* th) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nt0 = M.n_t;
  const int kc = t / (2 * nt0), jt = (t / 2) % nt0, ch = t % 2;
  if (kc >= M.n_c || M.nc_t_flag[kc] != 1 || M.tail_fix[jt] != 1) return;
  const int i = M.core_bead[kc], tb = kc * nt0 + jt, n3 = 3 * M.n, ot = 12 * M.n, of = 6 * M.n;
  R xin[16], yb[9], xb[8];
  for (int q = 0; q < 3; q++) xin[q] = R(x[ot + 3 * tb + q]);
  ld_bead(x, n3, i, xin + 3);
  xin[15] = R(M.h);
  for (int q = 0; q < 3; q++) {
    yb[q] = R(fb[of + 3 * tb + q]);
    yb[3 + q] = R(fb[3 * i + q]);
    yb[6 + q] = R(fb[n3 + 3 * i + q]);
  }
  const double* P = M.tail_pos + 3 * jt;
  vjp_chunk_g<8, 16, 9, G>([&](const auto* xd, auto* yd) { anchor_term(P, xd, xd + 3, xd[15], yd); }, xin, yb, ch, xb);
  for (int j = 0; j < 8; j++) {
    const int q = ch * 8 + j;
    const double v = (double)xb[j];
    if (q < 3) atomicAdd(lam + ot + 3 * tb + q, v);
    else if (q < 15) atomicAdd(lam + sidx(n3, i, q - 3), v);
    else atomicAdd(th + 0, v);
  }
}

// ------------------------------------------------------------ frames, moves
// adjoint of the first refresh pass: copy, with the refreshed DNA frame
// entries (recomputed by the pass) cleared, then the pass's VJP adds to it
__global__ void k_pass1_init(DevModel M, const double* lam_in, double* lam_out, int ns) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ns) return;
  const int n3 = 3 * M.n;
  double v = lam_in[t];
  if (t >= n3 && t < 4 * n3) {
    const int bead = (t % n3) / 3;
    if (bead < M.n - 1 && M.type[bead] == 0) v = 0.0;
  }
  lam_out[t] = v;
}

constexpr int kP1In = 21;
constexpr int kP1Chunks = (kP1In + kBW - 1) / kBW;

template <class R, class G = R>
__global__ void k_adj_pass1(DevModel M, const double* __restrict__ x, const double* __restrict__ lam_in,
                            double* lam_out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / kP1Chunks, ch = t % kP1Chunks;
  if (i >= M.n - 1 || M.type[i] != 0) return;
  const int n3 = 3 * M.n, tn = M.type[i + 1];
  R xin[kP1In], yb[9], xb[kBW];
  for (int q = 0; q < 3; q++) {
    xin[q] = R(x[3 * i + q]);
    xin[3 + q] = R(x[3 * (i + 1) + q]);
    xin[6 + q] = R(x[n3 + 3 * i + q]);
    xin[9 + q] = R(x[2 * n3 + 3 * i + q]);
    xin[12 + q] = R(x[n3 + 3 * (i + 1) + q]);
    xin[15 + q] = R(x[2 * n3 + 3 * (i + 1) + q]);
    xin[18 + q] = R(x[3 * n3 + 3 * (i + 1) + q]);
    yb[q] = R(lam_in[n3 + 3 * i + q]);
    yb[3 + q] = R(lam_in[2 * n3 + 3 * i + q]);
    yb[6 + q] = R(lam_in[3 * n3 + 3 * i + q]);
  }
  vjp_chunk_g<kBW, kP1In, 9, G>(
      [&](const auto* xd, auto* yd) { frame_pass1(tn, xd, xd + 3, xd + 6, xd + 9, xd + 12, xd + 15, xd + 18, yd); },
      xin, yb, ch, xb);
  for (int j = 0; j < kBW; j++) {
    const int q = ch * kBW + j;
    if (q >= kP1In) break;
    const double v = (double)xb[j];
    if (v == 0.0) continue;
    const int comp = q % 3, grp = q / 3;
    // r_i, r_{i+1}, a_i, b_i, a_{i+1}, b_{i+1}, c_{i+1}
    const int bead = (grp == 0 || grp == 2 || grp == 3) ? i : i + 1;
    const int field = (grp <= 1) ? 0 : (grp == 2 || grp == 4) ? 1 : (grp == 3 || grp == 5) ? 2 : 3;
    atomicAdd(lam_out + field * n3 + 3 * bead + comp, v);
  }
}

// adjoint of rotate (func.cpp:1607-1670) for one bead: torque and frame
template <class R, class G = R>
__global__ void k_adj_rotate(DevModel M, const double* __restrict__ x, const double* __restrict__ T,
                             const double* __restrict__ rr, const double* __restrict__ lamR, double* lamX,
                             double* Tbar) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M.n) return;
  const int n3 = 3 * M.n;
  R xin[12], yb[9], xb[12];
  for (int q = 0; q < 3; q++) {
    xin[q] = R(T[3 * i + q]);
    xin[3 + q] = R(x[n3 + 3 * i + q]);
    xin[6 + q] = R(x[2 * n3 + 3 * i + q]);
    xin[9 + q] = R(x[3 * n3 + 3 * i + q]);
    yb[q] = R(lamR[n3 + 3 * i + q]);
    yb[3 + q] = R(lamR[2 * n3 + 3 * i + q]);
    yb[6 + q] = R(lamR[3 * n3 + 3 * i + q]);
  }
  const int core = M.type[i] != 0;
  const double dt = M.dt;
  const double* rri = rr + 3 * i;
  vjp_chunk_g<12, 12, 9, G>([&](const auto* xd, auto* yd) { rotate_frame(core, dt, rri, xd, xd + 3, yd); }, xin, yb, 0,
                       xb);
  for (int q = 0; q < 3; q++) Tbar[3 * i + q] += (double)xb[q];
  for (int q = 3; q < 12; q++) lamX[sidx(n3, i, q)] += (double)xb[q];
}

// translation's identity parts: the state's positions and the noise rd
__global__ void k_pos_through(int n, int nt, const double* lamR, double* lamX, double* lv, double* rdb) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int n3 = 3 * n;
  if (t >= n3 + 3 * nt) return;
  const int s = t < n3 ? t : 4 * n3 + (t - n3);
  const double v = lamR[s];
  lamX[s] += v;
  lv[t] = v;
  rdb[t] += v;
}

// species-block RPY product (D_blk v)_I, added as scale * (D_blk v) to the
// force adjoint (chain F | tails tF); warp per bead
template <class R>
__global__ void k_dblk(DevModel M, const double* __restrict__ r_all, const double* __restrict__ v, double scale,
                       double* fb) {
  const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int n = M.n, nD = n + M.n_tail;
  if (I >= nD) return;
  const int lo = I < n ? 0 : n, hi = I < n ? n : nD;
  const R a1 = R(M.a1), a2 = R(M.a2), ri = R(M.rad_all[I]);
  R acc[3] = {R(0), R(0), R(0)};
  for (int J = lo + lane; J < hi; J += 32) {
    if (J == I) {
      for (int q = 0; q < 3; q++) acc[q] += (a1 / ri) * R(v[3 * I + q]);
      continue;
    }
    R s[3], B[9];
    for (int q = 0; q < 3; q++) s[q] = R(r_all[3 * I + q] - r_all[3 * J + q]);
    rpy_block(ri, R(M.rad_all[J]), a1, a2, s, B);
    for (int p = 0; p < 3; p++)
      for (int q = 0; q < 3; q++) acc[p] += B[3 * p + q] * R(v[3 * J + q]);
  }
  for (int q = 0; q < 3; q++) acc[q] = warp_sum(acc[q]);
  if (lane == 0) {
    const int o = I < n ? 3 * I : 6 * n + 3 * (I - n);
    for (int q = 0; q < 3; q++) fb[o + q] += scale * (double)acc[q];
  }
}

// forces of a DevForces in tensor order (chain | tails)
__global__ void k_stack(int n, int nt, const double* F, const double* tF, double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 3 * n) out[t] = F[t];
  else if (t < 3 * (n + nt)) out[t] = tF[t - 3 * n];
}

__global__ void k_half(int cnt, const double* a, double* b, double* c) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < cnt) b[t] = c[t] = 0.5 * a[t];
}

// r_bar += sum_J sum_ab W_ab dB_ab(r_I - r_J)/d r_I with W the adjoint of the
// (I, J) and (J, I) blocks: Cholesky part Db and, within a species, the two
// drift products del (lz Fa^T) and del (ly F0^T); warp per bead
template <class R>
__global__ void k_adj_rpy(DevModel M, const double* __restrict__ r_all, const R* __restrict__ Db, int ldd,
                          const double* __restrict__ lz, const double* __restrict__ ly,
                          const double* __restrict__ fa, const double* __restrict__ f0, double* lam) {
  const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int n = M.n, nD = n + M.n_tail;
  if (I >= nD) return;
  const R a1 = R(M.a1), a2 = R(M.a2), ri = R(M.rad_all[I]), del = R(M.del);
  R lzI[3], lyI[3], faI[3], f0I[3];
  for (int q = 0; q < 3; q++) {
    lzI[q] = R(lz[3 * I + q]);
    lyI[q] = R(ly[3 * I + q]);
    faI[q] = R(fa[3 * I + q]);
    f0I[q] = R(f0[3 * I + q]);
  }
  const bool chainI = I < n;
  R acc[3] = {R(0), R(0), R(0)};
  for (int J = lane; J < nD; J += 32) {
    if (J == I) continue;
    using D = Dual<R, 3>;
    D s[3], B[9];
    for (int q = 0; q < 3; q++) {
      s[q] = D(r_all[3 * I + q] - r_all[3 * J + q]);
      s[q].d[q] = R(1);
    }
    rpy_block(ri, R(M.rad_all[J]), a1, a2, s, B);
    const bool same = (J < n) == chainI;
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) {
        R w = Db[(size_t)(3 * I + a) * ldd + 3 * J + b] + Db[(size_t)(3 * J + b) * ldd + 3 * I + a];
        if (same)
          w += del * (lzI[a] * R(fa[3 * J + b]) + faI[a] * R(lz[3 * J + b]) + lyI[a] * R(f0[3 * J + b]) +
                      f0I[a] * R(ly[3 * J + b]));
        for (int g = 0; g < 3; g++) acc[g] += w * B[3 * a + b].d[g];
      }
  }
  for (int q = 0; q < 3; q++) acc[q] = warp_sum(acc[q]);
  if (lane == 0) {
    const int o = chainI ? 3 * I : 12 * n + 3 * (I - n);
    for (int q = 0; q < 3; q++) lam[o + q] += (double)acc[q];
  }
}

// ------------------------------------------------------------ observable
// |r_{n-1} - r_0|^2 + Rg over the chain beads, scaled; with lam != nullptr
// its gradient is added to lam.  One CTA.
__global__ void k_loss(int n, const double* __restrict__ x, double scale, double* loss, double* lam) {
  __shared__ double sh[3][256];
  __shared__ double cm[3], rg;
  double s[3] = {0, 0, 0};
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    for (int q = 0; q < 3; q++) s[q] += x[3 * i + q];
  for (int q = 0; q < 3; q++) sh[q][threadIdx.x] = s[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < 3; q++) {
      double t = 0;
      for (int k = 0; k < (int)blockDim.x; k++) t += sh[q][k];
      cm[q] = t / n;
    }
  }
  __syncthreads();
  double r2 = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    for (int q = 0; q < 3; q++) r2 += (x[3 * i + q] - cm[q]) * (x[3 * i + q] - cm[q]);
  sh[0][threadIdx.x] = r2;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < (int)blockDim.x; k++) t += sh[0][k];
    rg = sqrt(t / n);
    double e2 = 0;
    for (int q = 0; q < 3; q++) {
      double e = x[3 * (n - 1) + q] - x[q];
      e2 += e * e;
    }
    loss[0] += scale * (e2 + rg);
  }
  __syncthreads();
  if (!lam) return;
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    for (int q = 0; q < 3; q++) atomicAdd(lam + 3 * i + q, scale * (x[3 * i + q] - cm[q]) / (n * rg));
  if (threadIdx.x == 0)
    for (int q = 0; q < 3; q++) {
      double e = x[3 * (n - 1) + q] - x[q];
      atomicAdd(lam + 3 * (n - 1) + q, scale * 2 * e);
      atomicAdd(lam + q, -scale * 2 * e);
    }
}

// ------------------------------------------------------------ Cholesky backward
// U = L^T as a dense row-major mp x mp matrix (identity on the padding)
template <class R, bool DF>
__global__ void k_extract_u(int m, int mp, const double* __restrict__ A, int lda, R* U) {
  const int k = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= mp) return;
  R v = R(0);
  if (k < m && i < m) {
    if (i >= k) {
      if (DF) {
        const float2 e = reinterpret_cast<const float2*>(A)[(size_t)k * lda + i];
        v = R(e.x) + R(e.y);
      } else {
        v = R(A[(size_t)k * lda + i]);
      }
    }
  } else if (i == k) {
    v = R(1);
  }
  U[(size_t)k * mp + i] = v;
}

// u = U rd_bar (warp per row)
template <class R>
__global__ void k_trmv_u(int mp, const R* __restrict__ U, const double* __restrict__ rdb, R* u) {
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (k >= mp) return;
  R s = R(0);
  for (int i = k + lane; i < mp; i += 32) s += U[(size_t)k * mp + i] * R(rdb[i]);
  s = warp_sum(s);
  if (lane == 0) u[k] = s;
}

// inverse of each 64 x 64 diagonal block of the upper-triangular U
template <class R>
__global__ void __launch_bounds__(64) k_inv_leaf(int mp, const R* __restrict__ U, R* V) {
  extern __shared__ unsigned char smem_raw[];
  R(*Us)[65] = reinterpret_cast<R(*)[65]>(smem_raw);
  R(*Vs)[65] = reinterpret_cast<R(*)[65]>(smem_raw + 64 * 65 * sizeof(R));
  const int b0 = blockIdx.x * 64, c = threadIdx.x;
  for (int e = c; e < 64 * 64; e += 64) Us[e / 64][e % 64] = U[(size_t)(b0 + e / 64) * mp + b0 + e % 64];
  __syncthreads();
  for (int i = 63; i > c; i--) Vs[i][c] = R(0);
  for (int i = c; i >= 0; i--) {
    R s = (i == c) ? R(1) : R(0);
    for (int k = i + 1; k <= c; k++) s -= Us[i][k] * Vs[k][c];
    Vs[i][c] = s / Us[i][i];
  }
  __syncthreads();
  for (int e = c; e < 64 * 64; e += 64) V[(size_t)(b0 + e / 64) * mp + b0 + e % 64] = Vs[e / 64][e % 64];
}

// C = alpha A op(B) (row-major; op(B) = B or B^T), M, N, K multiples of 64;
// gridDim.z independent products with operands zstride elements apart.
// kmode restricts the k range of each 64 x 64 output tile (r0, c0) to
// the nonzero band of triangular operands: 1: k >= r0, 2: k >= c0,
// 4: k < c0 + 64.
constexpr int kGT = 64, kGK = 16;
template <class R, bool TB>
__global__ void __launch_bounds__(256) k_gemm(int K, R alpha, const R* __restrict__ A, int lda,
                                              const R* __restrict__ B, int ldb, R* C, int ldc, int kmode,
                                              long zstride) {
  const int r0 = blockIdx.y * kGT, c0 = blockIdx.x * kGT;
  A += blockIdx.z * zstride;  // batch item z: every operand shifted by z * zstride elements
  B += blockIdx.z * zstride;
  C += blockIdx.z * zstride;
  int kb = 0, ke = K;
  if (kmode & 1) kb = max(kb, r0);
  if (kmode & 2) kb = max(kb, c0);
  if (kmode & 4) ke = min(ke, c0 + kGT);
  __shared__ R As[kGK][kGT + 4];
  __shared__ R Bs[kGK][kGT + 4];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  R acc[4][4];
  for (int u = 0; u < 4; u++)
    for (int v = 0; v < 4; v++) acc[u][v] = R(0);
  for (int k0 = kb; k0 < ke; k0 += kGK) {
    for (int e = threadIdx.x; e < kGT * kGK; e += 256) {
      const int rr = e / kGK, kk = e % kGK;
      As[kk][rr] = A[(size_t)(r0 + rr) * lda + k0 + kk];
      if (TB) {
        Bs[kk][rr] = B[(size_t)(c0 + rr) * ldb + k0 + kk];
      } else {
        const int k2 = e / kGT, cc = e % kGT;
        Bs[k2][cc] = B[(size_t)(k0 + k2) * ldb + c0 + cc];
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kGK; kk++) {
      R a[4], b[4];
      for (int u = 0; u < 4; u++) {
        a[u] = As[kk][ty * 4 + u];
        b[u] = Bs[kk][tx * 4 + u];
      }
      for (int u = 0; u < 4; u++)
        for (int v = 0; v < 4; v++) acc[u][v] += a[u] * b[v];
    }
    __syncthreads();
  }
  for (int u = 0; u < 4; u++)
    for (int v = 0; v < 4; v++) C[(size_t)(r0 + ty * 4 + u) * ldc + c0 + tx * 4 + v] = alpha * acc[u][v];
}

// Xt[c][i] = s2dt u_i (sum_{j<=i} p_j V[c][j] - p_i V[c][i] / 2): row c of
// (Phi V^T)^T with Phi = tril(s2dt u p^T), diagonal halved; CTA per row
template <class R>
__global__ void __launch_bounds__(256) k_build_xt(int m, int mp, const R* __restrict__ V,
                                                  const double* __restrict__ p, const R* __restrict__ u, R s2dt,
                                                  R* Xt) {
  __shared__ R wsum[8];
  const int c = blockIdx.x, lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const R* row = V + (size_t)c * mp;
  R carry = R(0);
  for (int i0 = 0; i0 < mp; i0 += 256) {
    const int i = i0 + threadIdx.x;  // mp is a multiple of 64, not of 256: lanes past mp carry zeros
    const R pi = i < m ? R(p[i]) : R(0);
    const R vi = (i >= c && i < mp) ? row[i] : R(0);  // V is upper triangular; its lower blocks are never written
    R s = pi * vi;
    for (int o = 1; o < 32; o <<= 1) {
      R t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += t;
    }
    if (lane == 31) wsum[wid] = s;
    __syncthreads();
    R before = R(0), total = R(0);
    for (int w = 0; w < 8; w++) {
      if (w < wid) before += wsum[w];
      total += wsum[w];
    }
    const R pref = carry + before + s;
    if (i < mp) Xt[(size_t)c * mp + i] = s2dt * u[i] * (pref - R(0.5) * pi * vi);
    carry += total;
    __syncthreads();
  }
}

// ------------------------------------------------------------ host side
template <class R>
int gemm(cudaStream_t st, int M_, int N_, int K_, R alpha, const R* A, int lda, const R* B, int ldb, R* C, int ldc,
         bool tb, int kmode, int batch = 1, long zstride = 0) {
  dim3 grid(N_ / kGT, M_ / kGT, batch);
  if (tb) k_gemm<R, true><<<grid, 256, 0, st>>>(K_, alpha, A, lda, B, ldb, C, ldc, kmode, zstride);
  else k_gemm<R, false><<<grid, 256, 0, st>>>(K_, alpha, A, lda, B, ldb, C, ldc, kmode, zstride);
  return 0;
}

// The tensor-core form for FP32 operands whose tiles are 128 x 128
// (tcgen05, three BF16 slices, six products: FP32-class); FP64 operands and
// the 64-wide first doubling level stay on the SIMT kernel.
template <class R>
int gemm_tc(cudaStream_t st, int M_, int N_, int K_, R alpha, const R* A, int lda, const R* B, int ldb, R* C, int ldc,
            bool tb, int kmode, int* err, int batch = 1, long zstride = 0) {
  if constexpr (std::is_same<R, float>::value) {
    if (err && M_ % 128 == 0 && N_ % 128 == 0 && K_ % 64 == 0)
      return bdk::tc_gemm_f32(st, M_, N_, K_, alpha, A, lda, B, ldb, C, ldc, tb, kmode, batch, zstride, err);
  }
  return gemm<R>(st, M_, N_, K_, alpha, A, lda, B, ldb, C, ldc, tb, kmode, batch, zstride);
}

// V = U^-1 for the upper-triangular U of order mp = 64 * 2^k (diagonal
// 64-blocks already inverted), by doubling: at block size b every diagonal
// 2b-block [[V11, V12], [0, V22]] gets V12 = -V11 (U12 V22), all blocks of a
// level in one batched launch per product (2 launches per level).
template <class R>
int inv_upper(cudaStream_t st, int mp, const R* U, R* V, R* tmp, int& launches, int* err) {
  for (int b = 64; b < mp; b *= 2) {
    const int nodes = mp / (2 * b);
    const long zs = 2L * b * (mp + 1);
    // T = U12 V22 (V22 upper: k < c0 + tile), then V12 = -V11 T (V11 upper: k >= r0)
    int rc = gemm_tc<R>(st, b, b, b, R(1), U + b, mp, V + (size_t)b * mp + b, mp, tmp + b, mp, false, 4, err, nodes, zs);
    if (!rc) rc = gemm_tc<R>(st, b, b, b, R(-1), V, mp, tmp + b, mp, V + b, mp, false, 1, err, nodes, zs);
    if (rc) return rc;
    launches += 2;
  }
  return 0;
}

}  // namespace

// ------------------------------------------------------------ work buffers
struct bdh::AdjWork {
  int nsteps = 0, K = 0, mp = 0, rsize = 0;
  size_t ns = 0, nfull = 0, nf = 0;
  double *ckpt = nullptr, *seg = nullptr, *x0 = nullptr;
  // per step of the segment being reversed: the factor L (the context's A),
  // r_all, the forces F0 and Fa ([F | T | tF] each) and the predictor /
  // corrector states of the step
  double *segA = nullptr, *segR = nullptr, *segF = nullptr, *segS = nullptr;
  double *lam = nullptr, *lamX = nullptr, *lamZ = nullptr, *lamY = nullptr, *lamYr = nullptr;
  double *fbA = nullptr, *fb0 = nullptr, *fb1 = nullptr;
  double *lz = nullptr, *ly = nullptr, *fa = nullptr, *f0 = nullptr, *rdb = nullptr;
  double *th = nullptr, *loss = nullptr, *scratch = nullptr, *rr = nullptr, *p = nullptr;
  void *U = nullptr, *V = nullptr, *Xt = nullptr, *Db = nullptr, *u = nullptr;
  std::vector<void*> allocs;
  long launches = 0;
};

void bdh::adj_free(AdjWork* w) {
  if (!w) return;
  for (void* p : w->allocs) cudaFree(p);
  delete w;
}

namespace {

// the DevState fields a step reads (no linker histone), in a fixed order
std::vector<std::pair<double*, size_t>> full_fields(const bd_ctx* c, const DevState& X) {
  const size_t n = c->M.n, nc = c->M.n_c, nt = c->M.n_tail;
  return {{X.r, 3 * n},      {X.a, 3 * n},       {X.b, 3 * n},       {X.c, 3 * n},     {X.r_t, 3 * nt},
          {X.alpha, n},      {X.beta, n},        {X.gamma, n},       {X.length, n},    {X.a_dna, 3 * nc},
          {X.b_dna, 3 * nc}, {X.c_dna, 3 * nc},  {X.alpha_p, nc},    {X.beta_p, nc},   {X.gamma_p, nc},
          {X.beta_t, nt}};
}

int pack_full(bd_ctx* c, double* dst, bool store) {
  size_t o = 0;
  for (auto& f : full_fields(c, c->X)) {
    if (f.second) {
      if (store) CK(cudaMemcpyAsync(dst + o, f.first, f.second * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      else CK(cudaMemcpyAsync(f.first, dst + o, f.second * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    }
    o += f.second;
  }
  return BD_OK;
}

int ensure_work(bd_ctx* c, int N, int K, bool grad) {
  bdh::AdjWork*& w = c->adj;
  const int rsize = c->precision == BD_PREC_MIXED ? 4 : 8;
  if (w && w->nsteps >= N && w->K == K && w->rsize == rsize && (w->U || !grad)) return BD_OK;
  bdh::adj_free(w);
  w = new bdh::AdjWork();
  w->nsteps = N;
  w->K = K;
  w->rsize = rsize;
  const DevModel& M = c->M;
  const size_t n = M.n, nt = M.n_tail, m = c->m;
  w->ns = 12 * n + 3 * nt;
  w->nf = 6 * n + 3 * nt;
  size_t nfull = 0;
  for (auto& f : full_fields(c, c->X)) nfull += f.second;
  w->nfull = nfull;
  // the triangular inverse doubles 64-blocks: the matrices of the Cholesky
  // backward are padded (identity) to 64 * 2^k >= m
  w->mp = 64;
  while (w->mp < (int)m) w->mp *= 2;
  auto take = [&](void** p, size_t bytes) -> int {
    CK(cudaMalloc(p, bytes ? bytes : 256));
    w->allocs.push_back(*p);
    return BD_OK;
  };
  int rc = 0;
  const size_t d = sizeof(double);
  const int nck = (N + K - 1) / K;
  if ((rc = take((void**)&w->x0, nfull * d)) || (rc = take((void**)&w->loss, 8 * d)) ||
      (rc = take((void**)&w->scratch, 8 * d)) || (rc = take((void**)&w->rr, (size_t)N * 3 * n * d)) ||
      (rc = take((void**)&w->p, (size_t)N * m * d)))
    return rc;
  if (grad) {
    const size_t mp = w->mp, ns = w->ns, nf = w->nf;
    if ((rc = take((void**)&w->ckpt, nck * nfull * d)) || (rc = take((void**)&w->seg, (size_t)K * nfull * d)) ||
        (rc = take((void**)&w->lam, ns * d)) || (rc = take((void**)&w->lamX, ns * d)) ||
        (rc = take((void**)&w->lamZ, ns * d)) || (rc = take((void**)&w->lamY, ns * d)) ||
        (rc = take((void**)&w->lamYr, ns * d)) ||
        (rc = take((void**)&w->fbA, nf * d)) || (rc = take((void**)&w->fb0, nf * d)) ||
        (rc = take((void**)&w->fb1, nf * d)) || (rc = take((void**)&w->lz, m * d)) ||
        (rc = take((void**)&w->ly, m * d)) || (rc = take((void**)&w->fa, m * d)) ||
        (rc = take((void**)&w->f0, m * d)) || (rc = take((void**)&w->rdb, mp * d)) ||
        (rc = take((void**)&w->th, 8 * d)) || (rc = take((void**)&w->segA, (size_t)K * m * c->lda * d)) ||
        (rc = take((void**)&w->segR, (size_t)K * m * d)) || (rc = take((void**)&w->segF, (size_t)K * 2 * nf * d)) ||
        (rc = take((void**)&w->segS, (size_t)K * 3 * ns * d)) || (rc = take(&w->U, mp * mp * rsize)) ||
        (rc = take(&w->V, mp * mp * rsize)) || (rc = take(&w->Xt, mp * mp * rsize)) ||
        (rc = take(&w->Db, mp * mp * rsize)) || (rc = take(&w->u, mp * rsize)))
      return rc;
  }
  return BD_OK;
}

// adjoint of the forces at state x (fbar = [F | T | tF]) into lamOut and th.
// The O(n) terms built on Euler angles (acos of cosines near +-1, whose
// derivative FP32 cannot resolve) run in FP64 whatever R is; the pair sums
// run in R.
template <class R>
int forces_vjp(bd_ctx* c, const double* x, const double* fbar, double* lamOut, double* th, long& L) {
  const DevModel& M = c->M;
  cudaStream_t st = c->stream;
  const int n = M.n, nt = M.n_tail;
  if (std::is_same<R, float>::value)
    k_adj_bonds<double, float, kBondWm><<<cdiv((long)(n - 1) * bond_chunks(kBondWm), 64), 64, 0, st>>>(M, x, fbar,
                                                                                                    lamOut, th);
  else
    k_adj_bonds<double, double, kBondW><<<cdiv((long)(n - 1) * bond_chunks(kBondW), 64), 64, 0, st>>>(M, x, fbar,
                                                                                                   lamOut, th);
  k_adj_dnadna<R><<<cdiv((long)n * n, 128), 128, 0, st>>>(M, x, fbar, lamOut, th);
  if (M.n_dna > 0) k_adj_dnacore<R><<<M.n_dna * M.n_c, 128, 0, st>>>(M, x, fbar, lamOut, th);
  k_adj_corecore<R><<<dim3(M.n_c * M.n_c, cdiv(M.Nq, kCcThreads)), kCcThreads, 13 * M.Nq * sizeof(R), st>>>(
      M, x, fbar, lamOut, th);
  L += 4;
  if (nt > 0) {
    k_adj_tail_bonded<double, R><<<cdiv(nt, 128), 128, 0, st>>>(M, x, fbar, lamOut);
    k_adj_tail_pairs<R><<<cdiv((long)nt * (nt + n), 256), 256, 0, st>>>(M, x, fbar, lamOut, th);
    k_adj_anchor<double, R><<<cdiv((long)M.n_c * M.n_t * 2, 64), 64, 0, st>>>(M, x, fbar, lamOut, th);
    L += 3;
  }
  CK(cudaGetLastError());
  return BD_OK;
}

// run step `step` forward from the context's state, keeping its
// intermediates in slot `slot` of the segment buffers
int forward_saved(bd_ctx* c, bdh::AdjWork& w, int step, int slot) {
  cudaStream_t st = c->stream;
  const int n3 = 3 * c->M.n, nt3 = 3 * c->M.n_tail, m = c->m;
  const size_t ns = w.ns, nf = w.nf;
  double* S = w.segS + (size_t)slot * 3 * ns;
  double* sv[3] = {S, S + ns, S + 2 * ns};
  int rc = bdh::step_device(c, w.rr + (size_t)step * n3, w.p + (size_t)step * m, sv);
  if (rc) return rc;
  const size_t d = sizeof(double);
  CK(cudaMemcpyAsync(w.segA + (size_t)slot * m * c->lda, c->A, (size_t)m * c->lda * d, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(w.segR + (size_t)slot * m, c->r_all, (size_t)m * d, cudaMemcpyDeviceToDevice, st));
  double* F = w.segF + (size_t)slot * 2 * nf;
  const DevForces* fs[2] = {&c->F0, &c->Fa};
  for (int k = 0; k < 2; k++) {
    CK(cudaMemcpyAsync(F + k * nf, fs[k]->F, n3 * d, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(F + k * nf + n3, fs[k]->T, n3 * d, cudaMemcpyDeviceToDevice, st));
    if (nt3) CK(cudaMemcpyAsync(F + k * nf + 2 * n3, fs[k]->tF, nt3 * d, cudaMemcpyDeviceToDevice, st));
  }
  return BD_OK;
}

// one reverse step from the intermediates forward_saved kept in `slot`: lam
// holds the adjoint of x_{n+1}; on return, of x_n
template <class R>
int reverse_step(bd_ctx* c, bdh::AdjWork& w, int step, const double* xs, int slot) {
  const DevModel& M = c->M;
  cudaStream_t st = c->stream;
  const int n = M.n, nt = M.n_tail, n3 = 3 * n, m = c->m, mp = w.mp;
  const double* rr = w.rr + (size_t)step * n3;
  const double* p = w.p + (size_t)step * m;
  int rc = 0;
  const int ns = (int)w.ns, nf = (int)w.nf;
  const double* S = w.segS + (size_t)slot * 3 * ns;
  const double *Yraw = S, *Yref = S + ns, *Zraw = S + 2 * ns;
  const double* Lf = w.segA + (size_t)slot * m * c->lda;
  const double* r_all = w.segR + (size_t)slot * m;
  const double* F0 = w.segF + (size_t)slot * 2 * nf;  // [F | T | tF]
  const double* Fa = F0 + nf;
  long& L = w.launches;
  // corrector: refresh, rotation, translation
  k_pass1_init<<<cdiv(ns, 256), 256, 0, st>>>(M, w.lam, w.lamZ, ns);
  k_adj_pass1<double, R><<<cdiv((long)(n - 1) * kP1Chunks, 64), 64, 0, st>>>(M, Zraw, w.lam, w.lamZ);
  CK(cudaMemsetAsync(w.lamX, 0, ns * sizeof(double), st));
  CK(cudaMemsetAsync(w.fbA, 0, nf * sizeof(double), st));
  CK(cudaMemsetAsync(w.rdb, 0, mp * sizeof(double), st));
  k_adj_rotate<double, R><<<cdiv(n, 64), 64, 0, st>>>(M, xs, Fa + n3, rr, w.lamZ, w.lamX, w.fbA + n3);
  k_pos_through<<<cdiv(m, 256), 256, 0, st>>>(n, nt, w.lamZ, w.lamX, w.lz, w.rdb);
  k_dblk<R><<<cdiv((long)(n + nt) * 32, 256), 256, 0, st>>>(M, r_all, w.lz, M.del, w.fbA);
  k_half<<<cdiv(nf, 256), 256, 0, st>>>(nf, w.fbA, w.fb0, w.fb1);
  // forces at the refreshed predictor
  CK(cudaMemsetAsync(w.lamYr, 0, ns * sizeof(double), st));
  if ((rc = forces_vjp<R>(c, Yref, w.fb1, w.lamYr, w.th, L))) return rc;
  // predictor: refresh, rotation, translation
  k_pass1_init<<<cdiv(ns, 256), 256, 0, st>>>(M, w.lamYr, w.lamY, ns);
  k_adj_pass1<double, R><<<cdiv((long)(n - 1) * kP1Chunks, 64), 64, 0, st>>>(M, Yraw, w.lamYr, w.lamY);
  k_adj_rotate<double, R><<<cdiv(n, 64), 64, 0, st>>>(M, xs, F0 + n3, rr, w.lamY, w.lamX, w.fb0 + n3);
  k_pos_through<<<cdiv(m, 256), 256, 0, st>>>(n, nt, w.lamY, w.lamX, w.ly, w.rdb);
  k_dblk<R><<<cdiv((long)(n + nt) * 32, 256), 256, 0, st>>>(M, r_all, w.ly, M.del, w.fb0);
  // forces at the state
  if ((rc = forces_vjp<R>(c, xs, w.fb0, w.lamX, w.th, L))) return rc;
  // Cholesky backward: D_bar = V (Phi V^T), V = U^-1, U = L^T
  R *U = (R*)w.U, *V = (R*)w.V, *Xt = (R*)w.Xt, *Db = (R*)w.Db, *u = (R*)w.u;
  if (c->precision == BD_PREC_MIXED)
    k_extract_u<R, true><<<dim3(cdiv(mp, 256), mp), 256, 0, st>>>(m, mp, Lf, c->lda, U);
  else
    k_extract_u<R, false><<<dim3(cdiv(mp, 256), mp), 256, 0, st>>>(m, mp, Lf, c->lda, U);
  k_trmv_u<R><<<cdiv((long)mp * 32, 256), 256, 0, st>>>(mp, U, w.rdb, u);
  k_inv_leaf<R><<<mp / 64, 64, 2 * 64 * 65 * sizeof(R), st>>>(mp, U, V);
  int gl = 0;
  if (inv_upper<R>(st, mp, U, V, Xt, gl, c->d_err)) return set_error(BD_ERR_CUDA, "bd_adjoint: triangular inverse");
  k_build_xt<R><<<mp, 256, 0, st>>>(m, mp, V, p, u, R(M.s2dt), Xt);
  // D_bar tiles that k_adj_rpy reads (rows, columns < m); beyond m both
  // factors vanish along k (p and u are zero on the padding)
  const int mt = (std::is_same<R, float>::value && mp >= 128) ? (m + 127) / 128 * 128 : (m + 63) / 64 * 64;
  if (gemm_tc<R>(st, mt, mt, mt, R(1), V, mp, Xt, mp, Db, mp, true, 3, c->d_err))
    return set_error(BD_ERR_CUDA, "bd_adjoint: D_bar product");
  // the RPY tensor
  k_stack<<<cdiv(m, 256), 256, 0, st>>>(n, nt, Fa, Fa + 2 * n3, w.fa);
  k_stack<<<cdiv(m, 256), 256, 0, st>>>(n, nt, F0, F0 + 2 * n3, w.f0);
  k_adj_rpy<R><<<cdiv((long)(n + nt) * 32, 256), 256, 0, st>>>(M, r_all, Db, mp, w.lz, w.ly, w.fa, w.f0, w.lamX);
  L += 24 + gl;
  CK(cudaGetLastError());
  std::swap(w.lam, w.lamX);
  return BD_OK;
}

int check_ctx(bd_ctx* c, int N, int K, int Wn, const double* rr, const double* p) {
  if (!c || !rr || !p) return set_error(BD_ERR_ARG, "bd_adjoint: null argument");
  if (N < 1 || K < 1 || Wn < 1 || Wn > N) return set_error(BD_ERR_ARG, "bd_adjoint: bad n_steps / checkpoint / window");
  if (c->M.n_LH != 0) return set_error(BD_ERR_ARG, "bd_adjoint: fibers with linker histones are not supported");
  if (c->freq_rp != 1) return set_error(BD_ERR_ARG, "bd_adjoint: requires frequency_RP == 1");
  return BD_OK;
}

template <class R>
int run(bd_ctx* c, int N, int K, int Wn, const double* rr, const double* p, double* loss, double* grad4) {
  const bool grad = grad4 != nullptr;
  int rc = ensure_work(c, N, K, grad);
  if (rc) return rc;
  bdh::AdjWork& w = *c->adj;
  cudaStream_t st = c->stream;
  const DevModel& M = c->M;
  const int n3 = 3 * M.n, m = c->m;
  CK(cudaMemcpyAsync(w.rr, rr, (size_t)N * n3 * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(w.p, p, (size_t)N * m * sizeof(double), cudaMemcpyHostToDevice, st));
  if ((rc = pack_full(c, w.x0, true))) return rc;
  const long step0 = c->step_count;
  CK(cudaMemsetAsync(w.loss, 0, 8 * sizeof(double), st));
  const double scale = 1.0 / Wn;
  w.launches = 0;
  {
    bdh::Range fwd_range("bd_adjoint: forward sweep");
    for (int s = 0; s < N; s++) {
      if (grad && s % K == 0 && (rc = pack_full(c, w.ckpt + (size_t)(s / K) * w.nfull, true))) return rc;
      if ((rc = bdh::step_device(c, w.rr + (size_t)s * n3, w.p + (size_t)s * m))) return rc;
      if (s + 1 >= N - Wn + 1) k_loss<<<1, 256, 0, st>>>(M.n, c->X.r, scale, w.loss, nullptr);
    }
  }
  if (grad) {
    bdh::Range rev_range("bd_adjoint: reverse sweep");
    CK(cudaMemsetAsync(w.lam, 0, w.ns * sizeof(double), st));
    CK(cudaMemsetAsync(w.th, 0, 8 * sizeof(double), st));
    k_loss<<<1, 256, 0, st>>>(M.n, c->X.r, scale, w.scratch, w.lam);
    for (int sg = (N - 1) / K; sg >= 0; sg--) {
      const int s0 = sg * K, e = std::min(s0 + K, N);
      if ((rc = pack_full(c, w.ckpt + (size_t)sg * w.nfull, false))) return rc;
      for (int s = s0; s < e; s++) {
        if ((rc = pack_full(c, w.seg + (size_t)(s - s0) * w.nfull, true))) return rc;
        if ((rc = forward_saved(c, w, s, s - s0))) return rc;
      }
      for (int s = e - 1; s >= s0; s--) {
        double* xs = w.seg + (size_t)(s - s0) * w.nfull;
        if ((rc = reverse_step<R>(c, w, s, xs, s - s0))) return rc;
        if (s >= N - Wn + 1) k_loss<<<1, 256, 0, st>>>(M.n, xs, scale, w.scratch, w.lam);
      }
    }
  }
  if ((rc = pack_full(c, w.x0, false))) return rc;
  c->step_count = step0;
  double th[8] = {0};
  double lh = 0.0;
  int derr = 0;
  CK(cudaMemcpyAsync(&lh, w.loss, sizeof(double), cudaMemcpyDeviceToHost, st));
  if (grad) CK(cudaMemcpyAsync(th, w.th, 8 * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (c->d_err) CK(cudaMemcpyAsync(&derr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  if (derr) return set_error(BD_ERR_CUDA, "bd_adjoint: a tensor-core kernel timed out waiting on its copies/MMAs");
  if (!std::isfinite(lh)) return set_error(BD_ERR_NONFINITE, "bd_adjoint: non-finite observable");
  if (loss) *loss = lh;
  if (grad) {
    // Debye length lambda = 1 / debye; both screening constants scale as 1 / lambda
    grad4[0] = th[0];
    grad4[1] = th[1];
    grad4[2] = th[2];
    grad4[3] = -(th[3] * M.debye * M.debye + th[4] * M.debyell * M.debye);
    for (int k = 0; k < 4; k++)
      if (!std::isfinite(grad4[k])) {
        char b[200];
        snprintf(b, sizeof b, "bd_adjoint: non-finite gradient (h %g g %g s %g kappa %g kappa_ll %g)", th[0], th[1],
                 th[2], th[3], th[4]);
        return set_error(BD_ERR_NONFINITE, b);
      }
  }
  return BD_OK;
}

int set_leaf_smem() {
  static bool done = false;
  if (done) return BD_OK;
  CK(cudaFuncSetAttribute(k_inv_leaf<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * 64 * 65 * 8));
  CK(cudaFuncSetAttribute(k_inv_leaf<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * 64 * 65 * 4));
  if (bdk::tc_gemm_attributes()) return set_error(BD_ERR_CUDA, "bd_adjoint: kernel attributes (shared memory)");
  done = true;
  return BD_OK;
}

}  // namespace

extern "C" int bd_adjoint(bd_ctx* c, int n_steps, int checkpoint_every, int window, const double* rr,
                          const double* p, double* loss, double* grad4) {
  int rc = check_ctx(c, n_steps, checkpoint_every, window, rr, p);
  if (rc) return rc;
  if (!grad4) return set_error(BD_ERR_ARG, "bd_adjoint: null gradient");
  if ((rc = set_leaf_smem())) return rc;
  if (c->precision == BD_PREC_MIXED) return run<float>(c, n_steps, checkpoint_every, window, rr, p, loss, grad4);
  return run<double>(c, n_steps, checkpoint_every, window, rr, p, loss, grad4);
}

extern "C" int bd_rollout_loss(bd_ctx* c, int n_steps, int window, const double* rr, const double* p, double* loss) {
  int rc = check_ctx(c, n_steps, 1, window, rr, p);
  if (rc) return rc;
  if (!loss) return set_error(BD_ERR_ARG, "bd_rollout_loss: null loss");
  return run<double>(c, n_steps, n_steps, window, rr, p, loss, nullptr);
}

extern "C" int bd_adjoint_launches(bd_ctx* c, long* out) {
  if (!c || !out) return set_error(BD_ERR_ARG, "bd_adjoint_launches: null argument");
  *out = c->adj ? c->adj->launches : 0;
  return BD_OK;
}
