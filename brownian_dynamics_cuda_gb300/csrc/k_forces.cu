// Forces, torques and energy of one configuration (FP64 parity path).
//
// The reference sums every interaction into per-bead arrays in loop order
// (func.cpp:951-2781; its GPU version scatters into 6*maxrtlh^2 scratch
// arrays, func_cuda.cu:1299-1731).  Here every bead's total is gathered by
// the thread, warp or CTA that owns the bead: each pair is evaluated from
// both sides with the reference's formula (the two evaluations are bitwise
// negatives of each other), and the three interactions between rigid charge
// sets - core/core (300 x 300 sites), DNA/core (300 sites) and
// globular-head/core (6 x 300 sites) - are evaluated once per object pair
// into a slot and reduced per bead in a fixed order.  No atomics: results
// are bitwise reproducible run to run.
//
// Each pair energy is counted exactly once, on a fixed side.
#include <cuda_runtime.h>

#include "bd_internal.h"
#include "dev_physics.cuh"

using namespace bdp;

namespace {

inline int cdiv(int a, int b) { return (a + b - 1) / b; }

__device__ __forceinline__ bool chain_ok(const DevModel& M, int b) {
  // func.cpp:1316-1323: a bead next to a core takes no part in the
  // DNA/core electrostatics
  return (b == 0 || M.type[b - 1] == 0) && (b == M.n - 1 || M.type[b + 1] == 0);
}

__device__ __forceinline__ int lh_param(const DevModel& M, int bead) {
  int idx = bead % M.nlh;
  return idx < M.n_lh_n ? idx : idx + M.n_lh_g;
}

__device__ __forceinline__ double eps_of(const DevModel& M) { return 1 / (4 * kPi * M.k_e); }

__device__ __forceinline__ V3 site(const DevState& X, int bead, const double* p) {
  return body(ld3(X.r + 3 * bead), ld3(X.a + 3 * bead), ld3(X.b + 3 * bead), ld3(X.c + 3 * bead), p);
}

// Mixed path: a position as a double-float pair (hi, lo) of FP32 xyz.
struct PF {
  float4 h, l;
};
__device__ __forceinline__ PF ldpf(const DevScratch& S, int i) { return PF{S.ph[i], S.pl[i]}; }
// a - b
__device__ __forceinline__ float3 sepf(const PF& a, const PF& b) {
  return make_float3((a.h.x - b.h.x) + (a.l.x - b.l.x), (a.h.y - b.h.y) + (a.l.y - b.l.y),
                     (a.h.z - b.h.z) + (a.l.z - b.l.z));
}
__device__ __forceinline__ float3 crossf(const float3& u, const float3& v) {
  return make_float3(fmaf(u.y, v.z, -u.z * v.y), fmaf(u.z, v.x, -u.x * v.z), fmaf(u.x, v.y, -u.y * v.x));
}

// deterministic warp sum (fixed butterfly order)
__device__ __forceinline__ double wsum(double v) {
  for (int o = 16; o > 0; o >>= 1) v = v + __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// deterministic block sum of NV values per thread; result valid in thread 0
template <int NV>
__device__ void bsum(double (&v)[NV], double* sm /* [32*NV] */) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; k++) v[k] = wsum(v[k]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) sm[w * NV + k] = v[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) {
      double s = 0.0;
      for (int q = 0; q < nw; q++) s = s + sm[q * NV + k];
      v[k] = s;
    }
  }
  __syncthreads();
}

// Double-float (hi, lo) addition in FP32 (two-sum, then renormalised).
__device__ __forceinline__ void df_add(float& h, float& l, float h2, float l2) {
  const float s = h + h2, bb = s - h, e = (h - (s - bb)) + (h2 - bb);
  const float t = e + l + l2;
  h = s + t;
  l = t - (h - s);
}

// Deterministic block sum of NV double-float values per thread, in FP32
// two-sum arithmetic (fixed butterfly, then warps in order); the FP64
// totals are valid in thread 0.  sm: 32 * NV doubles.
template <int NV>
__device__ void bsum_df(float (&h)[NV], float (&l)[NV], double (&out)[NV], double* sm) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; k++)
    for (int o = 16; o > 0; o >>= 1) {
      const float h2 = __shfl_xor_sync(0xffffffffu, h[k], o), l2 = __shfl_xor_sync(0xffffffffu, l[k], o);
      df_add(h[k], l[k], h2, l2);
    }
  float2* smf = reinterpret_cast<float2*>(sm);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) smf[w * NV + k] = make_float2(h[k], l[k]);
  }
  __syncthreads();
  double* res = sm + 16 * NV;  // past the float2 table of up to 32 warps
  if (threadIdx.x < NV) {
    const int k = threadIdx.x;
    float H = 0.f, L = 0.f;
    for (int q = 0; q < nw; q++) df_add(H, L, smf[q * NV + k].x, smf[q * NV + k].y);
    res[k] = (double)H + (double)L;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) out[k] = res[k];
  }
  __syncthreads();
}

// ------------------------------------------------------------ G-head sites
__global__ void k_gpos(DevModel M, DevState X) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M.n_lhcore * M.n_lh_g) return;
  int lc = t / M.n_lh_g, m = t % M.n_lh_g;
  st3(X.gpos + 3 * t, site(X, M.lh_core_bead[lc], M.LH_g_pos + 3 * m));
}

// ------------------------------------------------------------ chain bonded
// One bond's stretch, bend and twist terms (func.cpp:978-1179).
struct BondOut {
  V3 f1[3], f2[3], t1[3], t2[3];  // [stretch, bend, twist]
  double E;
};

__device__ void bond_terms(const DevModel& M, const DevState& X, int i, BondOut& o) {
  const double si = sin(kTheta), co = cos(kTheta);
  V3 ri = ld3(X.r + 3 * i), ai = ld3(X.a + 3 * i), bi = ld3(X.b + 3 * i), ci = ld3(X.c + 3 * i);
  V3 rj = ld3(X.r + 3 * i + 3), aj = ld3(X.a + 3 * i + 3), bj = ld3(X.b + 3 * i + 3), cj = ld3(X.c + 3 * i + 3);
  V3 rf, rs;
  if (M.type[i + 1] == 0) {
    rf = rj;
  } else {
    V3 bm{-si * aj.x + co * bj.x, -si * aj.y + co * bj.y, -si * aj.z + co * bj.z};
    rf = V3{rj.x - kRo * bm.x + kD1 * cj.x, rj.y - kRo * bm.y + kD1 * cj.y, rj.z - kRo * bm.z + kD1 * cj.z};
  }
  if (M.type[i] == 0) rs = ri;
  else rs = V3{ri.x - (kRo * bi.x + kD1 * ci.x), ri.y - (kRo * bi.y + kD1 * ci.y), ri.z - (kRo * bi.z + kD1 * ci.z)};
  o.E = 0.0;
  // stretching (func.cpp:996)
  o.f1[0] = stretch_f1(M.h, rs, rf, kLo, o.E);
  o.f2[0] = stretch_f2(M.h, rs, rf, kLo);
  // bending (func.cpp:1049-1085)
  int ic = M.core_rank[i];
  const double* al = X.alpha;
  const double* be = X.beta;
  const double* ga = X.gamma;
  V3 af, ab, ao;
  double beta_b;
  if (M.type[i] == 0) {
    af = (M.type[i + 1] == 0) ? aj : V3{co * aj.x + si * bj.x, co * aj.y + si * bj.y, co * aj.z + si * bj.z};
    ab = (M.type[i - 1] == 0) ? ld3(X.a + 3 * i - 3) : ld3(X.a_dna + 3 * ic);
    ao = ai;
    beta_b = be[i - 1];
  } else {
    af = aj;
    ab = ai;
    ao = ld3(X.a_dna + 3 * ic);
    beta_b = X.beta_p[ic];
  }
  {
    double beta = be[i], len = X.length[i];
    o.E = o.E + M.g * (beta - beta_b) * (beta - beta_b) / 2;
    double g1 = (beta >= 1e-10) ? beta / (sin(beta) * len) : 1.0 / len;
    double cb1 = cos(beta);
    V3 A{g1 * (af.x - cb1 * ao.x), g1 * (af.y - cb1 * ao.y), g1 * (af.z - cb1 * ao.z)};
    double g2 = (beta_b >= 1e-10) ? beta_b / (sin(beta_b) * len) : 1.0 / len;
    double cb2 = cos(beta_b);
    V3 B{g2 * (ab.x - cb2 * ao.x), g2 * (ab.y - cb2 * ao.y), g2 * (ab.z - cb2 * ao.z)};
    o.f1[1] = V3{-M.g * (A.x + B.x), -M.g * (A.y + B.y), -M.g * (A.z + B.z)};
    o.f2[1] = V3{M.g * (A.x + B.x), M.g * (A.y + B.y), M.g * (A.z + B.z)};
  }
  // twisting (func.cpp:1137-1159)
  {
    double al_b, be_b, ga_b, ph_b, ga_n;
    V3 bo, cO;
    if (M.type[i] == 0) {
      al_b = al[i - 1]; be_b = be[i - 1]; ga_b = ga[i - 1]; ph_b = M.phi_o[i - 1]; ga_n = ga[i - 1];
      bo = bi; cO = ci;
    } else {
      al_b = al[i]; be_b = X.beta_p[ic]; ga_b = ga[i]; ph_b = M.phi_o[i]; ga_n = X.gamma_p[ic];
      bo = ld3(X.b_dna + 3 * ic); cO = ld3(X.c_dna + 3 * ic);
    }
    double alpha = al[i], beta = be[i], gamma = ga[i], phi = M.phi_o[i], len = X.length[i];
    o.E = o.E + M.s * ((alpha + gamma - phi) * (alpha + gamma - phi)) / 2;
    double g1 = (alpha + gamma - phi) * tan(0.5 * beta) / len;
    double c1 = cos(alpha), s1 = sin(alpha);
    double g2 = (al_b + ga_b - ph_b) * tan(0.5 * be_b) / len;
    double c2 = cos(ga_n), s2 = sin(ga_n);
    V3 Ch{g1 * (c1 * cO.x - s1 * bo.x), g1 * (c1 * cO.y - s1 * bo.y), g1 * (c1 * cO.z - s1 * bo.z)};
    V3 Zh{g2 * (c2 * cO.x + s2 * bo.x), g2 * (c2 * cO.y + s2 * bo.y), g2 * (c2 * cO.z + s2 * bo.z)};
    o.f1[2] = V3{M.s * (Ch.x + Zh.x), M.s * (Ch.y + Zh.y), M.s * (Ch.z + Zh.z)};
    o.f2[2] = V3{-M.s * (Ch.x + Zh.x), -M.s * (Ch.y + Zh.y), -M.s * (Ch.z + Zh.z)};
  }
  for (int q = 0; q < 3; q++) {
    o.t1[q] = torque_abs(o.f1[q], rs, ri, ai, bi, ci);
    o.t2[q] = torque_abs(o.f2[q], rf, rj, aj, bj, cj);
  }
}

// Mechanical torque of bead i (func.cpp:1185-1277); T holds the bonded
// force torques on entry.
__device__ V3 mech_torque(const DevModel& M, const DevState& X, int i, V3 T) {
  const double si = sin(kTheta), co = cos(kTheta);
  const double s = M.s, g = M.g;
  const double* al = X.alpha;
  const double* be = X.beta;
  const double* ga = X.gamma;
  const double* ph = M.phi_o;
  int im1 = i - 1;
  if (M.type[i] == 0) {
    return V3{s * (al[i] + ga[i] + ph[i] - al[im1] - ga[im1] - ph[im1]), 0.0, 0.0};
  }
  int ic = M.core_rank[i];
  V3 a = ld3(X.a + 3 * i), b = ld3(X.b + 3 * i), c = ld3(X.c + 3 * i);
  V3 ad = ld3(X.a_dna + 3 * ic), bd = ld3(X.b_dna + 3 * ic), cd = ld3(X.c_dna + 3 * ic);
  double ada = ad.x * a.x + ad.y * a.y + ad.z * a.z;
  double adb = ad.x * b.x + ad.y * b.y + ad.z * b.z;
  double adc = ad.x * c.x + ad.y * c.y + ad.z * c.z;
  double mag = s * (al[i] + ga[i] - ph[i]);
  T.x = T.x + mag * ada; T.y = T.y + mag * adb; T.z = T.z + mag * adc;
  if (i > 0) {
    mag = -s * (al[im1] + ga[im1] - ph[im1]);
    T.x = T.x + mag * co; T.y = T.y + mag * si; T.z = T.z + 0.0;
  }
  double bp = X.beta_p[ic];
  T.y = T.y - g * bp * adc / sin(bp);
  T.z = T.z + g * bp * adb / sin(bp);
  if (i > 0) {
    V3 ab = ld3(X.a + 3 * i - 3);
    ada = ab.x * a.x + ab.y * a.y + ab.z * a.z;
    adb = ab.x * b.x + ab.y * b.y + ab.z * b.z;
    adc = ab.x * c.x + ab.y * c.y + ab.z * c.z;
    T.x = T.x + g * be[im1] * (si * adc) / sin(be[im1]);
    T.y = T.y - g * be[im1] * (co * adc) / sin(be[im1]);
    T.z = T.z + g * be[im1] * (co * adb - si * ada) / sin(be[im1]);
  }
  double s1 = sin(X.alpha_p[ic]), c1 = cos(X.alpha_p[ic]);
  mag = s * (al[i] + ga[i] - ph[i]) * tan(0.5 * bp);
  double cda = cd.x * a.x + cd.y * a.y + cd.z * a.z;
  double bda = bd.x * a.x + bd.y * a.y + bd.z * a.z;
  double cdb = cd.x * b.x + cd.y * b.y + cd.z * b.z;
  double bdb = bd.x * b.x + bd.y * b.y + bd.z * b.z;
  double cdc = cd.x * c.x + cd.y * c.y + cd.z * c.z;
  double bdc = bd.x * c.x + bd.y * c.y + bd.z * c.z;
  T.x = T.x - mag * (s1 * cda + c1 * bda);
  T.y = T.y - mag * (s1 * cdb + c1 * bdb);
  T.z = T.z - mag * (s1 * cdc + c1 * bdc);
  if (i > 0) {
    s1 = sin(ga[im1]);
    c1 = cos(ga[im1]);
    mag = s * (al[im1] + ga[im1] - ph[im1]) * tan(0.5 * be[im1]);
    T.x = T.x - mag * (s1 * 0.0 - c1 * (-si));
    T.y = T.y - mag * (s1 * 0.0 - c1 * co);
    T.z = T.z - mag * (s1 * 1.0 - c1 * 0.0);
  }
  return T;
}

// Thread per chain bead: bonded forces and torques in the reference's
// accumulation order; energy of bond j on thread j.
// Bonded terms of each chain bond i (beads i, i+1), one thread per bond: the
// FP64 work of every bond done once (each bead used to evaluate both of its
// bonds).  Stored per bond: f1, f2, t1, t2 (3 V3 each), E.
constexpr int kBondDoubles = 37;
__global__ void k_chain_bonds(DevModel M, DevState X, double* B) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M.n - 1) return;
  BondOut o;
  bond_terms(M, X, i, o);
  double* b = B + (size_t)kBondDoubles * i;
  for (int q = 0; q < 3; q++) {
    st3(b + 3 * q, o.f1[q]);
    st3(b + 9 + 3 * q, o.f2[q]);
    st3(b + 18 + 3 * q, o.t1[q]);
    st3(b + 27 + 3 * q, o.t2[q]);
  }
  b[36] = o.E;
}

// Per chain bead j: the terms of bonds j-1 and j summed in the order of the
// reference's loop, then the mechanical torque.
__global__ void k_chain_bonded(DevModel M, DevState X, const double* __restrict__ B, double* Fm, double* Tm,
                               double* Ech) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M.n) return;
  V3 F{0.0, 0.0, 0.0}, T{0.0, 0.0, 0.0};
  const bool has_lo = j >= 1, has_hi = j <= M.n - 2;
  const double* lo = B + (size_t)kBondDoubles * (j - 1);  // bond j-1: f2, t2 act on bead j
  const double* hi = B + (size_t)kBondDoubles * j;        // bond j: f1, t1
  for (int q = 0; q < 3; q++) {
    if (has_lo) { acc(F, ld3(lo + 9 + 3 * q)); }
    if (has_hi) { acc(F, ld3(hi + 3 * q)); }
  }
  for (int q = 0; q < 3; q++) {
    if (has_lo) acc(T, ld3(lo + 27 + 3 * q));
    if (has_hi) acc(T, ld3(hi + 18 + 3 * q));
  }
  if (j <= M.n - 2) {
    T = mech_torque(M, X, j, T);
  } else {
    // func.cpp:1281-1287
    T = V3{-M.s * (X.alpha[M.n - 2] + X.gamma[M.n - 2] - M.phi_o[M.n - 2]), 0.0, 0.0};
  }
  st3(Fm + 3 * j, F);
  st3(Tm + 3 * j, T);
  Ech[j] = has_hi ? hi[36] : 0.0;
}

// ------------------------------------------------------------ charge sets
// Core/core (func.cpp:1489-1566), FP64 path: kCCSplit CTAs per core pair
// I < J (mixed contexts: k_core_core_mx below, split the same way).
constexpr int kCCThreads = 256;

__global__ void __launch_bounds__(kCCThreads) k_core_core(DevModel M, DevState X, double* slots) {
  extern __shared__ double sm[];
  int I = blockIdx.x, J = blockIdx.y;
  // gridDim.z CTAs share the pair, each its own interleaved share of the
  // charge pairs and its own slot (summed by k_cc_sum)
  double* out = slots + (((size_t)blockIdx.z * M.n_c + I) * M.n_c + J) * 10;
  if (I >= J) return;
  int i = M.core_bead[I], j = M.core_bead[J];
  V3 ri = ld3(X.r + 3 * i), rj = ld3(X.r + 3 * j);
  double d0 = sqrt((rj.x - ri.x) * (rj.x - ri.x) + (rj.y - ri.y) * (rj.y - ri.y) + (rj.z - ri.z) * (rj.z - ri.z));
  bool ok = !(d0 > 25.0) && chain_ok(M, i) && chain_ok(M, j);
  if (!ok) {
    if (threadIdx.x < 10) out[threadIdx.x] = 0.0;
    return;
  }
  const int Nq = M.Nq;
  double* si_ = sm;            // [3 Nq] sites of I
  double* sj_ = sm + 3 * Nq;   // [3 Nq] sites of J
  double* red = sm + 6 * Nq;   // [32*10]
  V3 ai = ld3(X.a + 3 * i), bi = ld3(X.b + 3 * i), ci = ld3(X.c + 3 * i);
  V3 aj = ld3(X.a + 3 * j), bj = ld3(X.b + 3 * j), cj = ld3(X.c + 3 * j);
  for (int k = threadIdx.x; k < Nq; k += blockDim.x) {
    st3(si_ + 3 * k, body(ri, ai, bi, ci, M.core_pos + 3 * k));
    st3(sj_ + 3 * k, body(rj, aj, bj, cj, M.core_pos + 3 * k));
  }
  __syncthreads();
  const double* cp = M.core_pos;
  const double* cq = M.core_q;
  const double ke = M.k_e, kap = M.debye, kex = M.k_ex, sg = M.sCC;
  double v[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  {
  for (int p = blockIdx.z * blockDim.x + threadIdx.x; p < Nq * Nq; p += blockDim.x * gridDim.z) {
      int k = p / Nq, l = p - k * Nq;
      V3 pk = ld3(si_ + 3 * k), pl = ld3(sj_ + 3 * l);
      V3 z{pk.x - pl.x, pk.y - pl.y, pk.z - pl.z};
      double dd = sqrt(z.x * z.x + z.y * z.y + z.z * z.z);
      double mi = 1.0 / dd;
      z = V3{mi * z.x, mi * z.y, mi * z.z};
      double ex = exp(-kap * dd);
      double g1 = ke * cq[k] * cq[l] * ex * (kap * dd + 1.0) / (dd * dd);
      v[9] = v[9] + (ke * cq[l] * cq[k] / dd) * ex;
      double gsum[2] = {g1, 0.0};
      int ng = 1;
      if (dd <= 8.0) {
        gsum[1] = kex * ((12.0 / sg) * pow((sg / dd), 13) - (6.0 / sg) * pow((sg / dd), 7));
        v[9] = v[9] + kex * (pow(sg / dd, 12) - pow(sg / dd, 6));
        ng = 2;
      }
      for (int q = 0; q < ng; q++) {
        double gg = gsum[q];
        v[0] = v[0] + gg * z.x; v[1] = v[1] + gg * z.y; v[2] = v[2] + gg * z.z;
        double fa = gg * (ai.x * z.x + ai.y * z.y + ai.z * z.z);
        double fb = gg * (bi.x * z.x + bi.y * z.y + bi.z * z.z);
        double fc = gg * (ci.x * z.x + ci.y * z.y + ci.z * z.z);
        v[3] = v[3] + (fc * cp[3 * k + 1] - fb * cp[3 * k + 2]);
        v[4] = v[4] + (fa * cp[3 * k + 2] - fc * cp[3 * k]);
        v[5] = v[5] + (fb * cp[3 * k] - fa * cp[3 * k + 1]);
        fa = -gg * (aj.x * z.x + aj.y * z.y + aj.z * z.z);
        fb = -gg * (bj.x * z.x + bj.y * z.y + bj.z * z.z);
        fc = -gg * (cj.x * z.x + cj.y * z.y + cj.z * z.z);
        v[6] = v[6] + (fc * cp[3 * l + 1] - fb * cp[3 * l + 2]);
        v[7] = v[7] + (fa * cp[3 * l + 2] - fc * cp[3 * l]);
        v[8] = v[8] + (fb * cp[3 * l] - fa * cp[3 * l + 1]);
      }
    }
  }
  bsum<10>(v, red);
  if (threadIdx.x == 0)
    for (int q = 0; q < 10; q++) out[q] = v[q];
}

// the FP64 core/core slots: the kCCSplit partials of each pair I < J, summed in order
__global__ void k_cc_sum(int nc, const double* __restrict__ part, double* __restrict__ slots) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nc * nc * 10) return;
  const int pr = e / 10, I = pr / nc, J = pr - I * nc;
  if (I >= J) return;
  double s = 0.0;
  for (int z = 0; z < kCCSplit; z++) s += part[(size_t)z * nc * nc * 10 + e];
  slots[e] = s;
}

// Core/core, mixed path: the same slot (force on I, body-frame torques on I
// and J, energy) with no FP64 arithmetic per charge pair.  Sites are set up
// once per CTA in FP64 and stored in FP32 relative to the midpoint of the
// two cores (|s| <= ~20 nm, so the FP32 separation carries ~1e-6 relative
// error at 1 nm); the torques are summed in the world frame as
// lever x f (lever = R cp) and turned into the body frame once at the end
// (R^T (lever x f) = cp x (R^T f), the reference's form); sums are FP32 over
// 32 pairs, then FP64.
constexpr int kCCFlush = 32;

__global__ void __launch_bounds__(kCCThreads) k_core_core_mx(DevModel M, DevState X, DevScratch S, double* slots) {
  extern __shared__ double sm[];
  const int I = blockIdx.x, J = blockIdx.y;
  // gridDim.z CTAs share the pair (interleaved sites k of core I), each
  // with its own slot, summed in order by k_cc_sum
  double* out = slots + (((size_t)blockIdx.z * M.n_c + I) * M.n_c + J) * 10;
  if (I >= J) return;
  const int i = M.core_bead[I], j = M.core_bead[J];
  // far-pair test and the centre offset in FP32, from the double-float mirror
  const float3 oij = sepf(ldpf(S, i), ldpf(S, j));  // r_i - r_j
  if (oij.x * oij.x + oij.y * oij.y + oij.z * oij.z > 625.f || !chain_ok(M, i) || !chain_ok(M, j)) {
    if (threadIdx.x < 10) out[threadIdx.x] = 0.0;
    return;
  }
  const int Nq = M.Nq;
  // SoA: site (x, y, z), lever (x, y, z), charge; I then J
  float* f = reinterpret_cast<float*>(sm);
  float *sIx = f, *sIy = f + Nq, *sIz = f + 2 * Nq, *lIx = f + 3 * Nq, *lIy = f + 4 * Nq, *lIz = f + 5 * Nq,
        *qI = f + 6 * Nq;
  float *sJx = f + 7 * Nq, *sJy = f + 8 * Nq, *sJz = f + 9 * Nq, *lJx = f + 10 * Nq, *lJy = f + 11 * Nq,
        *lJz = f + 12 * Nq, *qJ = f + 13 * Nq;
  double* red = sm + (14 * Nq + 1) / 2;
  const V3 ai = ld3(X.a + 3 * i), bi = ld3(X.b + 3 * i), ci = ld3(X.c + 3 * i);
  const V3 aj = ld3(X.a + 3 * j), bj = ld3(X.b + 3 * j), cj = ld3(X.c + 3 * j);
  // sites relative to the pair's midpoint, in FP32: the centre offset from
  // the mirror, the frames converted once, the lever arms in FP32 (no FP64
  // per site)
  const float oix = 0.5f * oij.x, oiy = 0.5f * oij.y, oiz = 0.5f * oij.z;
  const float aix = (float)ai.x, aiy = (float)ai.y, aiz = (float)ai.z, bix = (float)bi.x, biy = (float)bi.y,
              biz = (float)bi.z, cix = (float)ci.x, ciy = (float)ci.y, ciz = (float)ci.z;
  const float ajx = (float)aj.x, ajy = (float)aj.y, ajz = (float)aj.z, bjx = (float)bj.x, bjy = (float)bj.y,
              bjz = (float)bj.z, cjx = (float)cj.x, cjy = (float)cj.y, cjz = (float)cj.z;
  const float kef = (float)M.k_e;
  for (int k = threadIdx.x; k < Nq; k += blockDim.x) {
    const float p0 = M.core_pf[3 * k], p1 = M.core_pf[3 * k + 1], p2 = M.core_pf[3 * k + 2];
    const float lix = aix * p0 + bix * p1 + cix * p2, liy = aiy * p0 + biy * p1 + ciy * p2,
                liz = aiz * p0 + biz * p1 + ciz * p2;
    const float ljx = ajx * p0 + bjx * p1 + cjx * p2, ljy = ajy * p0 + bjy * p1 + cjy * p2,
                ljz = ajz * p0 + bjz * p1 + cjz * p2;
    sIx[k] = oix + lix; sIy[k] = oiy + liy; sIz[k] = oiz + liz;
    sJx[k] = ljx - oix; sJy[k] = ljy - oiy; sJz[k] = ljz - oiz;
    lIx[k] = lix; lIy[k] = liy; lIz[k] = liz;
    lJx[k] = ljx; lJy[k] = ljy; lJz[k] = ljz;
    qI[k] = kef * M.core_qf[k];
    qJ[k] = M.core_qf[k];
  }
  __syncthreads();
  const float kap = (float)M.debye, kex = (float)M.k_ex, sg = (float)M.sCC;
  // runs of kCCFlush terms in FP32, the runs added with Kahan compensation
  float a[10], ks[10], kc[10];
#pragma unroll
  for (int q = 0; q < 10; q++) a[q] = 0.f, ks[q] = 0.f, kc[q] = 0.f;
  int cnt = 0;
  // warp w takes sites k = w, w + nw, ... of core I against all sites l of
  // core J (lanes); the force and torque on I are summed per k first
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int k = (threadIdx.x >> 5) + nw * blockIdx.z; k < Nq; k += nw * gridDim.z) {
    const float sx = sIx[k], sy = sIy[k], sz = sIz[k], qk = qI[k];
    float fkx = 0.f, fky = 0.f, fkz = 0.f;
    for (int l = lane; l < Nq; l += 32) {
      const float zx = sx - sJx[l], zy = sy - sJy[l], zz = sz - sJz[l];
      const float ssq = fmaf(zx, zx, fmaf(zy, zy, zz * zz));
      const float rinv = rsqrtf(ssq);
      const float dd = ssq * rinv;
      const float ex = expf(-kap * dd);
      float e = qk * qJ[l] * ex * rinv;             // k_e q_k q_l e^{-kappa d} / d
      float g = e * fmaf(kap, dd, 1.f) * rinv;      // ... (kappa d + 1) / d^2
      if (dd <= 8.f) {
        const float sr = sg * rinv, sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
        g = fmaf(kex * (12.f * sr12 - 6.f * sr6), rinv, g);
        e = fmaf(kex, sr12 - sr6, e);
      }
      const float gz = g * rinv;
      const float fx = gz * zx, fy = gz * zy, fz = gz * zz;
      fkx += fx; fky += fy; fkz += fz;
      a[6] = fmaf(-lJy[l], fz, fmaf(lJz[l], fy, a[6]));
      a[7] = fmaf(-lJz[l], fx, fmaf(lJx[l], fz, a[7]));
      a[8] = fmaf(-lJx[l], fy, fmaf(lJy[l], fx, a[8]));
      a[9] += e;
      if (++cnt == kCCFlush) {
#pragma unroll
        for (int q = 0; q < 10; q++) {
          const float y = a[q] - kc[q], t = ks[q] + y;
          kc[q] = (t - ks[q]) - y;
          ks[q] = t;
          a[q] = 0.f;
        }
        cnt = 0;
      }
    }
    a[0] += fkx; a[1] += fky; a[2] += fkz;
    a[3] = fmaf(lIy[k], fkz, fmaf(-lIz[k], fky, a[3]));
    a[4] = fmaf(lIz[k], fkx, fmaf(-lIx[k], fkz, a[4]));
    a[5] = fmaf(lIx[k], fky, fmaf(-lIy[k], fkx, a[5]));
  }
  float vh[10], vl[10];
#pragma unroll
  for (int q = 0; q < 10; q++) {
    const float y = a[q] - kc[q], t = ks[q] + y;
    vh[q] = t;
    vl[q] = -((t - ks[q]) - y);
  }
  double v[10];
  bsum_df<10>(vh, vl, v, red);
  if (threadIdx.x == 0) {
    out[0] = v[0]; out[1] = v[1]; out[2] = v[2];
    out[3] = ai.x * v[3] + ai.y * v[4] + ai.z * v[5];
    out[4] = bi.x * v[3] + bi.y * v[4] + bi.z * v[5];
    out[5] = ci.x * v[3] + ci.y * v[4] + ci.z * v[5];
    out[6] = aj.x * v[6] + aj.y * v[7] + aj.z * v[8];
    out[7] = bj.x * v[6] + bj.y * v[7] + bj.z * v[8];
    out[8] = cj.x * v[6] + cj.y * v[7] + cj.z * v[8];
    out[9] = v[9];
  }
}

// DNA/core (func.cpp:1355-1488): one warp per (linker bead d, core J).
// Slot: force on the DNA bead (3), torque on the core (3), energy.
template <bool MX>
__global__ void k_dna_core(DevModel M, DevState X, DevScratch S, double* slots) {
  int lane = threadIdx.x & 31;
  int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= M.n_dna * M.n_c) return;
  int D = w / M.n_c, J = w - D * M.n_c;
  double* out = slots + (size_t)w * 7;
  int i = M.dna_bead[D], j = M.core_bead[J];
  V3 rd_ = ld3(X.r + 3 * i), rc = ld3(X.r + 3 * j);
  bool ok;
  if constexpr (MX) {  // far-pair test in FP32 from the double-float mirror
    const float3 z = sepf(ldpf(S, i), ldpf(S, j));
    ok = !(z.x * z.x + z.y * z.y + z.z * z.z > 625.f) && chain_ok(M, i) && chain_ok(M, j);
  } else {
    int lo = i < j ? i : j, hi = i < j ? j : i;
    V3 rl = ld3(X.r + 3 * lo), rh = ld3(X.r + 3 * hi);
    double d0 = sqrt((rh.x - rl.x) * (rh.x - rl.x) + (rh.y - rl.y) * (rh.y - rl.y) + (rh.z - rl.z) * (rh.z - rl.z));
    ok = !(d0 > 25.0) && chain_ok(M, i) && chain_ok(M, j);
  }
  if (!ok) {
    if (lane < 7) out[lane] = 0.0;
    return;
  }
  bool adj = abs(i - j) > 1;
  V3 ac = ld3(X.a + 3 * j), bc = ld3(X.b + 3 * j), cc = ld3(X.c + 3 * j);
  const double* cp = M.core_pos;
  const double ke = M.k_e, kap = M.debye, kex = M.k_ex, sg = M.sDC, ql = M.q_l;
  double v[7] = {0, 0, 0, 0, 0, 0, 0};
  if constexpr (MX) {
    // FP32: the core centre relative to the DNA bead once in FP64, the site
    // lever arms from the FP32 core sites and frames; ~Nq / 32 terms per lane
    const float kapf = (float)kap, kexf = (float)kex, sgf = (float)sg, qlk = (float)(ke * ql);
    const float acx = (float)ac.x, acy = (float)ac.y, acz = (float)ac.z, bcx = (float)bc.x, bcy = (float)bc.y,
                bcz = (float)bc.z, ccx = (float)cc.x, ccy = (float)cc.y, ccz = (float)cc.z;
    const float3 o = sepf(ldpf(S, j), ldpf(S, i));  // core centre relative to the DNA bead
    const float ox = o.x, oy = o.y, oz = o.z;
    float a[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int k = lane; k < M.Nq; k += 32) {
      const float c0 = M.core_pf[3 * k], c1 = M.core_pf[3 * k + 1], c2 = M.core_pf[3 * k + 2];
      float zx = -(ox + (acx * c0 + bcx * c1 + ccx * c2));
      float zy = -(oy + (acy * c0 + bcy * c1 + ccy * c2));
      float zz = -(oz + (acz * c0 + bcz * c1 + ccz * c2));
      float dd = sqrtf(zx * zx + zy * zy + zz * zz);
      float mi = 1.f / dd;
      zx *= mi; zy *= mi; zz *= mi;
      const float q = M.core_qf[k];
      float g = 0.f, e = 0.f;
      if (adj) {
        float ex = expf(-kapf * dd);
        float qq = qlk * q;
        g = qq * ex * (kapf * dd + 1.f) / (dd * dd);
        e = qq * ex / dd;
      }
      if (dd <= 8.f && q > 0.f) {
        float sr = sgf / dd, sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
        g += kexf * (12.f * sr12 - 6.f * sr6) / dd;
        e += kexf * (sr12 - sr6);
      }
      a[6] += e;
      a[0] += g * zx; a[1] += g * zy; a[2] += g * zz;
      float fa = -g * (acx * zx + acy * zy + acz * zz), fb = -g * (bcx * zx + bcy * zy + bcz * zz),
            fc = -g * (ccx * zx + ccy * zy + ccz * zz);
      a[3] += fc * c1 - fb * c2; a[4] += fa * c2 - fc * c0; a[5] += fb * c0 - fa * c1;
    }
    for (int q = 0; q < 7; q++) v[q] = (double)a[q];
  } else {
  for (int k = lane; k < M.Nq; k += 32) {
      V3 s = body(rc, ac, bc, cc, cp + 3 * k);
      V3 z{rd_.x - s.x, rd_.y - s.y, rd_.z - s.z};
      double dd = sqrt(z.x * z.x + z.y * z.y + z.z * z.z);
      double mi = 1.0 / dd;
      z = V3{mi * z.x, mi * z.y, mi * z.z};
      double q = M.core_q[k];
      double gs[2];
      int ng = 0;
      if (adj) {
        double ex = exp(-kap * dd);
        gs[ng++] = ke * ql * q * ex * (kap * dd + 1.0) / (dd * dd);
        v[6] = v[6] + (ke * ql * q / dd) * ex;
      }
      if (dd <= 8.0 && q > 0) {
        gs[ng++] = kex * ((12.0 / sg) * pow((sg / dd), 13) - (6.0 / sg) * pow((sg / dd), 7));
        v[6] = v[6] + kex * (pow(sg / dd, 12) - pow(sg / dd, 6));
      }
      for (int t = 0; t < ng; t++) {
        double g1 = gs[t];
        v[0] = v[0] + g1 * z.x; v[1] = v[1] + g1 * z.y; v[2] = v[2] + g1 * z.z;
        double fa = -g1 * (ac.x * z.x + ac.y * z.y + ac.z * z.z);
        double fb = -g1 * (bc.x * z.x + bc.y * z.y + bc.z * z.z);
        double fc = -g1 * (cc.x * z.x + cc.y * z.y + cc.z * z.z);
        v[3] = v[3] + (fc * cp[3 * k + 1] - fb * cp[3 * k + 2]);
        v[4] = v[4] + (fa * cp[3 * k + 2] - fc * cp[3 * k]);
        v[5] = v[5] + (fb * cp[3 * k] - fa * cp[3 * k + 1]);
      }
    }
  }
  for (int q = 0; q < 7; q++) v[q] = wsum(v[q]);
  if (lane == 0)
    for (int q = 0; q < 7; q++) out[q] = v[q];
}

// Globular head of LH core I against the charges of core L != I
// (func.cpp:2524-2586): one warp per (I, L).  Slot: force on I (3), torque
// on I (3), torque on L (3), energy.  Pairs beyond the 7 nm cut-off add
// exact zeros, so far object pairs are skipped.
template <bool MX>
__global__ void k_ghead_core(DevModel M, DevState X, double* slots) {
  int lane = threadIdx.x & 31;
  int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= M.n_lhcore * M.n_c) return;
  int I = w / M.n_c, L = w - I * M.n_c;
  double* out = slots + (size_t)w * 10;
  int i = M.lh_core_bead[I], l = M.core_bead[L];
  V3 ri = ld3(X.r + 3 * i), rl = ld3(X.r + 3 * l);
  double d0 = dist3(ri, rl);
  if (i == l || d0 > 7.0 + M.gmax + M.qmax_core + 1e-6) {
    if (lane < 10) out[lane] = 0.0;
    return;
  }
  V3 ai = ld3(X.a + 3 * i), bi = ld3(X.b + 3 * i), ci = ld3(X.c + 3 * i);
  V3 al = ld3(X.a + 3 * l), bl = ld3(X.b + 3 * l), cl = ld3(X.c + 3 * l);
  const double eps = eps_of(M);
  double v[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  const int ng = M.n_lh_g, Nq = M.Nq;
  for (int p = lane; p < ng * Nq; p += 32) {
    int jm = p / Nq, m = p - jm * Nq;
    V3 g = ld3(X.gpos + 3 * (I * ng + jm));
    V3 z = body(rl, al, bl, cl, M.core_pos + 3 * m);
    V3 f1 = pairF<true, true, MX>(M.LH_q[jm], M.core_q[m], eps, M.debye, M.k_ex, M.LH_vdw_hc[jm], g, z, &v[9]);
    V3 f2{-f1.x, -f1.y, -f1.z};
    v[0] = v[0] + f1.x; v[1] = v[1] + f1.y; v[2] = v[2] + f1.z;
    V3 t1 = torque_rel(f1, M.LH_g_pos + 3 * jm, ai, bi, ci);
    V3 t2 = torque_rel(f2, M.core_pos + 3 * m, al, bl, cl);
    v[3] = v[3] + t1.x; v[4] = v[4] + t1.y; v[5] = v[5] + t1.z;
    v[6] = v[6] + t2.x; v[7] = v[7] + t2.y; v[8] = v[8] + t2.z;
  }
  for (int q = 0; q < 10; q++) v[q] = wsum(v[q]);
  if (lane == 0)
    for (int q = 0; q < 10; q++) out[q] = v[q];
}

// ------------------------------------------------------------ chain gather
// One CTA per chain bead: every remaining contribution to its force and
// torque, plus the slot reductions; writes the bead's final F, T and its
// energy share.
// Block sum of a chain bead's pair terms, then the slot reductions in a
// fixed order and the bonded terms; thread 0 stores.
__device__ void chain_finish(const DevModel& M, const DevScratch& S, const double* Fm, const double* Tm,
                             const double* Ech, DevForces& out, double* Eout, int j, V3 F, V3 T, double E,
                             double* red) {
  const bool dna = M.type[j] == 0;
  double v[7] = {F.x, F.y, F.z, T.x, T.y, T.z, E};
  bsum<7>(v, red);
  if (threadIdx.x != 0) return;
  F = V3{v[0], v[1], v[2]};
  T = V3{v[3], v[4], v[5]};
  E = v[6];
  // slot reductions, fixed order
  if (dna) {
    const int D = j - M.core_rank[j] - 1;  // linker beads before j
    for (int J = 0; J < M.n_c; J++) {
      const double* s = S.dc + ((size_t)D * M.n_c + J) * 7;
      F.x = F.x + s[0]; F.y = F.y + s[1]; F.z = F.z + s[2];
    }
  } else {
    const int J = M.core_rank[j];
    for (int K = 0; K < M.n_c; K++) {
      if (K < J) {
        const double* s = S.cc + ((size_t)K * M.n_c + J) * 10;
        F.x = F.x - s[0]; F.y = F.y - s[1]; F.z = F.z - s[2];
        T.x = T.x + s[6]; T.y = T.y + s[7]; T.z = T.z + s[8];
      } else if (K > J) {
        const double* s = S.cc + ((size_t)J * M.n_c + K) * 10;
        F.x = F.x + s[0]; F.y = F.y + s[1]; F.z = F.z + s[2];
        T.x = T.x + s[3]; T.y = T.y + s[4]; T.z = T.z + s[5];
        E = E + s[9];
      }
    }
    for (int D = 0; D < M.n_dna; D++) {
      const double* s = S.dc + ((size_t)D * M.n_c + J) * 7;
      F.x = F.x - s[0]; F.y = F.y - s[1]; F.z = F.z - s[2];
      T.x = T.x + s[3]; T.y = T.y + s[4]; T.z = T.z + s[5];
      E = E + s[6];
    }
    const int lc = M.core_lh[J];
    for (int I = 0; I < M.n_lhcore; I++) {
      const double* s = S.gc + ((size_t)I * M.n_c + J) * 10;
      F.x = F.x - s[0]; F.y = F.y - s[1]; F.z = F.z - s[2];
      T.x = T.x + s[6]; T.y = T.y + s[7]; T.z = T.z + s[8];
    }
    if (lc >= 0) {
      for (int L = 0; L < M.n_c; L++) {
        const double* s = S.gc + ((size_t)lc * M.n_c + L) * 10;
        F.x = F.x + s[0]; F.y = F.y + s[1]; F.z = F.z + s[2];
        T.x = T.x + s[3]; T.y = T.y + s[4]; T.z = T.z + s[5];
        E = E + s[9];
      }
    }
  }
  V3 Fb = ld3(Fm + 3 * j), Tb = ld3(Tm + 3 * j);
  st3(out.F + 3 * j, V3{Fb.x + F.x, Fb.y + F.y, Fb.z + F.z});
  st3(out.T + 3 * j, V3{Tb.x + T.x, Tb.y + T.y, Tb.z + T.z});
  Eout[j] = Ech[j] + E;
}

// Mixed path: chain_finish with the slot sums spread over the CTA's threads
// (FP64, many lanes per instruction instead of one thread walking every
// slot) and folded into the block sum; same terms, another summation order.
__device__ void chain_finish_mx(const DevModel& M, const DevScratch& S, const double* Fm, const double* Tm,
                                const double* Ech, DevForces& out, double* Eout, int j, V3 F, V3 T, double E,
                                double* red) {
  const int tid = threadIdx.x, nt = blockDim.x;
  if (M.type[j] == 0) {
    const int D = j - M.core_rank[j] - 1;  // linker beads before j
    for (int J = tid; J < M.n_c; J += nt) {
      const double* s = S.dc + ((size_t)D * M.n_c + J) * 7;
      F.x = F.x + s[0]; F.y = F.y + s[1]; F.z = F.z + s[2];
    }
  } else {
    const int J = M.core_rank[j];
    for (int K = tid; K < M.n_c; K += nt) {
      if (K < J) {
        const double* s = S.cc + ((size_t)K * M.n_c + J) * 10;
        F.x = F.x - s[0]; F.y = F.y - s[1]; F.z = F.z - s[2];
        T.x = T.x + s[6]; T.y = T.y + s[7]; T.z = T.z + s[8];
      } else if (K > J) {
        const double* s = S.cc + ((size_t)J * M.n_c + K) * 10;
        F.x = F.x + s[0]; F.y = F.y + s[1]; F.z = F.z + s[2];
        T.x = T.x + s[3]; T.y = T.y + s[4]; T.z = T.z + s[5];
        E = E + s[9];
      }
    }
    for (int D = tid; D < M.n_dna; D += nt) {
      const double* s = S.dc + ((size_t)D * M.n_c + J) * 7;
      F.x = F.x - s[0]; F.y = F.y - s[1]; F.z = F.z - s[2];
      T.x = T.x + s[3]; T.y = T.y + s[4]; T.z = T.z + s[5];
      E = E + s[6];
    }
    for (int I = tid; I < M.n_lhcore; I += nt) {
      const double* s = S.gc + ((size_t)I * M.n_c + J) * 10;
      F.x = F.x - s[0]; F.y = F.y - s[1]; F.z = F.z - s[2];
      T.x = T.x + s[6]; T.y = T.y + s[7]; T.z = T.z + s[8];
    }
    const int lc = M.core_lh[J];
    if (lc >= 0) {
      for (int L = tid; L < M.n_c; L += nt) {
        const double* s = S.gc + ((size_t)lc * M.n_c + L) * 10;
        F.x = F.x + s[0]; F.y = F.y + s[1]; F.z = F.z + s[2];
        T.x = T.x + s[3]; T.y = T.y + s[4]; T.z = T.z + s[5];
        E = E + s[9];
      }
    }
  }
  double v[7] = {F.x, F.y, F.z, T.x, T.y, T.z, E};
  bsum<7>(v, red);
  if (tid != 0) return;
  V3 Fb = ld3(Fm + 3 * j), Tb = ld3(Tm + 3 * j);
  st3(out.F + 3 * j, V3{Fb.x + v[0], Fb.y + v[1], Fb.z + v[2]});
  st3(out.T + 3 * j, V3{Tb.x + v[3], Tb.y + v[4], Tb.z + v[5]});
  Eout[j] = Ech[j] + v[6];
}

constexpr int kGatherThreads = 256;
// FP64 thread-per-bead kernels: few beads per CTA, so that the CTAs spread
// over many SMs (FP64 throughput is per SM)
#ifndef BD_FP64_BEAD_THREADS
#define BD_FP64_BEAD_THREADS 32
#endif
constexpr int kBeadThreads = BD_FP64_BEAD_THREADS;

template <bool MX>
__global__ void __launch_bounds__(kGatherThreads) k_chain_gather(DevModel M, DevState X, const double* Fm,
                                                                const double* Tm, const double* Ech,
                                                                DevScratch S, DevForces out, double* Eout) {
  __shared__ double red[32 * 7];
  const int j = blockIdx.x;
  const int tid = threadIdx.x, nt = blockDim.x;
  const double eps = eps_of(M);
  V3 rj = ld3(X.r + 3 * j), aj = ld3(X.a + 3 * j), bj = ld3(X.b + 3 * j), cj = ld3(X.c + 3 * j);
  V3 F{0.0, 0.0, 0.0}, T{0.0, 0.0, 0.0};
  double E = 0.0;
  const bool dna = M.type[j] == 0;
  if (dna) {
    // DNA/DNA (func.cpp:1326-1354); energy on the lower index
    if (chain_ok(M, j)) {
      double qq = M.q_l * M.q_l;
      for (int i = tid; i < M.n; i += nt) {
        if (i == j || M.type[i] != 0 || abs(i - j) <= 1 || !chain_ok(M, i)) continue;
        V3 ri = ld3(X.r + 3 * i);
        double d = sqrt((rj.x - ri.x) * (rj.x - ri.x) + (rj.y - ri.y) * (rj.y - ri.y) + (rj.z - ri.z) * (rj.z - ri.z));
        if (d > 25.0) continue;
        if constexpr (MX) {
          float zx = (float)(rj.x - ri.x), zy = (float)(rj.y - ri.y), zz = (float)(rj.z - ri.z);
          float df = sqrtf(zx * zx + zy * zy + zz * zz), mi = 1.f / df;
          float kap = (float)M.debyell, ex = expf(-kap * df), qf = (float)(M.k_e * qq);
          float g = qf * ex * (kap * df + 1.f) / (df * df), e = qf * ex / df;
          if (df <= 8.f) {
            float sr = (float)M.sDD / df, sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
            g += (float)M.k_ex * (12.f * sr12 - 6.f * sr6) / df;
            e += (float)M.k_ex * (sr12 - sr6);
          }
          if (j < i) E = E + (double)e;
          F.x += (double)(g * zx * mi); F.y += (double)(g * zy * mi); F.z += (double)(g * zz * mi);
          continue;
        }
        double mi = 1.0 / d;
        V3 z{mi * (rj.x - ri.x), mi * (rj.y - ri.y), mi * (rj.z - ri.z)};
        double g1 = M.k_e * qq * exp(-M.debyell * d) * (M.debyell * d + 1.0) / (d * d);
        double e = (M.k_e * qq / d) * exp(-M.debyell * d);
        if (d <= 8) {
          double s1 = M.sDD;
          g1 = g1 + M.k_ex * ((12.0 / s1) * pow((s1 / d), 13) - (6.0 / s1) * pow((s1 / d), 7));
          e = e + M.k_ex * (pow(s1 / d, 12) - pow(s1 / d, 6));
        }
        if (j < i) E = E + e;
        F.x = F.x + g1 * z.x; F.y = F.y + g1 * z.y; F.z = F.z + g1 * z.z;
      }
    }
    // tails on this DNA bead (func.cpp:1898-1917); energy on the tail side
    for (int t = tid; t < M.n_tail; t += nt)
      acc(F, pairF<true, true, MX>(M.q_l, M.t_q[t], eps, M.debye, M.k_ex, M.sTL, rj, ld3(X.r_t + 3 * t), nullptr));
    // LH beads on this DNA bead (func.cpp:2249-2279); energy on the LH side
    for (int b = tid; b < M.n_LH; b += nt) {
      int p = lh_param(M, b);
      acc(F, pairF<true, true, MX>(M.q_l, M.LH_q[p], eps, M.debye, M.k_ex, M.LH_vdw_hl[p], rj, ld3(X.r_lh + 3 * b), nullptr));
    }
    // globular heads on this DNA bead (func.cpp:2481-2522); energy on the core side
    for (int s = tid; s < M.n_lhcore * M.n_lh_g; s += nt) {
      int m = s % M.n_lh_g;
      acc(F, pairF<true, true, MX>(M.q_l, M.LH_q[m], eps, M.debye, M.k_ex, M.LH_vdw_hl[m], rj, ld3(X.gpos + 3 * s), nullptr));
    }
  } else {
    const int J = M.core_rank[j];
    const int lc = M.core_lh[J];
    if (lc >= 0) {
      const int ng = M.n_lh_g;
      // G-head vs linker DNA, tails, LH beads of other LHs, other G-heads
      for (int s = tid; s < ng * M.n; s += nt) {  // func.cpp:2481-2522
        int m = s / M.n, l = s - m * M.n;
        if (M.type[l] != 0) continue;
        V3 g = ld3(X.gpos + 3 * (lc * ng + m));
        V3 f1 = pairF<true, true, MX>(M.LH_q[m], M.q_l, eps, M.debye, M.k_ex, M.LH_vdw_hl[m], g, ld3(X.r + 3 * l), &E);
        acc(F, f1);
        acc(T, torque_rel(f1, M.LH_g_pos + 3 * m, aj, bj, cj));
      }
      for (int s = tid; s < ng * M.n_tail; s += nt) {  // func.cpp:2403-2476
        int m = s / M.n_tail, t = s - m * M.n_tail;
        V3 g = ld3(X.gpos + 3 * (lc * ng + m));
        V3 f1 = pairF<true, true, MX>(M.LH_q[m], M.t_q[t], eps, M.debye, M.k_ex, M.LH_vdw_ht[m], g, ld3(X.r_t + 3 * t), &E);
        acc(F, f1);
        acc(T, torque_rel(f1, M.LH_g_pos + 3 * m, aj, bj, cj));
      }
      for (int s = tid; s < ng * M.n_LH; s += nt) {  // func.cpp:2590-2644
        int m = s / M.n_LH, b = s - m * M.n_LH;
        if (b / M.nlh == lc) continue;
        int p2 = lh_param(M, b);
        V3 g = ld3(X.gpos + 3 * (lc * ng + m));
        V3 f1 = pairF<true, true, MX>(M.LH_q[m], M.LH_q[p2], eps, M.debye, M.k_ex, (M.LH_vdw_hh[m] + M.LH_vdw_hh[p2]) / 2,
                                    g, ld3(X.r_lh + 3 * b), &E);
        acc(F, f1);
        acc(T, torque_rel(f1, M.LH_g_pos + 3 * m, aj, bj, cj));
      }
      for (int s = tid; s < ng * M.n_lhcore * ng; s += nt) {  // func.cpp:2649-2719; energy on the lower core
        int m = s / (M.n_lhcore * ng), rest = s - m * (M.n_lhcore * ng);
        int K = rest / ng, m1 = rest - K * ng;
        if (K == lc) continue;
        V3 g = ld3(X.gpos + 3 * (lc * ng + m));
        V3 g2 = ld3(X.gpos + 3 * (K * ng + m1));
        double e = 0.0;
        V3 f1 = pairF<true, true, MX>(M.LH_q[m], M.LH_q[m1], eps, M.debye, M.k_ex, (M.LH_vdw_hh[m] + M.LH_vdw_hh[m1]) / 2, g,
                                    g2, &e);
        if (lc < K) E = E + e;
        acc(F, f1);
        acc(T, torque_rel(f1, M.LH_g_pos + 3 * m, aj, bj, cj));
      }
      if (tid == 0) {  // G-head <-> first C-term bead anchor (func.cpp:2725-2777)
        for (int jj = 0; jj < ng; jj++) {
          int pj = jj + M.n_lh_n;
          if (M.LH_conn[pj] != 1) continue;
          V3 g = ld3(X.gpos + 3 * (lc * ng + jj));
          V3 q = ld3(X.r_lh + 3 * (lc * M.nlh));
          double d = sqrt((q.x - g.x) * (q.x - g.x) + (q.y - g.y) * (q.y - g.y) + (q.z - g.z) * (q.z - g.z));
          double kst = M.LH_kstr[pj], eq = M.LH_streq[pj];
          E = E + kst * (d - eq) * (d - eq) / 2;
          V3 st{(d - eq) * (q.x - g.x) / d, (d - eq) * (q.y - g.y) / d, (d - eq) * (q.z - g.z) / d};
          F.x = F.x + kst * st.x * 10; F.y = F.y + kst * st.y * 10; F.z = F.z + kst * st.z * 10;
          double fa = kst * (aj.x * st.x + aj.y * st.y + aj.z * st.z);
          double fb = kst * (bj.x * st.x + bj.y * st.y + bj.z * st.z);
          double fc = kst * (cj.x * st.x + cj.y * st.y + cj.z * st.z);
          const double* gp = M.LH_g_pos + 3 * jj;
          T.x = T.x + fc * gp[1] - fb * gp[2];
          T.y = T.y + fa * gp[2] - fc * gp[0];
          T.z = T.z + fb * gp[0] - fa * gp[1];
        }
      }
    }
    // tail anchors of this core (func.cpp:1971-2022); energy here
    if (M.nc_t_flag[J] == 1) {
      for (int jt = tid; jt < M.n_t; jt += nt) {
        if (M.tail_fix[jt] != 1) continue;
        V3 ro = body(rj, aj, bj, cj, M.tail_pos + 3 * jt);
        int tb = J * M.n_t + jt;
        V3 rt = ld3(X.r_t + 3 * tb);
        V3 st{rt.x - ro.x, rt.y - ro.y, rt.z - ro.z};
        E = E + M.h * (st.x * st.x + st.y * st.y + st.z * st.z) / 2;
        V3 hs{M.h * st.x, M.h * st.y, M.h * st.z};
        acc(F, hs);
        acc(T, torque_rel(hs, M.tail_pos + 3 * jt, aj, bj, cj));
      }
    }
    // LH and G-head forces on this core's anchored tail beads are applied to
    // the core (func.cpp:2361-2391, 2436-2465)
    for (int t0 = 0; t0 < M.n_tail; t0++) {
      if (M.t_fix[t0] == 0 || M.t_core_bead[t0] != j) continue;
      V3 rt = ld3(X.r_t + 3 * t0);
      for (int b = tid; b < M.n_LH; b += nt) {
        int p = lh_param(M, b);
        V3 f2 = pairF<true, true, MX>(M.t_q[t0], M.LH_q[p], eps, M.debye, M.k_ex, M.LH_vdw_ht[p], rt, ld3(X.r_lh + 3 * b), nullptr);
        acc(F, f2);
        acc(T, torque_abs(f2, rt, rj, aj, bj, cj));
      }
      for (int s = tid; s < M.n_lhcore * M.n_lh_g; s += nt) {
        int m = s % M.n_lh_g;
        V3 f2 = pairF<true, true, MX>(M.t_q[t0], M.LH_q[m], eps, M.debye, M.k_ex, M.LH_vdw_ht[m], rt, ld3(X.gpos + 3 * s), nullptr);
        acc(F, f2);
        acc(T, torque_abs(f2, rt, rj, aj, bj, cj));
      }
    }
  }
  chain_finish(M, S, Fm, Tm, Ech, out, Eout, j, F, T, E, red);
}

// ------------------------------------------------------------ tails
// One warp per tail bead (func.cpp:1809-1917, 2343-2476 for the LH side).
template <bool MX>
__global__ void k_tail_gather(DevModel M, DevState X, DevForces out, double* Eout) {
  int lane = threadIdx.x & 31;
  int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (t >= M.n_tail) return;
  const double eps = eps_of(M);
  V3 rt = ld3(X.r_t + 3 * t);
  V3 F{0.0, 0.0, 0.0};
  double E = 0.0;
  const int* grp = M.t_grp;
  const int nt = M.n_tail;
  if (lane == 0) {
    // stretching (func.cpp:1811-1827): bond (t-1,t) then (t,t+1)
    if (t >= 1 && grp[t - 1] == grp[t]) acc(F, stretch_f2(M.h_t[t - 1], ld3(X.r_t + 3 * t - 3), rt, M.lo_t[t - 1]));
    if (t + 1 < nt && grp[t] == grp[t + 1]) acc(F, stretch_f1(M.h_t[t], rt, ld3(X.r_t + 3 * t + 3), M.lo_t[t], E));
    // bending (func.cpp:1832-1858): angles starting at t-2, t-1, t
    for (int s = t - 2; s <= t; s++) {
      if (s < 0 || s + 2 >= nt) continue;
      if (!(grp[s] == grp[s + 1] && grp[s] == grp[s + 2])) continue;
      V3 f1, f2, f3;
      double e = 0.0;
      bend3(M.g_t[s], X.beta_t[s], M.beta_o_t[s], ld3(X.r_t + 3 * s), ld3(X.r_t + 3 * s + 3), ld3(X.r_t + 3 * s + 6), f1,
            f2, f3, e);
      if (s == t) E = E + e;
      dec(F, s == t ? f1 : (s == t - 1 ? f2 : f3));
    }
    // anchor of a fixed template bead (func.cpp:1994-1996); energy on the core
    int J = t / M.n_t, jt = t - J * M.n_t;
    if (M.nc_t_flag[J] == 1 && M.tail_fix[jt] == 1) {
      int cb = M.core_bead[J];
      V3 ro = site(X, cb, M.tail_pos + 3 * jt);
      V3 st{rt.x - ro.x, rt.y - ro.y, rt.z - ro.z};
      F.x = F.x - M.h * st.x; F.y = F.y - M.h * st.y; F.z = F.z - M.h * st.z;
    }
  }
  // tail/tail electrostatics (func.cpp:1863-1891); energy on the lower index
  for (int u = lane; u < nt; u += 32) {
    if (u == t) continue;
    int lo = t < u ? t : u, hi = t < u ? u : t;
    if (!(grp[lo] != grp[hi] || hi > lo + 2)) continue;
    double e = 0.0;
    acc(F, pairF<true, false, MX>(M.t_q[t], M.t_q[u], eps, M.debye, 0.0, 0.0, rt, ld3(X.r_t + 3 * u), &e));
    if (t < u) E = E + e;
  }
  // linker DNA (func.cpp:1898-1917); energy here
  for (int q = lane; q < M.n_dna; q += 32) {
    int j = M.dna_bead[q];
    acc(F, pairF<true, true, MX>(M.t_q[t], M.q_l, eps, M.debye, M.k_ex, M.sTL, rt, ld3(X.r + 3 * j), &E));
  }
  if (M.t_fix[t] == 0) {
    // LH beads and globular heads act on free tail beads (energies on their side)
    for (int b = lane; b < M.n_LH; b += 32) {
      int p = lh_param(M, b);
      acc(F, pairF<true, true, MX>(M.t_q[t], M.LH_q[p], eps, M.debye, M.k_ex, M.LH_vdw_ht[p], rt, ld3(X.r_lh + 3 * b), nullptr));
    }
    for (int s = lane; s < M.n_lhcore * M.n_lh_g; s += 32) {
      int m = s % M.n_lh_g;
      acc(F, pairF<true, true, MX>(M.t_q[t], M.LH_q[m], eps, M.debye, M.k_ex, M.LH_vdw_ht[m], rt, ld3(X.gpos + 3 * s), nullptr));
    }
  }
  F.x = wsum(F.x); F.y = wsum(F.y); F.z = wsum(F.z); E = wsum(E);
  if (lane == 0) {
    st3(out.tF + 3 * t, F);
    Eout[t] = E;
  }
}

// ------------------------------------------------------------ LH beads
// One warp per mobile LH bead (func.cpp:2109-2398, 2588-2644, 2725-2777).
template <bool MX>
__global__ void k_lh_gather(DevModel M, DevState X, DevForces out, double* Eout) {
  int lane = threadIdx.x & 31;
  int bI = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (bI >= M.n_LH) return;
  const double eps = eps_of(M);
  const int nL = M.n_LH, nlh = M.nlh;
  V3 rb = ld3(X.r_lh + 3 * bI);
  const int pb = lh_param(M, bI);
  V3 F{0.0, 0.0, 0.0};
  double E = 0.0;
  if (lane == 0) {
    // stretching: bond (b-1,b) then (b,b+1)
    if (bI >= 1) {
      int p = lh_param(M, bI - 1);
      if (M.LH_conn[p] == 1) acc(F, stretch_f2(M.LH_kstr[p], ld3(X.r_lh + 3 * bI - 3), rb, M.LH_streq[p]));
    }
    if (M.LH_conn[pb] == 1 && bI + 1 < nL) acc(F, stretch_f1(M.LH_kstr[pb], rb, ld3(X.r_lh + 3 * bI + 3), M.LH_streq[pb], E));
    // bending around centres b-1, b, b+1
    for (int s = bI - 1; s <= bI + 1; s++) {
      if (s < 0 || s >= nL) continue;
      if (!((s % M.n_lh_c != 0) && (s % M.n_lh_c != M.n_lh_c - 1))) continue;
      int ps = lh_param(M, s);
      V3 f1, f2, f3;
      double e = 0.0;
      bend3(M.LH_kben[ps], X.beta_lh[s], M.LH_betaeq[ps], ld3(X.r_lh + 3 * s - 3), ld3(X.r_lh + 3 * s),
            ld3(X.r_lh + 3 * s + 3), f1, f2, f3, e);
      if (s == bI) E = E + e;
      dec(F, s == bI - 1 ? f3 : (s == bI ? f2 : f1));
    }
    // anchor to the globular head (func.cpp:2750-2752); energy on the core
    if (bI % nlh == 0) {
      int lc = bI / nlh;
      for (int jj = 0; jj < M.n_lh_g; jj++) {
        int pj = jj + M.n_lh_n;
        if (M.LH_conn[pj] != 1) continue;
        V3 g = ld3(X.gpos + 3 * (lc * M.n_lh_g + jj));
        double d = sqrt((rb.x - g.x) * (rb.x - g.x) + (rb.y - g.y) * (rb.y - g.y) + (rb.z - g.z) * (rb.z - g.z));
        double kst = M.LH_kstr[pj], eq = M.LH_streq[pj];
        V3 st{(d - eq) * (rb.x - g.x) / d, (d - eq) * (rb.y - g.y) / d, (d - eq) * (rb.z - g.z) / d};
        F.x = F.x - kst * st.x * 10; F.y = F.y - kst * st.y * 10; F.z = F.z - kst * st.z * 10;
      }
    }
  }
  // LH/LH (func.cpp:2190-2244); energy on the lower index
  for (int u = lane; u < nL; u += 32) {
    if (u == bI) continue;
    int pu = lh_param(M, u);
    double e = 0.0;
    double sig = (M.LH_vdw_hh[pb] + M.LH_vdw_hh[pu]) / 2;
    if (bI / nlh == u / nlh) {
      int lo = bI < u ? bI : u, hi = bI < u ? u : bI;
      if (!(hi > lo + 1)) continue;
      acc(F, pairF<false, true, MX>(0.0, 0.0, eps, M.debye, M.k_ex, sig, rb, ld3(X.r_lh + 3 * u), &e));
    } else {
      acc(F, pairF<true, true, MX>(M.LH_q[pb], M.LH_q[pu], eps, M.debye, M.k_ex, sig, rb, ld3(X.r_lh + 3 * u), &e));
    }
    if (bI < u) E = E + e;
  }
  // linker DNA and tails (func.cpp:2249-2398); energies here
  for (int q = lane; q < M.n_dna; q += 32) {
    int j = M.dna_bead[q];
    acc(F, pairF<true, true, MX>(M.LH_q[pb], M.q_l, eps, M.debye, M.k_ex, M.LH_vdw_hl[pb], rb, ld3(X.r + 3 * j), &E));
  }
  for (int t = lane; t < M.n_tail; t += 32)
    acc(F, pairF<true, true, MX>(M.LH_q[pb], M.t_q[t], eps, M.debye, M.k_ex, M.LH_vdw_ht[pb], rb, ld3(X.r_t + 3 * t), &E));
  // globular heads of the other LHs (func.cpp:2588-2644); energy on the core
  const int own = bI / nlh;
  for (int s = lane; s < M.n_lhcore * M.n_lh_g; s += 32) {
    int K = s / M.n_lh_g, m = s - K * M.n_lh_g;
    if (K == own) continue;
    acc(F, pairF<true, true, MX>(M.LH_q[pb], M.LH_q[m], eps, M.debye, M.k_ex, (M.LH_vdw_hh[m] + M.LH_vdw_hh[pb]) / 2, rb,
                               ld3(X.gpos + 3 * s), nullptr));
  }
  F.x = wsum(F.x); F.y = wsum(F.y); F.z = wsum(F.z); E = wsum(E);
  if (lane == 0) {
    st3(out.lF + 3 * bI, F);
    Eout[bI] = E;
  }
}

// ------------------------------------------------------------ mixed path: FP32 pair loops
// The gather kernels of the mixed path evaluate every pair in FP32 from a
// per-pass mirror of the positions as double-float pairs (hi, lo): the
// separation (hi_a - hi_b) + (lo_a - lo_b) keeps the FP64 positions'
// accuracy without FP64 arithmetic.  Pair sums run in FP32 for 32 pairs,
// then in FP64; torques from pair forces are summed in the world frame
// (lever x f) and turned into the body frame once.  The pair formulas and
// cut-offs are those of pair_f1_mx (func.cpp:278-345).

__global__ void k_mirror(DevModel M, DevState X, float4* ph, float4* pl, int npos) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npos) return;
  const int n = M.n, nt = M.n_tail, nL = M.n_LH;
  const double* p = i < n ? X.r + 3 * i
                  : i < n + nt ? X.r_t + 3 * (i - n)
                  : i < n + nt + nL ? X.r_lh + 3 * (i - n - nt)
                  : X.gpos + 3 * (i - n - nt - nL);
  const double x = p[0], y = p[1], z = p[2];
  const float hx = (float)x, hy = (float)y, hz = (float)z;
  ph[i] = make_float4(hx, hy, hz, 0.f);
  pl[i] = make_float4((float)(x - hx), (float)(y - hy), (float)(z - hz), 0.f);
}

// The FP64 distance of two double-float positions, formed as dist3 forms it
// from the FP64 positions (hi + lo is the FP64 position to 2^-48 relative).
__device__ __noinline__ double dist_pf64(const PF& a, const PF& b) {
  const V3 u{(double)a.h.x + (double)a.l.x, (double)a.h.y + (double)a.l.y, (double)a.h.z + (double)a.l.z};
  const V3 v{(double)b.h.x + (double)b.l.x, (double)b.h.y + (double)b.l.y, (double)b.h.z + (double)b.l.z};
  return dist3(u, v);
}

// force on particle 1 (a) from particle 2 (b); qq = k_e q1 q2.  Near a
// cut-off the decision is the FP64 path's (near_cutoff).
template <bool DH, bool LJ>
__device__ __forceinline__ float3 pairf(float qq, float kap, float kev, float sig, const PF& a, const PF& b, float& E) {
  const float3 d = sepf(a, b);
  const float d2 = fmaf(d.x, d.x, fmaf(d.y, d.y, d.z * d.z));
  const float rinv = rsqrtf(d2);  // 1/d: one reciprocal square root instead of a root and divisions
  const float dd = d2 * rinv;
  bool in7 = dd < 7.f, in4 = dd < 4.f;
  if (near_cutoff(dd)) {
    const double d64 = dist_pf64(a, b);
    in7 = d64 < 7.0, in4 = d64 < 4.0;
  }
  float t = 0.f;
  if (DH && in7) {
    const float qe = qq * expf(-kap * dd) * rinv;  // k_e q1 q2 e^{-kappa d} / d
    t = qe * fmaf(kap, dd, 1.f) * rinv;
    E += qe;
  }
  if (LJ && in4) {
    const float sr = sig * rinv, sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
    t = t - kev * (6.f * sr6 - 12.f * sr12) * rinv;
    E += kev * (sr12 - sr6);
  }
  const float w = t * rinv;
  return make_float3(clamp09f(w * d.x), clamp09f(w * d.y), clamp09f(w * d.z));
}

// s = start, start + step, ... split as s = hi n + lo, advanced without a
// division per step (an integer division costs several conversion
// instructions).
struct Idx2 {
  int s, hi, lo, dh, dl, n;
  __device__ Idx2(int start, int step, int n_) : s(start), n(n_) {
    hi = start / n_;
    lo = start - hi * n_;
    dh = step / n_;
    dl = step - dh * n_;
  }
  __device__ void next() {
    s += dh * n + dl;
    hi += dh;
    lo += dl;
    if (lo >= n) lo -= n, hi++;
  }
};

// Partial sums of force, world torque and energy: runs of up to 32 terms in
// plain FP32, the runs added with Kahan compensation (still FP32: an FP64
// operation costs as much as ~64 FP32 ones on GB300); finish() forms the
// FP64 totals s[] once.  Compiled without FMA contraction, so the
// compensation is exact.
struct FAcc {
  float f[7], k[7], c[7];
  double s[7];
  int n;
  __device__ void init() {
#pragma unroll
    for (int q = 0; q < 7; q++) f[q] = 0.f, k[q] = 0.f, c[q] = 0.f;
    n = 0;
  }
  __device__ void flush() {
#pragma unroll
    for (int q = 0; q < 7; q++) {
      const float y = f[q] - c[q], t = k[q] + y;
      c[q] = (t - k[q]) - y;
      k[q] = t;
      f[q] = 0.f;
    }
    n = 0;
  }
  __device__ void tick() {
    if (++n == 32) flush();
  }
  __device__ void finish() {
    flush();
#pragma unroll
    for (int q = 0; q < 7; q++) s[q] = (double)k[q] - (double)c[q];
  }
  __device__ void force(const float3& v) { f[0] += v.x; f[1] += v.y; f[2] += v.z; }
  __device__ void torque(const float3& v) { f[3] += v.x; f[4] += v.y; f[5] += v.z; }
};

// LH bead-type parameters in FP32, per CTA: q, vdw_hh, vdw_hl, vdw_ht
struct LHf {
  float q[64], hh[64], hl[64], ht[64];
};
__device__ void load_lhf(const DevModel& M, LHf& P) {
  const int np = M.n_lh_n + M.n_lh_g + M.n_lh_c;
  for (int i = threadIdx.x; i < np && i < 64; i += blockDim.x) {
    P.q[i] = (float)M.LH_q[i];
    P.hh[i] = (float)M.LH_vdw_hh[i];
    P.hl[i] = (float)M.LH_vdw_hl[i];
    P.ht[i] = (float)M.LH_vdw_ht[i];
  }
  __syncthreads();
}

// Bonded terms and the anchor of each tail bead (func.cpp:1809-1862), FP64,
// one thread per bead: on GB300 an FP64 warp instruction costs the same
// with one active lane as with 32, so these per-bead terms are taken out
// of the one-warp-per-bead pair kernel.
__global__ void k_tail_bonded_mx(DevModel M, DevState X, DevScratch S) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M.n_tail) return;
  V3 rt = ld3(X.r_t + 3 * t);
  V3 F{0.0, 0.0, 0.0};
  double E = 0.0;
  const int* grp = M.t_grp;
  const int nt = M.n_tail;
  {
    if (t >= 1 && grp[t - 1] == grp[t]) acc(F, stretch_f2(M.h_t[t - 1], ld3(X.r_t + 3 * t - 3), rt, M.lo_t[t - 1]));
    if (t + 1 < nt && grp[t] == grp[t + 1]) acc(F, stretch_f1(M.h_t[t], rt, ld3(X.r_t + 3 * t + 3), M.lo_t[t], E));
    for (int s = t - 2; s <= t; s++) {
      if (s < 0 || s + 2 >= nt) continue;
      if (!(grp[s] == grp[s + 1] && grp[s] == grp[s + 2])) continue;
      V3 f1, f2, f3;
      double e = 0.0;
      bend3(M.g_t[s], X.beta_t[s], M.beta_o_t[s], ld3(X.r_t + 3 * s), ld3(X.r_t + 3 * s + 3), ld3(X.r_t + 3 * s + 6), f1,
            f2, f3, e);
      if (s == t) E = E + e;
      dec(F, s == t ? f1 : (s == t - 1 ? f2 : f3));
    }
    int J = t / M.n_t, jt = t - J * M.n_t;
    if (M.nc_t_flag[J] == 1 && M.tail_fix[jt] == 1) {
      int cb = M.core_bead[J];
      V3 ro = site(X, cb, M.tail_pos + 3 * jt);
      V3 st{rt.x - ro.x, rt.y - ro.y, rt.z - ro.z};
      F.x = F.x - M.h * st.x; F.y = F.y - M.h * st.y; F.z = F.z - M.h * st.z;
    }
  }
  double* bt = S.bond + 4 * (size_t)t;
  bt[0] = F.x; bt[1] = F.y; bt[2] = F.z; bt[3] = E;
}

// Tail beads, one warp each (func.cpp:1809-1917, 2343-2476 for the LH side).
constexpr int kTailTile = 256;
__global__ void __launch_bounds__(256) k_tail_gather_mx(DevModel M, DevState X, DevScratch S, DevForces out,
                                                        double* Eout) {
  __shared__ LHf P;
  __shared__ float4 th[kTailTile], tl[kTailTile];
  __shared__ float tq[kTailTile];
  __shared__ int tg[kTailTile];
  load_lhf(M, P);
  const int lane = threadIdx.x & 31;
  const int t_raw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const bool active = t_raw < M.n_tail;  // the CTA's warps share the staged tiles: none leaves early
  const int t = active ? t_raw : M.n_tail - 1;
  V3 rt = ld3(X.r_t + 3 * t);
  V3 F{0.0, 0.0, 0.0};
  double E = 0.0;
  const int* grp = M.t_grp;
  const int nt = M.n_tail;
  if (lane == 0) {  // bonded terms and the anchor (k_tail_bonded_mx)
    const double* bt = S.bond + 4 * (size_t)t;
    F = V3{bt[0], bt[1], bt[2]};
    E = bt[3];
  }
  const float ke = (float)M.k_e, kap = (float)M.debye, kex = (float)M.k_ex;
  const float qt = ke * M.t_qf[t];
  const PF pt = ldpf(S, S.ot + t);
  FAcc A;
  A.init();
  float dummy = 0.f;
  const int gt = grp[t];
  for (int base = 0; base < nt; base += kTailTile) {  // tail/tail (func.cpp:1863-1891); energy on the lower index
    __syncthreads();
    for (int x = threadIdx.x; x < kTailTile && base + x < nt; x += blockDim.x) {
      th[x] = S.ph[S.ot + base + x];
      tl[x] = S.pl[S.ot + base + x];
      tq[x] = M.t_qf[base + x];
      tg[x] = grp[base + x];
    }
    __syncthreads();
    const int ue = min(nt, base + kTailTile);
    for (int u = base + lane; u < ue; u += 32) {
      const int x = u - base;
      if (u == t || (tg[x] == gt && abs(u - t) <= 2)) continue;  // bonded neighbours of one tail
      float e = 0.f;
      A.force(pairf<true, false>(qt * tq[x], kap, 0.f, 0.f, pt, PF{th[x], tl[x]}, e));
      if (t < u) A.f[6] += e;
      A.tick();
    }
  }
  const float ql = (float)M.q_l, sTL = (float)M.sTL;
  for (int q = lane; q < M.n_dna; q += 32) {  // linker DNA (func.cpp:1898-1917); energy here
    A.force(pairf<true, true>(qt * ql, kap, kex, sTL, pt, ldpf(S, M.dna_bead[q]), A.f[6]));
    A.tick();
  }
  if (M.t_fix[t] == 0) {  // LH beads and globular heads on free tail beads (energies on their side)
    for (int b = lane; b < M.n_LH; b += 32) {
      int p = M.lh_p[b];
      A.force(pairf<true, true>(qt * P.q[p], kap, kex, P.ht[p], pt, ldpf(S, S.ol + b), dummy));
      A.tick();
    }
    for (Idx2 x(lane, 32, M.n_lh_g); x.s < M.n_lhcore * M.n_lh_g; x.next()) {
      const int m = x.lo;
      A.force(pairf<true, true>(qt * P.q[m], kap, kex, P.ht[m], pt, ldpf(S, S.og + x.s), dummy));
      A.tick();
    }
  }
  A.finish();
  F.x += A.s[0]; F.y += A.s[1]; F.z += A.s[2]; E += A.s[6];
  F.x = wsum(F.x); F.y = wsum(F.y); F.z = wsum(F.z); E = wsum(E);
  if (lane == 0 && active) {
    st3(out.tF + 3 * t, F);
    Eout[t] = E;
  }
}

// Bonded terms and the globular-head anchor of each LH bead
// (func.cpp:2109-2185, 2725-2777), FP64, one thread per bead (as
// k_tail_bonded_mx).
__global__ void k_lh_bonded_mx(DevModel M, DevState X, DevScratch S) {
  const int bI = blockIdx.x * blockDim.x + threadIdx.x;
  if (bI >= M.n_LH) return;
  const int nL = M.n_LH, nlh = M.nlh;
  V3 rb = ld3(X.r_lh + 3 * bI);
  const int pb = M.lh_p[bI];
  V3 F{0.0, 0.0, 0.0};
  double E = 0.0;
  {
    if (bI >= 1) {
      int p = M.lh_p[bI - 1];
      if (M.LH_conn[p] == 1) acc(F, stretch_f2(M.LH_kstr[p], ld3(X.r_lh + 3 * bI - 3), rb, M.LH_streq[p]));
    }
    if (M.LH_conn[pb] == 1 && bI + 1 < nL) acc(F, stretch_f1(M.LH_kstr[pb], rb, ld3(X.r_lh + 3 * bI + 3), M.LH_streq[pb], E));
    for (int s = bI - 1; s <= bI + 1; s++) {
      if (s < 0 || s >= nL) continue;
      if (!((s % M.n_lh_c != 0) && (s % M.n_lh_c != M.n_lh_c - 1))) continue;
      int ps = M.lh_p[s];
      V3 f1, f2, f3;
      double e = 0.0;
      bend3(M.LH_kben[ps], X.beta_lh[s], M.LH_betaeq[ps], ld3(X.r_lh + 3 * s - 3), ld3(X.r_lh + 3 * s),
            ld3(X.r_lh + 3 * s + 3), f1, f2, f3, e);
      if (s == bI) E = E + e;
      dec(F, s == bI - 1 ? f3 : (s == bI ? f2 : f1));
    }
    if (bI % nlh == 0) {
      int lc = bI / nlh;
      for (int jj = 0; jj < M.n_lh_g; jj++) {
        int pj = jj + M.n_lh_n;
        if (M.LH_conn[pj] != 1) continue;
        V3 g = ld3(X.gpos + 3 * (lc * M.n_lh_g + jj));
        double d = sqrt((rb.x - g.x) * (rb.x - g.x) + (rb.y - g.y) * (rb.y - g.y) + (rb.z - g.z) * (rb.z - g.z));
        double kst = M.LH_kstr[pj], eq = M.LH_streq[pj];
        V3 st{(d - eq) * (rb.x - g.x) / d, (d - eq) * (rb.y - g.y) / d, (d - eq) * (rb.z - g.z) / d};
        F.x = F.x - kst * st.x * 10; F.y = F.y - kst * st.y * 10; F.z = F.z - kst * st.z * 10;
      }
    }
  }
  double* bt = S.bond + 4 * ((size_t)M.n_tail + bI);
  bt[0] = F.x; bt[1] = F.y; bt[2] = F.z; bt[3] = E;
}

// Mobile LH beads, one warp each (func.cpp:2109-2398, 2588-2644, 2725-2777).
__global__ void __launch_bounds__(256) k_lh_gather_mx(DevModel M, DevState X, DevScratch S, DevForces out,
                                                      double* Eout) {
  __shared__ LHf P;
  __shared__ float4 th[kTailTile], tl[kTailTile];
  __shared__ float tq[kTailTile];
  load_lhf(M, P);
  const int lane = threadIdx.x & 31;
  const int b_raw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const bool active = b_raw < M.n_LH;  // the CTA's warps share the staged tiles: none leaves early
  const int bI = active ? b_raw : M.n_LH - 1;
  const int nL = M.n_LH, nlh = M.nlh;
  V3 rb = ld3(X.r_lh + 3 * bI);
  const int pb = M.lh_p[bI];
  V3 F{0.0, 0.0, 0.0};
  double E = 0.0;
  if (lane == 0) {  // bonded terms and the globular-head anchor (k_lh_bonded_mx)
    const double* bt = S.bond + 4 * ((size_t)M.n_tail + bI);
    F = V3{bt[0], bt[1], bt[2]};
    E = bt[3];
  }
  const float ke = (float)M.k_e, kap = (float)M.debye, kex = (float)M.k_ex;
  const float qb = ke * P.q[pb];
  const PF pp = ldpf(S, S.ol + bI);
  FAcc A;
  A.init();
  float dummy = 0.f;
  const int own0 = (bI / nlh) * nlh;
  for (int u = lane; u < nL; u += 32) {  // LH/LH (func.cpp:2190-2244); energy on the lower index
    if (u == bI) continue;
    const int pu = M.lh_p[u];
    const float sig = (P.hh[pb] + P.hh[pu]) * 0.5f;
    float e = 0.f;
    const PF pu4 = ldpf(S, S.ol + u);
    if ((unsigned)(u - own0) < (unsigned)nlh) {  // same LH molecule
      int lo = bI < u ? bI : u, hi = bI < u ? u : bI;
      if (!(hi > lo + 1)) continue;
      A.force(pairf<false, true>(0.f, kap, kex, sig, pp, pu4, e));
    } else {
      A.force(pairf<true, true>(qb * P.q[pu], kap, kex, sig, pp, pu4, e));
    }
    if (bI < u) A.f[6] += e;
    A.tick();
  }
  const float ql = (float)M.q_l;
  for (int q = lane; q < M.n_dna; q += 32) {  // linker DNA; energy here
    A.force(pairf<true, true>(qb * ql, kap, kex, P.hl[pb], pp, ldpf(S, M.dna_bead[q]), A.f[6]));
    A.tick();
  }
  for (int base = 0; base < M.n_tail; base += kTailTile) {  // tails; energy here
    __syncthreads();
    for (int x = threadIdx.x; x < kTailTile && base + x < M.n_tail; x += blockDim.x) {
      th[x] = S.ph[S.ot + base + x];
      tl[x] = S.pl[S.ot + base + x];
      tq[x] = M.t_qf[base + x];
    }
    __syncthreads();
    const int te = min(M.n_tail, base + kTailTile);
    for (int t = base + lane; t < te; t += 32) {
      const int x = t - base;
      A.force(pairf<true, true>(qb * tq[x], kap, kex, P.ht[pb], pp, PF{th[x], tl[x]}, A.f[6]));
      A.tick();
    }
  }
  const int own = bI / nlh;
  for (Idx2 x(lane, 32, M.n_lh_g); x.s < M.n_lhcore * M.n_lh_g; x.next()) {  // other LHs' globular heads; energy on the core
    const int K = x.hi, m = x.lo;
    if (K == own) continue;
    A.force(pairf<true, true>(qb * P.q[m], kap, kex, (P.hh[m] + P.hh[pb]) * 0.5f, pp, ldpf(S, S.og + x.s), dummy));
    A.tick();
  }
  A.finish();
  F.x += A.s[0]; F.y += A.s[1]; F.z += A.s[2]; E += A.s[6];
  F.x = wsum(F.x); F.y = wsum(F.y); F.z = wsum(F.z); E = wsum(E);
  if (lane == 0 && active) {
    st3(out.lF + 3 * bI, F);
    Eout[bI] = E;
  }
}

// Chain beads, one CTA each.
// One CTA per chain bead, beads[blockIdx.x]: launched once over the linker
// DNA beads (kGatherThreads threads) and once over the cores, whose pair
// lists (globular heads, anchored tails) are ~20x longer (kGatherCoreThreads).
constexpr int kGatherCoreThreads = 512;
__global__ void __launch_bounds__(kGatherCoreThreads) k_chain_gather_mx(DevModel M, DevState X, const double* Fm,
                                                                       const double* Tm, const double* Ech,
                                                                       DevScratch S, DevForces out, double* Eout,
                                                                       const int* __restrict__ beads) {
  __shared__ double red[32 * 7];
  __shared__ LHf P;
  load_lhf(M, P);
  const int j = beads[blockIdx.x];
  const int tid = threadIdx.x, nt = blockDim.x;
  V3 rj = ld3(X.r + 3 * j), aj = ld3(X.a + 3 * j), bj = ld3(X.b + 3 * j), cj = ld3(X.c + 3 * j);
  V3 F{0.0, 0.0, 0.0}, T{0.0, 0.0, 0.0};
  double E = 0.0;
  const float ke = (float)M.k_e, kap = (float)M.debye, kex = (float)M.k_ex, ql = (float)M.q_l;
  const PF pj = ldpf(S, j);
  FAcc A;
  A.init();
  float dummy = 0.f;
  if (M.type[j] == 0) {
    if (chain_ok(M, j)) {  // DNA/DNA (func.cpp:1326-1354); energy on the lower index
      const float kll = (float)M.debyell, qq = ke * ql * ql, sDD = (float)M.sDD;
      for (int i = tid; i < M.n; i += nt) {
        if (i == j || M.type[i] != 0 || abs(i - j) <= 1 || !chain_ok(M, i)) continue;
        const float3 z = sepf(pj, ldpf(S, i));
        const float d2 = fmaf(z.x, z.x, fmaf(z.y, z.y, z.z * z.z));
        const float mi = rsqrtf(d2), df = d2 * mi;  // 1/d and d
        if (df > 25.f) continue;
        const float ex = expf(-kll * df);
        float e = qq * ex * mi, g = e * fmaf(kll, df, 1.f) * mi;
        if (df <= 8.f) {
          const float sr = sDD * mi, sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
          g += kex * (12.f * sr12 - 6.f * sr6) * mi;
          e += kex * (sr12 - sr6);
        }
        if (j < i) A.f[6] += e;
        A.force(make_float3(g * z.x * mi, g * z.y * mi, g * z.z * mi));
        A.tick();
      }
    }
    const float qlk = ke * ql, sTL = (float)M.sTL;
    for (int t = tid; t < M.n_tail; t += nt) {  // tails on this DNA bead; energy on the tail side
      A.force(pairf<true, true>(qlk * M.t_qf[t], kap, kex, sTL, pj, ldpf(S, S.ot + t), dummy));
      A.tick();
    }
    for (int b = tid; b < M.n_LH; b += nt) {  // LH beads; energy on the LH side
      int p = M.lh_p[b];
      A.force(pairf<true, true>(qlk * P.q[p], kap, kex, P.hl[p], pj, ldpf(S, S.ol + b), dummy));
      A.tick();
    }
    for (Idx2 x(tid, nt, M.n_lh_g); x.s < M.n_lhcore * M.n_lh_g; x.next()) {  // globular heads; energy on the core side
      const int m = x.lo, s = x.s;
      A.force(pairf<true, true>(qlk * P.q[m], kap, kex, P.hl[m], pj, ldpf(S, S.og + s), dummy));
      A.tick();
    }
  } else {
    const int J = M.core_rank[j];
    const int lc = M.core_lh[J];
    if (lc >= 0) {
      const int ng = M.n_lh_g;
      for (Idx2 x(tid, nt, M.n); x.s < ng * M.n; x.next()) {  // G-head vs linker DNA (func.cpp:2481-2522); energy here
        const int m = x.hi, l = x.lo;
        if (M.type[l] != 0) continue;
        const PF g = ldpf(S, S.og + lc * ng + m);
        const float3 f1 = pairf<true, true>(ke * P.q[m] * ql, kap, kex, P.hl[m], g, ldpf(S, l), A.f[6]);
        A.force(f1);
        A.torque(crossf(sepf(g, pj), f1));
        A.tick();
      }
      for (Idx2 x(tid, nt, M.n_tail); x.s < ng * M.n_tail; x.next()) {  // G-head vs tails (func.cpp:2403-2476)
        const int m = x.hi, t = x.lo;
        const PF g = ldpf(S, S.og + lc * ng + m);
        const float3 f1 = pairf<true, true>(ke * P.q[m] * M.t_qf[t], kap, kex, P.ht[m], g, ldpf(S, S.ot + t),
                                            A.f[6]);
        A.force(f1);
        A.torque(crossf(sepf(g, pj), f1));
        A.tick();
      }
      for (Idx2 x(tid, nt, M.n_LH); x.s < ng * M.n_LH; x.next()) {  // G-head vs other LHs' beads (func.cpp:2590-2644)
        const int m = x.hi, b = x.lo;
        if ((unsigned)(b - lc * M.nlh) < (unsigned)M.nlh) continue;
        int p2 = M.lh_p[b];
        const PF g = ldpf(S, S.og + lc * ng + m);
        const float3 f1 = pairf<true, true>(ke * P.q[m] * P.q[p2], kap, kex, (P.hh[m] + P.hh[p2]) * 0.5f,
                                            g, ldpf(S, S.ol + b), A.f[6]);
        A.force(f1);
        A.torque(crossf(sepf(g, pj), f1));
        A.tick();
      }
      for (int s = tid; s < ng * M.n_lhcore * ng; s += nt) {  // G-head/G-head (func.cpp:2649-2719); lower core
        int m = s / (M.n_lhcore * ng), rest = s - m * (M.n_lhcore * ng);
        int K = rest / ng, m1 = rest - K * ng;
        if (K == lc) continue;
        const PF g = ldpf(S, S.og + lc * ng + m);
        float e = 0.f;
        const float3 f1 = pairf<true, true>(ke * P.q[m] * P.q[m1], kap, kex, (P.hh[m] + P.hh[m1]) * 0.5f,
                                            g, ldpf(S, S.og + K * ng + m1), e);
        if (lc < K) A.f[6] += e;
        A.force(f1);
        A.torque(crossf(sepf(g, pj), f1));
        A.tick();
      }
      if (tid == 0) {  // G-head <-> first C-term bead anchor (func.cpp:2725-2777), FP64
        for (int jj = 0; jj < ng; jj++) {
          int pjj = jj + M.n_lh_n;
          if (M.LH_conn[pjj] != 1) continue;
          V3 g = ld3(X.gpos + 3 * (lc * ng + jj));
          V3 q = ld3(X.r_lh + 3 * (lc * M.nlh));
          double d = sqrt((q.x - g.x) * (q.x - g.x) + (q.y - g.y) * (q.y - g.y) + (q.z - g.z) * (q.z - g.z));
          double kst = M.LH_kstr[pjj], eq = M.LH_streq[pjj];
          E = E + kst * (d - eq) * (d - eq) / 2;
          V3 st{(d - eq) * (q.x - g.x) / d, (d - eq) * (q.y - g.y) / d, (d - eq) * (q.z - g.z) / d};
          F.x = F.x + kst * st.x * 10; F.y = F.y + kst * st.y * 10; F.z = F.z + kst * st.z * 10;
          double fa = kst * (aj.x * st.x + aj.y * st.y + aj.z * st.z);
          double fb = kst * (bj.x * st.x + bj.y * st.y + bj.z * st.z);
          double fc = kst * (cj.x * st.x + cj.y * st.y + cj.z * st.z);
          const double* gp = M.LH_g_pos + 3 * jj;
          T.x = T.x + fc * gp[1] - fb * gp[2];
          T.y = T.y + fa * gp[2] - fc * gp[0];
          T.z = T.z + fb * gp[0] - fa * gp[1];
        }
      }
    }
    if (M.nc_t_flag[J] == 1) {  // tail anchors of this core (func.cpp:1971-2022), FP64
      for (int jt = tid; jt < M.n_t; jt += nt) {
        if (M.tail_fix[jt] != 1) continue;
        V3 ro = body(rj, aj, bj, cj, M.tail_pos + 3 * jt);
        int tb = J * M.n_t + jt;
        V3 rt = ld3(X.r_t + 3 * tb);
        V3 st{rt.x - ro.x, rt.y - ro.y, rt.z - ro.z};
        E = E + M.h * (st.x * st.x + st.y * st.y + st.z * st.z) / 2;
        V3 hs{M.h * st.x, M.h * st.y, M.h * st.z};
        acc(F, hs);
        acc(T, torque_rel(hs, M.tail_pos + 3 * jt, aj, bj, cj));
      }
    }
    // LH and G-head forces on this core's anchored tail beads go to the core
    // (func.cpp:2361-2391, 2436-2465)
    const int t_lo = M.tails_by_core ? J * M.n_t : 0;
    const int t_hi = M.tails_by_core ? min((J + 1) * M.n_t, M.n_tail) : M.n_tail;
    for (int t0 = t_lo; t0 < t_hi; t0++) {
      if (M.t_fix[t0] == 0 || M.t_core_bead[t0] != j) continue;
      const PF pt = ldpf(S, S.ot + t0);
      const float3 lever = sepf(pt, pj);
      const float qt = ke * M.t_qf[t0];
      for (int b = tid; b < M.n_LH; b += nt) {
        int p = M.lh_p[b];
        const float3 f2 = pairf<true, true>(qt * P.q[p], kap, kex, P.ht[p], pt, ldpf(S, S.ol + b), dummy);
        A.force(f2);
        A.torque(crossf(lever, f2));
        A.tick();
      }
      for (Idx2 x(tid, nt, M.n_lh_g); x.s < M.n_lhcore * M.n_lh_g; x.next()) {
        const int m = x.lo, s = x.s;
        const float3 f2 = pairf<true, true>(qt * P.q[m], kap, kex, P.ht[m], pt, ldpf(S, S.og + s), dummy);
        A.force(f2);
        A.torque(crossf(lever, f2));
        A.tick();
      }
    }
  }
  A.finish();
  F.x += A.s[0]; F.y += A.s[1]; F.z += A.s[2]; E += A.s[6];
  // world-frame torques of the pair terms into the body frame
  T.x += aj.x * A.s[3] + aj.y * A.s[4] + aj.z * A.s[5];
  T.y += bj.x * A.s[3] + bj.y * A.s[4] + bj.z * A.s[5];
  T.z += cj.x * A.s[3] + cj.y * A.s[4] + cj.z * A.s[5];
  chain_finish_mx(M, S, Fm, Tm, Ech, out, Eout, j, F, T, E, red);
}

// Total energy: chain, tail and LH shares in a fixed order.
__global__ void k_energy(int n0, const double* e0, double* E) {
  __shared__ double red[32];
  double v[1] = {0.0};
  for (int i = threadIdx.x; i < n0; i += blockDim.x) v[0] = v[0] + e0[i];
  bsum<1>(v, red);
  if (threadIdx.x == 0) E[0] = v[0];
}

}  // namespace

namespace bdk {

int forces(const DevModel& M, DevState& X, DevForces& out, DevScratch& S, int mixed, cudaStream_t st) {
  // energy layout in S.ebuf: [0,n) chain, [n, n+n_tail) tails, then LH
  double* Ech = S.ebuf;
  double* Et = S.ebuf + M.n;
  double* El = S.ebuf + M.n + M.n_tail;
  double* Ebond = S.ebuf + M.n + M.n_tail + M.n_LH;  // [n] bonded shares
  double* Fm = S.ebuf + 2 * M.n + M.n_tail + M.n_LH; // [3n]
  double* Tm = Fm + 3 * M.n;                          // [3n]
  int L = 0;
#define KSEL(name) (mixed ? name<true> : name<false>)
  auto k_dna_coreX = KSEL(k_dna_core);
  auto k_ghead_coreX = KSEL(k_ghead_core);
  auto k_tail_gatherX = KSEL(k_tail_gather);
  auto k_lh_gatherX = KSEL(k_lh_gather);
  auto k_chain_gatherX = KSEL(k_chain_gather);
#undef KSEL
  if (M.n_lhcore > 0) { k_gpos<<<cdiv(M.n_lhcore * M.n_lh_g, 128), 128, 0, st>>>(M, X); L++; }
  if (mixed) { k_mirror<<<cdiv(S.npos, 128), 128, 0, st>>>(M, X, S.ph, S.pl, S.npos); L++; }
  if (M.n > 1) {
    k_chain_bonds<<<cdiv(M.n - 1, kBeadThreads), kBeadThreads, 0, st>>>(M, X, S.bonds);
    L++;
  }
  k_chain_bonded<<<cdiv(M.n, kBeadThreads), kBeadThreads, 0, st>>>(M, X, S.bonds, Fm, Tm, Ebond);
  L++;
  if (M.n_c > 1) {
    if (mixed) {
      size_t sm = (size_t)((14 * M.Nq + 1) / 2 + 32 * 10) * sizeof(double);
      k_core_core_mx<<<dim3(M.n_c, M.n_c, kCCSplit), kCCThreads, sm, st>>>(M, X, S, S.ccp);
      k_cc_sum<<<cdiv(M.n_c * M.n_c * 10, 256), 256, 0, st>>>(M.n_c, S.ccp, S.cc);
      L++;
    } else {
      size_t sm = (size_t)(6 * M.Nq + 32 * 10) * sizeof(double);
      k_core_core<<<dim3(M.n_c, M.n_c, kCCSplit), kCCThreads, sm, st>>>(M, X, S.ccp);
      k_cc_sum<<<cdiv(M.n_c * M.n_c * 10, 256), 256, 0, st>>>(M.n_c, S.ccp, S.cc);
      L++;
    }
    L++;
  }
  if (M.n_dna > 0 && M.n_c > 0) { k_dna_coreX<<<cdiv(M.n_dna * M.n_c * 32, 256), 256, 0, st>>>(M, X, S, S.dc); L++; }
  if (M.n_lhcore > 0) { k_ghead_coreX<<<cdiv(M.n_lhcore * M.n_c * 32, 256), 256, 0, st>>>(M, X, S.gc); L++; }
  if (mixed) {
    if (M.n_tail > 0) { k_tail_bonded_mx<<<cdiv(M.n_tail, kBeadThreads), kBeadThreads, 0, st>>>(M, X, S); L++; }
    if (M.n_LH > 0) { k_lh_bonded_mx<<<cdiv(M.n_LH, kBeadThreads), kBeadThreads, 0, st>>>(M, X, S); L++; }
    if (M.n_tail > 0) { k_tail_gather_mx<<<cdiv(M.n_tail * 32, 256), 256, 0, st>>>(M, X, S, out, Et); L++; }
    if (M.n_LH > 0) { k_lh_gather_mx<<<cdiv(M.n_LH * 32, 256), 256, 0, st>>>(M, X, S, out, El); L++; }
    if (M.n_dna > 0) k_chain_gather_mx<<<M.n_dna, kGatherThreads, 0, st>>>(M, X, Fm, Tm, Ebond, S, out, Ech, M.dna_bead);
    if (M.n_c > 0) k_chain_gather_mx<<<M.n_c, kGatherCoreThreads, 0, st>>>(M, X, Fm, Tm, Ebond, S, out, Ech, M.core_bead);
    L += (M.n_dna > 0) + (M.n_c > 0) - 1;  // one chain launch is counted below
  } else {
    if (M.n_tail > 0) { k_tail_gatherX<<<cdiv(M.n_tail * 32, 256), 256, 0, st>>>(M, X, out, Et); L++; }
    if (M.n_LH > 0) { k_lh_gatherX<<<cdiv(M.n_LH * 32, 256), 256, 0, st>>>(M, X, out, El); L++; }
    k_chain_gatherX<<<M.n, kGatherThreads, 0, st>>>(M, X, Fm, Tm, Ebond, S, out, Ech);
  }
  k_energy<<<1, 256, 0, st>>>(M.n + M.n_tail + M.n_LH, S.ebuf, out.E);
  return L + 2;
}

}  // namespace bdk
