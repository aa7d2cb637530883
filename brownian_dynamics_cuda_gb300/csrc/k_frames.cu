// Internal coordinates and the Ermak-McCammon update.
//
//   frames()           update_Euler_Angle (func.cpp:433-685) as two ordered
//                      passes inside one CTA, plus update_tail_beta
//                      (func.cpp:1763-1790) and update_LH_beta (:2062-2089).
//                      The reference GPU version (func_cuda.cu:706-961) runs
//                      both passes in one thread per bead and races across
//                      blocks; here the passes are separated by a barrier.
//   rotate_translate() rotation_cal + rotate (func_cuda.cu:681-704,
//                      func.cpp:1607-1670) and translation_cal
//                      (func_cuda.cu:650-679).  The drift uses the
//                      species-block-diagonal RPY tensor, recomputed on the
//                      fly from positions (matrix-free) so the factorised
//                      matrix can overwrite D in place.
#include <cuda_runtime.h>

#include "bd_internal.h"
#include "dev_physics.cuh"

using namespace bdp;

namespace {

// FP64 throughout (GB300 runs ~2 FP64 operations per clock per SM), so the
// beads are spread over many small CTAs: one warp per CTA, 32 beads each.
#ifndef BD_FP64_BEAD_THREADS
#define BD_FP64_BEAD_THREADS 32
#endif
constexpr int kFrameThreads = BD_FP64_BEAD_THREADS;

// pass 1: DNA frames follow their bond; lengths (func.cpp:448-505)
__global__ void __launch_bounds__(kFrameThreads) k_frames_dna(DevModel M, DevState S) {
  const int n = M.n;
  double* r = S.r;
  double* a = S.a;
  double* b = S.b;
  double* c = S.c;
  const double si = sin(kTheta), co = cos(kTheta);
  {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int i1 = 3 * i, i2 = i1 + 1, i3 = i2 + 1, f1 = i1 + 3, f2 = f1 + 1, f3 = f2 + 1;
    double rf[3];
    if (M.type[i] == 0) {
      double ao[3] = {a[i1], a[i2], a[i3]};
      if (M.type[i + 1] == 0) {
        rf[0] = r[f1] - r[i1]; rf[1] = r[f2] - r[i2]; rf[2] = r[f3] - r[i3];
      } else {
        double bm[3] = {-si * a[f1] + co * b[f1], -si * a[f2] + co * b[f2], -si * a[f3] + co * b[f3]};
        rf[0] = r[f1] - kRo * bm[0] + kD1 * c[f1] - r[i1];
        rf[1] = r[f2] - kRo * bm[1] + kD1 * c[f2] - r[i2];
        rf[2] = r[f3] - kRo * bm[2] + kD1 * c[f3] - r[i3];
      }
      double len = sqrt(rf[0] * rf[0] + rf[1] * rf[1] + rf[2] * rf[2]);
      S.length[i] = len;
      double mi = 1.0 / len;
      double an[3] = {mi * rf[0], mi * rf[1], mi * rf[2]};
      double da[3] = {an[0] - ao[0], an[1] - ao[1], an[2] - ao[2]};
      double bn[3] = {b[i1], b[i2], b[i3]};
      double bda = bn[0] * da[0] + bn[1] * da[1] + bn[2] * da[2];
      bn[0] = bn[0] - bda * ao[0]; bn[1] = bn[1] - bda * ao[1]; bn[2] = bn[2] - bda * ao[2];
      bda = bn[0] * an[0] + bn[1] * an[1] + bn[2] * an[2];
      bn[0] = bn[0] - bda * an[0]; bn[1] = bn[1] - bda * an[1]; bn[2] = bn[2] - bda * an[2];
      mi = 1.0 / sqrt(bn[0] * bn[0] + bn[1] * bn[1] + bn[2] * bn[2]);
      bn[0] = mi * bn[0]; bn[1] = mi * bn[1]; bn[2] = mi * bn[2];
      a[i1] = an[0]; a[i2] = an[1]; a[i3] = an[2];
      b[i1] = bn[0]; b[i2] = bn[1]; b[i3] = bn[2];
      c[i1] = an[1] * bn[2] - an[2] * bn[1];
      c[i2] = an[2] * bn[0] - an[0] * bn[2];
      c[i3] = an[0] * bn[1] - an[1] * bn[0];
    } else {
      rf[0] = r[f1] - (r[i1] - kRo * b[i1] - kD1 * c[i1]);
      rf[1] = r[f2] - (r[i2] - kRo * b[i2] - kD1 * c[i2]);
      rf[2] = r[f3] - (r[i3] - kRo * b[i3] - kD1 * c[i3]);
      S.length[i] = sqrt(rf[0] * rf[0] + rf[1] * rf[1] + rf[2] * rf[2]);
    }
  }
}

// pass 2 (after pass 1 has finished for every bead): angles
// (func.cpp:507-681), then the tail and LH bend angles; thread index over
// the n - 1 chain beads, the tail beads, the LH beads in turn
__global__ void __launch_bounds__(kFrameThreads) k_frames_angles(DevModel M, DevState S) {
  const int n = M.n;
  double* r = S.r;
  double* a = S.a;
  double* b = S.b;
  double* c = S.c;
  const double si = sin(kTheta), co = cos(kTheta);
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n - 1) {
    const int i = g;
    int i1 = 3 * i, i2 = i1 + 1, i3 = i2 + 1, f1 = i1 + 3, f2 = f1 + 1, f3 = f2 + 1;
    if (M.type[i] == 0) {
      double af[3], bf[3], cf[3] = {c[f1], c[f2], c[f3]};
      if (M.type[i + 1] == 0) {
        af[0] = a[f1]; af[1] = a[f2]; af[2] = a[f3];
        bf[0] = b[f1]; bf[1] = b[f2]; bf[2] = b[f3];
      } else {
        af[0] = co * a[f1] + si * b[f1]; af[1] = co * a[f2] + si * b[f2]; af[2] = co * a[f3] + si * b[f3];
        bf[0] = -si * a[f1] + co * b[f1]; bf[1] = -si * a[f2] + co * b[f2]; bf[2] = -si * a[f3] + co * b[f3];
      }
      double ada = clamp1(a[i1] * af[0] + a[i2] * af[1] + a[i3] * af[2]);
      double be = acos(ada);
      double sb = sin(be);
      double x;
      if (be > 1e-10) x = (af[0] * b[i1] + af[1] * b[i2] + af[2] * b[i3]) / sb;
      else x = (bf[0] * b[i1] + bf[1] * b[i2] + bf[2] * b[i3]);
      double Ac = acos(clamp1(x));
      double y = af[0] * c[i1] + af[1] * c[i2] + af[2] * c[i3];
      double al = (y >= 0) ? Ac : -Ac;
      x = clamp1((b[i1] * bf[0] + b[i2] * bf[1] + b[i3] * bf[2] + c[i1] * cf[0] + c[i2] * cf[1] + c[i3] * cf[2]) /
                 (1.0 + ada));
      double apg = acos(x);
      y = (c[i1] * bf[0] + c[i2] * bf[1] + c[i3] * bf[2] - (b[i1] * cf[0] + b[i2] * cf[1] + b[i3] * cf[2])) /
          (1.0 + ada);
      S.beta[i] = be;
      S.alpha[i] = al;
      S.gamma[i] = (y >= 0.0) ? apg - al : -apg - al;
    } else {
      int ic = M.core_rank[i], c1 = 3 * ic;
      double len = S.length[i];
      double ad[3], bd[3], cd[3];
      ad[0] = (r[f1] - (r[i1] - kRo * b[i1] - kD1 * c[i1])) / len;
      ad[1] = (r[f2] - (r[i2] - kRo * b[i2] - kD1 * c[i2])) / len;
      ad[2] = (r[f3] - (r[i3] - kRo * b[i3] - kD1 * c[i3])) / len;
      double cb = clamp1(a[i1] * ad[0] + a[i2] * ad[1] + a[i3] * ad[2]);
      double bp = acos(cb);
      double sb = sin(bp);
      double alp = 0.0, gap = 0.0;
      bool have_p = bp >= 1e-10;
      if (have_p) {
        double bm[3] = {(ad[0] - cb * a[i1]) / sb, (ad[1] - cb * a[i2]) / sb, (ad[2] - cb * a[i3]) / sb};
        double ca = clamp1(bm[0] * b[i1] + bm[1] * b[i2] + bm[2] * b[i3]);
        double Ac = acos(ca);
        double y = ad[0] * c[i1] + ad[1] * c[i2] + ad[2] * c[i3];
        alp = (y >= 0) ? Ac : -Ac;
        gap = -alp;
        double sa = sin(alp), sg = sin(gap), cg = cos(gap);
        double R21 = -cg * sb, R22 = cg * cb * ca - sg * sa, R23 = cg * cb * sa + sg * ca;
        for (int k = 0; k < 3; k++) bd[k] = R21 * a[i1 + k] + R22 * b[i1 + k] + R23 * c[i1 + k];
        double R31 = sg * sb, R32 = -sg * cb * ca - cg * sa, R33 = -sg * cb * sa + cg * ca;
        for (int k = 0; k < 3; k++) cd[k] = R31 * a[i1 + k] + R32 * b[i1 + k] + R33 * c[i1 + k];
      } else {
        // alpha_p / gamma_p keep their previous values (func.cpp:640-647)
        alp = S.alpha_p[ic];
        gap = S.gamma_p[ic];
        for (int k = 0; k < 3; k++) { bd[k] = b[i1 + k]; cd[k] = c[i1 + k]; }
      }
      double ada = clamp1(ad[0] * a[f1] + ad[1] * a[f2] + ad[2] * a[f3]);
      double be = acos(ada);
      sb = sin(be);
      double x;
      if (be >= 1e-10) x = (a[f1] * bd[0] + a[f2] * bd[1] + a[f3] * bd[2]) / sb;
      else x = (b[f1] * bd[0] + b[f2] * bd[1] + b[f3] * bd[2]);
      double Ac = acos(clamp1(x));
      double y = a[f1] * cd[0] + a[f2] * cd[1] + a[f3] * cd[2];
      double al = (y >= 0) ? Ac : -Ac;
      x = clamp1((bd[0] * b[f1] + bd[1] * b[f2] + bd[2] * b[f3] + cd[0] * c[f1] + cd[1] * c[f2] + cd[2] * c[f3]) /
                 (1.0 + ada));
      double apg = acos(x);
      y = (cd[0] * b[f1] + cd[1] * b[f2] + cd[2] * b[f3] - (bd[0] * c[f1] + bd[1] * c[f2] + bd[2] * c[f3])) / (1.0 + ada);
      for (int k = 0; k < 3; k++) { S.a_dna[c1 + k] = ad[k]; S.b_dna[c1 + k] = bd[k]; S.c_dna[c1 + k] = cd[k]; }
      S.beta_p[ic] = bp;
      S.alpha_p[ic] = alp;
      S.gamma_p[ic] = gap;
      S.beta[i] = be;
      S.alpha[i] = al;
      S.gamma[i] = (y >= 0.0) ? apg - al : -apg - al;
    }
  }
  // tail bend angles (func.cpp:1763-1790, bounds test first)
  else if (g < n - 1 + M.n_tail) {
    const int i = g - (n - 1);
    const double* rt = S.r_t;
    double v = 0.0;
    if (i < M.n_tail - 2 && M.t_grp[i] == M.t_grp[i + 1] && M.t_grp[i] == M.t_grp[i + 2]) {
      double x12 = rt[i * 3] - rt[i * 3 + 3], y12 = rt[i * 3 + 1] - rt[i * 3 + 4], z12 = rt[i * 3 + 2] - rt[i * 3 + 5];
      double r12 = sqrt(x12 * x12 + y12 * y12 + z12 * z12);
      double x32 = rt[i * 3 + 6] - rt[i * 3 + 3], y32 = rt[i * 3 + 7] - rt[i * 3 + 4], z32 = rt[i * 3 + 8] - rt[i * 3 + 5];
      double r32 = sqrt(x32 * x32 + y32 * y32 + z32 * z32);
      v = acos((x12 * x32 + y12 * y32 + z12 * z32) / (r12 * r32));
    }
    S.beta_t[i] = v;
  }
  // LH bend angles (func.cpp:2062-2089)
  else if (g < n - 1 + M.n_tail + M.n_LH) {
    const int i = g - (n - 1) - M.n_tail;
    const double* rl = S.r_lh;
    double v = 0.0;
    if ((i % M.n_lh_c != 0) && (i % M.n_lh_c != M.n_lh_c - 1)) {
      double x12 = rl[i * 3 - 3] - rl[i * 3], y12 = rl[i * 3 - 2] - rl[i * 3 + 1], z12 = rl[i * 3 - 1] - rl[i * 3 + 2];
      double r12 = sqrt(x12 * x12 + y12 * y12 + z12 * z12);
      double x32 = rl[i * 3 + 3] - rl[i * 3], y32 = rl[i * 3 + 4] - rl[i * 3 + 1], z32 = rl[i * 3 + 5] - rl[i * 3 + 2];
      double r32 = sqrt(x32 * x32 + y32 * y32 + z32 * z32);
      v = acos((x12 * x32 + y12 * y32 + z12 * z32) / (r12 * r32));
    }
    S.beta_lh[i] = v;
  }
}

// rotation_cal + rotate for one chain bead (thread per bead)
__global__ void k_rotate(DevModel M, const double* __restrict__ T, const double* __restrict__ rr,
                         const double* __restrict__ a, const double* __restrict__ b, const double* __restrict__ c,
                         double* an, double* bn, double* cn) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M.n) return;
  double w[3];
  if (M.type[i] != 0) {
    for (int x = 0; x < 3; x++) w[x] = M.dt * T[3 * i + x] / (8 * kPi * kEta * 125.0) + rr[3 * i + x];
  } else {
    w[0] = M.dt * T[3 * i] / (4 * kPi * kEta * kRh * kRh * kLo) + rr[3 * i];
    w[1] = 0.0;
    w[2] = 0.0;
  }
  V3 A = ld3(a + 3 * i), B = ld3(b + 3 * i), C = ld3(c + 3 * i);
  double wa = w[0], wb = w[1], wc = w[2];
  double wa2 = wa * wa, wb2 = wb * wb, wc2 = wc * wc, z2 = wa2 + wb2 + wc2, z = sqrt(z2);
  double czt = cos(z * 1.0), szt = sin(z * 1.0), om = 1.0 - czt;
  if (z2 > 0.0) {
    double g1 = ((wb2 + wc2) * czt + wa2) / z2, g2 = wa * wb * om / z2 + wc * szt / z, g3 = wa * wc * om / z2 - wb * szt / z;
    st3(an + 3 * i, V3{g1 * A.x + g2 * B.x + g3 * C.x, g1 * A.y + g2 * B.y + g3 * C.y, g1 * A.z + g2 * B.z + g3 * C.z});
    g1 = wa * wb * om / z2 - wc * szt / z; g2 = ((wa2 + wc2) * czt + wb2) / z2; g3 = wb * wc * om / z2 + wa * szt / z;
    st3(bn + 3 * i, V3{g1 * A.x + g2 * B.x + g3 * C.x, g1 * A.y + g2 * B.y + g3 * C.y, g1 * A.z + g2 * B.z + g3 * C.z});
    g1 = wa * wc * om / z2 + wb * szt / z; g2 = wb * wc * om / z2 - wa * szt / z; g3 = ((wa2 + wb2) * czt + wc2) / z2;
    st3(cn + 3 * i, V3{g1 * A.x + g2 * B.x + g3 * C.x, g1 * A.y + g2 * B.y + g3 * C.y, g1 * A.z + g2 * B.z + g3 * C.z});
  } else {
    st3(an + 3 * i, A); st3(bn + 3 * i, B); st3(cn + 3 * i, C);
  }
}

// Drift + noise for one bead (a warp per bead): x_new = x + rd + del * D_ss F_s,
// D_ss the RPY block of the bead's own species (chain, tails or LH).
// The lanes split the partner loop; partial sums are combined in a fixed
// butterfly order so the result is deterministic.
__global__ void k_translate(DevModel M, const double* __restrict__ r_all, const double* __restrict__ Fc,
                            const double* __restrict__ Ft, const double* __restrict__ Fl, const double* __restrict__ rd,
                            const double* __restrict__ r0, const double* __restrict__ rt0,
                            const double* __restrict__ rl0, double* r1, double* rt1, double* rl1) {
  int lane = threadIdx.x & 31;
  int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= M.n_D) return;
  int lo, hi;
  const double* F;
  if (i < M.n) { lo = 0; hi = M.n; F = Fc; }
  else if (i < M.n + M.n_tail) { lo = M.n; hi = M.n + M.n_tail; F = Ft; }
  else { lo = M.n + M.n_tail; hi = M.n_D; F = Fl; }
  V3 ri = ld3(r_all + 3 * i);
  double radi = M.rad_all[i];
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int j = lo + lane; j < hi; j += 32) {
    const double* f = F + 3 * (j - lo);
    if (j == i) {
      double d = M.a1 / radi;
      s0 = s0 + M.del * d * f[0];
      s1 = s1 + M.del * d * f[1];
      s2 = s2 + M.del * d * f[2];
      continue;
    }
    V3 rj = ld3(r_all + 3 * j);
    V3 sij{ri.x - rj.x, ri.y - rj.y, ri.z - rj.z};
    double ssq = sij.x * sij.x + sij.y * sij.y + sij.z * sij.z;
    double s = sqrt(ssq);
    double radj = M.rad_all[j];
    double Db[3][3];
    rpy_block(sij, ssq, s, radi, radj, M.a1, M.a2, Db);
    for (int l = 0; l < 3; l++) {
      double fl = f[l];
      s0 = s0 + M.del * Db[0][l] * fl;
      s1 = s1 + M.del * Db[1][l] * fl;
      s2 = s2 + M.del * Db[2][l] * fl;
    }
    }
  for (int o = 16; o > 0; o >>= 1) {
    s0 = s0 + __shfl_xor_sync(0xffffffffu, s0, o);
    s1 = s1 + __shfl_xor_sync(0xffffffffu, s1, o);
    s2 = s2 + __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if (lane == 0) {
    double* out;
    const double* x0;
    int li;
    if (i < M.n) { out = r1; x0 = r0; li = i; }
    else if (i < M.n + M.n_tail) { out = rt1; x0 = rt0; li = i - M.n; }
    else { out = rl1; x0 = rl0; li = i - M.n - M.n_tail; }
    out[3 * li] = x0[3 * li] + rd[3 * i] + s0;
    out[3 * li + 1] = x0[3 * li + 1] + rd[3 * i + 1] + s1;
    out[3 * li + 2] = x0[3 * li + 2] + rd[3 * i + 2] + s2;
  }
}

// Mixed path: the same drift in FP32 arithmetic.  Separations from the
// double-float positions (hi differences plus lo differences), RPY blocks in
// FP32, each lane's terms summed in runs of 32 with the runs added under
// Kahan compensation (no FP64 in the pair loop: an FP64 operation costs as
// much as ~64 FP32 ones on GB300); the lane totals are reduced in FP64.  One
// warp per bead, 8 beads per CTA; the other beads' positions and forces are
// staged through shared memory in tiles shared by the CTA's warps.
constexpr int kTrTile = 256;
__device__ __forceinline__ void species_range(const DevModel& M, int i, int& lo, int& hi) {
  if (i < M.n) { lo = 0; hi = M.n; }
  else if (i < M.n + M.n_tail) { lo = M.n; hi = M.n + M.n_tail; }
  else { lo = M.n + M.n_tail; hi = M.n_D; }
}
__global__ void __launch_bounds__(256) k_translate_mx(DevModel M, const float4* __restrict__ qh,
                                                      const float4* __restrict__ ql, const float4* __restrict__ qf,
                                                      const double* __restrict__ rd, const double* __restrict__ r0,
                                                      const double* __restrict__ rt0, const double* __restrict__ rl0,
                                                      double* r1, double* rt1, double* rl1) {
  __shared__ float4 sh[kTrTile], sl[kTrTile], sf[kTrTile];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i0 = blockIdx.x * 8, i = i0 + warp;
  const bool active = i < M.n_D;
  int lo = 0, hi = 0, clo, chi, tmp;
  if (active) species_range(M, i, lo, hi);
  species_range(M, i0, clo, tmp);                      // the CTA's beads span [clo, chi)
  species_range(M, min(i0 + 7, M.n_D - 1), tmp, chi);
  const float4 hi_i = active ? qh[i] : make_float4(0.f, 0.f, 0.f, 1.f), lo_i = active ? ql[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float a1f = (float)M.a1, a2f = (float)M.a2, delf = (float)M.del;
  float run[3] = {0.f, 0.f, 0.f}, ks[3] = {0.f, 0.f, 0.f}, kc[3] = {0.f, 0.f, 0.f};
  int cnt = 0;
  for (int base = clo; base < chi; base += kTrTile) {
    __syncthreads();
    for (int x = threadIdx.x; x < kTrTile && base + x < chi; x += blockDim.x) {
      sh[x] = qh[base + x];
      sl[x] = ql[base + x];
      sf[x] = qf[base + x];
    }
    __syncthreads();
    if (!active) continue;
    const int je = min(hi, base + kTrTile);
    for (int j = max(lo, base) + lane; j < je; j += 32) {
      const int x = j - base;
      const float4 f = sf[x];
      if (j == i) {
        const float d = delf * (a1f / hi_i.w);
        run[0] += d * f.x;
        run[1] += d * f.y;
        run[2] += d * f.z;
      } else {
        const float4 hj = sh[x], lj = sl[x];
        float Db[3][3];
        rpy_block_f((hi_i.x - hj.x) + (lo_i.x - lj.x), (hi_i.y - hj.y) + (lo_i.y - lj.y),
                    (hi_i.z - hj.z) + (lo_i.z - lj.z), hi_i.w, hj.w, a1f, a2f, Db);
        run[0] += delf * (Db[0][0] * f.x + Db[0][1] * f.y + Db[0][2] * f.z);
        run[1] += delf * (Db[1][0] * f.x + Db[1][1] * f.y + Db[1][2] * f.z);
        run[2] += delf * (Db[2][0] * f.x + Db[2][1] * f.y + Db[2][2] * f.z);
      }
      if (++cnt == 32) {
#pragma unroll
        for (int q = 0; q < 3; q++) {
          const float y = run[q] - kc[q], t = ks[q] + y;
          kc[q] = (t - ks[q]) - y;
          ks[q] = t;
          run[q] = 0.f;
        }
        cnt = 0;
      }
    }
  }
  if (!active) return;
  double s[3];
#pragma unroll
  for (int q = 0; q < 3; q++) {
    const float y = run[q] - kc[q], t = ks[q] + y;
    s[q] = (double)t - (double)((t - ks[q]) - y);
  }
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int q = 0; q < 3; q++) s[q] = s[q] + __shfl_xor_sync(0xffffffffu, s[q], o);
  }
  if (lane == 0) {
    double* out;
    const double* x0;
    int li;
    if (i < M.n) { out = r1; x0 = r0; li = i; }
    else if (i < M.n + M.n_tail) { out = rt1; x0 = rt0; li = i - M.n; }
    else { out = rl1; x0 = rl0; li = i - M.n - M.n_tail; }
    out[3 * li] = x0[3 * li] + rd[3 * i] + s[0];
    out[3 * li + 1] = x0[3 * li + 1] + rd[3 * i + 1] + s[1];
    out[3 * li + 2] = x0[3 * li + 2] + rd[3 * i + 2] + s[2];
  }
}

// the move's forces in FP32, per bead of the tensor (chain | tails | LH)
__global__ void k_forces_f32(int n, int nt, int nl, const double* __restrict__ F, const double* __restrict__ tF,
                             const double* __restrict__ lF, float4* qf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n + nt + nl) return;
  const double* p = i < n ? F + 3 * i : (i < n + nt ? tF + 3 * (i - n) : lF + 3 * (i - n - nt));
  qf[i] = make_float4((float)p[0], (float)p[1], (float)p[2], 0.f);
}

// the tensor beads' positions as double-float pairs, radius in .w
__global__ void k_rall_mirror(int nD, const double* __restrict__ r_all, const double* __restrict__ rad, float4* qh,
                              float4* ql) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nD) return;
  const double x = r_all[3 * i], y = r_all[3 * i + 1], z = r_all[3 * i + 2];
  const float hx = (float)x, hy = (float)y, hz = (float)z;
  qh[i] = make_float4(hx, hy, hz, (float)rad[i]);
  ql[i] = make_float4((float)(x - hx), (float)(y - hy), (float)(z - hz), 0.f);
}

__global__ void k_average(int n3, int nt3, int nl3, const double* F0, const double* T0, const double* tF0,
                          const double* lF0, const double* F1, const double* T1, const double* tF1, const double* lF1,
                          double* F, double* T, double* tF, double* lF) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n3) { F[i] = 0.5 * (F0[i] + F1[i]); T[i] = 0.5 * (T0[i] + T1[i]); }
  if (i < nt3) tF[i] = 0.5 * (tF0[i] + tF1[i]);
  if (i < nl3) lF[i] = 0.5 * (lF0[i] + lF1[i]);
}

__global__ void k_gather_rall(int n, int nt, int nl, const double* r, const double* rt, const double* rl,
                              double* ra) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int n3 = 3 * n, nt3 = 3 * nt, nl3 = 3 * nl;
  if (i < n3) ra[i] = r[i];
  else if (i < n3 + nt3) ra[i] = rt[i - n3];
  else if (i < n3 + nt3 + nl3) ra[i] = rl[i - n3 - nt3];
}

inline int cdiv(int a, int b) { return (a + b - 1) / b; }

}  // namespace

namespace bdk {

void frames(const DevModel& M, DevState& S, cudaStream_t st) {
  const int nb = M.n - 1 > 0 ? M.n - 1 : 0;
  if (nb > 0) k_frames_dna<<<cdiv(nb, kFrameThreads), kFrameThreads, 0, st>>>(M, S);
  const int tot = nb + M.n_tail + M.n_LH;
  if (tot > 0) k_frames_angles<<<cdiv(tot, kFrameThreads), kFrameThreads, 0, st>>>(M, S);
}

void frame_angles(const DevModel& M, DevState& S, cudaStream_t st) {
  const int nb = M.n - 1 > 0 ? M.n - 1 : 0;
  const int tot = nb + M.n_tail + M.n_LH;
  if (tot > 0) k_frames_angles<<<cdiv(tot, kFrameThreads), kFrameThreads, 0, st>>>(M, S);
}

void gather_rall(const DevModel& M, const DevState& X, double* r_all, const DevScratch* S, cudaStream_t st) {
  int tot = 3 * M.n_D;
  k_gather_rall<<<cdiv(tot, 256), 256, 0, st>>>(M.n, M.n_tail, M.n_LH, X.r, X.r_t, X.r_lh, r_all);
  if (S) k_rall_mirror<<<cdiv(M.n_D, 256), 256, 0, st>>>(M.n_D, r_all, M.rad_all, S->qh, S->ql);
}

// X: state the move starts from; Y: receives the moved state.  r_all must
// hold X's positions (the tensor is evaluated at the start configuration).
void rotate_translate(const DevModel& M, const DevState& X, DevState& Y, const DevForces& Fo, const double* rr,
                      const double* rd, const double* r_all, int mixed, const DevScratch& S, cudaStream_t st) {
  k_rotate<<<cdiv(M.n, kFrameThreads), kFrameThreads, 0, st>>>(M, Fo.T, rr, X.a, X.b, X.c, Y.a, Y.b, Y.c);
  if (mixed) {
    k_forces_f32<<<cdiv(M.n_D, 256), 256, 0, st>>>(M.n, M.n_tail, M.n_LH, Fo.F, Fo.tF, Fo.lF, S.qf);
    k_translate_mx<<<cdiv(M.n_D * 32, 256), 256, 0, st>>>(M, S.qh, S.ql, S.qf, rd, X.r, X.r_t, X.r_lh, Y.r, Y.r_t,
                                                           Y.r_lh);
  } else {
    k_translate<<<cdiv(M.n_D * 32, 256), 256, 0, st>>>(M, r_all, Fo.F, Fo.tF, Fo.lF, rd, X.r, X.r_t, X.r_lh, Y.r,
                                                        Y.r_t, Y.r_lh);
  }
}

void average_forces(const DevModel& M, const DevForces& A, const DevForces& B, DevForces& o, cudaStream_t st) {
  int mx = 3 * M.n;
  if (3 * M.n_tail > mx) mx = 3 * M.n_tail;
  if (3 * M.n_LH > mx) mx = 3 * M.n_LH;
  k_average<<<cdiv(mx, 256), 256, 0, st>>>(3 * M.n, 3 * M.n_tail, 3 * M.n_LH, A.F, A.T, A.tF, A.lF, B.F, B.T, B.tF,
                                            B.lF, o.F, o.T, o.tF, o.lF);
}

}  // namespace bdk
