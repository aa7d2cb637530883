// Device-side pair and bonded primitives of the chromatin BD model.
// Formulas and operation order follow the reference CPU physics
// (BD_cuda/func.cpp line numbers given per function); the translation units
// that include this header are built with -fmad=false so that FP64 results
// round exactly as the reference's do.
#pragma once
#include <cuda_runtime.h>

namespace bdp {

constexpr double kPi = 3.141592653589790;   // constants.h:6
constexpr double kLo = 3.0;
constexpr double kRo = 4.8;
constexpr double kD1 = 1.8;
constexpr double kTheta = 1.2 * kPi / 2;
constexpr double kEta = 1.137076e-12;
constexpr double kRh = 1.2;

struct V3 {
  double x, y, z;
};
__device__ __forceinline__ V3 ld3(const double* p) { return V3{p[0], p[1], p[2]}; }
__device__ __forceinline__ void st3(double* p, V3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
__device__ __forceinline__ double c3(const V3& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

__device__ __forceinline__ double clamp09(double v) {
  if (v > 0.9) v = 0.9;
  if (v < -0.9) v = -0.9;
  return v;
}
__device__ __forceinline__ double clamp1(double v) {
  if (v > 1.0) v = 1.0;
  if (v < -1.0) v = -1.0;
  return v;
}

__device__ __forceinline__ double dist3(const V3& a, const V3& b) {
  return sqrt((a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y) + (a.z - b.z) * (a.z - b.z));
}

// body point r + a p0 + b p1 + c p2 (func.cpp:1364 and copies)
__device__ __forceinline__ V3 body(const V3& r, const V3& a, const V3& b, const V3& c, const double* p) {
  return V3{r.x + a.x * p[0] + b.x * p[1] + c.x * p[2], r.y + a.y * p[0] + b.y * p[1] + c.y * p[2],
            r.z + a.z * p[0] + b.z * p[1] + c.z * p[2]};
}

// func.cpp:134-151: force on c1 (f1); the force on c2 is -f1 exactly
__device__ __forceinline__ V3 stretch_f1(double h, const V3& c1, const V3& c2, double l0, double& E) {
  double d = dist3(c1, c2);
  E = E + h * (d - l0) * (d - l0) / 2;
  double f = -h * (d - l0);
  return V3{f * (c1.x - c2.x) / d, f * (c1.y - c2.y) / d, f * (c1.z - c2.z) / d};
}
// func.cpp:148 form of the force on c2 (bitwise -f1)
__device__ __forceinline__ V3 stretch_f2(double h, const V3& c1, const V3& c2, double l0) {
  double d = dist3(c1, c2);
  double f = -h * (d - l0);
  return V3{-f * (c1.x - c2.x) / d, -f * (c1.y - c2.y) / d, -f * (c1.z - c2.z) / d};
}

__device__ __forceinline__ V3 cross(const V3& u, const V3& v) {
  return V3{u.y * v.z - u.z * v.y, -1 * (u.x * v.z - u.z * v.x), u.x * v.y - u.y * v.x};
}
__device__ __forceinline__ double nrm(const V3& v) {
  double s = 0;
  s = s + v.x * v.x + v.y * v.y + v.z * v.z;
  return sqrt(s);
}

// func.cpp:153-196: forces on the three beads of an angle
__device__ __forceinline__ void bend3(double g, double beta, double beta0, const V3& c1, const V3& c2, const V3& c3,
                                      V3& f1, V3& f2, V3& f3, double& E) {
  E = E + g * (beta - beta0) * (beta - beta0) / 2;
  double f = -g * (beta - beta0);
  double d1 = dist3(c1, c2), d2 = dist3(c2, c3);
  V3 ji{c2.x - c1.x, c2.y - c1.y, c2.z - c1.z};
  V3 jk{c2.x - c3.x, c2.y - c3.y, c2.z - c3.z};
  V3 kj{c3.x - c2.x, c3.y - c2.y, c3.z - c2.z};
  V3 ri = cross(ji, cross(ji, jk));
  double nri = nrm(ri);
  f1 = V3{(f / d1) * ri.x / nri, (f / d1) * ri.y / nri, (f / d1) * ri.z / nri};
  f2 = V3{-(f / d1) * ri.x / nri, -(f / d1) * ri.y / nri, -(f / d1) * ri.z / nri};
  V3 rk = cross(kj, cross(ji, jk));
  double nrk = nrm(rk);
  f2 = V3{f2.x - (f / d2) * rk.x / nrk, f2.y - (f / d2) * rk.y / nrk, f2.z - (f / d2) * rk.z / nrk};
  f3 = V3{(f / d2) * rk.x / nrk, (f / d2) * rk.y / nrk, (f / d2) * rk.z / nrk};
}

// func.cpp:278-300, 318-340, 342-371: DH (cut 7), LJ (cut 4), both; force
// on c1, clamped per component to +-0.9.  The force on c2 is the same call
// with the beads swapped (bitwise the negation).
template <bool DH, bool LJ>
__device__ __forceinline__ V3 pair_f1(double q1, double q2, double eps, double kappa, double kev, double sig,
                                      const V3& c1, const V3& c2, double* E) {
  double f = 0.0, fl = 0.0;
  double d = dist3(c1, c2);
  if (DH && d < 7.0) {
    double ex = exp(-kappa * d);
    f = ((q1 * q2 * (kappa * d + 1)) / (4 * kPi * eps * d * d)) * ex;
    if (E) *E = *E + (q1 * q2 / (4 * kPi * eps * d)) * ex;
  }
  if (LJ && d < 4.0) {
    fl = -kev * ((6 * pow(sig, 6)) / pow(d, 7) - (12 * pow(sig, 12)) / pow(d, 13));
    if (E) *E = *E + kev * (pow(sig / d, 12) - pow(sig / d, 6));
  }
  double t = DH && LJ ? f + fl : (DH ? f : fl);
  return V3{clamp09(t * (c1.x - c2.x) / d), clamp09(t * (c1.y - c2.y) / d), clamp09(t * (c1.z - c2.z) / d)};
}

__device__ __forceinline__ float clamp09f(float v) { return fminf(fmaxf(v, -0.9f), 0.9f); }

// The Debye-Hueckel (7 nm) and Lennard-Jones (4 nm) cut-offs truncate the
// pair force without a shift, so it jumps there.  An FP32 distance carries an
// error of ~2e-6 nm near 7 nm; a pair closer than that to a cut-off can fall
// on the other side than in the FP64 path and move a bead by the whole jump.
// Inside this guard band (50x that error) the FP32 pair terms decide the
// cut-offs from the FP64 distance instead; the band holds ~3e-5 of the pairs.
constexpr float kCutGuard = 1e-4f;
__device__ __forceinline__ bool near_cutoff(float d) {
  return fabsf(d - 7.f) < kCutGuard || fabsf(d - 4.f) < kCutGuard;
}

// Mixed-precision form of pair_f1 for the tensor-core step: the separation
// is formed in FP64 (large absolute coordinates cost nothing), the rest of
// the pair in FP32 (sqrt, exp, powers of sigma/d by multiplication), and the
// result is widened back for FP64 accumulation.  Same formulas as pair_f1.
template <bool DH, bool LJ>
__device__ __forceinline__ V3 pair_f1_mx(double q1, double q2, double eps, double kappa, double kev, double sig,
                                         const V3& c1, const V3& c2, double* E) {
  const float dx = (float)(c1.x - c2.x), dy = (float)(c1.y - c2.y), dz = (float)(c1.z - c2.z);
  const float d2 = dx * dx + dy * dy + dz * dz;
  const float d = sqrtf(d2);
  bool in7 = d < 7.f, in4 = d < 4.f;
  if (near_cutoff(d)) {  // the cut-offs make the force jump: decide as the FP64 path does
    const double d64 = dist3(c1, c2);
    in7 = d64 < 7.0, in4 = d64 < 4.0;
  }
  float t = 0.f;
  if (DH && in7) {
    const float kap = (float)kappa;
    const float qq = (float)(q1 * q2 / (4 * kPi * eps));
    const float ex = expf(-kap * d);
    t = qq * (kap * d + 1.f) * ex / d2;
    if (E) *E = *E + (double)(qq * ex / d);
  }
  if (LJ && in4) {
    const float sr = (float)sig / d, sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
    const float kv = (float)kev;
    t = t - kv * (6.f * sr6 - 12.f * sr12) / d;
    if (E) *E = *E + (double)(kv * (sr12 - sr6));
  }
  const float w = t / d;
  return V3{(double)clamp09f(w * dx), (double)clamp09f(w * dy), (double)clamp09f(w * dz)};
}

// Dispatch on the step's precision.
template <bool DH, bool LJ, bool MX>
__device__ __forceinline__ V3 pairF(double q1, double q2, double eps, double kappa, double kev, double sig,
                                    const V3& c1, const V3& c2, double* E) {
  if constexpr (MX) return pair_f1_mx<DH, LJ>(q1, q2, eps, kappa, kev, sig, c1, c2, E);
  else return pair_f1<DH, LJ>(q1, q2, eps, kappa, kev, sig, c1, c2, E);
}

// func.cpp:374-394: torque about the body frame from a force at pf
__device__ __forceinline__ V3 torque_abs(const V3& F, const V3& pf, const V3& pc, const V3& a, const V3& b,
                                         const V3& c) {
  double c0 = (pf.x - pc.x) * a.x + (pf.y - pc.y) * a.y + (pf.z - pc.z) * a.z;
  double c1 = (pf.x - pc.x) * b.x + (pf.y - pc.y) * b.y + (pf.z - pc.z) * b.z;
  double c2 = (pf.x - pc.x) * c.x + (pf.y - pc.y) * c.y + (pf.z - pc.z) * c.z;
  double fa = a.x * F.x + a.y * F.y + a.z * F.z;
  double fb = b.x * F.x + b.y * F.y + b.z * F.z;
  double fc = c.x * F.x + c.y * F.y + c.z * F.z;
  return V3{fc * c1 - fb * c2, fa * c2 - fc * c0, fb * c0 - fa * c1};
}

// func.cpp:396-410: torque from a force at body-frame position comp
__device__ __forceinline__ V3 torque_rel(const V3& F, const double* comp, const V3& a, const V3& b, const V3& c) {
  double fa = a.x * F.x + a.y * F.y + a.z * F.z;
  double fb = b.x * F.x + b.y * F.y + b.z * F.z;
  double fc = c.x * F.x + c.y * F.y + c.z * F.z;
  return V3{fc * comp[1] - fb * comp[2], fa * comp[2] - fc * comp[0], fb * comp[0] - fa * comp[1]};
}

__device__ __forceinline__ void acc(V3& s, const V3& v) { s.x = s.x + v.x; s.y = s.y + v.y; s.z = s.z + v.z; }
__device__ __forceinline__ void dec(V3& s, const V3& v) { s.x = s.x - v.x; s.y = s.y - v.y; s.z = s.z - v.z; }

// RPY tensor element (row 3i+k, column 3j+l) for a bead pair i != j, with
// sij = r_i - r_j (either sign).  func.cpp:753-799 writes each off-diagonal
// element twice, leaving the value computed with the larger component
// index first; this returns that value.
__device__ __forceinline__ double rpy_elem(const V3& sij, double ssq, double s, double radi, double radj, double a1,
                                           double a2, int k, int l) {
  int kk = k > l ? k : l, ll = k > l ? l : k;
  double sk = c3(sij, kk), sl = c3(sij, ll);
  if (s >= radi + radj) {
    double f = (radi * radi + radj * radj) / ssq;
    double f1 = 1.0 + f / 3, f2 = 1.0 - f;
    if (k == l) return (a2 / s) * (f1 + f2 * sk * sk / ssq);
    return (a2 / s) * (f2 * sk * sl / ssq);
  }
  double se = pow((radi * radi * radi + radj * radj * radj) / 2.0, 1.0 / 3);
  if (k == l) return (a1 / se) * (1.0 - 9.0 * sqrt(ssq) / (32 * se) + 3.0 * sk * sk / (32.0 * se * sqrt(ssq)));
  return (a1 / se) * (3.0 * sk * sl / (32.0 * se * sqrt(ssq)));
}

// The full 3 x 3 block (same per-element expressions as rpy_elem, shared
// subexpressions evaluated once): out[k][l].
__device__ __forceinline__ void rpy_block(const V3& sij, double ssq, double s, double radi, double radj, double a1,
                                          double a2, double (&out)[3][3]) {
  const double sv[3] = {sij.x, sij.y, sij.z};
  if (s >= radi + radj) {
    double f = (radi * radi + radj * radj) / ssq;
    double f1 = 1.0 + f / 3, f2 = 1.0 - f;
    double as = a2 / s;
#pragma unroll
    for (int k = 0; k < 3; k++) out[k][k] = as * (f1 + f2 * sv[k] * sv[k] / ssq);
    double o10 = as * (f2 * sv[1] * sv[0] / ssq);
    double o20 = as * (f2 * sv[2] * sv[0] / ssq);
    double o21 = as * (f2 * sv[2] * sv[1] / ssq);
    out[1][0] = out[0][1] = o10;
    out[2][0] = out[0][2] = o20;
    out[2][1] = out[1][2] = o21;
    return;
  }
  double se = pow((radi * radi * radi + radj * radj * radj) / 2.0, 1.0 / 3);
  double as = a1 / se;
  double rs = sqrt(ssq);
#pragma unroll
  for (int k = 0; k < 3; k++) out[k][k] = as * (1.0 - 9.0 * rs / (32 * se) + 3.0 * sv[k] * sv[k] / (32.0 * se * rs));
  double o10 = as * (3.0 * sv[1] * sv[0] / (32.0 * se * rs));
  double o20 = as * (3.0 * sv[2] * sv[0] / (32.0 * se * rs));
  double o21 = as * (3.0 * sv[2] * sv[1] / (32.0 * se * rs));
  out[1][0] = out[0][1] = o10;
  out[2][0] = out[0][2] = o20;
  out[2][1] = out[1][2] = o21;
}

// FP32 form of rpy_block for the mixed path (drift and tensor; separation
// given in FP32, formed from double-float positions).
__device__ __forceinline__ void rpy_block_f(float sx, float sy, float sz, float radi, float radj, float a1, float a2,
                                            float (&out)[3][3]) {
  const float sv[3] = {sx, sy, sz};
  const float ssq = sx * sx + sy * sy + sz * sz;
  const float inv_s = rsqrtf(ssq);  // one reciprocal square root instead of a root and three divisions
  const float s = ssq * inv_s;
  if (s >= radi + radj) {
    const float inv_ssq = inv_s * inv_s;
    const float f = (radi * radi + radj * radj) * inv_ssq;
    const float f1 = 1.f + f * (1.f / 3.f), f2 = 1.f - f;
    const float as = a2 * inv_s, w = as * f2 * inv_ssq;
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
      for (int l = 0; l < 3; l++) out[k][l] = w * sv[k] * sv[l] + (k == l ? as * f1 : 0.f);
    return;
  }
  const float se = cbrtf((radi * radi * radi + radj * radj * radj) / 2.f);
  const float as = a1 / se, w = as * 3.f / (32.f * se * s);
#pragma unroll
  for (int k = 0; k < 3; k++)
#pragma unroll
    for (int l = 0; l < 3; l++) out[k][l] = w * sv[k] * sv[l] + (k == l ? as * (1.f - 9.f * s / (32.f * se)) : 0.f);
}

}  // namespace bdp
