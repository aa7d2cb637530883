// The force-field terms of the chromatin BD step (no linker histone) as
// scalar-generic functions, for the adjoint kernels.
//
// Each function restates one piece of the reference CPU physics
// (BD_cuda/func.cpp, line numbers per function) as a function of a small
// set of inputs, templated on the scalar type T: float / double evaluate it,
// adj::Dual<R, W> differentiates it.  The adjoint kernels contract these
// local Jacobians with the output adjoints (adj_dual.cuh).  The formulas are
// the same as the forward kernels'; the operation order is not kept (the
// adjoint needs derivatives, not bitwise values).
//
// Bead frame layout used throughout: x[0..2] = r, x[3..5] = a, x[6..8] = b,
// x[9..11] = c.
#pragma once
#include "adj_dual.cuh"

namespace adj {

constexpr double kPi = 3.141592653589790;  // constants.h:6-12
constexpr double kLo = 3.0;
constexpr double kRo = 4.8;
constexpr double kD1 = 1.8;
constexpr double kTheta = 1.2 * kPi / 2;
constexpr double kEta = 1.137076e-12;
constexpr double kRh = 1.2;

template <class T>
ADJ_HD T clamp09(const T& v) {
  if (val(v) > 0.9) return T(0.9);
  if (val(v) < -0.9) return T(-0.9);
  return v;
}
template <class T>
ADJ_HD T clamp1(const T& v) {
  if (val(v) > 1.0) return T(1.0);
  if (val(v) < -1.0) return T(-1.0);
  return v;
}

// internal coordinates of chain bead i (func.cpp:448-685, second pass, plus
// the bond length of the first pass), from the refreshed frames of beads i
// and i+1
template <class T>
struct Ang {
  T alpha, beta, gamma, length;
  T ad[3], bd[3], cd[3];
  T alpha_p, beta_p, gamma_p;
};

template <class T>
ADJ_HD void angles(int ti, int tn, const T* xi, const T* xn, Ang<T>& o) {
  using R = typename RealOf<T>::type;
  const R si = R(sin(kTheta)), co = R(cos(kTheta));
  const T *r = xi, *a = xi + 3, *b = xi + 6, *c = xi + 9;
  const T *rn = xn, *an = xn + 3, *bn = xn + 6, *cn = xn + 9;
  if (ti == 0) {
    T af[3], bf[3], rf[3];
    for (int x = 0; x < 3; x++) {
      if (tn == 0) {
        af[x] = an[x];
        bf[x] = bn[x];
        rf[x] = rn[x] - r[x];
      } else {
        af[x] = co * an[x] + si * bn[x];
        bf[x] = -si * an[x] + co * bn[x];
        rf[x] = rn[x] - R(kRo) * bf[x] + R(kD1) * cn[x] - r[x];
      }
    }
    o.length = norm3(rf);
    T ada = clamp1(dot3(a, af));
    o.beta = vacos(ada);
    T sb = vsin(o.beta);
    T x = (val(o.beta) > 1e-10) ? dot3(af, b) / sb : dot3(bf, b);
    x = clamp1(x);
    T Ac = vacos(x);
    T y = dot3(af, c);
    o.alpha = (val(y) >= 0) ? Ac : -Ac;
    x = clamp1((dot3(b, bf) + dot3(c, cn)) / (ada + R(1)));
    T apg = vacos(x);
    y = (dot3(c, bf) - dot3(b, cn)) / (ada + R(1));
    o.gamma = (val(y) >= 0.0) ? apg - o.alpha : -apg - o.alpha;
    o.alpha_p = o.beta_p = o.gamma_p = T(0.0);
    for (int k = 0; k < 3; k++) o.ad[k] = o.bd[k] = o.cd[k] = T(0.0);
  } else {
    T rf[3];
    for (int x = 0; x < 3; x++) rf[x] = rn[x] - (r[x] - R(kRo) * b[x] - R(kD1) * c[x]);
    o.length = norm3(rf);
    for (int x = 0; x < 3; x++) o.ad[x] = rf[x] / o.length;
    const T* ad = o.ad;
    T cb = clamp1(dot3(a, ad));
    o.beta_p = vacos(cb);
    T sb = vsin(o.beta_p);
    if (val(o.beta_p) >= 1e-10) {
      T bm[3];
      for (int x = 0; x < 3; x++) bm[x] = (ad[x] - cb * a[x]) / sb;
      T ca = clamp1(dot3(bm, b));
      T Ac = vacos(ca);
      T y = dot3(ad, c);
      o.alpha_p = (val(y) >= 0) ? Ac : -Ac;
      o.gamma_p = -o.alpha_p;
      T sa = vsin(o.alpha_p), sg = vsin(o.gamma_p), cg = vcos(o.gamma_p);
      T R21 = -cg * sb, R22 = cg * cb * ca - sg * sa, R23 = cg * cb * sa + sg * ca;
      T R31 = sg * sb, R32 = -sg * cb * ca - cg * sa, R33 = -sg * cb * sa + cg * ca;
      for (int x = 0; x < 3; x++) {
        o.bd[x] = R21 * a[x] + R22 * b[x] + R23 * c[x];
        o.cd[x] = R31 * a[x] + R32 * b[x] + R33 * c[x];
      }
    } else {
      o.alpha_p = o.gamma_p = T(0.0);
      for (int x = 0; x < 3; x++) {
        o.bd[x] = b[x];
        o.cd[x] = c[x];
      }
    }
    const T *bd = o.bd, *cd = o.cd;
    T ada = clamp1(dot3(ad, an));
    o.beta = vacos(ada);
    sb = vsin(o.beta);
    T x = (val(o.beta) >= 1e-10) ? dot3(an, bd) / sb : dot3(bn, bd);
    x = clamp1(x);
    T Ac = vacos(x);
    T y = dot3(an, cd);
    o.alpha = (val(y) >= 0) ? Ac : -Ac;
    x = clamp1((dot3(bd, bn) + dot3(cd, cn)) / (ada + R(1)));
    T apg = vacos(x);
    y = (dot3(cd, bn) - dot3(bd, cn)) / (ada + R(1));
    o.gamma = (val(y) >= 0.0) ? apg - o.alpha : -apg - o.alpha;
  }
}

// func.cpp:687-709 / 711-723: the bond's end points on beads i+1 and i
template <class T>
ADJ_HD void first_coord(int t, const T* x, T* rf) {
  using R = typename RealOf<T>::type;
  const R si = R(sin(kTheta)), co = R(cos(kTheta));
  for (int k = 0; k < 3; k++)
    rf[k] = (t == 0) ? x[k] : x[k] - R(kRo) * (-si * x[3 + k] + co * x[6 + k]) + R(kD1) * x[9 + k];
}
template <class T>
ADJ_HD void second_coord(int t, const T* x, T* rs) {
  using R = typename RealOf<T>::type;
  for (int k = 0; k < 3; k++) rs[k] = (t == 0) ? x[k] : x[k] - (R(kRo) * x[6 + k] + R(kD1) * x[9 + k]);
}

// func.cpp:374-394: torque of force F applied at pf on the body (pc; a, b, c)
template <class T>
ADJ_HD void torque_abs_add(const T* F, const T* pf, const T* x, T* t) {
  const T *pc = x, *a = x + 3, *b = x + 6, *c = x + 9;
  T d[3] = {pf[0] - pc[0], pf[1] - pc[1], pf[2] - pc[2]};
  T comp[3] = {dot3(d, a), dot3(d, b), dot3(d, c)};
  T fa = dot3(a, F), fb = dot3(b, F), fc = dot3(c, F);
  t[0] = t[0] + (fc * comp[1] - fb * comp[2]);
  t[1] = t[1] + (fa * comp[2] - fc * comp[0]);
  t[2] = t[2] + (fb * comp[0] - fa * comp[1]);
}

// Chain bond i: the stretching, bending and twisting forces of bond
// (i, i+1) with their torques (func.cpp:951-1195), the mechanical torque of
// bead i (func.cpp:1197-1280) and, on the last bond, the end torque of bead
// n-1 (func.cpp:1282-1285).  Inputs: beads i-1 (if has_prev), i, i+1 and the
// moduli h, g, s.  Outputs: F_i, F_{i+1}, T_i, T_{i+1}.
struct BondInfo {
  int tp, ti, tn;     // types of beads i-1, i, i+1
  int has_prev, last;
  double phi_p, phi_i;  // phi_o[i-1], phi_o[i]
};

template <class T>
ADJ_HD void bond_term(const BondInfo& k, const T* xp, const T* xi, const T* xn, const T& h, const T& g, const T& s,
                      T* out) {
  using R = typename RealOf<T>::type;
  const R si = R(sin(kTheta)), co = R(cos(kTheta));
  const R phi_p = R(k.phi_p), phi_i = R(k.phi_i);
  T *Fi = out, *Fn = out + 3, *Ti = out + 6, *Tn = out + 9;
  for (int x = 0; x < 12; x++) out[x] = T(0.0);
  Ang<T> Ai, Ap;
  angles(k.ti, k.tn, xi, xn, Ai);
  if (k.has_prev) angles(k.tp, k.ti, xp, xi, Ap);
  else Ap = Ai;  // unused
  const T *ai = xi + 3, *bi = xi + 6, *ci = xi + 9;
  const T *an = xn + 3, *bn = xn + 6;
  T rf[3], rs[3];
  first_coord(k.tn, xn, rf);
  second_coord(k.ti, xi, rs);
  auto apply = [&](const T* f1, const T* f2) {
    for (int x = 0; x < 3; x++) {
      Fi[x] = Fi[x] + f1[x];
      Fn[x] = Fn[x] + f2[x];
    }
    torque_abs_add(f1, rs, xi, Ti);
    torque_abs_add(f2, rf, xn, Tn);
  };
  T f1[3], f2[3];
  {  // stretching, func.cpp:134-151
    T dv[3] = {rs[0] - rf[0], rs[1] - rf[1], rs[2] - rf[2]};
    T d = norm3(dv);
    T f = -h * (d - R(kLo));
    for (int x = 0; x < 3; x++) {
      f1[x] = f * dv[x] / d;
      f2[x] = -f1[x];
    }
    apply(f1, f2);
  }
  {  // bending, func.cpp:198-232
    T af[3], ab[3], ao[3], beta_b;
    for (int x = 0; x < 3; x++) {
      if (k.ti == 0) {
        af[x] = (k.tn == 0) ? an[x] : co * an[x] + si * bn[x];
        ab[x] = (k.tp == 0) ? xp[3 + x] : Ap.ad[x];
        ao[x] = ai[x];
      } else {
        af[x] = an[x];
        ab[x] = ai[x];
        ao[x] = Ai.ad[x];
      }
    }
    beta_b = (k.ti == 0) ? Ap.beta : Ai.beta_p;
    const T& beta = Ai.beta;
    T g1 = (val(beta) >= 1e-10) ? beta / (vsin(beta) * Ai.length) : R(1) / Ai.length;
    T c1 = vcos(beta);
    T g2 = (val(beta_b) >= 1e-10) ? beta_b / (vsin(beta_b) * Ai.length) : R(1) / Ai.length;
    T c2 = vcos(beta_b);
    for (int x = 0; x < 3; x++) {
      T A = g1 * (af[x] - c1 * ao[x]);
      T B = g2 * (ab[x] - c2 * ao[x]);
      f1[x] = -g * (A + B);
      f2[x] = g * (A + B);
    }
    apply(f1, f2);
  }
  {  // twisting, func.cpp:234-260
    T al_b, be_b, ga_b, ga_n;
    R ph_b;
    const T *bo, *cO;
    if (k.ti == 0) {
      al_b = Ap.alpha; be_b = Ap.beta; ga_b = Ap.gamma; ph_b = phi_p; ga_n = Ap.gamma;
      bo = bi; cO = ci;
    } else {
      al_b = Ai.alpha; be_b = Ai.beta_p; ga_b = Ai.gamma; ph_b = phi_i; ga_n = Ai.gamma_p;
      bo = Ai.bd; cO = Ai.cd;
    }
    T g1 = (Ai.alpha + Ai.gamma - phi_i) * vtan(Ai.beta * R(0.5)) / Ai.length;
    T c1 = vcos(Ai.alpha), s1 = vsin(Ai.alpha);
    T g2 = (al_b + ga_b - ph_b) * vtan(be_b * R(0.5)) / Ai.length;
    T c2 = vcos(ga_n), s2 = vsin(ga_n);
    for (int x = 0; x < 3; x++) {
      T Ch = g1 * (c1 * cO[x] - s1 * bo[x]);
      T Zh = g2 * (c2 * cO[x] + s2 * bo[x]);
      f1[x] = s * (Ch + Zh);
      f2[x] = -s * (Ch + Zh);
    }
    apply(f1, f2);
  }
  // mechanical torque of bead i
  if (k.ti == 0) {
    Ti[0] = Ti[0] + s * (Ai.alpha + Ai.gamma + phi_i - Ap.alpha - Ap.gamma - phi_p);
  } else {
    const T *ad = Ai.ad, *bd = Ai.bd, *cd = Ai.cd;
    T mag = s * (Ai.alpha + Ai.gamma - phi_i);
    Ti[0] = Ti[0] + mag * dot3(ad, ai);
    Ti[1] = Ti[1] + mag * dot3(ad, bi);
    Ti[2] = Ti[2] + mag * dot3(ad, ci);
    if (k.has_prev) {
      mag = -s * (Ap.alpha + Ap.gamma - phi_p);
      Ti[0] = Ti[0] + mag * co;
      Ti[1] = Ti[1] + mag * si;
    }
    T sbp = vsin(Ai.beta_p);
    Ti[1] = Ti[1] - g * Ai.beta_p * dot3(ad, ci) / sbp;
    Ti[2] = Ti[2] + g * Ai.beta_p * dot3(ad, bi) / sbp;
    if (k.has_prev) {
      const T* ap = xp + 3;
      T ada = dot3(ap, ai), adb = dot3(ap, bi), adc = dot3(ap, ci);
      T gb = g * Ap.beta / vsin(Ap.beta);
      Ti[0] = Ti[0] + gb * (si * adc);
      Ti[1] = Ti[1] - gb * (co * adc);
      Ti[2] = Ti[2] + gb * (co * adb - si * ada);
    }
    T s1 = vsin(Ai.alpha_p), cc1 = vcos(Ai.alpha_p);
    mag = s * (Ai.alpha + Ai.gamma - phi_i) * vtan(Ai.beta_p * R(0.5));
    Ti[0] = Ti[0] - mag * (s1 * dot3(cd, ai) + cc1 * dot3(bd, ai));
    Ti[1] = Ti[1] - mag * (s1 * dot3(cd, bi) + cc1 * dot3(bd, bi));
    Ti[2] = Ti[2] - mag * (s1 * dot3(cd, ci) + cc1 * dot3(bd, ci));
    if (k.has_prev) {
      s1 = vsin(Ap.gamma);
      cc1 = vcos(Ap.gamma);
      mag = s * (Ap.alpha + Ap.gamma - phi_p) * vtan(Ap.beta * R(0.5));
      Ti[0] = Ti[0] - mag * (cc1 * si);
      Ti[1] = Ti[1] + mag * (cc1 * co);
      Ti[2] = Ti[2] - mag * s1;
    }
  }
  if (k.last) Tn[0] = Tn[0] - s * (Ai.alpha + Ai.gamma - phi_i);
}

// First pass of update_Euler_Angle for a linker-DNA bead i (func.cpp:448-492):
// a_i follows the bond, b_i is re-orthogonalised and normalised, c_i = a x b.
// Inputs: r_i, r_{i+1}, a_i, b_i and (next bead a core) a, b, c of bead i+1.
template <class T>
ADJ_HD void frame_pass1(int tn, const T* ri, const T* rn, const T* ao, const T* bi, const T* an, const T* bn,
                        const T* cn, T* out /* a', b', c' */) {
  using R = typename RealOf<T>::type;
  const R si = R(sin(kTheta)), co = R(cos(kTheta));
  T rf[3];
  for (int x = 0; x < 3; x++)
    rf[x] = (tn == 0) ? rn[x] - ri[x] : rn[x] - R(kRo) * (-si * an[x] + co * bn[x]) + R(kD1) * cn[x] - ri[x];
  T mi = R(1) / norm3(rf);
  T* a = out;
  T* b = out + 3;
  T* c = out + 6;
  for (int x = 0; x < 3; x++) a[x] = mi * rf[x];
  T da[3] = {a[0] - ao[0], a[1] - ao[1], a[2] - ao[2]};
  T bda = dot3(bi, da);
  for (int x = 0; x < 3; x++) b[x] = bi[x] - bda * ao[x];
  bda = dot3(b, a);
  for (int x = 0; x < 3; x++) b[x] = b[x] - bda * a[x];
  mi = R(1) / norm3(b);
  for (int x = 0; x < 3; x++) b[x] = mi * b[x];
  cross3(a, b, c);
}

// rotation_cal + rotate (func_cuda.cu:681-704, func.cpp:1607-1670): rotate
// the frame of one bead by w = dt tau / zeta + rr.  Inputs: torque (3), a,
// b, c (9).  Outputs a', b', c'.
template <class T>
ADJ_HD void rotate_frame(int core, double dt, const double* rr, const T* tq, const T* x, T* out) {
  using R = typename RealOf<T>::type;
  T w[3];
  if (core) {
    const R k = R(dt / (8 * kPi * kEta * 125.0));
    for (int i = 0; i < 3; i++) w[i] = tq[i] * k + R(rr[i]);
  } else {
    const R k = R(dt / (4 * kPi * kEta * kRh * kRh * kLo));
    w[0] = tq[0] * k + R(rr[0]);
    w[1] = T(0.0);
    w[2] = T(0.0);
  }
  const T *a = x, *b = x + 3, *c = x + 6;
  T wa = w[0], wb = w[1], wc = w[2];
  T wa2 = wa * wa, wb2 = wb * wb, wc2 = wc * wc, z2 = wa2 + wb2 + wc2;
  if (!(val(z2) > 0.0)) {
    for (int i = 0; i < 9; i++) out[i] = x[i];
    return;
  }
  T z = vsqrt(z2);
  T czt = vcos(z), szt = vsin(z), om = R(1) - czt;
  T sz = szt / z;
  T g[9] = {((wb2 + wc2) * czt + wa2) / z2, wa * wb * om / z2 + wc * sz, wa * wc * om / z2 - wb * sz,
            wa * wb * om / z2 - wc * sz,    ((wa2 + wc2) * czt + wb2) / z2, wb * wc * om / z2 + wa * sz,
            wa * wc * om / z2 + wb * sz,    wb * wc * om / z2 - wa * sz, ((wa2 + wb2) * czt + wc2) / z2};
  for (int row = 0; row < 3; row++)
    for (int i = 0; i < 3; i++) out[3 * row + i] = g[3 * row] * a[i] + g[3 * row + 1] * b[i] + g[3 * row + 2] * c[i];
}

// ---------------------------------------------------------------- pairs
// Debye-Hueckel + Lennard-Jones magnitudes of the DNA/core charge-site
// interactions (func.cpp:1291-1605): g(d) with the force g * z / d.
template <class T, class R>
ADJ_HD T dh_g(R qq, const T& kappa, const T& d) {
  return qq * vexp(-kappa * d) * (kappa * d + R(1)) / (d * d);
}
template <class T, class R>
ADJ_HD T lj_g(R kex, R sig, const T& d) {
  T u = T(sig) / d;
  return kex * ((R(12) / sig) * ipow(u, 13) - (R(6) / sig) * ipow(u, 7));
}

// DNA-DNA: force on bead i for z = r_i - r_j (func.cpp:1330-1360)
template <class T, class R>
ADJ_HD void pair_dna_dna(R keqq, R kex, R sig, const T* z, const T& kappa, T* f) {
  T d = norm3(z);
  T g1 = dh_g(keqq, kappa, d);
  if (val(d) <= 8.0) g1 = g1 + lj_g(kex, sig, d);
  for (int x = 0; x < 3; x++) f[x] = g1 * z[x] / d;
}

// one core charge site and a DNA bead / another site: force on the first
// point for z = p1 - p2; dh, lj select the terms (func.cpp:1362-1600)
template <class T, class R>
ADJ_HD void pair_site(R keqq, bool dh, bool lj, R kex, R sig, const T* z, const T& kappa, T* f) {
  T d = norm3(z);
  T g1 = dh ? dh_g(keqq, kappa, d) : T(0.0);
  if (lj && val(d) <= 8.0) g1 = g1 + lj_g(kex, sig, d);
  for (int x = 0; x < 3; x++) f[x] = g1 * z[x] / d;
}

// func.cpp:278-300 / 342-371: clamped Debye-Hueckel (+ LJ) between two
// tail / linker beads, force on the first for z = c1 - c2
template <class T, class R>
ADJ_HD void pair_clamped(R q1q2, R eps, bool lj, R kev, R sig, const T* z, const T& kappa, T* f) {
  T d = norm3(z);
  T fm = T(0.0);
  if (val(d) < 7.0) fm = (q1q2 * (kappa * d + R(1))) / (R(4 * kPi) * eps * d * d) * vexp(-kappa * d);
  if (lj && val(d) < 4.0) {
    T s6 = ipow(T(sig), 6);
    fm = fm - kev * ((R(6) * s6) / ipow(d, 7) - (R(12) * s6 * s6) / ipow(d, 13));
  }
  for (int x = 0; x < 3; x++) f[x] = clamp09(fm * z[x] / d);
}

// func.cpp:134-151 for a tail bond: force on c1 (the force on c2 is -f)
template <class T, class R>
ADJ_HD void stretch_f(R h, R l0, const T* c1, const T* c2, T* f) {
  T dv[3] = {c1[0] - c2[0], c1[1] - c2[1], c1[2] - c2[2]};
  T d = norm3(dv);
  T fm = (d - l0) * (-h);
  for (int x = 0; x < 3; x++) f[x] = fm * dv[x] / d;
}

// update_tail_beta (func.cpp:1763-1790) + the three-bead angle force
// (func.cpp:153-196); outputs f1, f2, f3 (subtracted from the tail forces)
template <class T, class R>
ADJ_HD void bend3_f(R g, R beta0, const T* c1, const T* c2, const T* c3, T* f) {
  T x12[3] = {c1[0] - c2[0], c1[1] - c2[1], c1[2] - c2[2]};
  T x32[3] = {c3[0] - c2[0], c3[1] - c2[1], c3[2] - c2[2]};
  T beta = vacos(dot3(x12, x32) / (norm3(x12) * norm3(x32)));
  T fm = -g * (beta - beta0);
  T d1 = norm3(x12), d2 = norm3(x32);
  T ji[3] = {-x12[0], -x12[1], -x12[2]};
  T jk[3] = {c2[0] - c3[0], c2[1] - c3[1], c2[2] - c3[2]};
  T t[3], ri[3], rk[3];
  cross3(ji, jk, t);
  cross3(ji, t, ri);
  T nri = norm3(ri);
  cross3(x32, t, rk);
  T nrk = norm3(rk);
  for (int x = 0; x < 3; x++) {
    f[x] = (fm / d1) * ri[x] / nri;
    f[6 + x] = (fm / d2) * rk[x] / nrk;
    f[3 + x] = -f[x] - f[6 + x];
  }
}

// func.cpp:2366-2391 (anchor of a template tail bead): spring h (r_t - body
// point) with its reaction and torque on the core.  Inputs r_t (3), core
// frame (12), h.  Outputs: tail force (3), core force (3), core torque (3).
template <class T>
ADJ_HD void anchor_term(const double* P, const T* rt, const T* x, const T& h, T* out) {
  using R = typename RealOf<T>::type;
  const R p0 = R(P[0]), p1 = R(P[1]), p2 = R(P[2]);
  const T *r = x, *a = x + 3, *b = x + 6, *c = x + 9;
  T hs[3];
  for (int k = 0; k < 3; k++) hs[k] = h * (rt[k] - (r[k] + a[k] * p0 + b[k] * p1 + c[k] * p2));
  for (int k = 0; k < 3; k++) {
    out[k] = -hs[k];
    out[3 + k] = hs[k];
  }
  T fa = dot3(a, hs), fb = dot3(b, hs), fc = dot3(c, hs);
  out[6] = fc * p1 - fb * p2;
  out[7] = fa * p2 - fc * p0;
  out[8] = fb * p0 - fa * p1;
}

// func.cpp:737-804: the RPY block of two distinct beads for s = r_i - r_j
template <class T, class R>
ADJ_HD void rpy_block(R radi, R radj, R a1, R a2, const T* s, T* B /* 3 x 3 */) {
  T ssq = dot3(s, s);
  T sn = vsqrt(ssq);
  if (val(sn) >= radi + radj) {
    T f = T(radi * radi + radj * radj) / ssq;
    T f1 = f * R(1.0 / 3) + R(1), f2 = R(1) - f;
    T k = T(a2) / sn;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        T v = f2 * s[i] * s[j] / ssq;
        B[3 * i + j] = k * ((i == j) ? f1 + v : v);
      }
  } else {
    const R se = R(cbrt((double(radi) * radi * radi + double(radj) * radj * radj) / 2.0));
    const R k = a1 / se;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        T v = R(3) * s[i] * s[j] / (R(32) * se * sn);
        B[3 * i + j] = k * ((i == j) ? (R(1) - R(9) * sn / (R(32) * se)) + v : v);
      }
  }
}

}  // namespace adj
