// Test infrastructure only (see bd_oracle.h): the CPU oracle for the
// Brownian-dynamics step.  Every function names the reference lines it
// restates.  The expressions keep the reference's operation order so that
// the results agree with the reference bit for bit when FMA contraction is
// off; the loops are reorganised only where that does not change any
// floating-point sum.
#include "bd_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace orc {

// constants.h:6-12
constexpr double kPi = 3.141592653589790;
constexpr double kLo = 3.0;
constexpr double kRo = 4.8;
constexpr double kD1 = 1.8;
constexpr double kTheta = 1.2 * kPi / 2;
constexpr double kEta = 1.137076e-12;
constexpr double kRh = 1.2;

using Vec = std::vector<double>;
using IVec = std::vector<int>;

// Host threads for the O(m^2) and O(m^3) parts of a step (RPY assembly,
// Cholesky, rd); none of them changes a floating-point sum.
static int g_threads = 1;

// ---------------------------------------------------------------- primitives
// func.cpp:134-151
static void stretch(double h, const double* c1, const double* c2, double l0, double* f1, double* f2, double& E) {
  double d = std::sqrt((c1[0] - c2[0]) * (c1[0] - c2[0]) + (c1[1] - c2[1]) * (c1[1] - c2[1]) +
                       (c1[2] - c2[2]) * (c1[2] - c2[2]));
  E = E + h * (d - l0) * (d - l0) / 2;
  double f = -h * (d - l0);
  for (int i = 0; i < 3; i++) {
    f1[i] = f * (c1[i] - c2[i]) / d;
    f2[i] = -f * (c1[i] - c2[i]) / d;
  }
}

// utilities.cpp cross_product / norm(vector)
static void cross3(const double* u, const double* v, double* w) {
  double w0 = u[1] * v[2] - u[2] * v[1];
  double w1 = -1 * (u[0] * v[2] - u[2] * v[0]);
  double w2 = u[0] * v[1] - u[1] * v[0];
  w[0] = w0; w[1] = w1; w[2] = w2;
}
static double norm3(const double* v) {
  double s = 0;
  s = s + v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  return std::sqrt(s);
}

// func.cpp:153-196 (three-bead angle force)
static void bend3(double g, double beta, double beta0, const double* c1, const double* c2, const double* c3,
                  double* f1, double* f2, double* f3, double& E) {
  E = E + g * (beta - beta0) * (beta - beta0) / 2;
  double f = -g * (beta - beta0);
  double d1 = std::sqrt((c1[0] - c2[0]) * (c1[0] - c2[0]) + (c1[1] - c2[1]) * (c1[1] - c2[1]) +
                        (c1[2] - c2[2]) * (c1[2] - c2[2]));
  double d2 = std::sqrt((c2[0] - c3[0]) * (c2[0] - c3[0]) + (c2[1] - c3[1]) * (c2[1] - c3[1]) +
                        (c2[2] - c3[2]) * (c2[2] - c3[2]));
  double ji[3] = {c2[0] - c1[0], c2[1] - c1[1], c2[2] - c1[2]};
  double jk[3] = {c2[0] - c3[0], c2[1] - c3[1], c2[2] - c3[2]};
  double kj[3] = {c3[0] - c2[0], c3[1] - c2[1], c3[2] - c2[2]};
  double t[3], ri[3], rk[3];
  cross3(ji, jk, t);
  cross3(ji, t, ri);
  double nri = norm3(ri);
  for (int i = 0; i < 3; i++) {
    f1[i] = (f / d1) * ri[i] / nri;
    f2[i] = -(f / d1) * ri[i] / nri;
  }
  cross3(ji, jk, t);
  cross3(kj, t, rk);
  double nrk = norm3(rk);
  for (int i = 0; i < 3; i++) {
    f2[i] = f2[i] - (f / d2) * rk[i] / nrk;
    f3[i] = (f / d2) * rk[i] / nrk;
  }
}

// func.cpp:198-232
static void bend_proj(double g, double beta, double beta_b, double len, const double* af, const double* ab,
                      const double* ao, double* f1, double* f2, double& E) {
  E = E + g * (beta - beta_b) * (beta - beta_b) / 2;
  double g1 = (beta >= 1e-10) ? beta / (std::sin(beta) * len) : 1.0 / len;
  double c1 = std::cos(beta);
  double A[3] = {g1 * (af[0] - c1 * ao[0]), g1 * (af[1] - c1 * ao[1]), g1 * (af[2] - c1 * ao[2])};
  double g2 = (beta_b >= 1e-10) ? beta_b / (std::sin(beta_b) * len) : 1.0 / len;
  double c2 = std::cos(beta_b);
  double B[3] = {g2 * (ab[0] - c2 * ao[0]), g2 * (ab[1] - c2 * ao[1]), g2 * (ab[2] - c2 * ao[2])};
  for (int i = 0; i < 3; i++) {
    f1[i] = -g * (A[i] + B[i]);
    f2[i] = g * (A[i] + B[i]);
  }
}

// func.cpp:234-260
static void twist_proj(double s, double alpha, double beta, double gamma, double phi, double len, double alpha_b,
                       double beta_b, double gamma_b, double phi_b, double gamma_n, const double* b,
                       const double* c, double* f1, double* f2, double& E) {
  E = E + s * ((alpha + gamma - phi) * (alpha + gamma - phi)) / 2;
  double g1 = (alpha + gamma - phi) * std::tan(0.5 * beta) / len;
  double c1 = std::cos(alpha), s1 = std::sin(alpha);
  double g2 = (alpha_b + gamma_b - phi_b) * std::tan(0.5 * beta_b) / len;
  double c2 = std::cos(gamma_n), s2 = std::sin(gamma_n);
  double Ch[3], Zh[3];
  for (int i = 0; i < 3; i++) Ch[i] = g1 * (c1 * c[i] - s1 * b[i]);
  for (int i = 0; i < 3; i++) Zh[i] = g2 * (c2 * c[i] + s2 * b[i]);
  for (int i = 0; i < 3; i++) {
    f1[i] = s * (Ch[i] + Zh[i]);
    f2[i] = -s * (Ch[i] + Zh[i]);
  }
}

static inline double clamp09(double v) {
  if (v > 0.9) v = 0.9;
  if (v < -0.9) v = -0.9;
  return v;
}

// func.cpp:278-300 (Debye-Hueckel, cut 7 nm, per-component clamp)
static void pair_dh(double q1, double q2, double eps, double kappa, const double* c1, const double* c2, double* f1,
                    double* f2, double& E) {
  double f = 0.0;
  double d = std::sqrt((c1[0] - c2[0]) * (c1[0] - c2[0]) + (c1[1] - c2[1]) * (c1[1] - c2[1]) +
                       (c1[2] - c2[2]) * (c1[2] - c2[2]));
  if (d < 7.0) {
    f = ((q1 * q2 * (kappa * d + 1)) / (4 * kPi * eps * d * d)) * std::exp(-kappa * d);
    E = E + (q1 * q2 / (4 * kPi * eps * d)) * std::exp(-kappa * d);
  }
  for (int i = 0; i < 3; i++) {
    f1[i] = clamp09(f * (c1[i] - c2[i]) / d);
    f2[i] = clamp09(-f * (c1[i] - c2[i]) / d);
  }
}

// func.cpp:318-340 (Lennard-Jones, cut 4 nm)
static void pair_lj(double kev, double sig, const double* c1, const double* c2, double* f1, double* f2, double& E) {
  double f = 0.0;
  double d = std::sqrt((c1[0] - c2[0]) * (c1[0] - c2[0]) + (c1[1] - c2[1]) * (c1[1] - c2[1]) +
                       (c1[2] - c2[2]) * (c1[2] - c2[2]));
  if (d < 4.0) {
    f = -kev * ((6 * std::pow(sig, 6)) / std::pow(d, 7) - (12 * std::pow(sig, 12)) / std::pow(d, 13));
    E = E + kev * (std::pow(sig / d, 12) - std::pow(sig / d, 6));
  }
  for (int i = 0; i < 3; i++) {
    f1[i] = clamp09(f * (c1[i] - c2[i]) / d);
    f2[i] = clamp09(-f * (c1[i] - c2[i]) / d);
  }
}

// func.cpp:342-371 (DH + LJ)
static void pair_dhlj(double q1, double q2, double eps, double kappa, double kev, double sig, const double* c1,
                      const double* c2, double* f1, double* f2, double& E) {
  double f = 0.0, fl = 0.0;
  double d = std::sqrt((c1[0] - c2[0]) * (c1[0] - c2[0]) + (c1[1] - c2[1]) * (c1[1] - c2[1]) +
                       (c1[2] - c2[2]) * (c1[2] - c2[2]));
  if (d < 7.0) {
    f = ((q1 * q2 * (kappa * d + 1)) / (4 * kPi * eps * d * d)) * std::exp(-kappa * d);
    E = E + (q1 * q2 / (4 * kPi * eps * d)) * std::exp(-kappa * d);
  }
  if (d < 4.0) {
    fl = -kev * ((6 * std::pow(sig, 6)) / std::pow(d, 7) - (12 * std::pow(sig, 12)) / std::pow(d, 13));
    E = E + kev * (std::pow(sig / d, 12) - std::pow(sig / d, 6));
  }
  for (int i = 0; i < 3; i++) {
    f1[i] = clamp09((f + fl) * (c1[i] - c2[i]) / d);
    f2[i] = clamp09(-(f + fl) * (c1[i] - c2[i]) / d);
  }
}

// func.cpp:374-394
static void torque_abs(const double* F, const double* pf, const double* pc, const double* a, const double* b,
                       const double* c, double* t) {
  double comp[3];
  comp[0] = (pf[0] - pc[0]) * a[0] + (pf[1] - pc[1]) * a[1] + (pf[2] - pc[2]) * a[2];
  comp[1] = (pf[0] - pc[0]) * b[0] + (pf[1] - pc[1]) * b[1] + (pf[2] - pc[2]) * b[2];
  comp[2] = (pf[0] - pc[0]) * c[0] + (pf[1] - pc[1]) * c[1] + (pf[2] - pc[2]) * c[2];
  double fa = a[0] * F[0] + a[1] * F[1] + a[2] * F[2];
  double fb = b[0] * F[0] + b[1] * F[1] + b[2] * F[2];
  double fc = c[0] * F[0] + c[1] * F[1] + c[2] * F[2];
  t[0] = fc * comp[1] - fb * comp[2];
  t[1] = fa * comp[2] - fc * comp[0];
  t[2] = fb * comp[0] - fa * comp[1];
}

// func.cpp:396-410
static void torque_rel(const double* F, const double* comp, const double* a, const double* b, const double* c,
                       double* t) {
  double fa = a[0] * F[0] + a[1] * F[1] + a[2] * F[2];
  double fb = b[0] * F[0] + b[1] * F[1] + b[2] * F[2];
  double fc = c[0] * F[0] + c[1] * F[1] + c[2] * F[2];
  t[0] = fc * comp[1] - fb * comp[2];
  t[1] = fa * comp[2] - fc * comp[0];
  t[2] = fb * comp[0] - fa * comp[1];
}

// body point r + a*p0 + b*p1 + c*p2 (func.cpp:1364 and its many copies)
static void body_point(const double* r, const double* a, const double* b, const double* c, const double* p,
                       double* out) {
  for (int x = 0; x < 3; x++) out[x] = r[x] + a[x] * p[0] + b[x] * p[1] + c[x] * p[2];
}

// func.cpp:687-709 / 711-723
static void first_coord(int t, const double* r, const double* a, const double* b, const double* c, double* rf) {
  if (t == 0) {
    for (int x = 0; x < 3; x++) rf[x] = r[x];
  } else {
    double si = std::sin(kTheta), co = std::cos(kTheta);
    double bm[3];
    for (int x = 0; x < 3; x++) bm[x] = -si * a[x] + co * b[x];
    for (int x = 0; x < 3; x++) rf[x] = r[x] - kRo * bm[x] + kD1 * c[x];
  }
}
static void second_coord(int t, const double* r, const double* b, const double* c, double* rs) {
  if (t == 0) {
    for (int x = 0; x < 3; x++) rs[x] = r[x];
  } else {
    for (int x = 0; x < 3; x++) rs[x] = r[x] - (kRo * b[x] + kD1 * c[x]);
  }
}

static inline double clamp1(double v) {
  if (v > 1.0) v = 1.0;
  if (v < -1.0) v = -1.0;
  return v;
}

// ---------------------------------------------------------------- system
struct Frames {
  Vec alpha, beta, gamma, length, a_dna, b_dna, c_dna, alpha_p, beta_p, gamma_p;
  void size(int n, int nc) {
    alpha.assign(n, 0); beta.assign(n, 0); gamma.assign(n, 0); length.assign(n, 0);
    a_dna.assign(3 * nc, 0); b_dna.assign(3 * nc, 0); c_dna.assign(3 * nc, 0);
    alpha_p.assign(nc, 0); beta_p.assign(nc, 0); gamma_p.assign(nc, 0);
  }
};

struct State {
  Vec r, a, b, c, r_t, r_lh;
  Frames fr;
  Vec beta_t, beta_lh;
};

struct Forces {
  Vec F, T, tF, lF;
  double E = 0.0;
  void zero(int n, int nt, int nl) {
    F.assign(3 * n, 0.0); T.assign(3 * n, 0.0); tF.assign(3 * nt, 0.0); lF.assign(3 * nl, 0.0); E = 0.0;
  }
};

struct System {
  int n, n_c, Nq, n_t, n_tail, n_lh_n, n_lh_g, n_lh_c, n_LH, n_D;
  double h, g, s, debyell, debye, q_l, k_e, k_ex, sDD, sDC, sCC, sTT, sTL, sTC, a1, a2, dt, del, s2dt;
  IVec type, tail_fix, nc_t_flag, t_grp, t_fix, LH_conn, nc_lh_flag;
  Vec rad, phi_o, core_pos, core_q, tail_pos, h_t, g_t, lo_t, beta_o_t, t_q, t_rad, LH_g_pos, LH_q, LH_vdw_hh,
      LH_vdw_hc, LH_vdw_hl, LH_vdw_ht, LH_kstr, LH_kben, LH_streq, LH_betaeq, lh_rad, rad_all;
  IVec core_rank;   // core ordinal of bead i (count of cores in [0, i]) - 1
  State st;
  Vec rd;
  Forces last;
};

// ---------------------------------------------------------------- frames
// func.cpp:433-685 (two full passes: frames, then angles)
static void euler_angles(const System& S, const Vec& r, Vec& a, Vec& b, Vec& c, Frames& o) {
  const int n = S.n;
  const double si = std::sin(kTheta), co = std::cos(kTheta);
  for (int i = 0; i < n - 1; i++) {
    int i1 = 3 * i, i2 = i1 + 1, i3 = i2 + 1, f1 = i1 + 3, f2 = f1 + 1, f3 = f2 + 1;
    double rf[3];
    if (S.type[i] == 0) {
      double ao[3] = {a[i1], a[i2], a[i3]};
      if (S.type[i + 1] == 0) {
        rf[0] = r[f1] - r[i1]; rf[1] = r[f2] - r[i2]; rf[2] = r[f3] - r[i3];
      } else {
        double bm[3] = {-si * a[f1] + co * b[f1], -si * a[f2] + co * b[f2], -si * a[f3] + co * b[f3]};
        rf[0] = r[f1] - kRo * bm[0] + kD1 * c[f1] - r[i1];
        rf[1] = r[f2] - kRo * bm[1] + kD1 * c[f2] - r[i2];
        rf[2] = r[f3] - kRo * bm[2] + kD1 * c[f3] - r[i3];
      }
      o.length[i] = std::sqrt(rf[0] * rf[0] + rf[1] * rf[1] + rf[2] * rf[2]);
      double mi = 1.0 / o.length[i];
      a[i1] = mi * rf[0]; a[i2] = mi * rf[1]; a[i3] = mi * rf[2];
      double da[3] = {a[i1] - ao[0], a[i2] - ao[1], a[i3] - ao[2]};
      double bda = b[i1] * da[0] + b[i2] * da[1] + b[i3] * da[2];
      b[i1] = b[i1] - bda * ao[0]; b[i2] = b[i2] - bda * ao[1]; b[i3] = b[i3] - bda * ao[2];
      bda = b[i1] * a[i1] + b[i2] * a[i2] + b[i3] * a[i3];
      b[i1] = b[i1] - bda * a[i1]; b[i2] = b[i2] - bda * a[i2]; b[i3] = b[i3] - bda * a[i3];
      mi = 1.0 / std::sqrt(b[i1] * b[i1] + b[i2] * b[i2] + b[i3] * b[i3]);
      b[i1] = mi * b[i1]; b[i2] = mi * b[i2]; b[i3] = mi * b[i3];
      c[i1] = a[i2] * b[i3] - a[i3] * b[i2];
      c[i2] = a[i3] * b[i1] - a[i1] * b[i3];
      c[i3] = a[i1] * b[i2] - a[i2] * b[i1];
    } else {
      rf[0] = r[f1] - (r[i1] - kRo * b[i1] - kD1 * c[i1]);
      rf[1] = r[f2] - (r[i2] - kRo * b[i2] - kD1 * c[i2]);
      rf[2] = r[f3] - (r[i3] - kRo * b[i3] - kD1 * c[i3]);
      o.length[i] = std::sqrt(rf[0] * rf[0] + rf[1] * rf[1] + rf[2] * rf[2]);
    }
  }
  for (int i = 0; i < n - 1; i++) {
    int i1 = 3 * i, i2 = i1 + 1, i3 = i2 + 1, f1 = i1 + 3, f2 = f1 + 1, f3 = f2 + 1;
    if (S.type[i] == 0) {
      // forward frame: the next DNA bead's frame, or the core's entry frame
      double af[3], bf[3], cf[3] = {c[f1], c[f2], c[f3]};
      if (S.type[i + 1] == 0) {
        af[0] = a[f1]; af[1] = a[f2]; af[2] = a[f3];
        bf[0] = b[f1]; bf[1] = b[f2]; bf[2] = b[f3];
      } else {
        af[0] = co * a[f1] + si * b[f1]; af[1] = co * a[f2] + si * b[f2]; af[2] = co * a[f3] + si * b[f3];
        bf[0] = -si * a[f1] + co * b[f1]; bf[1] = -si * a[f2] + co * b[f2]; bf[2] = -si * a[f3] + co * b[f3];
      }
      double ada = clamp1(a[i1] * af[0] + a[i2] * af[1] + a[i3] * af[2]);
      o.beta[i] = std::acos(ada);
      double sb = std::sin(o.beta[i]);
      double x;
      if (o.beta[i] > 1e-10) x = (af[0] * b[i1] + af[1] * b[i2] + af[2] * b[i3]) / sb;
      else x = (bf[0] * b[i1] + bf[1] * b[i2] + bf[2] * b[i3]);
      x = clamp1(x);
      double Ac = std::acos(x);
      double y = af[0] * c[i1] + af[1] * c[i2] + af[2] * c[i3];
      o.alpha[i] = (y >= 0) ? Ac : -Ac;
      // func.cpp:537 / :575 (the DNA-DNA and DNA-core forms differ only in
      // which forward b is used; the c of the next bead is used in both)
      x = clamp1((b[i1] * bf[0] + b[i2] * bf[1] + b[i3] * bf[2] + c[i1] * cf[0] + c[i2] * cf[1] + c[i3] * cf[2]) /
                 (1.0 + ada));
      double apg = std::acos(x);
      y = (c[i1] * bf[0] + c[i2] * bf[1] + c[i3] * bf[2] - (b[i1] * cf[0] + b[i2] * cf[1] + b[i3] * cf[2])) /
          (1.0 + ada);
      o.gamma[i] = (y >= 0.0) ? apg - o.alpha[i] : -apg - o.alpha[i];
    } else {
      int ic = S.core_rank[i], c1 = 3 * ic, c2 = c1 + 1, c3 = c2 + 1;
      o.a_dna[c1] = (r[f1] - (r[i1] - kRo * b[i1] - kD1 * c[i1])) / o.length[i];
      o.a_dna[c2] = (r[f2] - (r[i2] - kRo * b[i2] - kD1 * c[i2])) / o.length[i];
      o.a_dna[c3] = (r[f3] - (r[i3] - kRo * b[i3] - kD1 * c[i3])) / o.length[i];
      double cb = clamp1(a[i1] * o.a_dna[c1] + a[i2] * o.a_dna[c2] + a[i3] * o.a_dna[c3]);
      o.beta_p[ic] = std::acos(cb);
      double sb = std::sin(o.beta_p[ic]);
      if (o.beta_p[ic] >= 1e-10) {
        double bm[3] = {(o.a_dna[c1] - cb * a[i1]) / sb, (o.a_dna[c2] - cb * a[i2]) / sb,
                        (o.a_dna[c3] - cb * a[i3]) / sb};
        double ca = clamp1(bm[0] * b[i1] + bm[1] * b[i2] + bm[2] * b[i3]);
        double Ac = std::acos(ca);
        double y = o.a_dna[c1] * c[i1] + o.a_dna[c2] * c[i2] + o.a_dna[c3] * c[i3];
        o.alpha_p[ic] = (y >= 0) ? Ac : -Ac;
        o.gamma_p[ic] = -o.alpha_p[ic];
        double sa = std::sin(o.alpha_p[ic]), sg = std::sin(o.gamma_p[ic]), cg = std::cos(o.gamma_p[ic]);
        double R21 = -cg * sb, R22 = cg * cb * ca - sg * sa, R23 = cg * cb * sa + sg * ca;
        for (int x = 0; x < 3; x++) o.b_dna[c1 + x] = R21 * a[i1 + x] + R22 * b[i1 + x] + R23 * c[i1 + x];
        double R31 = sg * sb, R32 = -sg * cb * ca - cg * sa, R33 = -sg * cb * sa + cg * ca;
        for (int x = 0; x < 3; x++) o.c_dna[c1 + x] = R31 * a[i1 + x] + R32 * b[i1 + x] + R33 * c[i1 + x];
      } else {
        for (int x = 0; x < 3; x++) { o.b_dna[c1 + x] = b[i1 + x]; o.c_dna[c1 + x] = c[i1 + x]; }
      }
      const double* ad = &o.a_dna[c1];
      const double* bd = &o.b_dna[c1];
      const double* cd = &o.c_dna[c1];
      double ada = clamp1(ad[0] * a[f1] + ad[1] * a[f2] + ad[2] * a[f3]);
      o.beta[i] = std::acos(ada);
      sb = std::sin(o.beta[i]);
      double x;
      if (o.beta[i] >= 1e-10) x = (a[f1] * bd[0] + a[f2] * bd[1] + a[f3] * bd[2]) / sb;
      else x = (b[f1] * bd[0] + b[f2] * bd[1] + b[f3] * bd[2]);
      x = clamp1(x);
      double Ac = std::acos(x);
      double y = a[f1] * cd[0] + a[f2] * cd[1] + a[f3] * cd[2];
      o.alpha[i] = (y >= 0) ? Ac : -Ac;
      x = clamp1((bd[0] * b[f1] + bd[1] * b[f2] + bd[2] * b[f3] + cd[0] * c[f1] + cd[1] * c[f2] + cd[2] * c[f3]) /
                 (1.0 + ada));
      double apg = std::acos(x);
      y = (cd[0] * b[f1] + cd[1] * b[f2] + cd[2] * b[f3] - (bd[0] * c[f1] + bd[1] * c[f2] + bd[2] * c[f3])) /
          (1.0 + ada);
      o.gamma[i] = (y >= 0.0) ? apg - o.alpha[i] : -apg - o.alpha[i];
    }
  }
}

// func.cpp:1763-1790 (bounds test applied before the group lookups)
static void tail_beta(const System& S, const Vec& r_t, Vec& beta_t) {
  for (int i = 0; i < S.n_tail; i++) {
    if (i < S.n_tail - 2 && S.t_grp[i] == S.t_grp[i + 1] && S.t_grp[i] == S.t_grp[i + 2]) {
      double x12 = r_t[i * 3] - r_t[i * 3 + 3], y12 = r_t[i * 3 + 1] - r_t[i * 3 + 4], z12 = r_t[i * 3 + 2] - r_t[i * 3 + 5];
      double r12 = std::sqrt(x12 * x12 + y12 * y12 + z12 * z12);
      double x32 = r_t[i * 3 + 6] - r_t[i * 3 + 3], y32 = r_t[i * 3 + 7] - r_t[i * 3 + 4], z32 = r_t[i * 3 + 8] - r_t[i * 3 + 5];
      double r32 = std::sqrt(x32 * x32 + y32 * y32 + z32 * z32);
      beta_t[i] = std::acos((x12 * x32 + y12 * y32 + z12 * z32) / (r12 * r32));
    } else {
      beta_t[i] = 0.0;
    }
  }
}

// func.cpp:2062-2089
static void lh_beta(const System& S, const Vec& r_lh, Vec& beta_lh) {
  for (int i = 0; i < S.n_LH; i++) {
    if ((i % S.n_lh_c != 0) && (i % S.n_lh_c != S.n_lh_c - 1)) {
      double x12 = r_lh[i * 3 - 3] - r_lh[i * 3], y12 = r_lh[i * 3 - 2] - r_lh[i * 3 + 1], z12 = r_lh[i * 3 - 1] - r_lh[i * 3 + 2];
      double r12 = std::sqrt(x12 * x12 + y12 * y12 + z12 * z12);
      double x32 = r_lh[i * 3 + 3] - r_lh[i * 3], y32 = r_lh[i * 3 + 4] - r_lh[i * 3 + 1], z32 = r_lh[i * 3 + 5] - r_lh[i * 3 + 2];
      double r32 = std::sqrt(x32 * x32 + y32 * y32 + z32 * z32);
      beta_lh[i] = std::acos((x12 * x32 + y12 * y32 + z12 * z32) / (r12 * r32));
    } else {
      beta_lh[i] = 0.0;
    }
  }
}

static inline void add3(Vec& v, int i, const double* d) {
  v[3 * i] = v[3 * i] + d[0]; v[3 * i + 1] = v[3 * i + 1] + d[1]; v[3 * i + 2] = v[3 * i + 2] + d[2];
}
static inline void sub3(Vec& v, int i, const double* d) {
  v[3 * i] = v[3 * i] - d[0]; v[3 * i + 1] = v[3 * i + 1] - d[1]; v[3 * i + 2] = v[3 * i + 2] - d[2];
}

// ---------------------------------------------------------------- bonded
// func.cpp:951-1289
static void mechanical(const System& S, const State& X, Forces& out) {
  const int n = S.n;
  const Vec &r = X.r, &a = X.a, &b = X.b, &c = X.c;
  const Frames& fr = X.fr;
  const double si = std::sin(kTheta), co = std::cos(kTheta);
  double f1[3], f2[3], t1[3], t2[3], rf[3], rs[3];
  auto bond_torques = [&](int i) {
    torque_abs(f1, rs, &r[3 * i], &a[3 * i], &b[3 * i], &c[3 * i], t1);
    torque_abs(f2, rf, &r[3 * i + 3], &a[3 * i + 3], &b[3 * i + 3], &c[3 * i + 3], t2);
    add3(out.F, i, f1); add3(out.F, i + 1, f2);
    add3(out.T, i, t1); add3(out.T, i + 1, t2);
  };
  auto ends = [&](int i) {
    first_coord(S.type[i + 1], &r[3 * i + 3], &a[3 * i + 3], &b[3 * i + 3], &c[3 * i + 3], rf);
    second_coord(S.type[i], &r[3 * i], &b[3 * i], &c[3 * i], rs);
  };
  for (int i = 0; i < n - 1; i++) {  // stretching
    ends(i);
    stretch(S.h, rs, rf, kLo, f1, f2, out.E);
    bond_torques(i);
  }
  for (int i = 0; i < n - 1; i++) {  // bending
    int ic = S.core_rank[i];
    ends(i);
    double af[3], ab[3], ao[3], beta_b;
    if (S.type[i] == 0) {
      if (S.type[i + 1] == 0) {
        for (int x = 0; x < 3; x++) af[x] = a[3 * i + 3 + x];
      } else {
        for (int x = 0; x < 3; x++) af[x] = co * a[3 * i + 3 + x] + si * b[3 * i + 3 + x];
      }
      if (S.type[i - 1] == 0) {
        for (int x = 0; x < 3; x++) ab[x] = a[3 * i - 3 + x];
      } else {
        for (int x = 0; x < 3; x++) ab[x] = fr.a_dna[3 * ic + x];
      }
      for (int x = 0; x < 3; x++) ao[x] = a[3 * i + x];
      beta_b = fr.beta[i - 1];
    } else {
      for (int x = 0; x < 3; x++) { af[x] = a[3 * i + 3 + x]; ab[x] = a[3 * i + x]; ao[x] = fr.a_dna[3 * ic + x]; }
      beta_b = fr.beta_p[ic];
    }
    bend_proj(S.g, fr.beta[i], beta_b, fr.length[i], af, ab, ao, f1, f2, out.E);
    bond_torques(i);
  }
  for (int i = 0; i < n - 1; i++) {  // twisting
    int ic = S.core_rank[i];
    ends(i);
    double al_b, be_b, ga_b, ph_b, ga_n, bo[3], cO[3];
    if (S.type[i] == 0) {
      al_b = fr.alpha[i - 1]; be_b = fr.beta[i - 1]; ga_b = fr.gamma[i - 1]; ph_b = S.phi_o[i - 1];
      ga_n = fr.gamma[i - 1];
      for (int x = 0; x < 3; x++) { bo[x] = b[3 * i + x]; cO[x] = c[3 * i + x]; }
    } else {
      al_b = fr.alpha[i]; be_b = fr.beta_p[ic]; ga_b = fr.gamma[i]; ph_b = S.phi_o[i]; ga_n = fr.gamma_p[ic];
      for (int x = 0; x < 3; x++) { bo[x] = fr.b_dna[3 * ic + x]; cO[x] = fr.c_dna[3 * ic + x]; }
    }
    twist_proj(S.s, fr.alpha[i], fr.beta[i], fr.gamma[i], S.phi_o[i], fr.length[i], al_b, be_b, ga_b, ph_b, ga_n,
               bo, cO, f1, f2, out.E);
    bond_torques(i);
  }
  Vec& T = out.T;
  const double s = S.s, g = S.g;
  for (int i = 0; i < n - 1; i++) {  // mechanical torques
    int im1 = i - 1, i1 = 3 * i, i2 = i1 + 1, i3 = i2 + 1, ib1 = i1 - 3, ib2 = ib1 + 1, ib3 = ib2 + 1;
    int ic = S.core_rank[i], c1 = 3 * ic, c2 = c1 + 1, c3 = c2 + 1;
    if (S.type[i] == 0) {
      T[i1] = s * (fr.alpha[i] + fr.gamma[i] + S.phi_o[i] - fr.alpha[im1] - fr.gamma[im1] - S.phi_o[im1]);
      T[i2] = 0.0;
      T[i3] = 0.0;
    } else {
      const Vec &ad = fr.a_dna, &bd = fr.b_dna, &cd = fr.c_dna;
      double ada = ad[c1] * a[i1] + ad[c2] * a[i2] + ad[c3] * a[i3];
      double adb = ad[c1] * b[i1] + ad[c2] * b[i2] + ad[c3] * b[i3];
      double adc = ad[c1] * c[i1] + ad[c2] * c[i2] + ad[c3] * c[i3];
      double mag = s * (fr.alpha[i] + fr.gamma[i] - S.phi_o[i]);
      T[i1] = T[i1] + mag * ada; T[i2] = T[i2] + mag * adb; T[i3] = T[i3] + mag * adc;
      if (i > 0) {
        mag = -s * (fr.alpha[im1] + fr.gamma[im1] - S.phi_o[im1]);
        T[i1] = T[i1] + mag * co; T[i2] = T[i2] + mag * si; T[i3] = T[i3] + 0.0;
      }
      T[i2] = T[i2] - g * fr.beta_p[ic] * adc / std::sin(fr.beta_p[ic]);
      T[i3] = T[i3] + g * fr.beta_p[ic] * adb / std::sin(fr.beta_p[ic]);
      if (i > 0) {
        ada = a[ib1] * a[i1] + a[ib2] * a[i2] + a[ib3] * a[i3];
        adb = a[ib1] * b[i1] + a[ib2] * b[i2] + a[ib3] * b[i3];
        adc = a[ib1] * c[i1] + a[ib2] * c[i2] + a[ib3] * c[i3];
        T[i1] = T[i1] + g * fr.beta[im1] * (si * adc) / std::sin(fr.beta[im1]);
        T[i2] = T[i2] - g * fr.beta[im1] * (co * adc) / std::sin(fr.beta[im1]);
        T[i3] = T[i3] + g * fr.beta[im1] * (co * adb - si * ada) / std::sin(fr.beta[im1]);
      }
      double s1 = std::sin(fr.alpha_p[ic]), cc1 = std::cos(fr.alpha_p[ic]);
      mag = s * (fr.alpha[i] + fr.gamma[i] - S.phi_o[i]) * std::tan(0.5 * fr.beta_p[ic]);
      double cda = cd[c1] * a[i1] + cd[c2] * a[i2] + cd[c3] * a[i3];
      double bda = bd[c1] * a[i1] + bd[c2] * a[i2] + bd[c3] * a[i3];
      double cdb = cd[c1] * b[i1] + cd[c2] * b[i2] + cd[c3] * b[i3];
      double bdb = bd[c1] * b[i1] + bd[c2] * b[i2] + bd[c3] * b[i3];
      double cdc = cd[c1] * c[i1] + cd[c2] * c[i2] + cd[c3] * c[i3];
      double bdc = bd[c1] * c[i1] + bd[c2] * c[i2] + bd[c3] * c[i3];
      T[i1] = T[i1] - mag * (s1 * cda + cc1 * bda);
      T[i2] = T[i2] - mag * (s1 * cdb + cc1 * bdb);
      T[i3] = T[i3] - mag * (s1 * cdc + cc1 * bdc);
      if (i > 0) {
        s1 = std::sin(fr.gamma[im1]);
        cc1 = std::cos(fr.gamma[im1]);
        mag = s * (fr.alpha[im1] + fr.gamma[im1] - S.phi_o[im1]) * std::tan(0.5 * fr.beta[im1]);
        T[i1] = T[i1] - mag * (s1 * 0.0 - cc1 * (-si));
        T[i2] = T[i2] - mag * (s1 * 0.0 - cc1 * co);
        T[i3] = T[i3] - mag * (s1 * 1.0 - cc1 * 0.0);
      }
    }
  }
  T[3 * n - 3] = -s * (fr.alpha[n - 2] + fr.gamma[n - 2] - S.phi_o[n - 2]);
  T[3 * n - 2] = 0.0;
  T[3 * n - 1] = 0.0;
}

// ---------------------------------------------------------------- DNA/core pairs
// func.cpp:1291-1605
static void electrostatics(const System& S, const State& X, Forces& out) {
  const int n = S.n, Nq = S.Nq;
  const Vec &r = X.r, &a = X.a, &b = X.b, &c = X.c, &cp = S.core_pos, &cq = S.core_q;
  Vec &F = out.F, &T = out.T;
  double& E = out.E;
  const double qq = S.q_l * S.q_l, ke = S.k_e, kex = S.k_ex;
  // charge-site force g1*z on i, -g1*z on j, plus torque on the core whose
  // frame (fa, fb, fc along its a, b, c) carries charge k
  auto push = [&](int i, int j, double g1, const double* z) {
    F[3 * i] = F[3 * i] + g1 * z[0]; F[3 * i + 1] = F[3 * i + 1] + g1 * z[1]; F[3 * i + 2] = F[3 * i + 2] + g1 * z[2];
    F[3 * j] = F[3 * j] - g1 * z[0]; F[3 * j + 1] = F[3 * j + 1] - g1 * z[1]; F[3 * j + 2] = F[3 * j + 2] - g1 * z[2];
  };
  auto core_torque = [&](int j, double sgn_g1, const double* z, int k) {
    double fa = sgn_g1 * (a[3 * j] * z[0] + a[3 * j + 1] * z[1] + a[3 * j + 2] * z[2]);
    double fb = sgn_g1 * (b[3 * j] * z[0] + b[3 * j + 1] * z[1] + b[3 * j + 2] * z[2]);
    double fc = sgn_g1 * (c[3 * j] * z[0] + c[3 * j + 1] * z[1] + c[3 * j + 2] * z[2]);
    T[3 * j] = T[3 * j] + fc * cp[3 * k + 1] - fb * cp[3 * k + 2];
    T[3 * j + 1] = T[3 * j + 1] + fa * cp[3 * k + 2] - fc * cp[3 * k];
    T[3 * j + 2] = T[3 * j + 2] + fb * cp[3 * k] - fa * cp[3 * k + 1];
  };
  auto lj_g = [&](double sig, double d) {
    return kex * ((12.0 / sig) * std::pow((sig / d), 13) - (6.0 / sig) * std::pow((sig / d), 7));
  };
  auto lj_e = [&](double sig, double d) { return kex * (std::pow(sig / d, 12) - std::pow(sig / d, 6)); };
  for (int i = 0; i < n - 1; i++) {
    int i1 = 3 * i;
    for (int j = i + 1; j < n; j++) {
      int j1 = 3 * j;
      double d = std::sqrt((r[j1] - r[i1]) * (r[j1] - r[i1]) + (r[j1 + 1] - r[i1 + 1]) * (r[j1 + 1] - r[i1 + 1]) +
                           (r[j1 + 2] - r[i1 + 2]) * (r[j1 + 2] - r[i1 + 2]));
      bool ok = !(d > 25.0);
      if (S.type[i + 1] != 0) ok = false;
      if (i > 0 && S.type[i - 1] != 0) ok = false;
      if (j < n - 1 && S.type[j + 1] != 0) ok = false;
      if (S.type[j - 1] != 0) ok = false;
      if (!ok) continue;
      int adj = std::abs(i - j) > 1;
      if (S.type[i] == 0 && S.type[j] == 0) {
        if (!adj) continue;
        double mi = 1.0 / d;
        double z[3] = {mi * (r[i1] - r[j1]), mi * (r[i1 + 1] - r[j1 + 1]), mi * (r[i1 + 2] - r[j1 + 2])};
        double g1 = ke * qq * std::exp(-S.debyell * d) * (S.debyell * d + 1.0) / (d * d);
        E = E + (ke * qq / d) * std::exp(-S.debyell * d);
        if (d <= 8) {
          g1 = g1 + lj_g(S.sDD, d);
          E = E + lj_e(S.sDD, d);
        }
        push(i, j, g1, z);
      } else if (S.type[i] == 0 || S.type[j] == 0) {
        // one DNA bead (dn) and one core (co); z points from the charge
        // site to the DNA bead for DNA-core, from DNA to site for core-DNA
        bool dna_first = (S.type[i] == 0);
        int dn = dna_first ? i : j, cr = dna_first ? j : i;
        int d1 = 3 * dn, k1c = 3 * cr;
        for (int k = 0; k < Nq; k++) {
          double z[3];
          if (dna_first) {
            for (int x = 0; x < 3; x++)
              z[x] = (r[d1 + x] - (r[k1c + x] + a[k1c + x] * cp[3 * k] + b[k1c + x] * cp[3 * k + 1] + c[k1c + x] * cp[3 * k + 2]));
          } else {
            for (int x = 0; x < 3; x++)
              z[x] = (-r[d1 + x] + (r[k1c + x] + a[k1c + x] * cp[3 * k] + b[k1c + x] * cp[3 * k + 1] + c[k1c + x] * cp[3 * k + 2]));
          }
          double dd = std::sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
          double mi = 1.0 / dd;
          z[0] = mi * z[0]; z[1] = mi * z[1]; z[2] = mi * z[2];
          if (adj) {
            double g1 = ke * S.q_l * cq[k] * std::exp(-S.debye * dd) * (S.debye * dd + 1.0) / (dd * dd);
            E = E + (ke * S.q_l * cq[k] / dd) * std::exp(-S.debye * dd);
            push(i, j, g1, z);
            core_torque(cr, dna_first ? -g1 : g1, z, k);
          }
          if (dd <= 8.0 && cq[k] > 0) {
            double g1;
            if (dna_first) {
              g1 = lj_g(S.sDC, dd);
              E = E + lj_e(S.sDC, dd);
            } else {
              E = E + lj_e(S.sDC, dd);
              g1 = lj_g(S.sDC, dd);
            }
            push(i, j, g1, z);
            core_torque(cr, dna_first ? -g1 : g1, z, k);
          }
        }
      } else {
        for (int k = 0; k < Nq; k++) {
          double pk[3], pl[3];
          for (int l = 0; l < Nq; l++) {
            double z[3];
            for (int x = 0; x < 3; x++) {
              pk[x] = r[i1 + x] + a[i1 + x] * cp[3 * k] + b[i1 + x] * cp[3 * k + 1] + c[i1 + x] * cp[3 * k + 2];
              pl[x] = r[j1 + x] + a[j1 + x] * cp[3 * l] + b[j1 + x] * cp[3 * l + 1] + c[j1 + x] * cp[3 * l + 2];
              z[x] = (pk[x] - pl[x]);
            }
            double dd = std::sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2]);
            double mi = 1.0 / dd;
            z[0] = mi * z[0]; z[1] = mi * z[1]; z[2] = mi * z[2];
            double g1 = ke * cq[k] * cq[l] * std::exp(-S.debye * dd) * (S.debye * dd + 1.0) / (dd * dd);
            E = E + (ke * cq[l] * cq[k] / dd) * std::exp(-S.debye * dd);
            push(i, j, g1, z);
            core_torque(i, g1, z, k);
            core_torque(j, -g1, z, l);
            if (dd <= 8.0) {
              g1 = lj_g(S.sCC, dd);
              E = E + lj_e(S.sCC, dd);
              push(i, j, g1, z);
              core_torque(i, g1, z, k);
              core_torque(j, -g1, z, l);
            }
          }
        }
      }
    }
  }
}

// core bead index of the tail group t_grp (func.cpp:2366-2375)
static int tail_core_bead(const System& S, int grp) {
  int k = 0;
  for (int cc = 0; cc < S.n; cc++) {
    if (k == (grp - 1) / 10 && S.type[cc] == 1) return cc;
    if (S.type[cc] == 1) k = k + 1;
  }
  return -1;
}

// ---------------------------------------------------------------- tails
// func.cpp:1793-2026
static void tails(const System& S, const State& X, Forces& out) {
  const int n = S.n, nt = S.n_tail;
  const Vec &r = X.r, &a = X.a, &b = X.b, &c = X.c, &rt = X.r_t;
  double f1[3], f2[3], f3[3];
  const double eps = 1 / (4 * kPi * S.k_e);
  for (int i = 0; i < nt - 1; i++) {
    if (S.t_grp[i] == S.t_grp[i + 1]) {
      stretch(S.h_t[i], &rt[3 * i], &rt[3 * i + 3], S.lo_t[i], f1, f2, out.E);
      add3(out.tF, i, f1); add3(out.tF, i + 1, f2);
    }
  }
  for (int i = 0; i < nt - 2; i++) {
    if (S.t_grp[i] == S.t_grp[i + 1] && S.t_grp[i] == S.t_grp[i + 2]) {
      bend3(S.g_t[i], X.beta_t[i], S.beta_o_t[i], &rt[3 * i], &rt[3 * i + 3], &rt[3 * i + 6], f1, f2, f3, out.E);
      sub3(out.tF, i, f1); sub3(out.tF, i + 1, f2); sub3(out.tF, i + 2, f3);
    }
  }
  for (int i = 0; i < nt - 1; i++) {
    for (int j = i + 1; j < nt; j++) {
      if (S.t_grp[i] != S.t_grp[j] || j > i + 2) {
        pair_dh(S.t_q[i], S.t_q[j], eps, S.debye, &rt[3 * i], &rt[3 * j], f1, f2, out.E);
        add3(out.tF, i, f1); add3(out.tF, j, f2);
      }
    }
  }
  for (int i = 0; i < nt; i++) {
    for (int j = 0; j < n; j++) {
      if (S.type[j] == 0) {
        pair_dhlj(S.t_q[i], S.q_l, eps, S.debye, S.k_ex, S.sTL, &rt[3 * i], &r[3 * j], f1, f2, out.E);
        add3(out.tF, i, f1); add3(out.F, j, f2);
      }
    }
  }
  int k = 0;
  for (int i = 0; i < n; i++) {  // anchors of the fixed template beads
    if (S.type[i] != 1) continue;
    if (S.nc_t_flag[k] == 1) {
      for (int j = 0; j < S.n_t; j++) {
        if (S.tail_fix[j] != 1) continue;
        double ro[3], st[3], hs[3], tq[3];
        body_point(&r[3 * i], &a[3 * i], &b[3 * i], &c[3 * i], &S.tail_pos[3 * j], ro);
        int tb = k * S.n_t + j;
        for (int x = 0; x < 3; x++) st[x] = rt[3 * tb + x] - ro[x];
        out.E = out.E + S.h * (st[0] * st[0] + st[1] * st[1] + st[2] * st[2]) / 2;
        for (int x = 0; x < 3; x++) out.tF[3 * tb + x] = out.tF[3 * tb + x] - S.h * st[x];
        for (int x = 0; x < 3; x++) out.F[3 * i + x] = out.F[3 * i + x] + S.h * st[x];
        for (int x = 0; x < 3; x++) hs[x] = S.h * st[x];
        torque_rel(hs, &S.tail_pos[3 * j], &a[3 * i], &b[3 * i], &c[3 * i], tq);
        add3(out.T, i, tq);
      }
    }
    k = k + 1;
  }
}

// ---------------------------------------------------------------- linker histone
static inline int lh_param(const System& S, int bead) {
  int idx = bead % (S.n_lh_n + S.n_lh_c);
  return idx < S.n_lh_n ? idx : idx + S.n_lh_g;
}

// force on tail bead j: to the tail, or to its core when the bead is fixed
// (func.cpp:2361-2391)
static void tail_or_core(const System& S, const State& X, Forces& out, int j, const double* f) {
  if (S.t_fix[j] == 0) {
    add3(out.tF, j, f);
  } else {
    int cc = tail_core_bead(S, S.t_grp[j]);
    double tq[3];
    torque_abs(f, &X.r_t[3 * j], &X.r[3 * cc], &X.a[3 * cc], &X.b[3 * cc], &X.c[3 * cc], tq);
    add3(out.F, cc, f);
    add3(out.T, cc, tq);
  }
}

// func.cpp:2093-2781
static void linker_histone(const System& S, const State& X, Forces& out) {
  const int n = S.n, nL = S.n_LH, nt = S.n_tail, nlh = S.n_lh_n + S.n_lh_c, ng = S.n_lh_g;
  const Vec &r = X.r, &a = X.a, &b = X.b, &c = X.c, &rl = X.r_lh, &rt = X.r_t;
  const double eps = 1 / (4 * kPi * S.k_e);
  double f1[3], f2[3], f3[3], tq[3], tq2[3];
  for (int i = 0; i < nL; i++) {
    int p = lh_param(S, i);
    if (S.LH_conn[p] == 1) {
      stretch(S.LH_kstr[p], &rl[3 * i], &rl[3 * i + 3], S.LH_streq[p], f1, f2, out.E);
      add3(out.lF, i, f1); add3(out.lF, i + 1, f2);
    }
  }
  for (int i = 0; i < nL; i++) {
    int p = lh_param(S, i);
    if ((i % S.n_lh_c != 0) && (i % S.n_lh_c != S.n_lh_c - 1)) {
      bend3(S.LH_kben[p], X.beta_lh[i], S.LH_betaeq[p], &rl[3 * i - 3], &rl[3 * i], &rl[3 * i + 3], f1, f2, f3, out.E);
      sub3(out.lF, i - 1, f1); sub3(out.lF, i, f2); sub3(out.lF, i + 1, f3);
    }
  }
  for (int i = 0; i < nL; i++) {
    int p1 = lh_param(S, i);
    for (int j = i; j < nL; j++) {
      int p2 = lh_param(S, j);
      if ((i / nlh == j / nlh) && (j > i + 1)) {
        pair_lj(S.k_ex, (S.LH_vdw_hh[p1] + S.LH_vdw_hh[p2]) / 2, &rl[3 * i], &rl[3 * j], f1, f2, out.E);
        add3(out.lF, i, f1); add3(out.lF, j, f2);
      } else if (i / nlh != j / nlh) {
        pair_dhlj(S.LH_q[p1], S.LH_q[p2], eps, S.debye, S.k_ex, (S.LH_vdw_hh[p1] + S.LH_vdw_hh[p2]) / 2, &rl[3 * i],
                  &rl[3 * j], f1, f2, out.E);
        add3(out.lF, i, f1); add3(out.lF, j, f2);
      }
    }
  }
  for (int i = 0; i < nL; i++) {  // LH - DNA
    int p = lh_param(S, i);
    for (int j = 0; j < n; j++) {
      if (S.type[j] != 0) continue;
      pair_dhlj(S.LH_q[p], S.q_l, eps, S.debye, S.k_ex, S.LH_vdw_hl[p], &rl[3 * i], &r[3 * j], f1, f2, out.E);
      add3(out.lF, i, f1); add3(out.F, j, f2);
    }
  }
  for (int i = 0; i < nL; i++) {  // LH - tails
    int p = lh_param(S, i);
    for (int j = 0; j < nt; j++) {
      pair_dhlj(S.LH_q[p], S.t_q[j], eps, S.debye, S.k_ex, S.LH_vdw_ht[p], &rl[3 * i], &rt[3 * j], f1, f2, out.E);
      add3(out.lF, i, f1);
      tail_or_core(S, X, out, j, f2);
    }
  }
  // globular-head beads ride on the core frame of each LH-bearing core
  auto ghead = [&](int i, int m, double* pos) {
    body_point(&r[3 * i], &a[3 * i], &b[3 * i], &c[3 * i], &S.LH_g_pos[3 * m], pos);
  };
  int k2 = 0;
  for (int i = 0; i < n; i++) {  // G-head - tails
    if (S.type[i] != 1) continue;
    if (S.nc_lh_flag[k2] == 1) {
      for (int m = 0; m < ng; m++) {
        double g[3];
        ghead(i, m, g);
        for (int j = 0; j < nt; j++) {
          pair_dhlj(S.LH_q[m], S.t_q[j], eps, S.debye, S.k_ex, S.LH_vdw_ht[m], g, &rt[3 * j], f1, f2, out.E);
          add3(out.F, i, f1);
          torque_rel(f1, &S.LH_g_pos[3 * m], &a[3 * i], &b[3 * i], &c[3 * i], tq);
          add3(out.T, i, tq);
          tail_or_core(S, X, out, j, f2);
        }
      }
    }
    k2 = k2 + 1;
  }
  int k = 0;
  for (int i = 0; i < n; i++) {  // G-head - linker DNA
    if (S.type[i] != 1) continue;
    if (S.nc_lh_flag[k] == 1) {
      for (int j = 0; j < ng; j++) {
        double g[3];
        ghead(i, j, g);
        for (int l = 0; l < n; l++) {
          if (S.type[l] != 0) continue;
          pair_dhlj(S.LH_q[j], S.q_l, eps, S.debye, S.k_ex, S.LH_vdw_hl[j], g, &r[3 * l], f1, f2, out.E);
          add3(out.F, i, f1); add3(out.F, l, f2);
          torque_rel(f1, &S.LH_g_pos[3 * j], &a[3 * i], &b[3 * i], &c[3 * i], tq);
          add3(out.T, i, tq);
        }
      }
    }
    k = k + 1;
  }
  k = 0;
  for (int i = 0; i < n; i++) {  // G-head - other cores' charges
    if (S.type[i] != 1) continue;
    if (S.nc_lh_flag[k] == 1) {
      for (int j = 0; j < ng; j++) {
        double g[3];
        ghead(i, j, g);
        for (int l = 0; l < n; l++) {
          if (i == l || S.type[l] != 1) continue;
          for (int m = 0; m < S.Nq; m++) {
            double z[3];
            body_point(&r[3 * l], &a[3 * l], &b[3 * l], &c[3 * l], &S.core_pos[3 * m], z);
            pair_dhlj(S.LH_q[j], S.core_q[m], eps, S.debye, S.k_ex, S.LH_vdw_hc[j], g, z, f1, f2, out.E);
            add3(out.F, i, f1); add3(out.F, l, f2);
            torque_rel(f1, &S.LH_g_pos[3 * j], &a[3 * i], &b[3 * i], &c[3 * i], tq);
            add3(out.T, i, tq);
            torque_rel(f2, &S.core_pos[3 * m], &a[3 * l], &b[3 * l], &c[3 * l], tq2);
            add3(out.T, l, tq2);
          }
        }
      }
    }
    k = k + 1;
  }
  k2 = 0;
  int count = 0;
  for (int i = 0; i < n; i++) {  // G-head - LH beads of other LHs
    if (S.type[i] != 1) continue;
    if (S.nc_lh_flag[k2] == 1) {
      for (int m = 0; m < ng; m++) {
        double g[3];
        ghead(i, m, g);
        for (int j = 0; j < nL; j++) {
          if (j / nlh == count) continue;
          int p2 = lh_param(S, j);
          pair_dhlj(S.LH_q[m], S.LH_q[p2], eps, S.debye, S.k_ex, (S.LH_vdw_hh[m] + S.LH_vdw_hh[p2]) / 2, g, &rl[3 * j],
                    f1, f2, out.E);
          add3(out.F, i, f1); add3(out.lF, j, f2);
          torque_rel(f1, &S.LH_g_pos[3 * m], &a[3 * i], &b[3 * i], &c[3 * i], tq);
          add3(out.T, i, tq);
        }
      }
      count = count + 1;
    }
    k2 = k2 + 1;
  }
  k2 = 0;
  for (int i = 0; i < n; i++) {  // G-head - G-head
    if (S.type[i] != 1) continue;
    if (S.nc_lh_flag[k2] == 1) {
      for (int m = 0; m < ng; m++) {
        double g[3];
        ghead(i, m, g);
        int kk = k2 + 1;
        for (int j = i + 1; j < n; j++) {
          if (S.type[j] != 1) continue;
          if (S.nc_lh_flag[kk] == 1) {
            for (int m1 = 0; m1 < ng; m1++) {
              double g2[3];
              ghead(j, m1, g2);
              pair_dhlj(S.LH_q[m], S.LH_q[m1], eps, S.debye, S.k_ex, (S.LH_vdw_hh[m] + S.LH_vdw_hh[m1]) / 2, g, g2, f1,
                        f2, out.E);
              add3(out.F, i, f1); add3(out.F, j, f2);
              torque_rel(f1, &S.LH_g_pos[3 * m], &a[3 * i], &b[3 * i], &c[3 * i], tq);
              add3(out.T, i, tq);
              torque_rel(f2, &S.LH_g_pos[3 * m1], &a[3 * j], &b[3 * j], &c[3 * j], tq);
              add3(out.T, j, tq);
            }
          }
          kk = kk + 1;
        }
      }
    }
    k2 = k2 + 1;
  }
  k = 0;
  k2 = 0;
  for (int i = 0; i < n; i++) {  // G-head <-> first C-term bead anchor
    if (S.type[i] != 1) continue;
    if (S.nc_lh_flag[k2] == 1) {
      for (int j = 0; j < ng; j++) {
        int pj = j + S.n_lh_n;
        if (S.LH_conn[pj] != 1) continue;
        double g[3];
        ghead(i, j, g);
        const double* q = &rl[3 * (k * nlh)];
        double d = std::sqrt((q[0] - g[0]) * (q[0] - g[0]) + (q[1] - g[1]) * (q[1] - g[1]) + (q[2] - g[2]) * (q[2] - g[2]));
        out.E = out.E + S.LH_kstr[pj] * (d - S.LH_streq[pj]) * (d - S.LH_streq[pj]) / 2;
        double st[3];
        for (int x = 0; x < 3; x++) st[x] = (d - S.LH_streq[pj]) * (q[x] - g[x]) / d;
        for (int x = 0; x < 3; x++) out.lF[3 * k * nlh + x] = out.lF[3 * k * nlh + x] - S.LH_kstr[pj] * st[x] * 10;
        for (int x = 0; x < 3; x++) out.F[3 * i + x] = out.F[3 * i + x] + S.LH_kstr[pj] * st[x] * 10;
        double fa = S.LH_kstr[pj] * (a[3 * i] * st[0] + a[3 * i + 1] * st[1] + a[3 * i + 2] * st[2]);
        double fb = S.LH_kstr[pj] * (b[3 * i] * st[0] + b[3 * i + 1] * st[1] + b[3 * i + 2] * st[2]);
        double fc = S.LH_kstr[pj] * (c[3 * i] * st[0] + c[3 * i + 1] * st[1] + c[3 * i + 2] * st[2]);
        const double* gp = &S.LH_g_pos[3 * j];
        out.T[3 * i] = out.T[3 * i] + fc * gp[1] - fb * gp[2];
        out.T[3 * i + 1] = out.T[3 * i + 1] + fa * gp[2] - fc * gp[0];
        out.T[3 * i + 2] = out.T[3 * i + 2] + fb * gp[0] - fa * gp[1];
      }
      k = k + 1;
    }
    k2 = k2 + 1;
  }
}

static void all_forces(const System& S, const State& X, Forces& out) {
  out.zero(S.n, S.n_tail, S.n_LH);
  mechanical(S, X, out);
  electrostatics(S, X, out);
  if (S.n_tail > 0) tails(S, X, out);
  if (S.n_LH > 0) linker_histone(S, X, out);
}

static void refresh(const System& S, State& X) {
  euler_angles(S, X.r, X.a, X.b, X.c, X.fr);
  tail_beta(S, X.r_t, X.beta_t);
  lh_beta(S, X.r_lh, X.beta_lh);
}

// ---------------------------------------------------------------- tensor
static void rall(const System& S, const State& X, Vec& ra) {
  ra.assign(3 * S.n_D, 0.0);
  for (int i = 0; i < S.n; i++) for (int x = 0; x < 3; x++) ra[3 * i + x] = X.r[3 * i + x];
  for (int i = 0; i < S.n_tail; i++) for (int x = 0; x < 3; x++) ra[3 * (S.n + i) + x] = X.r_t[3 * i + x];
  for (int i = 0; i < S.n_LH; i++) for (int x = 0; x < 3; x++) ra[3 * (S.n + S.n_tail + i) + x] = X.r_lh[3 * i + x];
}

// func.cpp:728-804, row-major full symmetric D (m = 3 N_D)
static void rpy(const System& S, const Vec& r, Vec& D) {
  const int N = S.n_D, m = 3 * N;
  const Vec& rad = S.rad_all;
  D.assign((size_t)m * m, 0.0);
  auto at = [&](int i, int j) -> double& { return D[(size_t)i * m + j]; };
  // each pair (i, j >= i) writes only its own two 3x3 blocks
#pragma omp parallel for schedule(dynamic, 8) num_threads(g_threads)
  for (int i = 0; i < N; i++) {
    for (int j = i; j < N; j++) {
      if (i == j) {
        for (int k = 0; k < 3; k++)
          for (int l = 0; l < 3; l++) at(3 * i + k, 3 * j + l) = (k == l) ? S.a1 / rad[i] : 0.0;
        continue;
      }
      double sij[3] = {r[3 * i] - r[3 * j], r[3 * i + 1] - r[3 * j + 1], r[3 * i + 2] - r[3 * j + 2]};
      double ssq = sij[0] * sij[0] + sij[1] * sij[1] + sij[2] * sij[2];
      double s = std::sqrt(ssq);
      if (s >= rad[i] + rad[j]) {
        double f = (rad[i] * rad[i] + rad[j] * rad[j]) / ssq;
        double f1 = 1.0 + f / 3, f2 = 1.0 - f;
        // func.cpp:760-778 writes (k,l) and (l,k) at both iterations, so the
        // value left behind is the one with the larger component index first
        for (int k = 0; k < 3; k++)
          for (int l = 0; l < 3; l++) {
            int kk = k > l ? k : l, ll = k > l ? l : k;
            double v = (k == l) ? (S.a2 / s) * (f1 + f2 * sij[k] * sij[k] / ssq) : (S.a2 / s) * (f2 * sij[kk] * sij[ll] / ssq);
            at(3 * i + k, 3 * j + l) = v;
            at(3 * j + l, 3 * i + k) = v;
          }
      } else {
        double se = std::pow((rad[i] * rad[i] * rad[i] + rad[j] * rad[j] * rad[j]) / 2.0, 1.0 / 3);
        for (int k = 0; k < 3; k++)
          for (int l = 0; l < 3; l++) {
            int kk = k > l ? k : l, ll = k > l ? l : k;
            double v = (k == l) ? (S.a1 / se) * (1.0 - 9.0 * std::sqrt(ssq) / (32 * se) + 3.0 * sij[k] * sij[k] / (32.0 * se * std::sqrt(ssq)))
                                : (S.a1 / se) * (3.0 * sij[kk] * sij[ll] / (32.0 * se * std::sqrt(ssq)));
            at(3 * i + k, 3 * j + l) = v;
            at(3 * j + l, 3 * i + k) = v;
          }
      }
    }
  }
}

}  // namespace orc

using namespace orc;

extern "C" void orc_set_threads(int n) { g_threads = n > 0 ? n : 1; }

// Multi-threaded form of func.cpp:806-836 with the same result bit for bit.
// L[i][j] depends only on columns < j, and every inner product
//   ssq = 0.0; for k = 0 .. j-1: ssq = ssq + L[i][k] * L[j][k]
// is still summed one product at a time in increasing k, each product and
// each sum rounded on its own (the file is built without FMA contraction).
// Only the schedule changes: columns go in blocks of four; the four rows of
// the diagonal block are finished first, one after another as in the
// reference; then every group of four rows below carries the 16 running sums
// of its four rows against the block's four columns through k < j0 together
// (two-wide vectors whose lanes are separate sums, the block's columns packed
// k-major), and finishes each row's four entries in column order.
typedef double orc_v2d __attribute__((vector_size(16)));

static int chol_blocked(int m, const double* D, double* L, int nthreads) {
  constexpr int CB = 4;
  int neg = 0;
  std::vector<double> P((size_t)m * CB + 2 * CB, 0.0);
#pragma omp parallel num_threads(nthreads)
  for (int j0 = 0; j0 < m; j0 += CB) {
    const int cb = std::min(CB, m - j0);
#pragma omp single
    {
      // diagonal block: rows j0 .. j0+cb-1, columns j0 .. j, in the reference's order
      for (int j = j0; j < j0 + cb; j++) {
        double* Lj = L + (size_t)j * m;
        for (int c = j0; c < j; c++) {
          const double* Lc = L + (size_t)c * m;
          double s = 0.0;
          for (int k = 0; k < c; k++) s = s + Lj[k] * Lc[k];
          Lj[c] = (D[(size_t)j * m + c] - s) / Lc[c];
        }
        double s = 0.0;
        for (int k = 0; k < j; k++) s = s + Lj[k] * Lj[k];
        double f = D[(size_t)j * m + j] - s;
        if (f < 0) { neg++; f = -f; }
        Lj[j] = std::sqrt(f);
      }
      // the block's columns k-major: P[4k + c] = L[j0 + c][k], k < j0
      for (int k = 0; k < j0; k++)
        for (int c = 0; c < CB; c++) P[(size_t)CB * k + c] = c < cb ? L[(size_t)(j0 + c) * m + k] : 0.0;
    }
    const int first = j0 + cb, groups = (m - first + 3) / 4;
#pragma omp for schedule(static)
    for (int g = 0; g < groups; g++) {
      const int i0 = first + 4 * g, nr = std::min(4, m - i0);
      const double* Li[4];
      for (int r = 0; r < 4; r++) Li[r] = L + (size_t)(i0 + std::min(r, nr - 1)) * m;
      orc_v2d a00 = {0.0, 0.0}, a01 = a00, a10 = a00, a11 = a00, a20 = a00, a21 = a00, a30 = a00, a31 = a00;
      for (int k = 0; k < j0; k++) {
        orc_v2d p0, p1;
        std::memcpy(&p0, &P[(size_t)CB * k], sizeof p0);
        std::memcpy(&p1, &P[(size_t)CB * k + 2], sizeof p1);
        const orc_v2d b0 = {Li[0][k], Li[0][k]}, b1 = {Li[1][k], Li[1][k]};
        const orc_v2d b2 = {Li[2][k], Li[2][k]}, b3 = {Li[3][k], Li[3][k]};
        a00 = a00 + b0 * p0; a01 = a01 + b0 * p1;
        a10 = a10 + b1 * p0; a11 = a11 + b1 * p1;
        a20 = a20 + b2 * p0; a21 = a21 + b2 * p1;
        a30 = a30 + b3 * p0; a31 = a31 + b3 * p1;
      }
      const orc_v2d acc[4][2] = {{a00, a01}, {a10, a11}, {a20, a21}, {a30, a31}};
      for (int r = 0; r < nr; r++) {
        double* Lr = L + (size_t)(i0 + r) * m;
        for (int c = 0; c < cb; c++) {
          const int j = j0 + c;
          const double* Lj = L + (size_t)j * m;
          double s = acc[r][c >> 1][c & 1];
          for (int k = j0; k < j; k++) s = s + Lr[k] * Lj[k];
          Lr[j] = (D[(size_t)(i0 + r) * m + j] - s) / Lj[j];
        }
      }
    }
  }
  return neg;
}

// func.cpp:806-836.  One thread: the reference's row loop as written; more
// threads: chol_blocked, which gives the same factor bit for bit.
extern "C" int orc_cholesky(int m, const double* D, double* L, int nthreads) {
  int neg = 0;
  if (m <= 0) return 0;
  L[0] = std::sqrt(D[0]);
  if (nthreads <= 1) {
    for (int i = 1; i < m; i++) {
      double* Li = L + (size_t)i * m;
      Li[0] = D[(size_t)i * m] / L[0];
      for (int j = 1; j < i; j++) {
        const double* Lj = L + (size_t)j * m;
        double ssq = 0.0;
        for (int k = 0; k < j; k++) ssq = ssq + Li[k] * Lj[k];
        Li[j] = (D[(size_t)i * m + j] - ssq) / Lj[j];
      }
      double ssq = 0.0;
      for (int k = 0; k < i; k++) ssq = ssq + Li[k] * Li[k];
      double f = D[(size_t)i * m + i] - ssq;
      if (f < 0) { neg++; f = -f; }
      Li[i] = std::sqrt(f);
    }
    return neg;
  }
  return chol_blocked(m, D, L, nthreads);
}

// Diffusion_Tensor's assembly part alone (func.cpp:737-804) for nD beads,
// row-major m x m; used to time a bounded CPU sample of the step.
extern "C" void orc_rpy(int nD, const double* r, const double* rad, double a1, double a2, double* D) {
  System S;
  S.n_D = nD;
  S.a1 = a1;
  S.a2 = a2;
  S.rad_all.assign(rad, rad + nD);
  Vec ra(r, r + 3 * nD), Dv;
  rpy(S, ra, Dv);
  memcpy(D, Dv.data(), sizeof(double) * Dv.size());
}

namespace {
template <class T>
std::vector<T> copyv(const T* p, int cnt) {
  return (p && cnt > 0) ? std::vector<T>(p, p + cnt) : std::vector<T>();
}
}  // namespace

extern "C" void* orc_create(const orc_system* y, const double* r, const double* a, const double* b, const double* c,
                            const double* r_t, const double* r_lh, int do_refresh) {
  System* S = new System();
  S->n = y->n; S->n_c = y->n_c; S->Nq = y->Nq; S->n_t = y->n_t; S->n_tail = y->n_tail;
  S->n_lh_n = y->n_lh_n; S->n_lh_g = y->n_lh_g; S->n_lh_c = y->n_lh_c; S->n_LH = y->n_LH;
  S->n_D = S->n + S->n_tail + S->n_LH;
  S->h = y->h; S->g = y->g; S->s = y->s; S->debyell = y->debyell; S->debye = y->debye; S->q_l = y->q_l;
  S->k_e = y->k_e; S->k_ex = y->k_ex;
  S->sDD = y->sigma_DNA_DNA; S->sDC = y->sigma_DNA_Core; S->sCC = y->sigma_Core_Core;
  S->sTT = y->sigma_Tail_Tail; S->sTL = y->sigma_Tail_Linker; S->sTC = y->sigma_Tail_Core;
  S->a1 = y->a1; S->a2 = y->a2; S->dt = y->time_step; S->del = y->del; S->s2dt = y->s2dt;
  const int n = S->n, nt = S->n_tail, nL = S->n_LH, np = S->n_lh_n + S->n_lh_g + S->n_lh_c;
  S->type = copyv(y->type, n); S->rad = copyv(y->rad, n); S->phi_o = copyv(y->phi_o, n);
  S->core_pos = copyv(y->core_pos, 3 * S->Nq); S->core_q = copyv(y->core_q, S->Nq);
  S->tail_pos = copyv(y->tail_pos, 3 * S->n_t); S->tail_fix = copyv(y->tail_fix, S->n_t);
  S->nc_t_flag = copyv(y->nc_t_flag, S->n_c);
  S->h_t = copyv(y->h_t, nt); S->g_t = copyv(y->g_t, nt); S->lo_t = copyv(y->lo_t, nt);
  S->beta_o_t = copyv(y->beta_o_t, nt); S->t_q = copyv(y->t_q, nt); S->t_rad = copyv(y->t_rad, nt);
  S->t_grp = copyv(y->t_grp, nt); S->t_fix = copyv(y->t_fix, nt);
  S->LH_g_pos = copyv(y->LH_g_pos, 3 * S->n_lh_g); S->LH_conn = copyv(y->LH_conn, np);
  S->nc_lh_flag = copyv(y->nc_lh_flag, S->n_c);
  S->LH_q = copyv(y->LH_q, np); S->LH_vdw_hh = copyv(y->LH_vdw_hh, np); S->LH_vdw_hc = copyv(y->LH_vdw_hc, np);
  S->LH_vdw_hl = copyv(y->LH_vdw_hl, np); S->LH_vdw_ht = copyv(y->LH_vdw_ht, np);
  S->LH_kstr = copyv(y->LH_kstr, np); S->LH_kben = copyv(y->LH_kben, np); S->LH_streq = copyv(y->LH_streq, np);
  S->LH_betaeq = copyv(y->LH_betaeq, np); S->lh_rad = copyv(y->lh_rad, nL);
  S->core_rank.assign(n, -1);
  int cnt = 0;
  for (int i = 0; i < n; i++) { if (S->type[i] == 1) cnt++; S->core_rank[i] = cnt - 1; }
  S->rad_all.assign(S->n_D, 0.0);
  for (int i = 0; i < n; i++) S->rad_all[i] = S->rad[i];
  for (int i = 0; i < nt; i++) S->rad_all[n + i] = S->t_rad[i];
  for (int i = 0; i < nL; i++) S->rad_all[n + nt + i] = S->lh_rad[i];
  State& X = S->st;
  X.r = copyv(r, 3 * n); X.a = copyv(a, 3 * n); X.b = copyv(b, 3 * n); X.c = copyv(c, 3 * n);
  X.r_t = copyv(r_t, 3 * nt); X.r_lh = copyv(r_lh, 3 * nL);
  X.fr.size(n, S->n_c);
  X.beta_t.assign(nt, 0.0); X.beta_lh.assign(nL, 0.0);
  if (do_refresh) refresh(*S, X);
  return S;
}

extern "C" void orc_destroy(void* h) { delete static_cast<System*>(h); }

extern "C" double orc_forces(void* h, double* F, double* T, double* tF, double* lF) {
  System& S = *static_cast<System*>(h);
  Forces out;
  all_forces(S, S.st, out);
  if (F) memcpy(F, out.F.data(), sizeof(double) * 3 * S.n);
  if (T) memcpy(T, out.T.data(), sizeof(double) * 3 * S.n);
  if (tF && S.n_tail) memcpy(tF, out.tF.data(), sizeof(double) * 3 * S.n_tail);
  if (lF && S.n_LH) memcpy(lF, out.lF.data(), sizeof(double) * 3 * S.n_LH);
  return out.E;
}

extern "C" void orc_tensor(void* h, double* D, double* L) {
  System& S = *static_cast<System*>(h);
  Vec ra, Dv;
  rall(S, S.st, ra);
  rpy(S, ra, Dv);
  int m = 3 * S.n_D;
  if (D) memcpy(D, Dv.data(), sizeof(double) * Dv.size());
  if (L) {
    memset(L, 0, sizeof(double) * (size_t)m * m);
    orc_cholesky(m, Dv.data(), L, 1);
  }
}

namespace {
// rotation_cal (func_cuda.cu:681-704) then rotate (func.cpp:1607-1670)
void rotation(const System& S, const Vec& T, const double* rr, const State& X, Vec& an, Vec& bn, Vec& cn) {
  for (int i = 0; i < S.n; i++) {
    double w[3];
    if (S.type[i] != 0) {
      for (int x = 0; x < 3; x++) w[x] = S.dt * T[3 * i + x] / (8 * kPi * kEta * 125.0) + rr[3 * i + x];
    } else {
      w[0] = S.dt * T[3 * i] / (4 * kPi * kEta * kRh * kRh * kLo) + rr[3 * i];
      w[1] = 0.0;
      w[2] = 0.0;
    }
    const double *a = &X.a[3 * i], *b = &X.b[3 * i], *c = &X.c[3 * i];
    double wa = w[0], wb = w[1], wc = w[2];
    double wa2 = wa * wa, wb2 = wb * wb, wc2 = wc * wc, z2 = wa2 + wb2 + wc2, z = std::sqrt(z2);
    double czt = std::cos(z * 1.0), szt = std::sin(z * 1.0), om = 1.0 - czt;
    if (z2 > 0.0) {
      double g1 = ((wb2 + wc2) * czt + wa2) / z2, g2 = wa * wb * om / z2 + wc * szt / z, g3 = wa * wc * om / z2 - wb * szt / z;
      for (int x = 0; x < 3; x++) an[3 * i + x] = g1 * a[x] + g2 * b[x] + g3 * c[x];
      g1 = wa * wb * om / z2 - wc * szt / z; g2 = ((wa2 + wc2) * czt + wb2) / z2; g3 = wb * wc * om / z2 + wa * szt / z;
      for (int x = 0; x < 3; x++) bn[3 * i + x] = g1 * a[x] + g2 * b[x] + g3 * c[x];
      g1 = wa * wc * om / z2 + wb * szt / z; g2 = wb * wc * om / z2 - wa * szt / z; g3 = ((wa2 + wb2) * czt + wc2) / z2;
      for (int x = 0; x < 3; x++) cn[3 * i + x] = g1 * a[x] + g2 * b[x] + g3 * c[x];
    } else {
      for (int x = 0; x < 3; x++) { an[3 * i + x] = a[x]; bn[3 * i + x] = b[x]; cn[3 * i + x] = c[x]; }
    }
  }
}

// translation_cal (func_cuda.cu:650-679): drift inside each species block
void translation(const System& S, const Vec& D, const Forces& Fo, const State& X, const Vec& rd, State& Y) {
  const int m = 3 * S.n_D, n3 = 3 * S.n, nt3 = 3 * S.n_tail;
  for (int col = 0; col < m; col++) {
    const double* Drow = &D[(size_t)col * m];
    if (col < n3) {
      double v = X.r[col] + rd[col];
      for (int k = 0; k < n3; k++) v = v + S.del * Drow[k] * Fo.F[k];
      Y.r[col] = v;
    } else if (col < n3 + nt3) {
      double v = X.r_t[col - n3] + rd[col];
      for (int k = n3; k < n3 + nt3; k++) v = v + S.del * Drow[k] * Fo.tF[k - n3];
      Y.r_t[col - n3] = v;
    } else {
      double v = X.r_lh[col - n3 - nt3] + rd[col];
      for (int k = n3 + nt3; k < m; k++) v = v + S.del * Drow[k] * Fo.lF[k - n3 - nt3];
      Y.r_lh[col - n3 - nt3] = v;
    }
  }
}
}  // namespace

extern "C" double orc_step(void* h, const double* rr, const double* p) {
  System& S = *static_cast<System*>(h);
  State& X = S.st;
  const int m = 3 * S.n_D;
  lh_beta(S, X.r_lh, X.beta_lh);
  Vec ra, D, L((size_t)m * m, 0.0);
  rall(S, X, ra);
  rpy(S, ra, D);
  orc_cholesky(m, D.data(), L.data(), g_threads);
  S.rd.assign(m, 0.0);
#pragma omp parallel for schedule(dynamic, 64) num_threads(g_threads)
  for (int col = 0; col < m; col++) {  // rd_cal, func_cuda.cu:634-647
    double v = 0.0;
    for (int k = 0; k <= col; k++) v += S.s2dt * L[(size_t)col * m + k] * p[k];
    S.rd[col] = v;
  }
  L.clear(); L.shrink_to_fit();
  Forces f0;
  all_forces(S, X, f0);
  S.last = f0;
  State Y = X;
  rotation(S, f0.T, rr, X, Y.a, Y.b, Y.c);
  translation(S, D, f0, X, S.rd, Y);
  refresh(S, Y);
  Forces f1;
  all_forces(S, Y, f1);
  Forces avg = f0;
  for (size_t i = 0; i < avg.F.size(); i++) { avg.F[i] = 0.5 * (f0.F[i] + f1.F[i]); avg.T[i] = 0.5 * (f0.T[i] + f1.T[i]); }
  for (size_t i = 0; i < avg.tF.size(); i++) avg.tF[i] = 0.5 * (f0.tF[i] + f1.tF[i]);
  for (size_t i = 0; i < avg.lF.size(); i++) avg.lF[i] = 0.5 * (f0.lF[i] + f1.lF[i]);
  rotation(S, avg.T, rr, X, Y.a, Y.b, Y.c);
  translation(S, D, avg, X, S.rd, Y);
  X.r = Y.r; X.a = Y.a; X.b = Y.b; X.c = Y.c; X.r_t = Y.r_t; X.r_lh = Y.r_lh;
  refresh(S, X);
  return f0.E;
}

// One move with caller forces and noise: rotation_cal + rotate, then
// translation_cal with the RPY tensor of the current state, then the
// frame refresh (the body of one predictor or corrector half of orc_step).
extern "C" int orc_em_update(void* h, const double* F, const double* T, const double* tF, const double* lF,
                             const double* rr, const double* rd) {
  System& S = *static_cast<System*>(h);
  State& X = S.st;
  const int m = 3 * S.n_D;
  Vec ra, D;
  rall(S, X, ra);
  rpy(S, ra, D);
  Forces f;
  f.zero(S.n, S.n_tail, S.n_LH);
  for (size_t i = 0; i < f.F.size(); i++) { f.F[i] = F[i]; f.T[i] = T[i]; }
  for (size_t i = 0; i < f.tF.size(); i++) f.tF[i] = tF[i];
  for (size_t i = 0; i < f.lF.size(); i++) f.lF[i] = lF[i];
  Vec rdv(rd, rd + m);
  State Y = X;
  rotation(S, f.T, rr, X, Y.a, Y.b, Y.c);
  translation(S, D, f, X, rdv, Y);
  X.r = Y.r; X.a = Y.a; X.b = Y.b; X.c = Y.c; X.r_t = Y.r_t; X.r_lh = Y.r_lh;
  refresh(S, X);
  return 0;
}

extern "C" int orc_get(void* h, const char* nm, double* out) {
  System& S = *static_cast<System*>(h);
  State& X = S.st;
  const Vec* v = nullptr;
  std::string s(nm);
  if (s == "r") v = &X.r; else if (s == "a") v = &X.a; else if (s == "b") v = &X.b; else if (s == "c") v = &X.c;
  else if (s == "r_t") v = &X.r_t; else if (s == "r_lh") v = &X.r_lh;
  else if (s == "alpha") v = &X.fr.alpha; else if (s == "beta") v = &X.fr.beta; else if (s == "gamma") v = &X.fr.gamma;
  else if (s == "length") v = &X.fr.length; else if (s == "a_dna") v = &X.fr.a_dna; else if (s == "b_dna") v = &X.fr.b_dna;
  else if (s == "c_dna") v = &X.fr.c_dna; else if (s == "alpha_p") v = &X.fr.alpha_p; else if (s == "beta_p") v = &X.fr.beta_p;
  else if (s == "gamma_p") v = &X.fr.gamma_p; else if (s == "beta_t") v = &X.beta_t; else if (s == "beta_lh") v = &X.beta_lh;
  else if (s == "rd") v = &S.rd; else if (s == "force") v = &S.last.F; else if (s == "torque") v = &S.last.T;
  else if (s == "t_force") v = &S.last.tF; else if (s == "LH_force") v = &S.last.lF;
  if (!v) return -1;
  if (out && !v->empty()) memcpy(out, v->data(), sizeof(double) * v->size());
  return (int)v->size();
}

extern "C" int orc_set(void* h, const char* nm, const double* in) {
  System& S = *static_cast<System*>(h);
  State& X = S.st;
  Vec* v = nullptr;
  std::string s(nm);
  if (s == "r") v = &X.r; else if (s == "a") v = &X.a; else if (s == "b") v = &X.b; else if (s == "c") v = &X.c;
  else if (s == "r_t") v = &X.r_t; else if (s == "r_lh") v = &X.r_lh;
  if (!v) return -1;
  memcpy(v->data(), in, sizeof(double) * v->size());
  refresh(S, X);
  return (int)v->size();
}

// ---------------------------------------------------------------- noise
// MT19937 (Matsumoto & Nishimura 1998) and the polar Box-Muller method as
// used by utilities.cpp:304-336 (one cached deviate carried across calls).
namespace {
struct Noise {
  uint32_t st[624];
  int idx = 625;
  double cached = 0.0;
  bool have = false;
  void seed(uint32_t s) {
    st[0] = s;
    for (int i = 1; i < 624; i++) st[i] = 1812433253u * (st[i - 1] ^ (st[i - 1] >> 30)) + (uint32_t)i;
    idx = 624;
  }
  uint32_t next() {
    if (idx >= 624) {
      if (idx == 625) seed(5489u);
      for (int i = 0; i < 624; i++) {
        uint32_t y = (st[i] & 0x80000000u) | (st[(i + 1) % 624] & 0x7fffffffu);
        st[i] = st[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
      }
      idx = 0;
    }
    uint32_t y = st[idx++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
  }
  double real1() { return next() * (1.0 / 4294967295.0); }
  double normal(double mean, double sd) {
    if (!have) {
      double x, y, rr;
      do {
        x = 2.0 * real1() - 1;
        y = 2.0 * real1() - 1;
        rr = x * x + y * y;
      } while (rr == 0.0 || rr > 1.0);
      double d = std::sqrt(-2.0 * std::log(rr) / rr);
      cached = y * d;
      have = true;
      return x * d * sd + mean;
    }
    have = false;
    return cached * sd + mean;
  }
};
}  // namespace

extern "C" void* orc_noise_create(unsigned long seed) {
  Noise* g = new Noise();
  g->seed((uint32_t)(seed & 0xffffffffUL));
  return g;
}
extern "C" void orc_noise_destroy(void* g) { delete static_cast<Noise*>(g); }
extern "C" unsigned int orc_noise_u32(void* g) { return static_cast<Noise*>(g)->next(); }
extern "C" double orc_noise_real1(void* g) { return static_cast<Noise*>(g)->real1(); }
extern "C" double orc_noise_normal(void* g, double mean, double sd) { return static_cast<Noise*>(g)->normal(mean, sd); }
extern "C" void orc_noise_step(void* gp, int step, int n3, const double* r_var, int nD3, double* rr, double* p) {
  Noise& g = *static_cast<Noise*>(gp);
  if (step % 100 == 0) { (void)g.real1(); (void)g.real1(); }
  for (int i = 0; i < n3; i++) rr[i] = g.normal(0, r_var[i]);
  for (int i = 0; i < nD3; i++) p[i] = g.normal(0, 1);
}
