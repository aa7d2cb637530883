// Test harness (built by tests/test_adjoint_terms.py with g++; not part of
// the library): the scalar-generic force-field terms of the adjoint kernels
// (adj_terms.cuh) compiled for the host.
//   adjh_forces      sums the terms exactly as the adjoint kernels split
//                    them, in double, for comparison with the CPU oracle's
//                    forces on the same state;
//   adjh_vjp_check   compares every term's dual-number vector-Jacobian
//                    product with central finite differences of the same
//                    term at random inputs.
#include <cmath>
#include <random>
#include <vector>

#include "adj_terms.cuh"

using namespace adj;

namespace {
struct Sys {
  int n, nc, Nq, n_t, nt;
  const int *type, *tail_fix, *nc_t_flag, *t_grp;
  const double *phi_o, *core_pos, *core_q, *tail_pos, *h_t, *g_t, *lo_t, *beta_o_t, *t_q;
  double h, g, s, debyell, debye, q_l, k_e, k_ex, sDD, sDC, sCC, sTL;
};

int sidx(int n3, int i, int q) { return (q / 3) * n3 + 3 * i + q % 3; }

bool pair_ok(const Sys& S, int i, int j) {
  if (S.type[i + 1] != 0) return false;
  if (i > 0 && S.type[i - 1] != 0) return false;
  if (j < S.n - 1 && S.type[j + 1] != 0) return false;
  if (S.type[j - 1] != 0) return false;
  return true;
}
}  // namespace

extern "C" int adjh_forces(const int* isz, const int* const* iarr, const double* const* darr, const double* par,
                           const double* x, double* F, double* T, double* tF) {
  Sys S;
  S.n = isz[0]; S.nc = isz[1]; S.Nq = isz[2]; S.n_t = isz[3]; S.nt = isz[4];
  S.type = iarr[0]; S.tail_fix = iarr[1]; S.nc_t_flag = iarr[2]; S.t_grp = iarr[3];
  S.phi_o = darr[0]; S.core_pos = darr[1]; S.core_q = darr[2]; S.tail_pos = darr[3]; S.h_t = darr[4];
  S.g_t = darr[5]; S.lo_t = darr[6]; S.beta_o_t = darr[7]; S.t_q = darr[8];
  S.h = par[0]; S.g = par[1]; S.s = par[2]; S.debyell = par[3]; S.debye = par[4]; S.q_l = par[5];
  S.k_e = par[6]; S.k_ex = par[7]; S.sDD = par[8]; S.sDC = par[9]; S.sCC = par[10]; S.sTL = par[11];
  const int n = S.n, n3 = 3 * n, nt = S.nt;
  for (int i = 0; i < n3; i++) F[i] = T[i] = 0.0;
  for (int i = 0; i < 3 * nt; i++) tF[i] = 0.0;
  std::vector<int> core_bead;
  for (int i = 0; i < n; i++)
    if (S.type[i] == 1) core_bead.push_back(i);
  auto bead = [&](int i, double* o) {
    for (int q = 0; q < 12; q++) o[q] = x[sidx(n3, i, q)];
  };
  for (int i = 0; i < n - 1; i++) {
    BondInfo k;
    k.ti = S.type[i]; k.tn = S.type[i + 1]; k.has_prev = i > 0; k.tp = i > 0 ? S.type[i - 1] : 1;
    k.last = i == n - 2; k.phi_i = S.phi_o[i]; k.phi_p = i > 0 ? S.phi_o[i - 1] : 0.0;
    double xp[12] = {0}, xi[12], xn[12], out[12];
    if (i > 0) bead(i - 1, xp);
    bead(i, xi);
    bead(i + 1, xn);
    bond_term(k, xp, xi, xn, S.h, S.g, S.s, out);
    for (int q = 0; q < 3; q++) {
      F[3 * i + q] += out[q];
      F[3 * i + 3 + q] += out[3 + q];
      T[3 * i + q] += out[6 + q];
      T[3 * i + 3 + q] += out[9 + q];
    }
  }
  for (int i = 0; i < n; i++)
    for (int j = i + 1; j < n; j++) {
      if (!pair_ok(S, i, j)) continue;
      double dd[3] = {x[3 * i] - x[3 * j], x[3 * i + 1] - x[3 * j + 1], x[3 * i + 2] - x[3 * j + 2]};
      if (norm3(dd) > 25.0) continue;
      const bool adj = j - i > 1;
      if (S.type[i] == 0 && S.type[j] == 0) {
        if (!adj) continue;
        double f[3];
        pair_dna_dna(S.k_e * S.q_l * S.q_l, S.k_ex, S.sDD, dd, S.debyell, f);
        for (int q = 0; q < 3; q++) {
          F[3 * i + q] += f[q];
          F[3 * j + q] -= f[q];
        }
      } else if (S.type[i] == 0 || S.type[j] == 0) {
        const int dn = S.type[i] == 0 ? i : j, cr = S.type[i] == 0 ? j : i;
        double xc[12];
        bead(cr, xc);
        for (int s = 0; s < S.Nq; s++) {
          const double* cp = S.core_pos + 3 * s;
          double z[3], f[3];
          for (int q = 0; q < 3; q++) z[q] = x[3 * dn + q] - (xc[q] + xc[3 + q] * cp[0] + xc[6 + q] * cp[1] + xc[9 + q] * cp[2]);
          pair_site(S.k_e * S.q_l * S.core_q[s], adj, S.core_q[s] > 0, S.k_ex, S.sDC, z, S.debye, f);
          double Fb[3] = {-dot3(xc + 3, f), -dot3(xc + 6, f), -dot3(xc + 9, f)}, t[3];
          cross3(cp, Fb, t);
          for (int q = 0; q < 3; q++) {
            F[3 * dn + q] += f[q];
            F[3 * cr + q] -= f[q];
            T[3 * cr + q] += t[q];
          }
        }
      } else {
        double xi[12], xj[12];
        bead(i, xi);
        bead(j, xj);
        for (int k = 0; k < S.Nq; k++)
          for (int l = 0; l < S.Nq; l++) {
            const double *ck = S.core_pos + 3 * k, *cl = S.core_pos + 3 * l;
            double z[3], f[3];
            for (int q = 0; q < 3; q++)
              z[q] = (xi[q] + xi[3 + q] * ck[0] + xi[6 + q] * ck[1] + xi[9 + q] * ck[2]) -
                     (xj[q] + xj[3 + q] * cl[0] + xj[6 + q] * cl[1] + xj[9 + q] * cl[2]);
            pair_site(S.k_e * S.core_q[k] * S.core_q[l], true, true, S.k_ex, S.sCC, z, S.debye, f);
            double Fi[3] = {dot3(xi + 3, f), dot3(xi + 6, f), dot3(xi + 9, f)};
            double Fj[3] = {-dot3(xj + 3, f), -dot3(xj + 6, f), -dot3(xj + 9, f)}, ti[3], tj[3];
            cross3(ck, Fi, ti);
            cross3(cl, Fj, tj);
            for (int q = 0; q < 3; q++) {
              F[3 * i + q] += f[q];
              F[3 * j + q] -= f[q];
              T[3 * i + q] += ti[q];
              T[3 * j + q] += tj[q];
            }
          }
      }
    }
  const double* rt = x + 4 * n3;
  const double eps = 1.0 / (4 * kPi * S.k_e);
  for (int i = 0; i < nt; i++) {
    if (i < nt - 1 && S.t_grp[i] == S.t_grp[i + 1]) {
      double f[3];
      stretch_f(S.h_t[i], S.lo_t[i], rt + 3 * i, rt + 3 * i + 3, f);
      for (int q = 0; q < 3; q++) {
        tF[3 * i + q] += f[q];
        tF[3 * i + 3 + q] -= f[q];
      }
    }
    if (i < nt - 2 && S.t_grp[i] == S.t_grp[i + 1] && S.t_grp[i] == S.t_grp[i + 2]) {
      double f[9];
      bend3_f(S.g_t[i], S.beta_o_t[i], rt + 3 * i, rt + 3 * i + 3, rt + 3 * i + 6, f);
      for (int q = 0; q < 9; q++) tF[3 * i + q] -= f[q];
    }
    for (int j = 0; j < nt + n; j++) {
      const bool tt = j < nt;
      if (tt ? !(i < j && (S.t_grp[i] != S.t_grp[j] || j > i + 2)) : S.type[j - nt] != 0) continue;
      const int jj = tt ? j : j - nt;
      const double* xj = tt ? rt + 3 * jj : x + 3 * jj;
      double z[3] = {rt[3 * i] - xj[0], rt[3 * i + 1] - xj[1], rt[3 * i + 2] - xj[2]}, f[3];
      if (tt) pair_clamped(S.t_q[i] * S.t_q[jj], eps, false, 0.0, 1.0, z, S.debye, f);
      else pair_clamped(S.t_q[i] * S.q_l, eps, true, S.k_ex, S.sTL, z, S.debye, f);
      double* Fj = tt ? tF + 3 * jj : F + 3 * jj;
      for (int q = 0; q < 3; q++) {
        tF[3 * i + q] += f[q];
        Fj[q] -= f[q];
      }
    }
  }
  for (int kc = 0; kc < S.nc; kc++) {
    if (S.nc_t_flag[kc] != 1) continue;
    const int i = core_bead[kc];
    double xc[12];
    bead(i, xc);
    for (int jt = 0; jt < S.n_t; jt++) {
      if (S.tail_fix[jt] != 1) continue;
      const int tb = kc * S.n_t + jt;
      double out[9];
      anchor_term(S.tail_pos + 3 * jt, rt + 3 * tb, xc, S.h, out);
      for (int q = 0; q < 3; q++) {
        tF[3 * tb + q] += out[q];
        F[3 * i + q] += out[3 + q];
        T[3 * i + q] += out[6 + q];
      }
    }
  }
  return 0;
}

namespace {
// max over inputs of |vjp - fd| / max |fd| for y = f(x), fd the Richardson
// extrapolation of central differences with steps h and h/2; -1 when the
// two steps disagree (a branch switch or a near-singular input within h)
template <int NIN, int NOUT, class F>
double check(const F& f, const double* x0, std::mt19937& g) {
  std::normal_distribution<double> N(0.0, 1.0);
  double yb[NOUT];
  for (int o = 0; o < NOUT; o++) yb[o] = N(g);
  double vj[NIN], fd[NIN];
  for (int c = 0; c * 8 < NIN; c++) {
    double xb[8];
    vjp_chunk<8, NIN, NOUT>(f, x0, yb, c, xb);
    for (int j = 0; j < 8 && c * 8 + j < NIN; j++) vj[c * 8 + j] = xb[j];
  }
  auto cd = [&](int k, double h) {
    double xp[NIN], xm[NIN], yp[NOUT], ym[NOUT];
    for (int q = 0; q < NIN; q++) xp[q] = xm[q] = x0[q];
    xp[k] += h;
    xm[k] -= h;
    f(xp, yp);
    f(xm, ym);
    double s = 0.0;
    for (int o = 0; o < NOUT; o++) s += yb[o] * (yp[o] - ym[o]) / (2 * h);
    return s;
  };
  double scale = 0.0, err = 0.0;
  bool rough = false;
  for (int k = 0; k < NIN; k++) {
    const double h = 1e-5 * (1.0 + std::fabs(x0[k]));
    const double f1 = cd(k, h), f2 = cd(k, h / 2);
    fd[k] = (4 * f2 - f1) / 3;
    if (std::fabs(f1 - f2) > 1e-4 * (std::fabs(f2) + 1e-3)) rough = true;
    scale = std::fmax(scale, std::fabs(fd[k]));
  }
  if (rough) return -1.0;
  for (int k = 0; k < NIN; k++) err = std::fmax(err, std::fabs(vj[k] - fd[k]));
  return err / (scale + 1e-30);
}

void frame(std::mt19937& g, double* x, double spread) {
  std::normal_distribution<double> N(0.0, 1.0);
  double a[3] = {N(g), N(g), N(g)}, b[3] = {N(g), N(g), N(g)}, c[3];
  double na = norm3(a);
  for (double& v : a) v /= na;
  double ba = dot3(a, b);
  for (int q = 0; q < 3; q++) b[q] -= ba * a[q];
  double nb = norm3(b);
  for (double& v : b) v /= nb;
  cross3(a, b, c);
  for (int q = 0; q < 3; q++) {
    x[q] = spread * N(g);
    x[3 + q] = a[q];
    x[6 + q] = b[q];
    x[9 + q] = c[q];
  }
}
}  // namespace

// out[k]: worst relative VJP error of term k over `trials` random inputs,
// out[10 + k]: the number of inputs smooth enough to be checked:
// 0 bond (DNA-DNA-DNA), 1 bond (core-DNA), 2 bond (DNA-core-DNA),
// 3 frame refresh, 4 rotation, 5 RPY block, 6 DNA pair, 7 clamped pair,
// 8 tail bend, 9 anchor
extern "C" int adjh_vjp_check(int trials, unsigned seed, double* out) {
  std::mt19937 g(seed);
  std::normal_distribution<double> N(0.0, 1.0);
  for (int k = 0; k < 20; k++) out[k] = 0.0;
  // out[k] = worst error of term k, out[10 + k] = trials it was checked on
  auto put = [&](int k, double e) {
    if (e < 0) return;
    out[k] = std::fmax(out[k], e);
    out[10 + k] += 1;
  };
  for (int t = 0; t < trials; t++) {
    // a straight-ish chain: bead i at 3 nm steps with its a along the bond
    for (int variant = 0; variant < 3; variant++) {
      BondInfo k;
      const int tps[3] = {1, 0, 0}, tis[3] = {0, 1, 0}, tns[3] = {0, 0, 1};
      k.tp = tps[variant];
      k.ti = tis[variant];
      k.tn = tns[variant];
      k.has_prev = variant != 1 ? 1 : (t % 2);
      k.last = t % 3 == 0;
      k.phi_p = 0.3 * N(g);
      k.phi_i = 0.3 * N(g);
      double x[39];
      for (int b = 0; b < 3; b++) {
        frame(g, x + 12 * b, 0.3);
        x[12 * b] += 3.0 * b;
      }
      // align each a with the next bond roughly (as a refreshed chain has)
      x[36] = 1.0 + 0.1 * N(g);
      x[37] = 0.5 + 0.1 * N(g);
      x[38] = 0.7 + 0.1 * N(g);
      auto f = [&](const auto* xd, auto* yd) { bond_term(k, xd, xd + 12, xd + 24, xd[36], xd[37], xd[38], yd); };
      put(variant, check<39, 12>(f, x, g));
    }
    {
      double x[21], f1[12], f2[12];
      frame(g, f1, 0.0);
      frame(g, f2, 0.0);
      for (int q = 0; q < 3; q++) {
        x[q] = 0.3 * N(g);
        x[3 + q] = x[q] + (q == 0 ? 3.0 : 0.0) + 0.3 * N(g);
        x[6 + q] = f1[3 + q];
        x[9 + q] = f1[6 + q];
        x[12 + q] = f2[3 + q];
        x[15 + q] = f2[6 + q];
        x[18 + q] = f2[9 + q];
      }
      const int tn = t % 2;
      auto f = [&](const auto* xd, auto* yd) { frame_pass1(tn, xd, xd + 3, xd + 6, xd + 9, xd + 12, xd + 15, xd + 18, yd); };
      put(3, check<21, 9>(f, x, g));
    }
    {
      double x[12], fr[12];
      frame(g, fr, 0.0);
      for (int q = 0; q < 3; q++) x[q] = 1e-3 * N(g);
      for (int q = 0; q < 9; q++) x[3 + q] = fr[3 + q];
      double rr[3] = {0.05 * N(g), 0.05 * N(g), 0.05 * N(g)};
      const int core = t % 2;
      auto f = [&](const auto* xd, auto* yd) { rotate_frame(core, 1e-12, rr, xd, xd + 3, yd); };
      put(4, check<12, 9>(f, x, g));
    }
    {
      double s[3] = {N(g), N(g), N(g)};
      const double sc = (t % 2) ? 4.0 : 1.2;
      for (double& v : s) v *= sc;
      auto f = [&](const auto* xd, auto* yd) { rpy_block(1.5, 0.6, 0.7, 0.9, xd, yd); };
      put(5, check<3, 9>(f, s, g));
    }
    {
      double z[4] = {3 * N(g), 3 * N(g), 3 * N(g), 0.8};
      auto f = [&](const auto* xd, auto* yd) { pair_dna_dna(2.0, 0.01, 3.0, xd, xd[3], yd); };
      put(6, check<4, 3>(f, z, g));
      auto f2 = [&](const auto* xd, auto* yd) { pair_clamped(0.5, 0.3, true, 0.01, 1.8, xd, xd[3], yd); };
      put(7, check<4, 3>(f2, z, g));
    }
    {
      double x[9];
      for (int q = 0; q < 9; q++) x[q] = 0.7 * (q / 3) * (q % 3 == 0) + 0.2 * N(g);
      auto f = [&](const auto* xd, auto* yd) { bend3_f(0.4, 2.5, xd, xd + 3, xd + 6, yd); };
      put(8, check<9, 9>(f, x, g));
    }
    {
      double x[16], fr[12];
      frame(g, fr, 1.0);
      for (int q = 0; q < 3; q++) x[q] = 2.0 + N(g);
      for (int q = 0; q < 12; q++) x[3 + q] = fr[q];
      x[15] = 1.3;
      const double P[3] = {1.0, -2.0, 0.5};
      auto f = [&](const auto* xd, auto* yd) { anchor_term(P, xd, xd + 3, xd[15], yd); };
      put(9, check<16, 9>(f, x, g));
    }
  }
  return 0;
}
