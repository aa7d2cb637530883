// Test infrastructure only: a C-ABI driver around the reference's own CPU
// physics (func.cpp, readfile.cpp, mt.cpp, utilities.cpp), compiled from the
// reference sources where they lie by oracle/Makefile into oracle/_ref/.
// It is the checker that pins oracle/bd_oracle.cpp; nothing in the product
// links it.
//
// Setup restates main.cpp:38-372 (file readers, update_phi_o,
// update_Euler_Angle, build_tail, build_LH, betas, r_var).  One step restates
// the order of main_cuda (func_cuda.cu:3434-3680) with the CPU functions of
// func.cpp; the GPU-only pieces are restated from func_cuda.cu:
//   rd_cal            func_cuda.cu:634-647
//   translation_cal   func_cuda.cu:650-679  (species-block-diagonal drift)
//   rotation_cal      func_cuda.cu:681-704  (d_theta, then rotate())
//   force_torque_tmp  func_cuda.cu:2626-2641
//   final_updates     func_cuda.cu:2643-2662
// Noise: the reference's MT19937 + polar Box-Muller stream in main.cpp order
// (main.cpp:386-388 two uniforms every 100 steps; :479-486 rr then p).
#include "constants.h"
#include "readfile.h"
#include "func.h"
#include "utilities.h"
#include <unistd.h>
#include <cstring>

namespace {

struct RefSys {
  // sizes
  int n = 0, n_c = 0, n3 = 0, nc3 = 0;
  int Nq = 0, Nq3 = 0, n_t = 0, n_tail = 0, n_tail3 = 0;
  int n_lh_n = 0, n_lh_g = 0, n_lh_c = 0, n_LH = 0, n_LH3 = 0, nc_lh = 0;
  int n_D = 0, n_D3 = 0;
  // constants (main.cpp:42-99)
  double T, Cs, unbind, Pbind;
  int nsteps, freq, freq_RP, Mg;
  double sDD, sDC, sCC, sTT, sTL, sTC;
  double q_l, debye, debyell, k_e, k_ex, k_h1, a1, a2, h, g, s, time_step, del, s2dt, kbt;
  // chain
  std::vector<int> type;
  std::vector<double> r, a, b, c, Er, rad, alpha, beta, gamma, phi_o, length;
  std::vector<double> a_dna, b_dna, c_dna, alpha_p, beta_p, gamma_p, r_var;
  // tails
  std::vector<double> core_pos, core_q, tail_pos, tail_q, tail_rad, tail_bond_c, tail_bond_v, tail_angle_c, tail_angle_v;
  std::vector<int> tail_grp, tail_fix;
  std::vector<int> nc_t_flag;
  std::vector<double> r_t, beta_t, h_t, g_t, lo_t, beta_o_t, t_q, t_rad;
  std::vector<int> t_grp, t_fix;   // padded by 2 sentinels (update_tail_beta reads i+2)
  // LH
  std::vector<double> LH_n_pos, LH_g_pos, LH_c_pos, LH_q, LH_vdw_hh, LH_vdw_hc, LH_vdw_hl, LH_vdw_ht,
      LH_kstr, LH_kben, LH_streq, LH_betaeq, LH_radius;
  std::vector<int> LH_conn, nc_lh_flag;
  std::vector<double> r_lh, lh_rad, beta_lh;
  std::vector<double> rad_all;
  // last step's diagnostics
  std::vector<std::vector<double>> D, Chol;
  std::vector<double> rd, force, torque, t_force, LH_force;
  double energy = 0.0;
};

RefSys* S = nullptr;

void forces(RefSys& s, std::vector<double>& r, std::vector<double>& a, std::vector<double>& b,
            std::vector<double>& c, std::vector<double>& alpha, std::vector<double>& beta,
            std::vector<double>& gamma, std::vector<double>& length, std::vector<double>& a_dna,
            std::vector<double>& b_dna, std::vector<double>& c_dna, std::vector<double>& alpha_p,
            std::vector<double>& beta_p, std::vector<double>& gamma_p, std::vector<double>& r_t,
            std::vector<double>& beta_t, std::vector<double>& r_lh, std::vector<double>& beta_lh,
            std::vector<double>& F, std::vector<double>& Tq, std::vector<double>& tF,
            std::vector<double>& lF, double& E) {
  F.assign(s.n3, 0.0); Tq.assign(s.n3, 0.0); tF.assign(std::max(s.n_tail3, 1), 0.0);
  lF.assign(std::max(s.n_LH3, 1), 0.0); E = 0.0;
  // mechanical first: it assigns DNA torques (func.cpp:1206-1209,1283-1285)
  mechanical_force_and_torque(s.n_c, s.nc3, s.n, s.n3, s.type.data(), r.data(), a.data(), b.data(), c.data(),
      alpha.data(), beta.data(), gamma.data(), length.data(), a_dna.data(), b_dna.data(), c_dna.data(),
      alpha_p.data(), beta_p.data(), gamma_p.data(), s.h, s.g, s.s, s.phi_o.data(), F.data(), Tq.data(), E, 0, 1);
  Electrostatic_and_Excluded_volume_force(s.n, s.n3, s.n_c, s.nc3, s.type.data(), r.data(), a.data(), b.data(),
      c.data(), s.debyell, s.debye, s.q_l, s.k_e, s.k_ex, s.k_h1, s.sDD, s.sDC, s.sCC, s.Nq, s.Nq3, s.core_pos,
      s.core_q, F.data(), Tq.data(), E, 0, 1);
  if (s.n_tail > 0)
    tail_force(s.n, s.n_t, s.type.data(), s.n_tail, s.n_tail3, s.tail_pos, s.tail_fix, s.nc_t_flag.data(),
        r_t.data(), beta_t.data(), s.h_t.data(), s.g_t.data(), s.lo_t.data(), s.beta_o_t.data(), s.h, s.k_e,
        s.debye, s.k_ex, s.t_q.data(), s.t_rad.data(), s.t_grp.data(), s.t_fix.data(), r.data(), a.data(),
        b.data(), c.data(), s.q_l, s.Nq, s.Nq3, s.core_pos, s.core_q, tF.data(), F.data(), Tq.data(), s.sTT,
        s.sTL, s.sTC, E, 0, 1);
  if (s.n_LH > 0)
    Linker_Histone_force(s.n, s.n_tail, s.n_lh_n, s.n_lh_g, s.n_lh_c, s.t_grp.data(), s.t_fix.data(),
        s.type.data(), s.n_LH, s.n_LH3, s.LH_g_pos, s.LH_conn, s.nc_lh_flag.data(), beta_lh.data(), r_lh.data(),
        s.LH_q, s.k_e, s.debye, s.k_ex, s.LH_vdw_hh, s.LH_vdw_hc, s.LH_vdw_hl, s.LH_vdw_ht, s.LH_kstr, s.LH_kben,
        s.LH_streq, s.LH_betaeq, r.data(), a.data(), b.data(), c.data(), s.q_l, s.Nq, s.Nq3, s.core_pos,
        s.core_q, r_t.data(), s.t_q.data(), tF.data(), lF.data(), F.data(), Tq.data(), E, 0, 1);
}

// rotation_cal (func_cuda.cu:681-704) with sequential semantics, then rotate()
void rotation(RefSys& s, const std::vector<double>& torque, const double* rr, std::vector<double>& a,
              std::vector<double>& b, std::vector<double>& c, std::vector<double>& a_n,
              std::vector<double>& b_n, std::vector<double>& c_n) {
  std::vector<double> dth(s.n3);
  for (int j = 0; j < s.n; j++) {
    int j1 = 3 * j;
    if (s.type[j] != 0) {
      for (int x = 0; x < 3; x++) dth[j1 + x] = s.time_step * torque[j1 + x] / (8 * PI * eta * 125.0) + rr[j1 + x];
    } else {
      dth[j1] = s.time_step * torque[j1] / (4 * PI * eta * r_h * r_h * lo) + rr[j1];
      dth[j1 + 1] = 0.0;
      dth[j1 + 2] = 0.0;
    }
  }
  rotate(s.n, s.n3, a.data(), b.data(), c.data(), a_n.data(), b_n.data(), c_n.data(), dth.data(), 1.0);
}

// translation_cal (func_cuda.cu:650-679): drift only inside the species blocks
void translation(RefSys& s, const std::vector<double>& F, const std::vector<double>& tF,
                 const std::vector<double>& lF, std::vector<double>& r_n, std::vector<double>& r_t_n,
                 std::vector<double>& r_lh_n) {
  const int n3 = s.n3, nt3 = s.n_tail3, nl3 = s.n_LH3;
  for (int col = 0; col < s.n_D3; col++) {
    if (col < n3) {
      double v = s.r[col] + s.rd[col];
      for (int k = 0; k < n3; k++) v = v + s.del * s.D[col][k] * F[k];
      r_n[col] = v;
    } else if (col < n3 + nt3) {
      double v = s.r_t[col - n3] + s.rd[col];
      for (int k = n3; k < n3 + nt3; k++) v = v + s.del * s.D[col][k] * tF[k - n3];
      r_t_n[col - n3] = v;
    } else {
      double v = s.r_lh[col - n3 - nt3] + s.rd[col];
      for (int k = n3 + nt3; k < n3 + nt3 + nl3; k++) v = v + s.del * s.D[col][k] * lF[k - n3 - nt3];
      r_lh_n[col - n3 - nt3] = v;
    }
  }
}

void refresh_rall(RefSys& s, std::vector<double>& r_all) {
  r_all.assign(s.n_D3, 0.0);
  for (int i = 0; i < s.n_D; i++) {
    for (int x = 0; x < 3; x++) {
      if (i < s.n) r_all[i * 3 + x] = s.r[i * 3 + x];
      else if (i < s.n + s.n_tail) r_all[i * 3 + x] = s.r_t[i * 3 - s.n3 + x];
      else r_all[i * 3 + x] = s.r_lh[i * 3 - s.n3 - s.n_tail3 + x];
    }
  }
}

void build_tensor(RefSys& s) {
  std::vector<double> r_all;
  refresh_rall(s, r_all);
  s.D.assign(s.n_D3, std::vector<double>(s.n_D3, 0.0));
  s.Chol.assign(s.n_D3, std::vector<double>(s.n_D3, 0.0));
  Diffusion_Tensor(s.n_D, s.n_D3, r_all.data(), s.a1, s.a2, s.rad_all.data(), s.D, s.Chol);
}

}  // namespace

extern "C" {

// Reads the reference input files from `dir` (setup.txt, data_mod, LH.in and
// the three named parameter files) with the reference readers and sets the
// system up exactly as main.cpp:38-372 does; the MT19937 stream is seeded
// with `seed` (main.cpp:60-62 uses time(0)).
int ref_init(const char* dir, const char* core_file, const char* tail_file, const char* lh_file,
             unsigned long seed) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof cwd)) return -1;
  if (chdir(dir) != 0) return -2;
  delete S;
  S = new RefSys();
  RefSys& s = *S;
  std::vector<double> ic = Read_const("setup.txt");
  if (ic.size() < 15) { chdir(cwd); return -3; }
  s.T = ic[0]; s.nsteps = (int)ic[1]; s.freq = (int)ic[2]; s.freq_RP = (int)ic[3];
  s.sDD = ic[4]; s.sDC = ic[5]; s.sCC = ic[6]; s.sTT = ic[7]; s.sTL = ic[8]; s.sTC = ic[9];
  s.Mg = (int)ic[10]; s.Cs = ic[11]; s.unbind = ic[13]; s.Pbind = ic[14];
  init_genrand(seed);
  double kb = 1.380649e-5;
  s.kbt = kb * 300.0;
  s.q_l = lo * (-5.8824) * (1.901912136835033e-8 * pow((s.Cs * 1000), 3.0) + -8.211102025728157e-6 * pow((s.Cs * 1000), 2.0)
        + 7.554037628581672e-3 * (s.Cs * 1000) + 3.524292543853884e-1);
  double per;
  s.debye = 0.736 * sqrt((s.Cs / 0.05) * (298 / s.T));
  if (s.Mg == 0) { per = 50; s.debyell = s.debye; } else { per = 30; s.debyell = 2.5; }
  s.k_e = 0.4151 * kb * 300; s.k_ex = 0.001 * s.kbt; s.k_h1 = 10.0 * s.kbt;
  s.a1 = s.kbt / (6 * PI * eta); s.a2 = s.kbt / (8 * PI * eta);
  s.h = 100 * s.kbt / (lo * lo); s.g = per * s.kbt / lo; s.s = 72.429 * s.kbt / lo;
  s.time_step = 1e-12; s.del = s.time_step / s.kbt; s.s2dt = sqrt(2 * s.time_step);

  std::vector<double> tr, ta, tb, tc, trad, tEr; std::vector<int> ttype;
  Read_initial_struc(s.n, s.n_c, s.n3, s.nc3, tr, ta, tb, tc, trad, tEr, ttype, "data_mod");
  s.r = tr; s.a = ta; s.b = tb; s.c = tc; s.Er = tEr; s.rad = trad; s.type = ttype;
  const bool restart = (int)ic[12] == 1;  // main.cpp:143-153
  if (restart) Read_restart_ini(s.n3, s.r.data(), s.a.data(), s.b.data(), s.c.data(), s.Er.data());
  s.alpha.assign(s.n, 0); s.beta.assign(s.n, 0); s.gamma.assign(s.n, 0); s.phi_o.assign(s.n, 0); s.length.assign(s.n, 0);
  s.a_dna.assign(std::max(s.nc3, 1), 0); s.b_dna = s.a_dna; s.c_dna = s.a_dna;
  s.alpha_p.assign(std::max(s.n_c, 1), 0); s.beta_p = s.alpha_p; s.gamma_p = s.alpha_p;
  update_phi_o(s.n, s.type.data(), s.phi_o.data());
  update_Euler_Angle(s.n_c, s.nc3, s.n, s.n3, s.type.data(), s.r.data(), s.a.data(), s.b.data(), s.c.data(),
      s.alpha.data(), s.beta.data(), s.gamma.data(), s.length.data(), s.a_dna.data(), s.b_dna.data(), s.c_dna.data(),
      s.alpha_p.data(), s.beta_p.data(), s.gamma_p.data());
  Read_core(s.Nq, s.Nq3, s.core_pos, s.core_q, core_file);
  Read_tail(s.n_t, s.tail_pos, s.tail_q, s.tail_grp, s.tail_fix, s.tail_rad, s.tail_bond_c, s.tail_bond_v,
            s.tail_angle_c, s.tail_angle_v, tail_file);
  s.nc_t_flag.assign(s.n_c, 1);
  s.n_tail = s.n_c * s.n_t; s.n_tail3 = s.n_tail * 3;
  int ntp = std::max(s.n_tail, 1);
  s.r_t.assign(3 * ntp, 0); s.beta_t.assign(ntp, 0); s.h_t.assign(ntp, 0); s.g_t.assign(ntp, 0);
  s.lo_t.assign(ntp, 0); s.beta_o_t.assign(ntp, 0); s.t_q.assign(ntp, 0); s.t_rad.assign(ntp, 0);
  s.t_grp.assign(ntp + 2, -1); s.t_fix.assign(ntp + 2, 0);
  build_tail(s.n, s.type.data(), s.n_t, s.tail_pos, s.tail_q, s.tail_grp, s.tail_fix, s.tail_rad, s.tail_bond_c,
      s.tail_bond_v, s.tail_angle_c, s.tail_angle_v, s.r.data(), s.a.data(), s.b.data(), s.c.data(), s.n_tail,
      s.nc_t_flag.data(), s.r_t.data(), s.h_t.data(), s.g_t.data(), s.lo_t.data(), s.beta_o_t.data(), s.t_q.data(),
      s.t_rad.data(), s.t_grp.data(), s.t_fix.data());
  if (restart && s.n_tail3 > 0) Read_restart_tail(s.n_tail3, s.r_t.data());  // main.cpp:218-220
  update_tail_beta(s.n_tail, s.r_t.data(), s.beta_t.data(), s.t_grp.data());
  Read_LH(s.n_lh_g, s.n_lh_n, s.n_lh_c, s.LH_g_pos, s.LH_n_pos, s.LH_c_pos, s.LH_conn, s.LH_q, s.LH_vdw_hh,
      s.LH_vdw_hc, s.LH_vdw_hl, s.LH_vdw_ht, s.LH_kstr, s.LH_kben, s.LH_streq, s.LH_betaeq, s.LH_radius, lh_file);
  s.nc_lh_flag.assign(std::max(s.n_c, 1), 0);
  Read_LH_core(s.n_c, s.nc_lh, s.nc_lh_flag.data());
  int nlh = s.n_lh_n + s.n_lh_c;
  // main.cpp:246 sizes the build buffer for every core, then counts flagged ones
  s.n_LH = 0;
  for (int i = 0; i < s.n_c; i++) if (s.nc_lh_flag[i] == 1) s.n_LH += nlh;
  s.n_LH3 = 3 * s.n_LH;
  std::vector<double> rlh_tmp(3 * std::max(nlh * s.n_c, 1), 0.0), lrad_tmp(std::max(nlh * s.n_c, 1), 0.0);
  build_LH(s.n, s.type.data(), s.n_LH, s.LH_n_pos, s.LH_c_pos, s.LH_radius, s.r.data(), s.a.data(), s.b.data(),
           s.c.data(), s.n_lh_n, s.n_lh_c, s.nc_lh_flag.data(), rlh_tmp.data(), lrad_tmp.data());
  s.r_lh.assign(rlh_tmp.begin(), rlh_tmp.begin() + std::max(s.n_LH3, 3));
  s.lh_rad.assign(lrad_tmp.begin(), lrad_tmp.begin() + std::max(s.n_LH, 1));
  s.beta_lh.assign(std::max(s.n_LH, 1), 0.0);
  if (restart && s.n_LH3 > 0) Read_restart_LH(s.n_LH3, s.r_lh.data());  // main.cpp:279-281
  if (s.n_LH > 0) update_LH_beta(s.n_LH, s.n_lh_c, s.r_lh.data(), s.beta_lh.data());
  s.r_var.assign(s.n3, 0.0);
  for (int i = 0; i < s.n; i++) {
    if (s.type[i] != 0) {
      for (int x = 0; x < 3; x++) s.r_var[i * 3 + x] = 2.0 * s.time_step * s.kbt / (8 * PI * eta * 125.0);
    } else {
      s.r_var[i * 3] = 2.0 * s.time_step * s.kbt / (4 * PI * eta * r_h * r_h * lo);
      s.r_var[i * 3 + 1] = 0.0; s.r_var[i * 3 + 2] = 0.0;
    }
  }
  s.n_D = s.n + s.n_tail + s.n_LH; s.n_D3 = 3 * s.n_D;
  s.rad_all.assign(s.n_D, 0.0);
  for (int i = 0; i < s.n_D; i++) {
    if (i < s.n) s.rad_all[i] = s.rad[i];
    else if (i < s.n + s.n_tail) s.rad_all[i] = s.t_rad[i - s.n];
    else s.rad_all[i] = s.lh_rad[i - s.n - s.n_tail];
  }
  chdir(cwd);
  return 0;
}

// sizes: n n_c n_tail n_LH n_D Nq n_t n_lh_n n_lh_g n_lh_c nsteps freq Mg
void ref_sizes(int* o) {
  RefSys& s = *S;
  int v[13] = {s.n, s.n_c, s.n_tail, s.n_LH, s.n_D, s.Nq, s.n_t, s.n_lh_n, s.n_lh_g, s.n_lh_c, s.nsteps, s.freq, s.Mg};
  memcpy(o, v, sizeof v);
}

// scalars: T Cs q_l debye debyell k_e k_ex k_h1 a1 a2 h g s time_step del s2dt kbt sDD sDC sCC sTT sTL sTC unbind Pbind energy
void ref_scalars(double* o) {
  RefSys& s = *S;
  double v[26] = {s.T, s.Cs, s.q_l, s.debye, s.debyell, s.k_e, s.k_ex, s.k_h1, s.a1, s.a2, s.h, s.g, s.s,
                  s.time_step, s.del, s.s2dt, s.kbt, s.sDD, s.sDC, s.sCC, s.sTT, s.sTL, s.sTC, s.unbind, s.Pbind,
                  s.energy};
  memcpy(o, v, sizeof v);
}

static const void* ref_field(const char* name, int* count, int* is_int) {
  RefSys& s = *S;
  *is_int = 0;
#define F(nm, vec, cnt) if (!strcmp(name, nm)) { *count = (cnt); return (vec).data(); }
#define FI(nm, vec, cnt) if (!strcmp(name, nm)) { *count = (cnt); *is_int = 1; return (vec).data(); }
  F("r", s.r, s.n3) F("a", s.a, s.n3) F("b", s.b, s.n3) F("c", s.c, s.n3) F("rad", s.rad, s.n)
  F("alpha", s.alpha, s.n) F("beta", s.beta, s.n) F("gamma", s.gamma, s.n) F("length", s.length, s.n)
  F("phi_o", s.phi_o, s.n) F("a_dna", s.a_dna, s.nc3) F("b_dna", s.b_dna, s.nc3) F("c_dna", s.c_dna, s.nc3)
  F("alpha_p", s.alpha_p, s.n_c) F("beta_p", s.beta_p, s.n_c) F("gamma_p", s.gamma_p, s.n_c)
  F("r_var", s.r_var, s.n3) F("core_pos", s.core_pos, s.Nq3) F("core_q", s.core_q, s.Nq)
  F("tail_pos", s.tail_pos, 3 * s.n_t) F("r_t", s.r_t, s.n_tail3) F("beta_t", s.beta_t, s.n_tail)
  F("h_t", s.h_t, s.n_tail) F("g_t", s.g_t, s.n_tail) F("lo_t", s.lo_t, s.n_tail) F("beta_o_t", s.beta_o_t, s.n_tail)
  F("t_q", s.t_q, s.n_tail) F("t_rad", s.t_rad, s.n_tail)
  FI("t_grp", s.t_grp, s.n_tail) FI("t_fix", s.t_fix, s.n_tail) FI("tail_fix", s.tail_fix, s.n_t)
  FI("type", s.type, s.n) FI("nc_lh_flag", s.nc_lh_flag, s.n_c) FI("LH_conn", s.LH_conn, (int)s.LH_conn.size())
  F("LH_g_pos", s.LH_g_pos, 3 * s.n_lh_g) F("LH_q", s.LH_q, (int)s.LH_q.size())
  F("LH_vdw_hh", s.LH_vdw_hh, (int)s.LH_q.size()) F("LH_vdw_hc", s.LH_vdw_hc, (int)s.LH_q.size())
  F("LH_vdw_hl", s.LH_vdw_hl, (int)s.LH_q.size()) F("LH_vdw_ht", s.LH_vdw_ht, (int)s.LH_q.size())
  F("LH_kstr", s.LH_kstr, (int)s.LH_q.size()) F("LH_kben", s.LH_kben, (int)s.LH_q.size())
  F("LH_streq", s.LH_streq, (int)s.LH_q.size()) F("LH_betaeq", s.LH_betaeq, (int)s.LH_q.size())
  F("r_lh", s.r_lh, s.n_LH3) F("lh_rad", s.lh_rad, s.n_LH) F("beta_lh", s.beta_lh, s.n_LH)
  F("rad_all", s.rad_all, s.n_D) F("rd", s.rd, (int)s.rd.size()) F("force", s.force, (int)s.force.size())
  F("torque", s.torque, (int)s.torque.size()) F("t_force", s.t_force, s.n_tail3) F("LH_force", s.LH_force, s.n_LH3)
#undef F
#undef FI
  *count = -1;
  return nullptr;
}

// Copies a named array out (ints widened to double); returns its length or -1.
int ref_get(const char* name, double* out) {
  int cnt, isint;
  const void* p = ref_field(name, &cnt, &isint);
  if (!p) return -1;
  if (out) {
    if (isint) for (int i = 0; i < cnt; i++) out[i] = ((const int*)p)[i];
    else memcpy(out, p, sizeof(double) * cnt);
  }
  return cnt;
}

// Overwrites a named double array (used to set frames/positions for force checks).
int ref_set(const char* name, const double* in) {
  int cnt, isint;
  const void* p = ref_field(name, &cnt, &isint);
  if (!p || isint) return -1;
  memcpy((void*)p, in, sizeof(double) * cnt);
  return cnt;
}

// Noise for `step` in the order of main.cpp:386-388 and :479-486.
void ref_draw_noise(int step, double* rr, double* p) {
  RefSys& s = *S;
  if (step % 100 == 0) { (void)genrand_real1(); (void)genrand_real1(); }
  for (int i = 0; i < s.n3; i++) rr[i] = rand_normal(0, s.r_var[i]);
  for (int i = 0; i < s.n_D3; i++) p[i] = rand_normal(0, 1);
}

// Raw uniform stream of the reference MT19937 (genrand_int32) for bitwise checks.
void ref_mt_raw(unsigned long seed, int count, unsigned int* out) {
  init_genrand(seed);
  for (int i = 0; i < count; i++) out[i] = (unsigned int)genrand_int32();
}

// Forces/torques at the current state (no state change); energy returned.
double ref_forces(double* F, double* Tq, double* tF, double* lF) {
  RefSys& s = *S;
  std::vector<double> f, t, tf, lf; double E;
  forces(s, s.r, s.a, s.b, s.c, s.alpha, s.beta, s.gamma, s.length, s.a_dna, s.b_dna, s.c_dna, s.alpha_p,
         s.beta_p, s.gamma_p, s.r_t, s.beta_t, s.r_lh, s.beta_lh, f, t, tf, lf, E);
  memcpy(F, f.data(), sizeof(double) * s.n3); memcpy(Tq, t.data(), sizeof(double) * s.n3);
  if (s.n_tail3) memcpy(tF, tf.data(), sizeof(double) * s.n_tail3);
  if (s.n_LH3) memcpy(lF, lf.data(), sizeof(double) * s.n_LH3);
  return E;
}

// Diffusion tensor and its Cholesky factor (both row-major n_D3 x n_D3).
void ref_tensor(double* Dout, double* Lout) {
  RefSys& s = *S;
  build_tensor(s);
  for (int i = 0; i < s.n_D3; i++) {
    if (Dout) memcpy(Dout + (size_t)i * s.n_D3, s.D[i].data(), sizeof(double) * s.n_D3);
    if (Lout) memcpy(Lout + (size_t)i * s.n_D3, s.Chol[i].data(), sizeof(double) * s.n_D3);
  }
}

// Recomputes the internal coordinates (update_Euler_Angle + betas) at the
// current state, as done after a step (func_cuda.cu:3656-3660).
void ref_refresh_angles() {
  RefSys& s = *S;
  update_Euler_Angle(s.n_c, s.nc3, s.n, s.n3, s.type.data(), s.r.data(), s.a.data(), s.b.data(), s.c.data(),
      s.alpha.data(), s.beta.data(), s.gamma.data(), s.length.data(), s.a_dna.data(), s.b_dna.data(),
      s.c_dna.data(), s.alpha_p.data(), s.beta_p.data(), s.gamma_p.data());
  if (s.n_tail) update_tail_beta(s.n_tail, s.r_t.data(), s.beta_t.data(), s.t_grp.data());
  if (s.n_LH) update_LH_beta(s.n_LH, s.n_lh_c, s.r_lh.data(), s.beta_lh.data());
}

// One BD step in the order of main_cuda (func_cuda.cu:3434-3680); returns
// the pass-1 energy (the value main.cpp writes to Energy.txt).
double ref_step(const double* rr, const double* p) {
  RefSys& s = *S;
  if (s.n_LH) update_LH_beta(s.n_LH, s.n_lh_c, s.r_lh.data(), s.beta_lh.data());
  build_tensor(s);
  s.rd.assign(s.n_D3, 0.0);
  for (int col = 0; col < s.n_D3; col++) {           // rd_cal
    double v = 0.0;
    for (int k = 0; k <= col; k++) v += s.s2dt * s.Chol[col][k] * p[k];
    s.rd[col] = v;
  }
  std::vector<double> F, Tq, tF, lF; double E;
  forces(s, s.r, s.a, s.b, s.c, s.alpha, s.beta, s.gamma, s.length, s.a_dna, s.b_dna, s.c_dna, s.alpha_p,
         s.beta_p, s.gamma_p, s.r_t, s.beta_t, s.r_lh, s.beta_lh, F, Tq, tF, lF, E);
  s.force = F; s.torque = Tq; s.t_force = tF; s.LH_force = lF; s.energy = E;
  std::vector<double> a_n(s.n3), b_n(s.n3), c_n(s.n3), r_n(s.n3), r_t_n(std::max(s.n_tail3, 3)),
      r_lh_n(std::max(s.n_LH3, 3));
  rotation(s, Tq, rr, s.a, s.b, s.c, a_n, b_n, c_n);
  translation(s, F, tF, lF, r_n, r_t_n, r_lh_n);
  std::vector<double> beta_t_n(std::max(s.n_tail, 1)), beta_lh_n(std::max(s.n_LH, 1));
  std::vector<double> al(s.n), be(s.n), ga(s.n), le(s.n), ad(s.a_dna.size()), bd(s.a_dna.size()),
      cd(s.a_dna.size()), ap(s.alpha_p.size()), bp(s.alpha_p.size()), gp(s.alpha_p.size());
  if (s.n_tail) update_tail_beta(s.n_tail, r_t_n.data(), beta_t_n.data(), s.t_grp.data());
  if (s.n_LH) update_LH_beta(s.n_LH, s.n_lh_c, r_lh_n.data(), beta_lh_n.data());
  update_Euler_Angle(s.n_c, s.nc3, s.n, s.n3, s.type.data(), r_n.data(), a_n.data(), b_n.data(), c_n.data(),
      al.data(), be.data(), ga.data(), le.data(), ad.data(), bd.data(), cd.data(), ap.data(), bp.data(), gp.data());
  std::vector<double> Fn, Tn, tFn, lFn; double En;
  forces(s, r_n, a_n, b_n, c_n, al, be, ga, le, ad, bd, cd, ap, bp, gp, r_t_n, beta_t_n, r_lh_n, beta_lh_n,
         Fn, Tn, tFn, lFn, En);
  for (int i = 0; i < s.n3; i++) { F[i] = 0.5 * (F[i] + Fn[i]); Tq[i] = 0.5 * (Tq[i] + Tn[i]); }
  for (int i = 0; i < s.n_tail3; i++) tF[i] = 0.5 * (tF[i] + tFn[i]);
  for (int i = 0; i < s.n_LH3; i++) lF[i] = 0.5 * (lF[i] + lFn[i]);
  rotation(s, Tq, rr, s.a, s.b, s.c, a_n, b_n, c_n);
  translation(s, F, tF, lF, r_n, r_t_n, r_lh_n);
  for (int i = 0; i < s.n3; i++) { s.r[i] = r_n[i]; s.a[i] = a_n[i]; s.b[i] = b_n[i]; s.c[i] = c_n[i]; }
  for (int i = 0; i < s.n_tail3; i++) s.r_t[i] = r_t_n[i];
  for (int i = 0; i < s.n_LH3; i++) s.r_lh[i] = r_lh_n[i];
  ref_refresh_angles();
  return E;
}

void ref_free() { delete S; S = nullptr; }

}  // extern "C"
