// Drop-in shim: the four C++ entry points of the reference's GPU step
// (BD_cuda/func_cuda.h:37-52), implemented on top of the C ABI so that the
// reference's main.cpp links against libbdgb300.so unchanged.
//
//   cuda_application_init_D_Chol  func_cuda.cu:2665  (no-op: bd_create sizes D)
//   cuda_application_init_data    func_cuda.cu:2676  (copies the host arrays)
//   main_cuda                     func_cuda.cu:3434  (creates the context on
//                                  its first call - it carries a1, a2, dt,
//                                  del and s2dt - then runs one step)
//   free_all                      func_cuda.cu:3682
//
// Like the reference, the shim keeps one simulation per process.  The LH
// binding Monte Carlo of main.cpp:386-465 may change n_LH; the shim then
// resizes the context (bd_set_lh_flags) from its current device state and
// the host's new LH beads.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "bd_internal.h"

namespace {

struct Saved {
  bool have = false;
  int n_c, n, Nq, n_t, n_tail, n_lh_n, n_lh_g, n_lh_c, n_LH;
  double h, g, s, debyell, debye, q_l, k_e, k_ex, k_h1, sDD, sDC, sCC, sTT, sTL, sTC;
  std::vector<int> type, tail_fix, nc_t_flag, t_grp, t_fix, LH_conn, nc_lh_flag;
  std::vector<double> r, a, b, c, alpha, beta, gamma, length, a_dna, b_dna, c_dna, alpha_p, beta_p, gamma_p, phi_o,
      core_pos, core_q, tail_pos, r_t, h_t, g_t, lo_t, beta_o_t, t_q, t_rad, LH_g_pos, r_lh, LH_q, LH_vdw_hh, LH_vdw_hc,
      LH_vdw_hl, LH_vdw_ht, LH_kstr, LH_kben, LH_streq, LH_betaeq, rad_all, rad, lh_rad;
};

Saved g_sv;
bd_ctx* g_ctx = nullptr;

template <class T>
std::vector<T> cp(const T* p, int n) {
  return (p && n > 0) ? std::vector<T>(p, p + n) : std::vector<T>();
}

void die(const char* where, int rc) {
  fprintf(stderr, "%s: %s (status %d)\n", where, bd_last_error(), rc);
  exit(1);
}

}  // namespace

extern "C++" void cuda_application_init_D_Chol(int n3) { (void)n3; }

extern "C++" void cuda_application_init_data(
    int n_c, int nc3, int n, int n3, int* type, double* r, double* a, double* b, double* c, double* alpha,
    double* beta, double* gamma, double* length, double* a_dna, double* b_dna, double* c_dna, double* alpha_p,
    double* beta_p, double* gamma_p, double h, double g, double s, double* phi_o, double debyell, double debye,
    double q_l, double k_e, double k_ex, double k_h1, double sigma_DNA_DNA, double sigma_DNA_Core,
    double sigma_Core_Core, double sigma_Tail_Tail, double sigma_Tail_Linker, double sigma_Tail_Core, int Nq, int Nq3,
    double* core_pos, double* core_q, int n_t, int n_tail, int n_tail3, double* tail_pos, int* tail_fix,
    int* nc_t_flag, double* r_t, double* beta_t, double* h_t, double* g_t, double* lo_t, double* beta_o_t,
    double* t_q, double* t_rad, int* t_grp, int* t_fix, int n_lh_n, int n_lh_g, int n_lh_c, int n_LH, int n_LH3,
    double* LH_g_pos, int* LH_conn, int* nc_lh_flag, double* beta_lh, double* r_lh, double* LH_q, double* LH_vdw_hh,
    double* LH_vdw_hc, double* LH_vdw_hl, double* LH_vdw_ht, double* LH_kstr, double* LH_kben, double* LH_streq,
    double* LH_betaeq, double* LH_force, double* t_force, double* force, double* torque, double* Energy,
    double* r_all, double* rad_all) {
  (void)nc3; (void)n3; (void)Nq3; (void)n_tail3; (void)n_LH3; (void)beta_t; (void)beta_lh; (void)LH_force;
  (void)t_force; (void)force; (void)torque; (void)Energy; (void)r_all;
  Saved& S = g_sv;
  int np = n_lh_n + n_lh_g + n_lh_c;
  S.n_c = n_c; S.n = n; S.Nq = Nq; S.n_t = n_t; S.n_tail = n_tail;
  S.n_lh_n = n_lh_n; S.n_lh_g = n_lh_g; S.n_lh_c = n_lh_c; S.n_LH = n_LH;
  S.h = h; S.g = g; S.s = s; S.debyell = debyell; S.debye = debye; S.q_l = q_l; S.k_e = k_e; S.k_ex = k_ex; S.k_h1 = k_h1;
  S.sDD = sigma_DNA_DNA; S.sDC = sigma_DNA_Core; S.sCC = sigma_Core_Core;
  S.sTT = sigma_Tail_Tail; S.sTL = sigma_Tail_Linker; S.sTC = sigma_Tail_Core;
  S.type = cp(type, n); S.r = cp(r, 3 * n); S.a = cp(a, 3 * n); S.b = cp(b, 3 * n); S.c = cp(c, 3 * n);
  S.alpha = cp(alpha, n); S.beta = cp(beta, n); S.gamma = cp(gamma, n); S.length = cp(length, n);
  S.a_dna = cp(a_dna, 3 * n_c); S.b_dna = cp(b_dna, 3 * n_c); S.c_dna = cp(c_dna, 3 * n_c);
  S.alpha_p = cp(alpha_p, n_c); S.beta_p = cp(beta_p, n_c); S.gamma_p = cp(gamma_p, n_c); S.phi_o = cp(phi_o, n);
  S.core_pos = cp(core_pos, 3 * Nq); S.core_q = cp(core_q, Nq); S.tail_pos = cp(tail_pos, 3 * n_t);
  S.tail_fix = cp(tail_fix, n_t); S.nc_t_flag = cp(nc_t_flag, n_c); S.r_t = cp(r_t, 3 * n_tail);
  S.h_t = cp(h_t, n_tail); S.g_t = cp(g_t, n_tail); S.lo_t = cp(lo_t, n_tail); S.beta_o_t = cp(beta_o_t, n_tail);
  S.t_q = cp(t_q, n_tail); S.t_rad = cp(t_rad, n_tail); S.t_grp = cp(t_grp, n_tail); S.t_fix = cp(t_fix, n_tail);
  S.LH_g_pos = cp(LH_g_pos, 3 * n_lh_g); S.LH_conn = cp(LH_conn, np); S.nc_lh_flag = cp(nc_lh_flag, n_c);
  S.r_lh = cp(r_lh, 3 * n_LH); S.LH_q = cp(LH_q, np); S.LH_vdw_hh = cp(LH_vdw_hh, np); S.LH_vdw_hc = cp(LH_vdw_hc, np);
  S.LH_vdw_hl = cp(LH_vdw_hl, np); S.LH_vdw_ht = cp(LH_vdw_ht, np); S.LH_kstr = cp(LH_kstr, np);
  S.LH_kben = cp(LH_kben, np); S.LH_streq = cp(LH_streq, np); S.LH_betaeq = cp(LH_betaeq, np);
  int nD = n + n_tail + n_LH;
  S.rad_all = cp(rad_all, nD);
  S.rad.assign(S.rad_all.begin(), S.rad_all.begin() + n);
  S.lh_rad.assign(S.rad_all.begin() + n + n_tail, S.rad_all.end());
  S.have = true;
}

extern "C++" void main_cuda(int n_c, int nc3, int step, int number_of_steps, double time_step, double del,
                            int frequency_RP, int frequency_of_sampling, double h, double g, double s, double debyell,
                            double debye, double q_l, double k_e, double k_ex, double k_h1, double sigma_DNA_DNA,
                            double sigma_DNA_Core, double sigma_Core_Core, double sigma_Tail_Tail,
                            double sigma_Tail_Linker, double sigma_Tail_Core, int Nq, int Nq3, int n_t, int n_lh_n,
                            int n_lh_g, int n_lh_c, int n, int n3, int n_tail, int n_tail3, int n_LH, int n_LH3,
                            double a1, double a2, double s2dt, double* rr, double* p, double* Energy, double* h_r,
                            double* h_a, double* h_b, double* h_c, double* h_r_t, double* h_r_lh, double* h_rad_all,
                            int* nc_lh_flag) {
  (void)nc3; (void)frequency_RP; (void)h; (void)g; (void)s; (void)debyell; (void)debye; (void)q_l; (void)k_e;
  (void)k_ex; (void)k_h1; (void)sigma_DNA_DNA; (void)sigma_DNA_Core; (void)sigma_Core_Core; (void)sigma_Tail_Tail;
  (void)sigma_Tail_Linker; (void)sigma_Tail_Core; (void)Nq; (void)Nq3; (void)n_t; (void)n_lh_n; (void)n_lh_g;
  (void)n_lh_c; (void)n; (void)n3; (void)n_tail; (void)n_tail3; (void)n_LH3;
  Saved& S = g_sv;
  if (!S.have) {
    fprintf(stderr, "main_cuda: cuda_application_init_data was not called\n");
    exit(1);
  }
  bool flags_changed = false;
  for (int i = 0; i < n_c; i++) flags_changed |= (S.nc_lh_flag[i] != nc_lh_flag[i]);
  if (g_ctx && (flags_changed || n_LH != S.n_LH)) {
    // LH binding changed: the chain, tails and frames stay as the device has
    // them (the reference keeps them on the device); the LH beads and their
    // radii come from the host, which main.cpp rebuilt (main.cpp:418-465)
    for (int i = 0; i < n_c; i++) S.nc_lh_flag[i] = nc_lh_flag[i];
    S.n_LH = n_LH;
    int rc = bd_set_lh_flags(g_ctx, nc_lh_flag, h_r_lh, h_rad_all ? h_rad_all + S.n + S.n_tail : nullptr);
    if (rc) die("main_cuda/bd_set_lh_flags", rc);
  }
  if (!g_ctx) {
    bd_model m{};
    m.n = S.n; m.n_c = S.n_c; m.Nq = S.Nq; m.n_t = S.n_t; m.n_tail = S.n_tail;
    m.n_lh_n = S.n_lh_n; m.n_lh_g = S.n_lh_g; m.n_lh_c = S.n_lh_c; m.n_LH = S.n_LH;
    m.h = S.h; m.g = S.g; m.s = S.s; m.debyell = S.debyell; m.debye = S.debye; m.q_l = S.q_l; m.k_e = S.k_e;
    m.k_ex = S.k_ex; m.k_h1 = S.k_h1;
    m.sigma_DNA_DNA = S.sDD; m.sigma_DNA_Core = S.sDC; m.sigma_Core_Core = S.sCC;
    m.sigma_Tail_Tail = S.sTT; m.sigma_Tail_Linker = S.sTL; m.sigma_Tail_Core = S.sTC;
    m.a1 = a1; m.a2 = a2; m.time_step = time_step; m.del = del; m.s2dt = s2dt;
    m.type = S.type.data(); m.rad = S.rad.data(); m.phi_o = S.phi_o.data(); m.r_var = nullptr;
    m.core_pos = S.core_pos.data(); m.core_q = S.core_q.data(); m.tail_pos = S.tail_pos.data();
    m.tail_fix = S.tail_fix.data(); m.nc_t_flag = S.nc_t_flag.data(); m.h_t = S.h_t.data(); m.g_t = S.g_t.data();
    m.lo_t = S.lo_t.data(); m.beta_o_t = S.beta_o_t.data(); m.t_q = S.t_q.data(); m.t_rad = S.t_rad.data();
    m.t_grp = S.t_grp.data(); m.t_fix = S.t_fix.data(); m.LH_g_pos = S.LH_g_pos.data(); m.LH_conn = S.LH_conn.data();
    m.nc_lh_flag = S.nc_lh_flag.data(); m.LH_q = S.LH_q.data(); m.LH_vdw_hh = S.LH_vdw_hh.data();
    m.LH_vdw_hc = S.LH_vdw_hc.data(); m.LH_vdw_hl = S.LH_vdw_hl.data(); m.LH_vdw_ht = S.LH_vdw_ht.data();
    m.LH_kstr = S.LH_kstr.data(); m.LH_kben = S.LH_kben.data(); m.LH_streq = S.LH_streq.data();
    m.LH_betaeq = S.LH_betaeq.data(); m.lh_rad = S.lh_rad.data();
    bd_state st{};
    st.r = S.r.data(); st.a = S.a.data(); st.b = S.b.data(); st.c = S.c.data(); st.r_t = S.r_t.data();
    st.r_lh = S.r_lh.data();
    st.refresh_frames = 0;
    st.alpha = S.alpha.data(); st.beta = S.beta.data(); st.gamma = S.gamma.data(); st.length = S.length.data();
    st.a_dna = S.a_dna.data(); st.b_dna = S.b_dna.data(); st.c_dna = S.c_dna.data();
    st.alpha_p = S.alpha_p.data(); st.beta_p = S.beta_p.data(); st.gamma_p = S.gamma_p.data();
    if (g_ctx == nullptr && step > 0) st.refresh_frames = 1;  // rebuilt mid-run: angles follow the state
    bd_options o{};
    o.precision = BD_PREC_FP64;
    o.frequency_RP = 1;
    o.use_graph = 1;
    const char* pe = getenv("BD_PRECISION");
    if (pe && pe[0] == 'm') o.precision = BD_PREC_MIXED;
    int rc = bd_create(&m, &st, &o, &g_ctx);
    if (rc) die("main_cuda/bd_create", rc);
  }
  int rc = bd_step_reference(g_ctx, step, number_of_steps, frequency_of_sampling, rr, p, Energy, h_r, h_a, h_b, h_c,
                             h_r_t, h_r_lh);
  if (rc) die("main_cuda/bd_step", rc);
}

extern "C++" void free_all() {
  bd_destroy(g_ctx);
  g_ctx = nullptr;
}
