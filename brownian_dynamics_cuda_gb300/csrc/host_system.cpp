// Host side of the drop-in boundary: the reference's input readers and
// start-up model construction, the MT19937 noise stream and the out.xyz
// writer.  Pure C++ (no CUDA); compiled into libbdgb300.so.
//
//   readers          readfile.cpp:14-337, :563-584
//   constants        main.cpp:68-99
//   phi_o            func.cpp:13-99 (twist_angle_phi), :412-431
//   tails, LH        func.cpp:1672-1713 (build_tail), :2029-2059 (build_LH)
//   r_var            main.cpp:292-303
//   out.xyz          readfile.cpp:346-405
//   noise            mt.cpp (MT19937), utilities.cpp:304-336, main.cpp:386-388,479-486
#include "cr_log.cuh"
#include "bd_internal.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace bdh {

namespace {

constexpr double kPi = 3.141592653589790;
constexpr double kLo = 3.0;
constexpr double kEta = 1.137076e-12;
constexpr double kRh = 1.2;

std::vector<std::string> tokens(const std::string& line) {
  std::istringstream is(line);
  std::vector<std::string> t;
  std::string w;
  while (is >> w) t.push_back(w);
  return t;
}

double num(const std::string& s) {
  std::istringstream is(s);
  double v = 0;
  is >> v;
  return v;
}

int inum(const std::string& s) {
  std::istringstream is(s);
  int v = 0;
  is >> v;
  return v;
}

std::string join(const std::string& dir, const std::string& f) {
  if (f.empty() || f[0] == '/') return f;
  return dir + "/" + f;
}

// Read_restart_ini / _tail / _LH (readfile.cpp:443-630): the first value of
// each line, `count` of them
int read_restart_column(const std::string& dir, const char* name, size_t count, std::vector<double>& out,
                        std::string& err) {
  std::ifstream in(join(dir, name));
  if (!in) { err = std::string("restart = 1 in setup.txt but ") + name + " cannot be opened"; return BD_ERR_IO; }
  out.resize(count);
  size_t i = 0;
  std::string line;
  while (i < count && std::getline(in, line)) {
    auto t = tokens(line);
    if (t.empty()) continue;
    out[i++] = num(t[0]);
  }
  if (i < count) { err = std::string(name) + ": fewer values than the system has"; return BD_ERR_IO; }
  return BD_OK;
}

// func.cpp:13-99: intrinsic twist per linker segment for w linker beads
double twist_angle(int w, bool* ok) {
  static const double table[12] = {0, 0, 0.9007, -0.6754, -0.3519, -0.1463, 0.0215, 0.1178, 0.2025, 0.2726, -0.2415, -0.15};
  *ok = true;
  if (w <= 11) {
    if (w < 2) { *ok = false; return 0.0; }
    return table[w];
  }
  double nbp = (w + 1) * 3 / 0.34;
  double turns = nbp / 10.3;
  double rot = std::round(turns);
  double per_bp = rot * 360 / nbp;
  double dtw = per_bp - 34.95;
  double whole = nbp * dtw;
  double seg = whole / (w + 1);
  return kPi * seg / 180.00;
}

}  // namespace

int load_system(const char* dir_c, const char* data_f, const char* core_f, const char* tail_f, const char* lh_f,
                const char* lhflag_f, HostSystem& S, std::string& err) {
  std::string dir = dir_c ? dir_c : ".";
  // setup.txt: second token of every line after the first (readfile.cpp:14-38)
  {
    std::ifstream in(join(dir, "setup.txt"));
    if (!in) { err = "cannot open setup.txt"; return BD_ERR_IO; }
    std::string line;
    int i = 0;
    S.setup.clear();
    while (std::getline(in, line)) {
      if (i++ == 0) continue;
      auto t = tokens(line);
      if (t.size() < 2) { err = "setup.txt: short line"; return BD_ERR_IO; }
      S.setup.push_back(num(t[1]));
    }
    if (S.setup.size() < 15) { err = "setup.txt: expected 15 values"; return BD_ERR_IO; }
  }
  const double T = S.setup[0], Cs = S.setup[11];
  const int Mg = (int)S.setup[10];
  // main.cpp:68-99
  const double kb = 1.380649e-5, kbt = kb * 300.0;
  bd_model& m = S.m;
  memset(&m, 0, sizeof m);
  m.q_l = kLo * (-5.8824) *
          (1.901912136835033e-8 * pow((Cs * 1000), 3.0) + -8.211102025728157e-6 * pow((Cs * 1000), 2.0) +
           7.554037628581672e-3 * (Cs * 1000) + 3.524292543853884e-1);
  m.debye = 0.736 * sqrt((Cs / 0.05) * (298 / T));
  double per;
  if (Mg == 0) { per = 50; m.debyell = m.debye; } else { per = 30; m.debyell = 2.5; }
  m.k_e = 0.4151 * kb * 300;
  m.k_ex = 0.001 * kbt;
  m.k_h1 = 10.0 * kbt;
  m.a1 = kbt / (6 * kPi * kEta);
  m.a2 = kbt / (8 * kPi * kEta);
  m.h = 100 * kbt / (kLo * kLo);
  m.g = per * kbt / kLo;
  m.s = 72.429 * kbt / kLo;
  m.time_step = 1e-12;
  m.del = m.time_step / kbt;
  m.s2dt = sqrt(2 * m.time_step);
  m.sigma_DNA_DNA = S.setup[4]; m.sigma_DNA_Core = S.setup[5]; m.sigma_Core_Core = S.setup[6];
  m.sigma_Tail_Tail = S.setup[7]; m.sigma_Tail_Linker = S.setup[8]; m.sigma_Tail_Core = S.setup[9];

  // data_mod: 4 lines per bead (readfile.cpp:40-142)
  {
    std::ifstream in(join(dir, data_f ? data_f : "data_mod"));
    if (!in) { err = "cannot open data file"; return BD_ERR_IO; }
    std::string line;
    int i = 0;
    S.type.clear(); S.r.clear(); S.a.clear(); S.b.clear(); S.c.clear(); S.rad.clear();
    while (std::getline(in, line)) {
      auto t = tokens(line);
      int k = i % 4;
      if (t.size() < (k == 0 ? 4u : 3u)) { err = "data file: short line"; return BD_ERR_IO; }
      std::vector<double>* dst = k == 0 ? &S.r : k == 1 ? &S.a : k == 2 ? &S.b : &S.c;
      for (int x = 0; x < 3; x++) dst->push_back(num(t[x]));
      if (k == 0) {
        int ty = inum(t[3]);
        S.type.push_back(ty);
        S.rad.push_back(ty == 1 ? 5.0 : 1.5);
      }
      i++;
    }
    if (i % 4 != 0 || S.type.empty()) { err = "data file: incomplete bead record"; return BD_ERR_IO; }
  }
  const int n = (int)S.type.size();
  int n_c = 0;
  for (int t : S.type) n_c += (t == 1);
  // restart = 1 in setup.txt: positions and frames from the text restart
  // files, before the tails and linker histones are built on them
  // (main.cpp:143-153)
  const bool restart = S.setup.size() > 12 && (int)S.setup[12] == 1;
  if (restart) {
    int rc = 0;
    if ((rc = read_restart_column(dir, "restart_r.txt", 3 * (size_t)n, S.r, err)) ||
        (rc = read_restart_column(dir, "restart_a.txt", 3 * (size_t)n, S.a, err)) ||
        (rc = read_restart_column(dir, "restart_b.txt", 3 * (size_t)n, S.b, err)) ||
        (rc = read_restart_column(dir, "restart_c.txt", 3 * (size_t)n, S.c, err)))
      return rc;
  }
  m.n = n; m.n_c = n_c;
  if (S.type[0] != 1 || S.type[n - 1] != 0) {
    err = "chain must start with a core and end with linker DNA (func.cpp:1062,1283)";
    return BD_ERR_IO;
  }
  // update_phi_o (func.cpp:412-431)
  S.phi_o.assign(n, 0.0);
  for (int i = 0; i < n; i++) {
    if (S.type[i] != 1) continue;
    int k = 1;
    while (i + k < n && S.type[i + k] == 0) k++;
    bool ok;
    double tw = twist_angle(k - 1, &ok);
    if (!ok) { err = "linker with fewer than 2 DNA beads (twist_angle_phi)"; return BD_ERR_IO; }
    for (int l = 0; l < k; l++) S.phi_o[i + l] = tw;
  }
  // r_var (main.cpp:292-303)
  S.r_var.assign(3 * n, 0.0);
  for (int i = 0; i < n; i++) {
    if (S.type[i] != 0) {
      for (int x = 0; x < 3; x++) S.r_var[3 * i + x] = 2.0 * m.time_step * kbt / (8 * kPi * kEta * 125.0);
    } else {
      S.r_var[3 * i] = 2.0 * m.time_step * kbt / (4 * kPi * kEta * kRh * kRh * kLo);
    }
  }
  // core charges: 3-token lines are positions in Angstrom, others charges
  {
    std::ifstream in(join(dir, core_f));
    if (!in) { err = "cannot open core charge file"; return BD_ERR_IO; }
    std::string line;
    S.core_pos.clear(); S.core_q.clear();
    while (std::getline(in, line)) {
      auto t = tokens(line);
      if (t.empty()) continue;
      if (t.size() == 3) {
        for (int x = 0; x < 3; x++) S.core_pos.push_back(num(t[x]) / 10);
      } else {
        S.core_q.push_back(num(t[0]));
      }
    }
    if (S.core_q.size() * 3 != S.core_pos.size()) { err = "core file: positions/charges mismatch"; return BD_ERR_IO; }
    m.Nq = (int)S.core_q.size();
  }
  // tail table (readfile.cpp:183-250)
  {
    std::ifstream in(join(dir, tail_f));
    if (!in) { err = "cannot open tail file"; return BD_ERR_IO; }
    std::string line;
    S.tail_pos.clear(); S.tail_fix.clear();
    std::vector<double> tq, trad, bc, bv, ac, av;
    std::vector<int> tg;
    while (std::getline(in, line)) {
      auto t = tokens(line);
      if (t.empty()) continue;
      if (t.size() < 13) { err = "tail file: expected 13 columns"; return BD_ERR_IO; }
      tg.push_back(inum(t[1]));
      S.tail_fix.push_back(inum(t[2]));
      tq.push_back(num(t[3]) * 1.12);
      trad.push_back(num(t[4]) / 10);
      for (int x = 0; x < 3; x++) S.tail_pos.push_back(num(t[6 + x]) / 10);
      bv.push_back(num(t[9]) / 10);
      bc.push_back(num(t[10]) * 100 * 4.142e-3 / 0.5962);
      av.push_back(num(t[11]) * kPi / 180);
      ac.push_back(num(t[12]) * 4.142e-3 / 0.5962);
    }
    const int n_t = (int)tg.size();
    m.n_t = n_t;
    int n_grp = n_t > 0 ? 1 : 0;
    for (int i = 1; i < n_t; i++) if (tg[i] != tg[i - 1]) n_grp++;
    S.nc_t_flag.assign(n_c, 1);
    // build_tail (func.cpp:1672-1713) with every core carrying tails
    const int n_tail = n_c * n_t;
    m.n_tail = n_tail;
    S.r_t.assign(3 * n_tail, 0.0);
    S.h_t.assign(n_tail, 0); S.g_t.assign(n_tail, 0); S.lo_t.assign(n_tail, 0); S.beta_o_t.assign(n_tail, 0);
    S.t_q.assign(n_tail, 0); S.t_rad.assign(n_tail, 0); S.t_grp.assign(n_tail, 0); S.t_fix.assign(n_tail, 0);
    int k = 0;
    for (int i = 0; i < n; i++) {
      if (S.type[i] != 1) continue;
      for (int j = 0; j < n_t; j++) {
        int tb = k * n_t + j;
        for (int x = 0; x < 3; x++)
          S.r_t[3 * tb + x] = S.r[3 * i + x] + S.a[3 * i + x] * S.tail_pos[3 * j] + S.b[3 * i + x] * S.tail_pos[3 * j + 1] +
                              S.c[3 * i + x] * S.tail_pos[3 * j + 2];
        S.t_q[tb] = tq[j]; S.t_rad[tb] = trad[j]; S.t_fix[tb] = S.tail_fix[j]; S.t_grp[tb] = tg[j] + k * n_grp;
        S.h_t[tb] = bc[j]; S.lo_t[tb] = bv[j]; S.g_t[tb] = ac[j]; S.beta_o_t[tb] = av[j];
      }
      k++;
    }
    if (n_t > 0 && n_grp != 10) {
      err = "tail template must have 10 groups (the core lookup (t_grp-1)/10 of func.cpp:2368 assumes it)";
      return BD_ERR_IO;
    }
    if (restart && n_tail > 0) {  // main.cpp:218-220
      int rc = read_restart_column(dir, "restart_tail.txt", 3 * (size_t)n_tail, S.r_t, err);
      if (rc) return rc;
    }
  }
  // LH table (readfile.cpp:252-337)
  {
    std::ifstream in(join(dir, lh_f));
    if (!in) { err = "cannot open LH file"; return BD_ERR_IO; }
    std::string line, kind;
    std::vector<double> npos, cpos;
    S.LH_g_pos.clear(); S.LH_conn.clear(); S.LH_q.clear(); S.LH_vdw_hh.clear(); S.LH_vdw_hc.clear();
    S.LH_vdw_hl.clear(); S.LH_vdw_ht.clear(); S.LH_kstr.clear(); S.LH_kben.clear(); S.LH_streq.clear();
    S.LH_betaeq.clear();
    std::vector<double> radius;
    int nn = 0, ng = 0, nc = 0;
    while (std::getline(in, line)) {
      auto t = tokens(line);
      if (t.empty()) continue;
      if (t.size() >= 2 && t[1] == "N-term") { kind = "N"; continue; }
      if (t.size() >= 2 && t[1] == "G-head") { kind = "G"; continue; }
      if (t.size() >= 2 && t[1] == "C-term") { kind = "C"; continue; }
      if (t[0] == "#") continue;
      if (t.size() < 15) { err = "LH file: expected 15 columns"; return BD_ERR_IO; }
      double x = num(t[0]), y = num(t[1]), z = num(t[2]);
      if (kind == "N") { nn++; npos.insert(npos.end(), {x, y, z}); }
      else if (kind == "G") { ng++; S.LH_g_pos.insert(S.LH_g_pos.end(), {x, y, z}); }
      else if (kind == "C") { nc++; cpos.insert(cpos.end(), {x, y, z}); }
      S.LH_q.push_back(num(t[3]) * 0.66);
      S.LH_vdw_hh.push_back(num(t[4])); S.LH_vdw_hc.push_back(num(t[5]));
      S.LH_vdw_hl.push_back(num(t[6])); S.LH_vdw_ht.push_back(num(t[7]));
      S.LH_kstr.push_back(num(t[8]) * 4.142e-3 / 0.5962);
      S.LH_kben.push_back(num(t[9]) * 4.142e-3 / 0.5962);
      S.LH_streq.push_back(num(t[13]));
      S.LH_betaeq.push_back(num(t[14]) * kPi / 180);
      S.LH_conn.push_back(inum(t[12]));
      radius.push_back(0.5);
    }
    m.n_lh_n = nn; m.n_lh_g = ng; m.n_lh_c = nc;
    if (nn != 0) {
      err = "LH models with N-terminal beads are not supported (G-head parameters are indexed from 0, func.cpp:2422)";
      return BD_ERR_IO;
    }
    // LH.in flags (readfile.cpp:563-584): one int per line, first n_c lines
    S.nc_lh_flag.assign(n_c, 0);
    {
      std::ifstream fin(join(dir, lhflag_f ? lhflag_f : "LH.in"));
      if (!fin) { err = "cannot open LH flag file"; return BD_ERR_IO; }
      int i = 0;
      while (std::getline(fin, line) && i < n_c) {
        auto t = tokens(line);
        if (t.empty()) continue;
        S.nc_lh_flag[i++] = inum(t[0]);
      }
    }
    // build_LH (func.cpp:2029-2059)
    const int nlh = nn + nc;
    S.lh_tpos.clear();
    S.lh_trad.clear();
    for (int j = 0; j < nlh; j++) {
      const double* p = j < nn ? &npos[3 * j] : &cpos[3 * j];
      S.lh_tpos.insert(S.lh_tpos.end(), {p[0], p[1], p[2]});
      S.lh_trad.push_back(radius[j]);
    }
    int nLH = 0;
    for (int f : S.nc_lh_flag) if (f == 1) nLH += nlh;
    m.n_LH = nLH;
    S.r_lh.assign(3 * nLH, 0.0);
    S.lh_rad.assign(nLH, 0.0);
    int k = 0, k1 = 0;
    for (int i = 0; i < n; i++) {
      if (S.type[i] != 1) continue;
      if (S.nc_lh_flag[k1] == 1) {
        for (int j = 0; j < nlh; j++) {
          const double* p = j < nn ? &npos[3 * j] : &cpos[3 * j];
          int lb = k * nlh + j;
          for (int x = 0; x < 3; x++)
            S.r_lh[3 * lb + x] = S.r[3 * i + x] + S.a[3 * i + x] * p[0] + S.b[3 * i + x] * p[1] + S.c[3 * i + x] * p[2];
          S.lh_rad[lb] = radius[j];
        }
        k++;
      }
      k1++;
    }
    if (restart && nLH > 0) {  // main.cpp:279-281
      int rc = read_restart_column(dir, "restart_lh.txt", 3 * (size_t)nLH, S.r_lh, err);
      if (rc) return rc;
    }
  }
  refresh_model_pointers(S);
  return BD_OK;
}

void refresh_model_pointers(HostSystem& S) {
  bd_model& m = S.m;
  m.type = S.type.data(); m.rad = S.rad.data(); m.phi_o = S.phi_o.data(); m.r_var = S.r_var.data();
  m.core_pos = S.core_pos.data(); m.core_q = S.core_q.data();
  m.tail_pos = S.tail_pos.data(); m.tail_fix = S.tail_fix.data(); m.nc_t_flag = S.nc_t_flag.data();
  m.h_t = S.h_t.data(); m.g_t = S.g_t.data(); m.lo_t = S.lo_t.data(); m.beta_o_t = S.beta_o_t.data();
  m.t_q = S.t_q.data(); m.t_rad = S.t_rad.data(); m.t_grp = S.t_grp.data(); m.t_fix = S.t_fix.data();
  m.LH_g_pos = S.LH_g_pos.data(); m.LH_conn = S.LH_conn.data(); m.nc_lh_flag = S.nc_lh_flag.data();
  m.LH_q = S.LH_q.data(); m.LH_vdw_hh = S.LH_vdw_hh.data(); m.LH_vdw_hc = S.LH_vdw_hc.data();
  m.LH_vdw_hl = S.LH_vdw_hl.data(); m.LH_vdw_ht = S.LH_vdw_ht.data(); m.LH_kstr = S.LH_kstr.data();
  m.LH_kben = S.LH_kben.data(); m.LH_streq = S.LH_streq.data(); m.LH_betaeq = S.LH_betaeq.data();
  m.lh_rad = S.lh_rad.data();
}

// readfile.cpp:346-405 (default ostream precision: 6 significant digits)
int write_xyz(const bd_model* m, const double* r, const double* a, const double* b, const double* c,
              const double* r_t, const double* r_lh, const char* path) {
  std::ofstream out(path, std::ios_base::app);
  if (!out) return BD_ERR_IO;
  int nc_lh = 0;
  for (int i = 0; i < m->n_c; i++) nc_lh += (m->nc_lh_flag[i] == 1);
  out << m->n * 4 + m->n_c * m->Nq + m->n_tail + m->n_LH + nc_lh * m->n_lh_g << "\n";
  out << "comments zl3765" << "\n";
  auto body = [&](int i, const double* p, double* z) {
    for (int x = 0; x < 3; x++) z[x] = r[3 * i + x] + a[3 * i + x] * p[0] + b[3 * i + x] * p[1] + c[3 * i + x] * p[2];
  };
  for (int i = 0; i < m->n; i++) {
    out << (m->type[i] == 0 ? "CA" : "OC") << " " << r[3 * i] << " " << r[3 * i + 1] << " " << r[3 * i + 2] << "\n";
    out << "H1" << " " << a[3 * i] << " " << a[3 * i + 1] << " " << a[3 * i + 2] << "\n";
    out << "H2" << " " << b[3 * i] << " " << b[3 * i + 1] << " " << b[3 * i + 2] << "\n";
    out << "H3" << " " << c[3 * i] << " " << c[3 * i + 1] << " " << c[3 * i + 2] << "\n";
    if (m->type[i] != 0) {
      for (int j = 0; j < m->Nq; j++) {
        double z[3];
        body(i, &m->core_pos[3 * j], z);
        out << "NC" << " " << z[0] << " " << z[1] << " " << z[2] << "\n";
      }
    }
  }
  for (int i = 0; i < m->n_tail; i++) out << "HT" << " " << r_t[3 * i] << " " << r_t[3 * i + 1] << " " << r_t[3 * i + 2] << "\n";
  int k = 0;
  for (int i = 0; i < m->n; i++) {
    if (m->type[i] != 1) continue;
    if (m->nc_lh_flag[k] == 1) {
      for (int j = 0; j < m->n_lh_g; j++) {
        double z[3];
        body(i, &m->LH_g_pos[3 * j], z);
        out << "LHG" << " " << z[0] << " " << z[1] << " " << z[2] << "\n";
      }
    }
    k++;
  }
  for (int i = 0; i < m->n_LH; i++) out << "LH" << " " << r_lh[3 * i] << " " << r_lh[3 * i + 1] << " " << r_lh[3 * i + 2] << "\n";
  out.flush();
  return out ? BD_OK : BD_ERR_IO;
}

// ---------------------------------------------------------------- noise
// MT19937 (Matsumoto & Nishimura, ACM TOMACS 8(1), 1998): 624-word state,
// twist with the published matrix 0x9908b0df and tempering masks.
void Mt19937::seed(uint32_t s) {
  st[0] = s;
  for (int i = 1; i < 624; i++) st[i] = 1812433253u * (st[i - 1] ^ (st[i - 1] >> 30)) + (uint32_t)i;
  idx = 624;
}

uint32_t Mt19937::next() {
  if (idx >= 624) {
    int i = 0;
    for (; i < 624 - 397; i++) {
      uint32_t y = (st[i] & 0x80000000u) | (st[i + 1] & 0x7fffffffu);
      st[i] = st[i + 397] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    for (; i < 623; i++) {
      uint32_t y = (st[i] & 0x80000000u) | (st[i + 1] & 0x7fffffffu);
      st[i] = st[i + 397 - 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    uint32_t y = (st[623] & 0x80000000u) | (st[0] & 0x7fffffffu);
    st[623] = st[396] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    idx = 0;
  }
  uint32_t y = st[idx++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= (y >> 18);
  return y;
}

// Polar (Marsaglia) Box-Muller with one cached deviate, as utilities.cpp:304-336.
double Mt19937::normal(double mean, double sd) {
  if (have) {
    have = false;
    return cached * sd + mean;
  }
  double x, y, q;
  do {
    x = 2.0 * real1() - 1;
    y = 2.0 * real1() - 1;
    q = x * x + y * y;
  } while (q == 0.0 || q > 1.0);
  double d = std::sqrt(-2.0 * (cr_log ? crlog::log_cr(q) : std::log(q)) / q);
  cached = y * d;
  have = true;
  return x * d * sd + mean;
}

}  // namespace bdh

// ---------------------------------------------------------------- C ABI
using namespace bdh;

extern "C" int bd_system_load(const char* dir, const char* data_file, const char* core_file, const char* tail_file,
                              const char* lh_file, const char* lh_flags_file, bd_system** out) {
  if (!out || !core_file || !tail_file || !lh_file) return set_error(BD_ERR_ARG, "bd_system_load: null argument");
  HostSystem* S = new HostSystem();
  std::string err;
  int rc = load_system(dir, data_file, core_file, tail_file, lh_file, lh_flags_file, *S, err);
  if (rc != BD_OK) {
    delete S;
    return set_error(rc, ("bd_system_load: " + err).c_str());
  }
  *out = reinterpret_cast<bd_system*>(S);
  return BD_OK;
}

extern "C" int bd_system_model(const bd_system* sys, bd_model* out) {
  if (!sys || !out) return set_error(BD_ERR_ARG, "bd_system_model: null argument");
  *out = reinterpret_cast<const HostSystem*>(sys)->m;
  return BD_OK;
}

extern "C" int bd_system_state(const bd_system* sys, bd_state* out) {
  if (!sys || !out) return set_error(BD_ERR_ARG, "bd_system_state: null argument");
  const HostSystem* S = reinterpret_cast<const HostSystem*>(sys);
  memset(out, 0, sizeof *out);
  out->r = S->r.data(); out->a = S->a.data(); out->b = S->b.data(); out->c = S->c.data();
  out->r_t = S->r_t.data(); out->r_lh = S->r_lh.data();
  out->refresh_frames = 1;
  return BD_OK;
}

extern "C" int bd_system_setup(const bd_system* sys, double* out15) {
  if (!sys || !out15) return set_error(BD_ERR_ARG, "bd_system_setup: null argument");
  const HostSystem* S = reinterpret_cast<const HostSystem*>(sys);
  for (int i = 0; i < 15; i++) out15[i] = S->setup[i];
  return BD_OK;
}

extern "C" void bd_system_free(bd_system* sys) { delete reinterpret_cast<HostSystem*>(sys); }

extern "C" int bd_write_xyz(const bd_model* m, const double* r, const double* a, const double* b, const double* c,
                            const double* r_t, const double* r_lh, const char* path) {
  if (!m || !r || !a || !b || !c || !path) return set_error(BD_ERR_ARG, "bd_write_xyz: null argument");
  int rc = write_xyz(m, r, a, b, c, r_t, r_lh, path);
  return rc == BD_OK ? BD_OK : set_error(rc, "bd_write_xyz: write failed");
}

extern "C" int bd_noise_create(unsigned long seed, bd_noise** out) {
  if (!out) return set_error(BD_ERR_ARG, "bd_noise_create: null argument");
  Mt19937* g = new Mt19937();
  g->seed((uint32_t)(seed & 0xffffffffUL));
  *out = reinterpret_cast<bd_noise*>(g);
  return BD_OK;
}

extern "C" int bd_noise_step(bd_noise* gp, int step, int n3, const double* r_var, int n_D3, double* rr, double* p) {
  if (!gp || (n3 > 0 && (!r_var || !rr)) || (n_D3 > 0 && !p)) return set_error(BD_ERR_ARG, "bd_noise_step: null argument");
  Mt19937& g = *reinterpret_cast<Mt19937*>(gp);
  if (step % 100 == 0) { (void)g.real1(); (void)g.real1(); }
  for (int i = 0; i < n3; i++) rr[i] = g.normal(0, r_var[i]);
  for (int i = 0; i < n_D3; i++) p[i] = g.normal(0, 1);
  return BD_OK;
}

extern "C" int bd_noise_u32(bd_noise* gp, int count, uint32_t* out) {
  if (!gp || (count > 0 && !out)) return set_error(BD_ERR_ARG, "bd_noise_u32: null argument");
  Mt19937& g = *reinterpret_cast<Mt19937*>(gp);
  for (int i = 0; i < count; i++) out[i] = g.next();
  return BD_OK;
}

extern "C" void bd_noise_free(bd_noise* g) { delete reinterpret_cast<Mt19937*>(g); }

extern "C" int bd_noise_set_log(bd_noise* gp, int mode) {
  if (!gp || (mode != BD_LOG_LIBM && mode != BD_LOG_CR)) return set_error(BD_ERR_ARG, "bd_noise_set_log: bad argument");
  reinterpret_cast<Mt19937*>(gp)->cr_log = mode == BD_LOG_CR;
  return BD_OK;
}

extern "C" int bd_noise_get_state(const bd_noise* gp, uint32_t* words624, int* index, int* have_cached,
                                  double* cached) {
  if (!gp || !words624 || !index || !have_cached || !cached) return set_error(BD_ERR_ARG, "bd_noise_get_state: null argument");
  const Mt19937& g = *reinterpret_cast<const Mt19937*>(gp);
  std::memcpy(words624, g.st, sizeof g.st);
  *index = g.idx;
  *have_cached = g.have ? 1 : 0;
  *cached = g.cached;
  return BD_OK;
}

extern "C" int bd_noise_set_state(bd_noise* gp, const uint32_t* words624, int index, int have_cached, double cached) {
  if (!gp || !words624 || index < 0 || index > 625) return set_error(BD_ERR_ARG, "bd_noise_set_state: bad argument");
  Mt19937& g = *reinterpret_cast<Mt19937*>(gp);
  std::memcpy(g.st, words624, sizeof g.st);
  g.idx = index;
  g.have = have_cached != 0;
  g.cached = cached;
  return BD_OK;
}

// ---------------------------------------------------------------- restart
namespace {
const char kRestartMagic[8] = {'B', 'D', 'R', 'S', 'T', '0', '0', '1'};

struct RestartHead {
  char magic[8];
  int32_t n, n_c, n_tail, n_LH, has_noise, pad;
  int64_t step;
};

// the arrays of a restart in file order, with their lengths
std::vector<std::pair<double*, size_t>> restart_arrays(const bd_restart& r) {
  const size_t n = r.n, nc = r.n_c, nt = r.n_tail, nl = r.n_LH;
  return {{r.r, 3 * n},       {r.a, 3 * n},       {r.b, 3 * n},       {r.c, 3 * n},      {r.alpha, n},
          {r.beta, n},        {r.gamma, n},       {r.length, n},      {r.a_dna, 3 * nc}, {r.b_dna, 3 * nc},
          {r.c_dna, 3 * nc},  {r.alpha_p, nc},    {r.beta_p, nc},     {r.gamma_p, nc},   {r.r_t, 3 * nt},
          {r.r_lh, 3 * nl}};
}

bool sizes_ok(const bd_restart& r) { return r.n > 0 && r.n_c > 0 && r.n_tail >= 0 && r.n_LH >= 0; }
}  // namespace

extern "C" int bd_restart_write(const char* path, const bd_restart* rs, const bd_noise* g) {
  if (!path || !rs || !sizes_ok(*rs) || !rs->nc_lh_flag) return set_error(BD_ERR_ARG, "bd_restart_write: bad argument");
  for (auto& a : restart_arrays(*rs))
    if (a.second && !a.first) return set_error(BD_ERR_ARG, "bd_restart_write: missing array");
  FILE* f = std::fopen(path, "wb");
  if (!f) return set_error(BD_ERR_IO, "bd_restart_write: cannot open file");
  RestartHead h{};
  std::memcpy(h.magic, kRestartMagic, 8);
  h.n = rs->n, h.n_c = rs->n_c, h.n_tail = rs->n_tail, h.n_LH = rs->n_LH, h.has_noise = g ? 1 : 0;
  h.step = rs->step;
  bool ok = std::fwrite(&h, sizeof h, 1, f) == 1;
  for (auto& a : restart_arrays(*rs))
    if (a.second) ok = ok && std::fwrite(a.first, sizeof(double), a.second, f) == a.second;
  ok = ok && std::fwrite(rs->nc_lh_flag, sizeof(int32_t), rs->n_c, f) == (size_t)rs->n_c;
  if (g) {
    const Mt19937& m = *reinterpret_cast<const Mt19937*>(g);
    const int32_t idx = m.idx, have = m.have ? 1 : 0;
    ok = ok && std::fwrite(m.st, sizeof m.st, 1, f) == 1 && std::fwrite(&idx, 4, 1, f) == 1 &&
         std::fwrite(&have, 4, 1, f) == 1 && std::fwrite(&m.cached, 8, 1, f) == 1;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? BD_OK : set_error(BD_ERR_IO, "bd_restart_write: write failed");
}

static int read_head(FILE* f, RestartHead& h) {
  if (std::fread(&h, sizeof h, 1, f) != 1 || std::memcmp(h.magic, kRestartMagic, 8) != 0)
    return set_error(BD_ERR_IO, "bd_restart: not a restart file");
  if (h.n <= 0 || h.n_c <= 0 || h.n_tail < 0 || h.n_LH < 0) return set_error(BD_ERR_IO, "bd_restart: bad sizes");
  return BD_OK;
}

extern "C" int bd_restart_info(const char* path, bd_restart* rs, int* has_noise) {
  if (!path || !rs) return set_error(BD_ERR_ARG, "bd_restart_info: null argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(BD_ERR_IO, "bd_restart_info: cannot open file");
  RestartHead h{};
  int rc = read_head(f, h);
  std::fclose(f);
  if (rc) return rc;
  rs->step = (long)h.step, rs->n = h.n, rs->n_c = h.n_c, rs->n_tail = h.n_tail, rs->n_LH = h.n_LH;
  if (has_noise) *has_noise = h.has_noise;
  return BD_OK;
}

extern "C" int bd_restart_read(const char* path, bd_restart* rs, bd_noise* g) {
  if (!path || !rs || !rs->nc_lh_flag) return set_error(BD_ERR_ARG, "bd_restart_read: bad argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(BD_ERR_IO, "bd_restart_read: cannot open file");
  RestartHead h{};
  int rc = read_head(f, h);
  if (!rc && (h.n != rs->n || h.n_c != rs->n_c || h.n_tail != rs->n_tail || h.n_LH != rs->n_LH))
    rc = set_error(BD_ERR_ARG, "bd_restart_read: sizes differ from the file's");
  bool ok = !rc;
  for (auto& a : restart_arrays(*rs)) {
    if (!ok) break;
    if (a.second && !a.first) {
      rc = set_error(BD_ERR_ARG, "bd_restart_read: missing array");
      ok = false;
      break;
    }
    if (a.second) ok = std::fread(a.first, sizeof(double), a.second, f) == a.second;
  }
  ok = ok && std::fread(rs->nc_lh_flag, sizeof(int32_t), rs->n_c, f) == (size_t)rs->n_c;
  bool bad_idx = false;
  if (ok && g && h.has_noise) {
    // read into a copy first: the generator is changed only by a complete,
    // valid state (its index must lie in [0, 625]; next() reads st[idx])
    Mt19937 tmp;
    int32_t idx = 0, have = 0;
    double cached = 0.0;
    ok = std::fread(tmp.st, sizeof tmp.st, 1, f) == 1 && std::fread(&idx, 4, 1, f) == 1 &&
         std::fread(&have, 4, 1, f) == 1 && std::fread(&cached, 8, 1, f) == 1;
    bad_idx = ok && (idx < 0 || idx > 625);
    if (ok && !bad_idx) {
      Mt19937& m = *reinterpret_cast<Mt19937*>(g);
      std::memcpy(m.st, tmp.st, sizeof m.st);
      m.idx = idx, m.have = have != 0, m.cached = cached;
    }
  }
  std::fclose(f);
  if (rc) return rc;
  if (!ok) return set_error(BD_ERR_IO, "bd_restart_read: truncated file");
  if (bad_idx) return set_error(BD_ERR_IO, "bd_restart_read: generator index out of range");
  rs->step = (long)h.step;
  return BD_OK;
}

// ---------------------------------------------------------------- LH binding
extern "C" int bd_system_lh_template(const bd_system* sys, double* pos, double* rad) {
  if (!sys || !pos || !rad) return set_error(BD_ERR_ARG, "bd_system_lh_template: null argument");
  const HostSystem* S = reinterpret_cast<const HostSystem*>(sys);
  std::memcpy(pos, S->lh_tpos.data(), S->lh_tpos.size() * sizeof(double));
  std::memcpy(rad, S->lh_trad.data(), S->lh_trad.size() * sizeof(double));
  return BD_OK;
}

// main.cpp:386-412
extern "C" int bd_lh_mc(int n_c, double u_random, double u_core, double unbind, double Pbind, int* nc_lh_flag,
                        int* changed) {
  if (n_c <= 0 || !nc_lh_flag) return set_error(BD_ERR_ARG, "bd_lh_mc: bad argument");
  int n_b = (int)(n_c * u_core);
  if (n_b >= n_c) n_b = n_c - 1;
  const int before = nc_lh_flag[n_b];
  if (nc_lh_flag[n_b] > 0.5) {
    if (u_random <= unbind) nc_lh_flag[n_b] = 0;
  } else {
    if (u_random <= Pbind) nc_lh_flag[n_b] = 1;
  }
  if (changed) *changed = nc_lh_flag[n_b] != before;
  return BD_OK;
}

// main.cpp:414-447 with build_LH (func.cpp:2029-2059): every bound core's
// beads placed from the template in its frame, then the beads of the cores
// bound before overwritten with their previous positions
extern "C" int bd_lh_rebind(int n, const int* type, int n_c, const double* r, const double* a, const double* b,
                            const double* c, int nlh, const double* tpos, const double* trad, const int* old_flags,
                            const double* old_r_lh, const int* new_flags, double* new_r_lh, double* new_lh_rad) {
  if (n <= 0 || n_c <= 0 || nlh <= 0 || !type || !r || !a || !b || !c || !tpos || !trad || !old_flags || !new_flags ||
      !new_r_lh || !new_lh_rad)
    return set_error(BD_ERR_ARG, "bd_lh_rebind: null argument");
  int k = 0, k1 = 0;
  for (int i = 0; i < n; i++) {
    if (type[i] != 1) continue;
    if (k1 >= n_c) return set_error(BD_ERR_ARG, "bd_lh_rebind: more cores in type[] than n_c");
    if (new_flags[k1] == 1) {
      for (int j = 0; j < nlh; j++) {
        const double* p = tpos + 3 * j;
        for (int x = 0; x < 3; x++)
          new_r_lh[(k * nlh + j) * 3 + x] =
              r[i * 3 + x] + a[i * 3 + x] * p[0] + b[i * 3 + x] * p[1] + c[i * 3 + x] * p[2];
        new_lh_rad[k * nlh + j] = trad[j];
      }
      k++;
    }
    k1++;
  }
  k = 0;
  k1 = 0;
  for (int i = 0; i < n_c; i++) {
    if (new_flags[i] == 1) {
      if (old_flags[i] == 1) {
        if (!old_r_lh) return set_error(BD_ERR_ARG, "bd_lh_rebind: previous LH positions required");
        for (int j = 0; j < nlh; j++)
          for (int x = 0; x < 3; x++) new_r_lh[(k * nlh + j) * 3 + x] = old_r_lh[(k1 * nlh + j) * 3 + x];
        k1++;
      }
      k++;
    } else if (old_flags[i] == 1) {
      k1++;
    }
  }
  return BD_OK;
}

extern "C" int bd_noise_uniforms(bd_noise* gp, int count, double* out) {
  if (!gp || count < 0 || (count > 0 && !out)) return set_error(BD_ERR_ARG, "bd_noise_uniforms: bad argument");
  Mt19937& g = *reinterpret_cast<Mt19937*>(gp);
  for (int i = 0; i < count; i++) out[i] = g.real1();
  return BD_OK;
}

extern "C" int bd_noise_draws(bd_noise* gp, int n3, const double* r_var, int n_D3, double* rr, double* p) {
  if (!gp || (n3 > 0 && (!r_var || !rr)) || (n_D3 > 0 && !p)) return set_error(BD_ERR_ARG, "bd_noise_draws: null argument");
  Mt19937& g = *reinterpret_cast<Mt19937*>(gp);
  for (int i = 0; i < n3; i++) rr[i] = g.normal(0, r_var[i]);
  for (int i = 0; i < n_D3; i++) p[i] = g.normal(0, 1);
  return BD_OK;
}



// write_restart (readfile.cpp:404-439): one value per line, fixed notation
// with 15 decimals, one file per array, in dir
extern "C" int bd_write_restart_text(const char* dir, int n, int n_tail, int n_LH, const double* r, const double* a,
                                     const double* b, const double* c, const double* Er, const double* r_t,
                                     const double* r_lh) {
  if (!dir || n <= 0 || !r || !a || !b || !c || (n_tail > 0 && !r_t) || (n_LH > 0 && !r_lh))
    return set_error(BD_ERR_ARG, "bd_write_restart_text: bad argument");
  const std::vector<double> zero(3 * (size_t)n, 0.0);
  struct F { const char* name; const double* v; size_t cnt; } files[] = {
      {"restart_r.txt", r, 3 * (size_t)n},        {"restart_a.txt", a, 3 * (size_t)n},
      {"restart_b.txt", b, 3 * (size_t)n},        {"restart_c.txt", c, 3 * (size_t)n},
      {"restart_Er.txt", Er ? Er : zero.data(), 3 * (size_t)n},
      {"restart_tail.txt", r_t, 3 * (size_t)n_tail}, {"restart_lh.txt", r_lh, 3 * (size_t)n_LH}};
  for (auto& f : files) {
    FILE* fp = std::fopen(join(dir, f.name).c_str(), "w");
    if (!fp) return set_error(BD_ERR_IO, "bd_write_restart_text: cannot open a file");
    bool ok = true;
    for (size_t i = 0; i < f.cnt && ok; i++) ok = std::fprintf(fp, "%.15f\n", f.v[i]) > 0;
    ok = (std::fclose(fp) == 0) && ok;
    if (!ok) return set_error(BD_ERR_IO, "bd_write_restart_text: write failed");
  }
  return BD_OK;
}

