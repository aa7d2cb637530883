// Device context and step orchestration behind include/bd_capi.h.
//
// One context owns every device buffer of one fiber (no file-scope
// globals, unlike func_cuda.cu:3-104).  All buffers are allocated once at
// creation; a step allocates nothing (the reference frees and re-allocates
// D, Chol, the cuSOLVER handle and workspace every step,
// func_cuda.cu:3436-3534).  The device part of a step is stream-ordered and
// can be captured once into a CUDA graph and replayed.
//
// Step order follows main_cuda (func_cuda.cu:3434-3680):
//   r_all <- state; D <- RPY(r_all); L <- chol(D) in place; rd <- s2dt L p;
//   F0 <- forces(X); Y <- move(X, F0); frames(Y); F1 <- forces(Y);
//   Fa <- (F0 + F1)/2; Y <- move(X, Fa); X <- Y; frames(X).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
#define BD_HAVE_NVTX 1
#endif

#include "bd_internal.h"

namespace bdh {
#ifdef BD_HAVE_NVTX
Range::Range(const char* name) { nvtxRangePushA(name); }
Range::~Range() { nvtxRangePop(); }
#else
Range::Range(const char*) {}
Range::~Range() {}
#endif

static thread_local std::string g_err;
int set_error(int code, const char* msg) {
  g_err = msg ? msg : "";
  return code;
}
}  // namespace bdh

using bdh::set_error;

extern "C" const char* bd_last_error(void) { return bdh::g_err.c_str(); }
extern "C" const char* bd_version(void) { return "bd-gb300 0.1 (sm_103a)"; }

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

// Bump allocator over one device allocation (256-byte aligned slices).
struct Arena {
  char* base = nullptr;
  size_t size = 0, used = 0;
  template <class T>
  T* take(size_t count) {
    size_t bytes = ((count * sizeof(T)) + 255) & ~size_t(255);
    if (bytes == 0) bytes = 256;
    T* p = reinterpret_cast<T*>(base + used);
    used += bytes;
    return p;
  }
};

template <class T>
size_t slab(size_t count) {
  size_t b = ((count * sizeof(T)) + 255) & ~size_t(255);
  return b ? b : 256;
}

}  // namespace


namespace {

int validate(const bd_model* m) {
  if (!m || m->n < 3 || m->n_c < 1 || !m->type || !m->phi_o || !m->rad) return set_error(BD_ERR_ARG, "bd_create: model sizes/arrays");
  if (m->type[0] != 1 || m->type[m->n - 1] != 0)
    return set_error(BD_ERR_ARG, "bd_create: chain must start with a core and end with linker DNA");
  int nc = 0;
  for (int i = 0; i < m->n; i++) nc += m->type[i] == 1;
  if (nc != m->n_c) return set_error(BD_ERR_ARG, "bd_create: n_c does not match type[]");
  if (m->Nq < 1 || !m->core_pos || !m->core_q) return set_error(BD_ERR_ARG, "bd_create: core charges");
  if (m->n_tail != m->n_c * m->n_t) return set_error(BD_ERR_ARG, "bd_create: n_tail must be n_c * n_t");
  if (m->n_lh_n != 0) return set_error(BD_ERR_ARG, "bd_create: LH N-terminal beads are not supported");
  int nlh = m->n_lh_n + m->n_lh_c;
  int nlhc = 0;
  for (int i = 0; i < m->n_c; i++) nlhc += m->nc_lh_flag && m->nc_lh_flag[i] == 1;
  if (m->n_LH != nlhc * nlh) return set_error(BD_ERR_ARG, "bd_create: n_LH does not match nc_lh_flag");
  return BD_OK;
}

template <class T>
int up(T* d, const T* h, size_t cnt, cudaStream_t st) {
  if (cnt == 0) return BD_OK;
  if (!h) return set_error(BD_ERR_ARG, "bd_create: missing array");
  CK(cudaMemcpyAsync(d, h, cnt * sizeof(T), cudaMemcpyHostToDevice, st));
  return BD_OK;
}

int record(bd_ctx* c, int k) {
  if (c->timing) CK(cudaEventRecord(c->ev[k], c->stream));
  return BD_OK;
}

// The device part of one step (stream-ordered, capturable).
}  // namespace

// [r a b c r_t] of a state into one buffer (12n + 3 n_tail doubles)
static int pack_ns(bd_ctx* c, const DevState& Y, double* dst) {
  const size_t n3 = 3 * (size_t)c->M.n, b = n3 * sizeof(double);
  CK(cudaMemcpyAsync(dst, Y.r, b, cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaMemcpyAsync(dst + n3, Y.a, b, cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaMemcpyAsync(dst + 2 * n3, Y.b, b, cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaMemcpyAsync(dst + 3 * n3, Y.c, b, cudaMemcpyDeviceToDevice, c->stream));
  if (c->M.n_tail)
    CK(cudaMemcpyAsync(dst + 4 * n3, Y.r_t, 3 * (size_t)c->M.n_tail * sizeof(double), cudaMemcpyDeviceToDevice,
                       c->stream));
  return BD_OK;
}

// The phases of one step: kPre (positions, RPY tensor), kChol (its
// factorisation), kPost (noise displacement, forces, moves, frames).  A
// batch runs kPre of every replica, one batched factorisation, then kPost.
enum { kPre = 1, kChol = 2, kPost = 4 };

static int step_phases(bd_ctx* c, const double* d_rr, const double* d_p, double* const* saves, int phases) {
  bdh::Range range(phases == (kPre | kChol | kPost) ? "bd_step" : phases == kPre ? "bd_step: positions, tensor"
                                                                  : phases == kPost ? "bd_step: forces, moves"
                                                                                    : "bd_step: factorisation");
  DevModel& M = c->M;
  cudaStream_t st = c->stream;
  int L = 0, rc = 0;
  const bool mixed = c->precision == BD_PREC_MIXED;
  const bool krylov = c->noise_mode == BD_NOISE_KRYLOV;
  // a Krylov step needs D itself: rebuilt when A holds a factor
  bool rebuild = (c->step_count % c->freq_rp) == 0 || (krylov && c->a_holds_factor) || c->need_rebuild;
  if (phases & kPre) {
    record(c, 0);
    bdk::gather_rall(M, c->X, c->r_all, mixed ? &c->S : nullptr, st);
    L += mixed ? 2 : 1;
    if (rebuild && !(krylov && mixed)) {  // mixed Krylov products are matrix-free: no tensor
      bdk::rpy_assemble(M.n_D, c->r_all, M.rad_all, M.a1, M.a2, c->A, c->lda, st, mixed ? c->S.qh : nullptr,
                        mixed ? c->S.ql : nullptr);
      L++;
      CK(cudaMemsetAsync(c->negpiv, 0, sizeof(int), st));
      c->a_holds_factor = false;
      c->need_rebuild = false;
    }
    record(c, 1);
  }
  if ((phases & kChol) && rebuild && !krylov) {
    c->a_holds_factor = true;
    if (mixed) {
      const bool kt = c->timing && !c->kev.empty();
      c->kflop = 0.0;
      c->kbytes = 0.0;
      c->kev_pairs = 0;
      L += bdk::potrf_mixed(c->m, c->A, c->lda, c->PS, c->negpiv, c->d_err, st, kt ? c->kev.data() : nullptr,
                            kt ? &c->kev_pairs : nullptr, kt ? &c->kflop : nullptr,
                            kt ? &c->kbytes : nullptr, c->mixed_passes);
    }
    else L += bdk::potrf_fp64(c->m, c->A, c->lda, nullptr, nullptr, 0.0, c->negpiv, st);
  }
  if (!(phases & kPost)) {
    c->last_launches = L;
    return BD_OK;
  }
  record(c, 2);
  if (krylov) {
    rc = bdk::krylov_sqrt(c->m, mixed ? nullptr : c->A, c->lda, mixed, c->S.qh, c->S.ql, M.a1, M.a2, d_p, M.s2dt,
                          c->krylov_tol, c->krylov_kmax, c->rd, c->kscratch, st, &c->krylov_iters, &c->krylov_change,
                          &c->kgraphs);
    if (rc) return set_error(rc, "bd_step: Krylov noise displacement failed");
    L += 10 * c->krylov_iters + 4;
  } else {
    bdk::trmv_lower_ws(c->m, c->A, c->lda, d_p, M.s2dt, c->rd, c->rd_part, st, mixed);
    L += 2;
  }
  record(c, 3);
  L += bdk::forces(M, c->X, c->F0, c->S, c->precision, st);
  record(c, 4);
  bdk::rotate_translate(M, c->X, c->Y, c->F0, d_rr, c->rd, c->r_all, c->precision, c->S, st);
  L += mixed ? 3 : 2;
  if (saves && (rc = pack_ns(c, c->Y, saves[0]))) return rc;
  record(c, 5);
  bdk::frames(M, c->Y, st);
  L += 2;
  if (saves && (rc = pack_ns(c, c->Y, saves[1]))) return rc;
  record(c, 6);
  L += bdk::forces(M, c->Y, c->F1, c->S, c->precision, st);
  record(c, 7);
  bdk::average_forces(M, c->F0, c->F1, c->Fa, st);
  bdk::rotate_translate(M, c->X, c->Y, c->Fa, d_rr, c->rd, c->r_all, c->precision, c->S, st);
  L += mixed ? 4 : 3;
  if (saves && (rc = pack_ns(c, c->Y, saves[2]))) return rc;
  // X <- Y (final_updates, func_cuda.cu:2643-2662), then refresh frames
  size_t n3 = 3 * (size_t)M.n;
  CK(cudaMemcpyAsync(c->X.r, c->Y.r, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(c->X.a, c->Y.a, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(c->X.b, c->Y.b, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(c->X.c, c->Y.c, n3 * sizeof(double), cudaMemcpyDeviceToDevice, st));
  if (M.n_tail) CK(cudaMemcpyAsync(c->X.r_t, c->Y.r_t, 3 * (size_t)M.n_tail * sizeof(double), cudaMemcpyDeviceToDevice, st));
  if (M.n_LH) CK(cudaMemcpyAsync(c->X.r_lh, c->Y.r_lh, 3 * (size_t)M.n_LH * sizeof(double), cudaMemcpyDeviceToDevice, st));
  bdk::frames(M, c->X, st);
  L += 2;
  record(c, 8);
  CK(cudaGetLastError());
  c->last_launches = L;
  return BD_OK;
}

int bdh::step_device(bd_ctx* c, const double* d_rr, const double* d_p, double* const* saves) {
  return step_phases(c, d_rr, d_p, saves, kPre | kChol | kPost);
}

using bdh::step_device;


namespace {
template <class T>
std::vector<T> vec(const T* p, long n) {
  return (p && n > 0) ? std::vector<T>(p, p + n) : std::vector<T>();
}
template <class T>
const T* ptr(const std::vector<T>& v) {
  return v.empty() ? nullptr : v.data();
}
}  // namespace

void bdh::ModelCopy::take(const bd_model& s) {
  m = s;
  const long n = s.n, nc = s.n_c, Nq = s.Nq, nt0 = s.n_t, nt = s.n_tail, np = s.n_lh_n + s.n_lh_g + s.n_lh_c;
  type = vec(s.type, n); rad = vec(s.rad, n); phi_o = vec(s.phi_o, n); r_var = vec(s.r_var, 3 * n);
  core_pos = vec(s.core_pos, 3 * Nq); core_q = vec(s.core_q, Nq); tail_pos = vec(s.tail_pos, 3 * nt0);
  tail_fix = vec(s.tail_fix, nt0); nc_t_flag = vec(s.nc_t_flag, nc);
  h_t = vec(s.h_t, nt); g_t = vec(s.g_t, nt); lo_t = vec(s.lo_t, nt); beta_o_t = vec(s.beta_o_t, nt);
  t_q = vec(s.t_q, nt); t_rad = vec(s.t_rad, nt); t_grp = vec(s.t_grp, nt); t_fix = vec(s.t_fix, nt);
  LH_g_pos = vec(s.LH_g_pos, 3L * s.n_lh_g); LH_conn = vec(s.LH_conn, np); nc_lh_flag = vec(s.nc_lh_flag, nc);
  LH_q = vec(s.LH_q, np); LH_vdw_hh = vec(s.LH_vdw_hh, np); LH_vdw_hc = vec(s.LH_vdw_hc, np);
  LH_vdw_hl = vec(s.LH_vdw_hl, np); LH_vdw_ht = vec(s.LH_vdw_ht, np); LH_kstr = vec(s.LH_kstr, np);
  LH_kben = vec(s.LH_kben, np); LH_streq = vec(s.LH_streq, np); LH_betaeq = vec(s.LH_betaeq, np);
  lh_rad = vec(s.lh_rad, s.n_LH);
  bind();
}

void bdh::ModelCopy::bind() {
  m.type = ptr(type); m.rad = ptr(rad); m.phi_o = ptr(phi_o); m.r_var = ptr(r_var);
  m.core_pos = ptr(core_pos); m.core_q = ptr(core_q); m.tail_pos = ptr(tail_pos); m.tail_fix = ptr(tail_fix);
  m.nc_t_flag = ptr(nc_t_flag); m.h_t = ptr(h_t); m.g_t = ptr(g_t); m.lo_t = ptr(lo_t); m.beta_o_t = ptr(beta_o_t);
  m.t_q = ptr(t_q); m.t_rad = ptr(t_rad); m.t_grp = ptr(t_grp); m.t_fix = ptr(t_fix); m.LH_g_pos = ptr(LH_g_pos);
  m.LH_conn = ptr(LH_conn); m.nc_lh_flag = ptr(nc_lh_flag); m.LH_q = ptr(LH_q); m.LH_vdw_hh = ptr(LH_vdw_hh);
  m.LH_vdw_hc = ptr(LH_vdw_hc); m.LH_vdw_hl = ptr(LH_vdw_hl); m.LH_vdw_ht = ptr(LH_vdw_ht); m.LH_kstr = ptr(LH_kstr);
  m.LH_kben = ptr(LH_kben); m.LH_streq = ptr(LH_streq); m.LH_betaeq = ptr(LH_betaeq); m.lh_rad = ptr(lh_rad);
}

extern "C" int bd_create(const bd_model* m, const bd_state* s, const bd_options* opt, bd_ctx** out) {
  if (!out || !s) return set_error(BD_ERR_ARG, "bd_create: null argument");
  int rc = validate(m);
  if (rc) return rc;
  if (!s->r || !s->a || !s->b || !s->c || (m->n_tail && !s->r_t) || (m->n_LH && !s->r_lh))
    return set_error(BD_ERR_ARG, "bd_create: state arrays");
  if (!s->refresh_frames && (!s->alpha || !s->beta || !s->gamma || !s->length || !s->a_dna || !s->b_dna || !s->c_dna ||
                             !s->alpha_p || !s->beta_p || !s->gamma_p))
    return set_error(BD_ERR_ARG, "bd_create: angles required when refresh_frames == 0");
  bd_ctx* c = new bd_ctx();
  c->model = std::make_shared<bdh::ModelCopy>();
  c->model->take(*m);
  if (opt) {
    c->precision = opt->precision;
    c->freq_rp = opt->frequency_RP > 0 ? opt->frequency_RP : 1;
    c->use_graph = opt->use_graph;
    c->device = opt->device;
    c->stream = (cudaStream_t)opt->stream;
  }
  auto fail = [&](int code) {
    bd_destroy(c);
    return code;
  };
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) {
    delete c;
    return set_error(BD_ERR_CUDA, (std::string("bd_create: cudaSetDevice: ") + cudaGetErrorString(e)).c_str());
  }
  if (!c->stream) {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete c;
      return set_error(BD_ERR_CUDA, "bd_create: stream creation failed");
    }
    c->own_stream = true;
  }
  DevModel& M = c->M;
  M.n = m->n; M.n_c = m->n_c; M.Nq = m->Nq; M.n_t = m->n_t; M.n_tail = m->n_tail;
  M.n_lh_n = m->n_lh_n; M.n_lh_g = m->n_lh_g; M.n_lh_c = m->n_lh_c; M.n_LH = m->n_LH;
  M.n_D = M.n + M.n_tail + M.n_LH;
  M.nlh = M.n_lh_n + M.n_lh_c;
  M.h = m->h; M.g = m->g; M.s = m->s; M.debyell = m->debyell; M.debye = m->debye; M.q_l = m->q_l;
  M.k_e = m->k_e; M.k_ex = m->k_ex;
  M.sDD = m->sigma_DNA_DNA; M.sDC = m->sigma_DNA_Core; M.sCC = m->sigma_Core_Core;
  M.sTT = m->sigma_Tail_Tail; M.sTL = m->sigma_Tail_Linker; M.sTC = m->sigma_Tail_Core;
  M.a1 = m->a1; M.a2 = m->a2; M.dt = m->time_step; M.del = m->del; M.s2dt = m->s2dt;
  const int n = M.n, nc = M.n_c, nt = M.n_tail, nL = M.n_LH, np = M.n_lh_n + M.n_lh_g + M.n_lh_c;
  // host-side derived index arrays
  std::vector<int> core_rank(n), core_bead, dna_bead, lh_core_bead, core_lh(nc, -1), t_core_bead(nt, -1);
  {
    int cnt = 0;
    for (int i = 0; i < n; i++) {
      if (m->type[i] == 1) { cnt++; core_bead.push_back(i); } else dna_bead.push_back(i);
      core_rank[i] = cnt - 1;
    }
    for (int k = 0; k < nc; k++)
      if (m->nc_lh_flag && m->nc_lh_flag[k] == 1) { core_lh[k] = (int)lh_core_bead.size(); lh_core_bead.push_back(core_bead[k]); }
    for (int t = 0; t < nt; t++) {
      int grp = m->t_grp[t], k = (grp - 1) / 10;
      t_core_bead[t] = (k >= 0 && k < nc) ? core_bead[k] : -1;  // func.cpp:2366-2375
    }
  }
  M.n_dna = (int)dna_bead.size();
  M.n_lhcore = (int)lh_core_bead.size();
  c->h_type.assign(m->type, m->type + n);
  if (m->r_var) c->h_rvar.assign(m->r_var, m->r_var + 3 * (size_t)n);
  double qmax = 0, gmax = 0;
  for (int k = 0; k < M.Nq; k++) {
    const double* p = m->core_pos + 3 * k;
    qmax = fmax(qmax, sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]));
  }
  for (int k = 0; k < M.n_lh_g; k++) {
    const double* p = m->LH_g_pos + 3 * k;
    gmax = fmax(gmax, sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]));
  }
  M.qmax_core = qmax;
  M.gmax = gmax;
  std::vector<double> rad_all(M.n_D);
  for (int i = 0; i < n; i++) rad_all[i] = m->rad[i];
  for (int i = 0; i < nt; i++) rad_all[n + i] = m->t_rad[i];
  for (int i = 0; i < nL; i++) rad_all[n + nt + i] = m->lh_rad[i];
  // sizes.  Every buffer that depends on the linker-histone binding is sized
  // for every core bound (capacity), so that bd_set_lh_flags resizes the
  // context in place; the logical sizes (M.n_LH, M.n_D, c->m) follow the flags.
  c->m = 3 * M.n_D;
  const int nL_cap = M.nlh * nc, nD_cap = n + nt + nL_cap, m_cap = 3 * nD_cap;
  c->m_cap = m_cap;
  c->lda = (m_cap + 31) & ~31;
  const size_t ndna = M.n_dna, nlhc = M.n_lhcore;
  const size_t nlhc_cap = (M.nlh > 0 || M.n_lh_g > 0) ? (size_t)nc : nlhc;
  size_t ebuf = (size_t)8 * n + nt + nL;
  const size_t ebuf_cap = (size_t)8 * n + nt + nL_cap;
  size_t tot = 0;
  auto addD = [&](size_t k) { tot += slab<double>(k); };
  auto addI = [&](size_t k) { tot += slab<int>(k); };
  // model
  addI(n); addI(n); addI(nc); addI(ndna); addI(nlhc_cap); addI(nc); addD(n); addD(nD_cap); addD(3 * M.Nq); addD(M.Nq);
  addD(3 * M.n_t); addI(M.n_t); addI(nc); for (int q = 0; q < 5; q++) addD(nt); addI(nt + 2); addI(nt); addI(nt);
  addD(3 * M.n_lh_g); addI(np); addI(nc); for (int q = 0; q < 9; q++) addD(np);
  // two states
  for (int q = 0; q < 2; q++) {
    for (int k = 0; k < 4; k++) addD(3 * n);
    addD(3 * nt); addD(3 * (size_t)nL_cap);
    for (int k = 0; k < 4; k++) addD(n);
    for (int k = 0; k < 3; k++) addD(3 * nc);
    for (int k = 0; k < 3; k++) addD(nc);
    addD(nt); addD(nL_cap); addD(3 * nlhc_cap * M.n_lh_g);
  }
  for (int q = 0; q < 3; q++) { addD(3 * n); addD(3 * n); addD(3 * nt); addD(3 * (size_t)nL_cap); addD(1); }
  addD((size_t)nc * nc * 10); addD((size_t)kCCSplit * nc * nc * 10); addD(ndna * nc * 7); addD(nlhc_cap * nc * 10); addD(ebuf_cap);
  addD(3 * (size_t)nD_cap); addD(m_cap); addD(m_cap); addD(3 * n); addD(bdk::trmv_scratch_doubles(m_cap)); addD(1); addI(1);
  const int npos = n + nt + nL + (int)nlhc * M.n_lh_g;
  const int npos_cap = n + nt + nL_cap + (int)nlhc_cap * M.n_lh_g;
  addD((nt + 4 * (size_t)M.Nq + 1) / 2); addD(2 * (size_t)npos_cap); addD(2 * (size_t)npos_cap);
  for (int q = 0; q < 3; q++) addD(2 * (size_t)nD_cap);
  addD(4 * ((size_t)nt + nL_cap));
  addI(nL_cap);
  addD(37 * (size_t)n);
  e = cudaMalloc(&c->arena_base, tot);
  if (e != cudaSuccess) return fail(set_error(BD_ERR_NOMEM, "bd_create: device arena allocation failed"));
  if (c->precision != BD_PREC_MIXED && c->precision != BD_PREC_FP64)
    return fail(set_error(BD_ERR_ARG, "bd_create: unknown precision"));
  e = cudaMalloc((void**)&c->A, (size_t)m_cap * c->lda * sizeof(double));
  if (e != cudaSuccess) return fail(set_error(BD_ERR_NOMEM, "bd_create: tensor allocation failed"));
  if (c->precision == BD_PREC_MIXED) {
    if (bdk::set_mixed_attributes()) return fail(set_error(BD_ERR_CUDA, "bd_create: kernel attributes (shared memory)"));
    e = cudaMalloc((void**)&c->PS, bdk::mixed_panel_bytes(m_cap));
    if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_err, sizeof(int));
    if (e != cudaSuccess) return fail(set_error(BD_ERR_NOMEM, "bd_create: tensor allocation failed"));
    if (cudaMemset(c->d_err, 0, sizeof(int)) != cudaSuccess) return fail(set_error(BD_ERR_CUDA, "bd_create: memset failed"));
  }
  Arena ar{(char*)c->arena_base, tot, 0};
  int *d_type = ar.take<int>(n), *d_core_rank = ar.take<int>(n), *d_core_bead = ar.take<int>(nc),
      *d_dna_bead = ar.take<int>(ndna), *d_lhcb = ar.take<int>(nlhc_cap), *d_core_lh = ar.take<int>(nc);
  double *d_phi = ar.take<double>(n), *d_rad_all = ar.take<double>(nD_cap), *d_cpos = ar.take<double>(3 * M.Nq),
         *d_cq = ar.take<double>(M.Nq), *d_tpos = ar.take<double>(3 * M.n_t);
  int *d_tfix_tmpl = ar.take<int>(M.n_t), *d_nct = ar.take<int>(nc);
  double *d_ht = ar.take<double>(nt), *d_gt = ar.take<double>(nt), *d_lot = ar.take<double>(nt),
         *d_bot = ar.take<double>(nt), *d_tq = ar.take<double>(nt);
  int *d_tgrp = ar.take<int>(nt + 2), *d_tfix = ar.take<int>(nt), *d_tcb = ar.take<int>(nt);
  double* d_gpos0 = ar.take<double>(3 * M.n_lh_g);
  int *d_conn = ar.take<int>(np), *d_nclh = ar.take<int>(nc);
  double* d_lhp[9];
  for (int q = 0; q < 9; q++) d_lhp[q] = ar.take<double>(np);
  DevState* sts[2] = {&c->X, &c->Y};
  for (int q = 0; q < 2; q++) {
    DevState& D = *sts[q];
    D.r = ar.take<double>(3 * n); D.a = ar.take<double>(3 * n); D.b = ar.take<double>(3 * n); D.c = ar.take<double>(3 * n);
    D.r_t = ar.take<double>(3 * nt); D.r_lh = ar.take<double>(3 * (size_t)nL_cap);
    D.alpha = ar.take<double>(n); D.beta = ar.take<double>(n); D.gamma = ar.take<double>(n); D.length = ar.take<double>(n);
    D.a_dna = ar.take<double>(3 * nc); D.b_dna = ar.take<double>(3 * nc); D.c_dna = ar.take<double>(3 * nc);
    D.alpha_p = ar.take<double>(nc); D.beta_p = ar.take<double>(nc); D.gamma_p = ar.take<double>(nc);
    D.beta_t = ar.take<double>(nt); D.beta_lh = ar.take<double>(nL_cap);
    D.gpos = ar.take<double>(3 * nlhc_cap * M.n_lh_g);
  }
  DevForces* fs[3] = {&c->F0, &c->F1, &c->Fa};
  for (int q = 0; q < 3; q++) {
    fs[q]->F = ar.take<double>(3 * n); fs[q]->T = ar.take<double>(3 * n); fs[q]->tF = ar.take<double>(3 * nt);
    fs[q]->lF = ar.take<double>(3 * (size_t)nL_cap); fs[q]->E = ar.take<double>(1);
  }
  c->S.cc = ar.take<double>((size_t)nc * nc * 10);
  c->S.ccp = ar.take<double>((size_t)kCCSplit * nc * nc * 10);
  c->S.dc = ar.take<double>(ndna * nc * 7);
  c->S.gc = ar.take<double>(nlhc_cap * nc * 10);
  c->S.ebuf = ar.take<double>(ebuf_cap);
  c->S.nE = (int)ebuf;
  c->r_all = ar.take<double>(3 * (size_t)nD_cap);
  c->rd = ar.take<double>(m_cap);
  c->p = ar.take<double>(m_cap);
  c->rr = ar.take<double>(3 * n);
  c->rd_part = ar.take<double>(bdk::trmv_scratch_doubles(m_cap));
  c->energy = ar.take<double>(1);
  float* d_tqf = ar.take<float>(nt + 4 * (size_t)m->Nq);  // tail charges, core sites, core charges (FP32)
  c->S.ph = ar.take<float4>(npos_cap);
  c->S.pl = ar.take<float4>(npos_cap);
  c->S.qh = ar.take<float4>(nD_cap);
  c->S.ql = ar.take<float4>(nD_cap);
  c->S.qf = ar.take<float4>(nD_cap);
  c->S.bond = ar.take<double>(4 * ((size_t)nt + nL_cap));
  int* d_lhp_idx = ar.take<int>(nL_cap);
  c->S.bonds = ar.take<double>(37 * (size_t)n);
  c->S.ot = n; c->S.ol = n + nt; c->S.og = n + nt + nL; c->S.npos = npos;
  c->negpiv = ar.take<int>(1);
  cudaStream_t st = c->stream;
  std::vector<int> tgrp_pad(nt + 2, -1);
  for (int t = 0; t < nt; t++) tgrp_pad[t] = m->t_grp[t];
  if ((rc = up(d_type, m->type, n, st)) || (rc = up(d_core_rank, core_rank.data(), n, st)) ||
      (rc = up(d_core_bead, core_bead.data(), nc, st)) || (rc = up(d_dna_bead, dna_bead.data(), ndna, st)) ||
      (rc = up(d_lhcb, lh_core_bead.data(), nlhc, st)) || (rc = up(d_core_lh, core_lh.data(), nc, st)) ||
      (rc = up(d_phi, m->phi_o, n, st)) || (rc = up(d_rad_all, rad_all.data(), M.n_D, st)) ||
      (rc = up(d_cpos, m->core_pos, 3 * M.Nq, st)) || (rc = up(d_cq, m->core_q, M.Nq, st)) ||
      (rc = up(d_tpos, m->tail_pos, 3 * M.n_t, st)) || (rc = up(d_tfix_tmpl, m->tail_fix, M.n_t, st)) ||
      (rc = up(d_nct, m->nc_t_flag, nc, st)) || (rc = up(d_ht, m->h_t, nt, st)) || (rc = up(d_gt, m->g_t, nt, st)) ||
      (rc = up(d_lot, m->lo_t, nt, st)) || (rc = up(d_bot, m->beta_o_t, nt, st)) || (rc = up(d_tq, m->t_q, nt, st)) ||
      (rc = up(d_tgrp, tgrp_pad.data(), nt + 2, st)) || (rc = up(d_tfix, m->t_fix, nt, st)) ||
      (rc = up(d_tcb, t_core_bead.data(), nt, st)) || (rc = up(d_gpos0, m->LH_g_pos, 3 * M.n_lh_g, st)) ||
      (rc = up(d_conn, m->LH_conn, np, st)) || (rc = up(d_nclh, m->nc_lh_flag, nc, st)))
    return fail(rc);
  const double* lhsrc[9] = {m->LH_q, m->LH_vdw_hh, m->LH_vdw_hc, m->LH_vdw_hl, m->LH_vdw_ht,
                            m->LH_kstr, m->LH_kben, m->LH_streq, m->LH_betaeq};
  for (int q = 0; q < 9; q++)
    if ((rc = up(d_lhp[q], lhsrc[q], np, st))) return fail(rc);
  M.type = d_type; M.core_rank = d_core_rank; M.core_bead = d_core_bead; M.dna_bead = d_dna_bead;
  M.lh_core_bead = d_lhcb; M.core_lh = d_core_lh; M.phi_o = d_phi; M.rad_all = d_rad_all;
  M.core_pos = d_cpos; M.core_q = d_cq; M.tail_pos = d_tpos; M.tail_fix = d_tfix_tmpl; M.nc_t_flag = d_nct;
  M.h_t = d_ht; M.g_t = d_gt; M.lo_t = d_lot; M.beta_o_t = d_bot; M.t_q = d_tq; M.t_grp = d_tgrp; M.t_fix = d_tfix;
  M.t_core_bead = d_tcb; M.LH_g_pos = d_gpos0; M.LH_conn = d_conn; M.nc_lh_flag = d_nclh;
  M.LH_q = d_lhp[0]; M.LH_vdw_hh = d_lhp[1]; M.LH_vdw_hc = d_lhp[2]; M.LH_vdw_hl = d_lhp[3]; M.LH_vdw_ht = d_lhp[4];
  M.LH_kstr = d_lhp[5]; M.LH_kben = d_lhp[6]; M.LH_streq = d_lhp[7]; M.LH_betaeq = d_lhp[8];
  {
    const int nq = m->Nq;
    std::vector<float> tqf(nt + 4 * (size_t)nq);
    for (int t = 0; t < nt; t++) tqf[t] = (float)m->t_q[t];
    for (int k = 0; k < 3 * nq; k++) tqf[nt + k] = (float)m->core_pos[k];
    for (int k = 0; k < nq; k++) tqf[nt + 3 * nq + k] = (float)m->core_q[k];
    if (!tqf.empty() &&
        cudaMemcpyAsync(d_tqf, tqf.data(), tqf.size() * sizeof(float), cudaMemcpyHostToDevice, st) != cudaSuccess)
      return fail(set_error(BD_ERR_CUDA, "bd_create: upload failed"));
    if (!tqf.empty() && cudaStreamSynchronize(st) != cudaSuccess)
      return fail(set_error(BD_ERR_CUDA, "bd_create: upload failed"));
    std::vector<int> lhp(nL);
    for (int b = 0; b < nL; b++) {  // as the bead-type lookup of the FP64 path: position in the molecule
      const int idx = b % M.nlh;
      lhp[b] = idx < M.n_lh_n ? idx : idx + M.n_lh_g;
    }
    if (nL && (cudaMemcpyAsync(d_lhp_idx, lhp.data(), nL * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
               cudaStreamSynchronize(st) != cudaSuccess))
      return fail(set_error(BD_ERR_CUDA, "bd_create: upload failed"));
    M.lh_p = d_lhp_idx;
    M.t_qf = d_tqf;
    M.core_pf = d_tqf + nt;
    M.core_qf = d_tqf + nt + 3 * nq;
    M.tails_by_core = M.n_t > 0;
    for (int t = 0; t < nt && M.tails_by_core; t++)
      if (t_core_bead[t] != -1 && (t / M.n_t >= nc || t_core_bead[t] != core_bead[t / M.n_t])) M.tails_by_core = 0;
  }
  if ((nL > 0 || nlhc > 0) && np > 64) return fail(set_error(BD_ERR_ARG, "bd_create: more than 64 LH bead types"));
  // state
  if ((rc = up(c->X.r, s->r, 3 * n, st)) || (rc = up(c->X.a, s->a, 3 * n, st)) || (rc = up(c->X.b, s->b, 3 * n, st)) ||
      (rc = up(c->X.c, s->c, 3 * n, st)) || (rc = up(c->X.r_t, s->r_t, 3 * nt, st)) ||
      (rc = up(c->X.r_lh, s->r_lh, 3 * nL, st)))
    return fail(rc);
  // angle slots the reference never writes (the last bead's) read as zero
  for (DevState* D : {&c->X, &c->Y})
    if (cudaMemsetAsync(D->alpha, 0, n * sizeof(double), st) != cudaSuccess ||
        cudaMemsetAsync(D->beta, 0, n * sizeof(double), st) != cudaSuccess ||
        cudaMemsetAsync(D->gamma, 0, n * sizeof(double), st) != cudaSuccess ||
        cudaMemsetAsync(D->length, 0, n * sizeof(double), st) != cudaSuccess)
      return fail(set_error(BD_ERR_CUDA, "bd_create: memset failed"));
  if (cudaMemsetAsync(c->X.alpha_p, 0, nc * sizeof(double), st) != cudaSuccess ||
      cudaMemsetAsync(c->X.gamma_p, 0, nc * sizeof(double), st) != cudaSuccess ||
      cudaMemsetAsync(c->Y.alpha_p, 0, nc * sizeof(double), st) != cudaSuccess ||
      cudaMemsetAsync(c->Y.gamma_p, 0, nc * sizeof(double), st) != cudaSuccess ||
      cudaMemsetAsync(c->negpiv, 0, sizeof(int), st) != cudaSuccess)
    return fail(set_error(BD_ERR_CUDA, "bd_create: memset failed"));
  bdk::frames(M, c->X, st);   // also the tail and LH bend angles
  if (!s->refresh_frames) {
    // keep the caller's frames and angles (cuda_application_init_data form)
    if ((rc = up(c->X.a, s->a, 3 * n, st)) || (rc = up(c->X.b, s->b, 3 * n, st)) || (rc = up(c->X.c, s->c, 3 * n, st)) ||
        (rc = up(c->X.alpha, s->alpha, n, st)) || (rc = up(c->X.beta, s->beta, n, st)) ||
        (rc = up(c->X.gamma, s->gamma, n, st)) || (rc = up(c->X.length, s->length, n, st)) ||
        (rc = up(c->X.a_dna, s->a_dna, 3 * nc, st)) || (rc = up(c->X.b_dna, s->b_dna, 3 * nc, st)) ||
        (rc = up(c->X.c_dna, s->c_dna, 3 * nc, st)) || (rc = up(c->X.alpha_p, s->alpha_p, nc, st)) ||
        (rc = up(c->X.beta_p, s->beta_p, nc, st)) || (rc = up(c->X.gamma_p, s->gamma_p, nc, st)))
      return fail(rc);
  }
  for (int k = 0; k < 10; k++) cudaEventCreate(&c->ev[k]);
  if (c->precision == BD_PREC_MIXED) {
    c->kev.resize(2 * (size_t)bdk::mixed_max_launches(c->m_cap));
    for (auto& ev : c->kev) cudaEventCreate(&ev);
  }
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(set_error(BD_ERR_CUDA, (std::string("bd_create: ") + cudaGetErrorString(e)).c_str()));
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(set_error(BD_ERR_CUDA, (std::string("bd_create: ") + cudaGetErrorString(e)).c_str()));
  *out = c;
  return BD_OK;
}

extern "C" int bd_destroy(bd_ctx* c) {
  if (!c) return BD_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->graph) cudaGraphExecDestroy(c->graph);
  bdh::adj_free(c->adj);
  for (int k = 0; k < 10; k++)
    if (c->ev[k]) cudaEventDestroy(c->ev[k]);
  for (auto ev : c->kev) cudaEventDestroy(ev);
  if (c->A) cudaFree(c->A);
  if (c->PS) cudaFree(c->PS);
  if (c->d_err) cudaFree(c->d_err);
  c->kgraphs.clear();
  if (c->kscratch) cudaFree(c->kscratch);
  if (c->arena_base) cudaFree(c->arena_base);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return BD_OK;
}

extern "C" int bd_sizes(const bd_ctx* c, int* o) {
  if (!c || !o) return set_error(BD_ERR_ARG, "bd_sizes: null argument");
  o[0] = c->M.n; o[1] = c->M.n_c; o[2] = c->M.n_tail; o[3] = c->M.n_LH; o[4] = c->M.n_D; o[5] = c->m; o[6] = c->lda;
  o[7] = c->precision;
  return BD_OK;
}

static int run_step(bd_ctx* c, const double* d_rr, const double* d_p) {
  int rc;
  if (c->use_graph && d_rr == c->rr && d_p == c->p && c->freq_rp == 1 && c->noise_mode == BD_NOISE_CHOLESKY) {
    if (!c->graph) {
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      bool t = c->timing;
      c->timing = false;
      rc = step_device(c, d_rr, d_p);
      c->timing = t;
      cudaError_t e = cudaStreamEndCapture(c->stream, &g);
      if (rc) return rc;
      if (e != cudaSuccess) return set_error(BD_ERR_CUDA, "bd_step: graph capture failed");
      e = cudaGraphInstantiate(&c->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return set_error(BD_ERR_CUDA, "bd_step: graph instantiation failed");
    }
    CK(cudaGraphLaunch(c->graph, c->stream));
  } else {
    if ((rc = step_device(c, d_rr, d_p))) return rc;
  }
  c->step_count++;
  return BD_OK;
}

extern "C" int bd_step_device(bd_ctx* c, const double* d_rr, const double* d_p, double* d_energy) {
  if (!c || !d_rr || !d_p) return set_error(BD_ERR_ARG, "bd_step_device: null argument");
  // stage the noise into the context's buffers so a captured graph can replay
  if (d_rr != c->rr)
    CK(cudaMemcpyAsync(c->rr, d_rr, 3 * (size_t)c->M.n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  if (d_p != c->p) CK(cudaMemcpyAsync(c->p, d_p, (size_t)c->m * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  int rc = run_step(c, c->rr, c->p);
  if (rc) return rc;
  if (d_energy) CK(cudaMemcpyAsync(d_energy, c->F0.E, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  return BD_OK;
}

extern "C" int bd_step(bd_ctx* c, const double* rr, const double* p, double* energy) {
  if (!c || !rr || !p) return set_error(BD_ERR_ARG, "bd_step: null argument");
  // host noise is checked before anything is launched: a NaN or Inf would
  // otherwise reach the positions and only show in the next step's energy
  for (size_t i = 0, n = 3 * (size_t)c->M.n; i < n; i++)
    if (!std::isfinite(rr[i])) return set_error(BD_ERR_NONFINITE, "bd_step: non-finite rotational noise");
  for (size_t i = 0; i < (size_t)c->m; i++)
    if (!std::isfinite(p[i])) return set_error(BD_ERR_NONFINITE, "bd_step: non-finite translational noise");
  CK(cudaMemcpyAsync(c->rr, rr, 3 * (size_t)c->M.n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->p, p, (size_t)c->m * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  int rc = run_step(c, c->rr, c->p);
  if (rc) return rc;
  double e = 0.0;
  int derr = 0;
  CK(cudaMemcpyAsync(&e, c->F0.E, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (c->d_err) CK(cudaMemcpyAsync(&derr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (derr) return set_error(BD_ERR_CUDA, "bd_step: a tensor-core kernel timed out waiting on its copies/MMAs");
  if (!std::isfinite(e)) return set_error(BD_ERR_NONFINITE, "bd_step: non-finite energy");
  if (energy) *energy = e;
  return BD_OK;
}

extern "C" int bd_step_reference(bd_ctx* c, int step, int number_of_steps, int freq, const double* rr, const double* p,
                                 double* energy, double* h_r, double* h_a, double* h_b, double* h_c, double* h_r_t,
                                 double* h_r_lh) {
  int rc = bd_step(c, rr, p, energy);
  if (rc) return rc;
  cudaStream_t st = c->stream;
  size_t n3 = 3 * (size_t)c->M.n;
  if (h_r_lh && c->M.n_LH) CK(cudaMemcpyAsync(h_r_lh, c->X.r_lh, 3 * (size_t)c->M.n_LH * sizeof(double), cudaMemcpyDeviceToHost, st));
  if ((freq > 0 && step % freq == 0) || step == number_of_steps - 1) {
    if (h_r) CK(cudaMemcpyAsync(h_r, c->X.r, n3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (h_a) CK(cudaMemcpyAsync(h_a, c->X.a, n3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (h_b) CK(cudaMemcpyAsync(h_b, c->X.b, n3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (h_c) CK(cudaMemcpyAsync(h_c, c->X.c, n3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (h_r_t && c->M.n_tail) CK(cudaMemcpyAsync(h_r_t, c->X.r_t, 3 * (size_t)c->M.n_tail * sizeof(double), cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  return BD_OK;
}

extern "C" int bd_forces(bd_ctx* c, double* F, double* T, double* tF, double* lF, double* E) {
  if (!c) return set_error(BD_ERR_ARG, "bd_forces: null context");
  bdk::forces(c->M, c->X, c->F0, c->S, c->precision, c->stream);
  CK(cudaGetLastError());
  cudaStream_t st = c->stream;
  size_t n3 = 3 * (size_t)c->M.n;
  if (F) CK(cudaMemcpyAsync(F, c->F0.F, n3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (T) CK(cudaMemcpyAsync(T, c->F0.T, n3 * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (tF && c->M.n_tail) CK(cudaMemcpyAsync(tF, c->F0.tF, 3 * (size_t)c->M.n_tail * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (lF && c->M.n_LH) CK(cudaMemcpyAsync(lF, c->F0.lF, 3 * (size_t)c->M.n_LH * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (E) CK(cudaMemcpyAsync(E, c->F0.E, sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return BD_OK;
}

static int copy_lower(bd_ctx* c, double* out, bool mirror) {
  const int lda = c->lda;
  std::vector<double> h((size_t)c->m * lda);
  CK(cudaMemcpyAsync(h.data(), c->A, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  const int m = c->m;
  if (c->precision == BD_PREC_MIXED) {  // double-float pairs (hi, lo) -> FP64
    for (size_t e = 0; e < h.size(); e++) {
      float f[2];
      std::memcpy(f, &h[e], sizeof f);
      h[e] = (double)f[0] + (double)f[1];
    }
  }
  for (int i = 0; i < m; i++)
    for (int j = 0; j < m; j++) {
      double v;
      if (i >= j) v = h[(size_t)j * lda + i];
      else v = mirror ? h[(size_t)i * lda + j] : 0.0;
      out[(size_t)i * m + j] = v;
    }
  return BD_OK;
}

static void assemble_now(bd_ctx* c) {
  const bool mixed = c->precision == BD_PREC_MIXED;
  c->a_holds_factor = false;
  bdk::gather_rall(c->M, c->X, c->r_all, mixed ? &c->S : nullptr, c->stream);
  bdk::rpy_assemble(c->M.n_D, c->r_all, c->M.rad_all, c->M.a1, c->M.a2, c->A, c->lda, c->stream,
                    mixed ? c->S.qh : nullptr, mixed ? c->S.ql : nullptr);
}

extern "C" int bd_diffusion_tensor(bd_ctx* c, double* D) {
  if (!c || !D) return set_error(BD_ERR_ARG, "bd_diffusion_tensor: null argument");
  assemble_now(c);
  CK(cudaGetLastError());
  return copy_lower(c, D, true);
}

static int factor_now(bd_ctx* c) {
  assemble_now(c);
  c->a_holds_factor = true;
  CK(cudaMemsetAsync(c->negpiv, 0, sizeof(int), c->stream));
  if (c->precision == BD_PREC_MIXED) {
    bdk::potrf_mixed(c->m, c->A, c->lda, c->PS, c->negpiv, c->d_err, c->stream, nullptr, nullptr, nullptr, nullptr,
                     c->mixed_passes);
    int derr = 0;
    CK(cudaMemcpyAsync(&derr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (derr) return set_error(BD_ERR_CUDA, "factor: a tensor-core kernel timed out");
  } else {
    bdk::potrf_fp64(c->m, c->A, c->lda, nullptr, nullptr, 0.0, c->negpiv, c->stream);
  }
  CK(cudaGetLastError());
  return BD_OK;
}

extern "C" int bd_cholesky(bd_ctx* c, double* L) {
  if (!c || !L) return set_error(BD_ERR_ARG, "bd_cholesky: null argument");
  int rc = factor_now(c);
  if (rc) return rc;
  return copy_lower(c, L, false);
}

extern "C" int bd_noise_displacement(bd_ctx* c, const double* p, double* rd) {
  if (!c || !p || !rd) return set_error(BD_ERR_ARG, "bd_noise_displacement: null argument");
  const bool mixed = c->precision == BD_PREC_MIXED;
  if (c->noise_mode == BD_NOISE_KRYLOV) {
    assemble_now(c);
    CK(cudaMemcpyAsync(c->p, p, (size_t)c->m * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    int rc = bdk::krylov_sqrt(c->m, mixed ? nullptr : c->A, c->lda, mixed, c->S.qh, c->S.ql, c->M.a1, c->M.a2, c->p,
                              c->M.s2dt, c->krylov_tol, c->krylov_kmax, c->rd, c->kscratch, c->stream,
                              &c->krylov_iters, &c->krylov_change, &c->kgraphs);
    if (rc) return set_error(rc, "bd_noise_displacement: Krylov iteration failed");
  } else {
    int rc = factor_now(c);
    if (rc) return rc;
    CK(cudaMemcpyAsync(c->p, p, (size_t)c->m * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    bdk::trmv_lower_ws(c->m, c->A, c->lda, c->p, c->M.s2dt, c->rd, c->rd_part, c->stream, mixed);
  }
  CK(cudaMemcpyAsync(rd, c->rd, (size_t)c->m * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return BD_OK;
}

static double* state_field(bd_ctx* c, const char* nm, int* cnt) {
  DevState& X = c->X;
  const int n = c->M.n, nc = c->M.n_c, nt = c->M.n_tail, nL = c->M.n_LH;
  struct F { const char* k; double* p; int n; } tab[] = {
      {"r", X.r, 3 * n}, {"a", X.a, 3 * n}, {"b", X.b, 3 * n}, {"c", X.c, 3 * n}, {"r_t", X.r_t, 3 * nt},
      {"r_lh", X.r_lh, 3 * nL}, {"alpha", X.alpha, n}, {"beta", X.beta, n}, {"gamma", X.gamma, n},
      {"length", X.length, n}, {"a_dna", X.a_dna, 3 * nc}, {"b_dna", X.b_dna, 3 * nc}, {"c_dna", X.c_dna, 3 * nc},
      {"alpha_p", X.alpha_p, nc}, {"beta_p", X.beta_p, nc}, {"gamma_p", X.gamma_p, nc}, {"beta_t", X.beta_t, nt},
      {"beta_lh", X.beta_lh, nL}, {"rd", c->rd, c->m}, {"force", c->F0.F, 3 * n}, {"torque", c->F0.T, 3 * n},
      {"t_force", c->F0.tF, 3 * nt}, {"LH_force", c->F0.lF, 3 * nL}};
  for (auto& f : tab)
    if (!strcmp(f.k, nm)) { *cnt = f.n; return f.p; }
  return nullptr;
}

extern "C" int bd_get_state(bd_ctx* c, const char* name, double* out, int* count) {
  if (!c || !name) return set_error(BD_ERR_ARG, "bd_get_state: null argument");
  int cnt = 0;
  double* p = state_field(c, name, &cnt);
  if (!p) return set_error(BD_ERR_ARG, "bd_get_state: unknown name");
  if (count) *count = cnt;
  if (out && cnt) {
    CK(cudaMemcpyAsync(out, p, cnt * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return BD_OK;
}

extern "C" int bd_set_state(bd_ctx* c, const char* name, const double* in) {
  if (!c || !name || !in) return set_error(BD_ERR_ARG, "bd_set_state: null argument");
  static const char* ok[] = {"r", "a", "b", "c", "r_t", "r_lh"};
  bool allowed = false;
  for (auto k : ok) allowed |= !strcmp(k, name);
  if (!allowed) return set_error(BD_ERR_ARG, "bd_set_state: only r a b c r_t r_lh can be set");
  int cnt = 0;
  double* p = state_field(c, name, &cnt);
  if (cnt) CK(cudaMemcpyAsync(p, in, cnt * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  bdk::frames(c->M, c->X, c->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->stream));
  return BD_OK;
}

extern "C" int bd_dev_rpy(bd_ctx* c, int nb, const double* d_r, const double* d_rad, double a1, double a2, double* d_D,
                          int lda) {
  if (!c || !d_r || !d_rad || !d_D || nb <= 0 || lda < 3 * nb) return set_error(BD_ERR_ARG, "bd_dev_rpy: bad argument");
  bdk::rpy_assemble(nb, d_r, d_rad, a1, a2, d_D, lda, c->stream);
  CK(cudaGetLastError());
  return BD_OK;
}

extern "C" int bd_dev_potrf(bd_ctx* c, int m, double* d_A, int lda, int precision, int* d_info) {
  if (!c || !d_A || m <= 0 || lda < m || !d_info) return set_error(BD_ERR_ARG, "bd_dev_potrf: bad argument");
  if (precision != BD_PREC_FP64) return set_error(BD_ERR_ARG, "bd_dev_potrf: only BD_PREC_FP64 is available");
  bdk::potrf_fp64(m, d_A, lda, nullptr, nullptr, 0.0, d_info, c->stream);
  CK(cudaGetLastError());
  return BD_OK;
}

extern "C" int bd_phase_times(bd_ctx* c, float* out9) {
  if (!c || !out9) return set_error(BD_ERR_ARG, "bd_phase_times: null argument");
  if (!c->timing) {
    c->timing = true;  // enabled from the next step on
    for (int k = 0; k < 9; k++) out9[k] = 0.f;
    return BD_OK;
  }
  CK(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < 8; k++) cudaEventElapsedTime(&out9[k], c->ev[k], c->ev[k + 1]);
  cudaEventElapsedTime(&out9[8], c->ev[0], c->ev[8]);
  return BD_OK;
}

extern "C" int bd_kernel_bytes(bd_ctx* c, double* bytes) {
  if (!c || !bytes) return set_error(BD_ERR_ARG, "bd_kernel_bytes: null argument");
  *bytes = c->kbytes;
  return BD_OK;
}

extern "C" int bd_kernel_times(bd_ctx* c, float* out_ms, int max, int* launches) {
  if (!c || !launches || (max > 0 && !out_ms)) return set_error(BD_ERR_ARG, "bd_kernel_times: bad argument");
  *launches = 0;
  if (c->precision != BD_PREC_MIXED || !c->timing) return BD_OK;
  CK(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < c->kev_pairs; k++) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->kev[2 * k], c->kev[2 * k + 1]) != cudaSuccess) ms = -1.f;
    if (*launches < max) out_ms[*launches] = ms;
    (*launches)++;
  }
  return BD_OK;
}

extern "C" int bd_kernel_time(bd_ctx* c, float* total_ms, int* launches, double* tensor_flop) {
  if (!c || !total_ms || !launches) return set_error(BD_ERR_ARG, "bd_kernel_time: null argument");
  *total_ms = 0.f;
  *launches = 0;
  if (tensor_flop) *tensor_flop = c->kflop;
  if (c->precision != BD_PREC_MIXED || !c->timing) return BD_OK;
  CK(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < c->kev_pairs; k++) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->kev[2 * k], c->kev[2 * k + 1]) == cudaSuccess) {
      *total_ms += ms;
      (*launches)++;
    }
  }
  return BD_OK;
}

extern "C" int bd_launch_count(bd_ctx* c, int* out) {
  if (!c || !out) return set_error(BD_ERR_ARG, "bd_launch_count: null argument");
  *out = c->last_launches;
  return BD_OK;
}

extern "C" int bd_negative_pivots(bd_ctx* c, int* out) {
  if (!c || !out) return set_error(BD_ERR_ARG, "bd_negative_pivots: null argument");
  CK(cudaMemcpyAsync(&c->host_negpiv, c->negpiv, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  *out = c->host_negpiv;
  return BD_OK;
}

// ------------------------------------------------------------ batches
struct bd_batch {
  std::vector<bd_ctx*> ctx;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int use_graph = 0;
  cudaGraphExec_t graph = nullptr;
  std::vector<bd_noise*> noise;
  std::vector<std::vector<double>> h_rr, h_p;
  bdk::NoiseBatch* dnoise = nullptr;  // bd_batch_run_device: every replica's device noise stream
  bdk::MixedBatch* chol = nullptr;  // the replicas' factorisations as one launch per schedule step
  // side streams: the replicas' position / tensor and move phases run on
  // kBatchLanes streams side by side (no tensor-core kernel among them)
  std::vector<cudaStream_t> lane;
  std::vector<cudaEvent_t> ev;  // [0]: fork, [1 + k]: join of lane k
  // phase timing (bd_batch_phase_times): while on, steps run eagerly with
  // events around the three phases of a batched mixed step
  bool timing = false, timed = false;
  cudaEvent_t tev[4] = {nullptr, nullptr, nullptr, nullptr};
  int launches = 0;  // kernel launches of the last batch step enqueued
};

#ifndef BD_BATCH_LANES
#define BD_BATCH_LANES 64
#endif
constexpr int kBatchLanes = BD_BATCH_LANES;

// One step of every replica.  Mixed precision, D rebuilt every step: the
// positions and tensors of all replicas, then one batched factorisation
// (bdk::mixed_batch_run: launch i carries step i of every replica's
// schedule), then the rest of every replica's step.  Otherwise the replicas'
// steps run one after another.
static bool batch_together(const bd_batch* b) {
  bool together = true;
  for (bd_ctx* c : b->ctx) together = together && c->precision == BD_PREC_MIXED && c->freq_rp == 1;
  return together;
}

// the batched factorisation's plan (allocates and copies: never inside a
// stream capture)
static int batch_prepare(bd_batch* b) {
  if (batch_together(b) && !b->chol) {
    const size_t nr = b->ctx.size();
    std::vector<int> m(nr), lda(nr);
    std::vector<double*> A(nr);
    std::vector<unsigned char*> PS(nr);
    std::vector<int*> np(nr), er(nr);
    for (size_t i = 0; i < nr; i++) {
      bd_ctx* c = b->ctx[i];
      m[i] = c->m, lda[i] = c->lda, A[i] = c->A, PS[i] = c->PS, np[i] = c->negpiv, er[i] = c->d_err;
    }
    b->chol = bdk::mixed_batch_create((int)nr, m.data(), A.data(), lda.data(), PS.data(), np.data(), er.data(),
                                      b->ctx[0]->mixed_passes);
    if (!b->chol) return set_error(BD_ERR_NOMEM, "bd_batch: batched factorisation plan");
    if (b->lane.empty()) {  // kept when the plan is rebuilt (bd_batch_set_mixed_passes)
      const int nl = (int)std::min<size_t>(nr, kBatchLanes);
      b->lane.resize(nl, nullptr);
      b->ev.resize(1 + nl, nullptr);
      for (auto& s : b->lane) CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
      for (auto& e : b->ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
  }
  return BD_OK;
}

// run phase `ph` of every replica on the side streams, between a fork from
// and a join back into the batch stream
static int batch_lanes(bd_batch* b, int ph) {
  const int nl = (int)b->lane.size();
  CK(cudaEventRecord(b->ev[0], b->stream));
  for (int k = 0; k < nl; k++) CK(cudaStreamWaitEvent(b->lane[k], b->ev[0], 0));
  int rc = BD_OK;
  for (size_t i = 0; i < b->ctx.size() && !rc; i++) {
    bd_ctx* c = b->ctx[i];
    c->stream = b->lane[i % nl];
    rc = step_phases(c, c->rr, c->p, nullptr, ph);
    c->stream = b->stream;
    b->launches += c->last_launches;
  }
  for (int k = 0; k < nl; k++) {
    CK(cudaEventRecord(b->ev[1 + k], b->lane[k]));
    CK(cudaStreamWaitEvent(b->stream, b->ev[1 + k], 0));
  }
  return rc;
}

static int batch_enqueue(bd_batch* b) {
  int rc = BD_OK;
  b->launches = 0;
  if (!b->chol) {
    for (bd_ctx* c : b->ctx) {
      if (!rc) rc = step_device(c, c->rr, c->p);
      b->launches += c->last_launches;
    }
    return rc;
  }
  const bool ev = b->timing;
  if (ev) CK(cudaEventRecord(b->tev[0], b->stream));
  if ((rc = batch_lanes(b, kPre))) return rc;
  if (ev) CK(cudaEventRecord(b->tev[1], b->stream));
  {
    bdh::Range range("bd_batch: factorisations");
    b->launches += bdk::mixed_batch_run(b->chol, b->stream);  // alone on the GPU: the only tensor-core kernel of the step
  }
  CK(cudaGetLastError());
  if (ev) CK(cudaEventRecord(b->tev[2], b->stream));
  rc = batch_lanes(b, kPost);
  if (ev && !rc) {
    CK(cudaEventRecord(b->tev[3], b->stream));
    b->timed = true;
  }
  return rc;
}

static int batch_device_step(bd_batch* b) {
  int prc = batch_prepare(b);
  if (prc) return prc;
  bool graph_ok = b->use_graph && !b->timing;
  for (bd_ctx* c : b->ctx) graph_ok = graph_ok && c->freq_rp == 1;
  if (graph_ok) {
    if (!b->graph) {
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      int rc = batch_enqueue(b);
      cudaError_t e = cudaStreamEndCapture(b->stream, &g);
      if (rc) return rc;
      if (e != cudaSuccess) return set_error(BD_ERR_CUDA, "bd_batch: graph capture failed");
      e = cudaGraphInstantiate(&b->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return set_error(BD_ERR_CUDA, "bd_batch: graph instantiation failed");
    }
    CK(cudaGraphLaunch(b->graph, b->stream));
  } else {
    int rc = batch_enqueue(b);
    if (rc) return rc;
  }
  for (bd_ctx* c : b->ctx) c->step_count++;
  return BD_OK;
}

extern "C" int bd_batch_create(int nrep, const bd_model* models, const bd_state* states, const bd_options* opt,
                               bd_batch** out) {
  if (nrep <= 0 || !models || !states || !out) return set_error(BD_ERR_ARG, "bd_batch_create: bad argument");
  bd_batch* b = new bd_batch();
  bd_options o{};
  if (opt) o = *opt;
  else o.precision = BD_PREC_FP64, o.frequency_RP = 1;
  if (cudaSetDevice(o.device) != cudaSuccess) {
    delete b;
    return set_error(BD_ERR_CUDA, "bd_batch_create: cudaSetDevice failed");
  }
  b->stream = static_cast<cudaStream_t>(o.stream);
  if (!b->stream) {
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete b;
      return set_error(BD_ERR_CUDA, "bd_batch_create: stream creation failed");
    }
    b->own_stream = true;
  }
  b->use_graph = o.use_graph;
  o.stream = b->stream;
  o.use_graph = 0;  // the batch captures one graph for all replicas
  for (int i = 0; i < nrep; i++) {
    bd_ctx* c = nullptr;
    int rc = bd_create(&models[i], &states[i], &o, &c);
    if (rc) {
      bd_batch_destroy(b);
      return rc;
    }
    c->in_batch = true;
    b->ctx.push_back(c);
  }
  *out = b;
  return BD_OK;
}

extern "C" int bd_batch_destroy(bd_batch* b) {
  if (!b) return BD_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  bdk::mixed_batch_free(b->chol);
  for (auto s : b->lane)
    if (s) cudaStreamDestroy(s);
  for (auto e : b->ev)
    if (e) cudaEventDestroy(e);
  for (auto e : b->tev)
    if (e) cudaEventDestroy(e);
  for (bd_ctx* c : b->ctx) bd_destroy(c);
  for (bd_noise* g : b->noise) bd_noise_free(g);
  bdk::noise_batch_free(b->dnoise);
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return BD_OK;
}

extern "C" int bd_batch_size(const bd_batch* b, int* nrep) {
  if (!b || !nrep) return set_error(BD_ERR_ARG, "bd_batch_size: null argument");
  *nrep = (int)b->ctx.size();
  return BD_OK;
}

extern "C" int bd_set_noise_mode(bd_ctx* c, int mode, double tol, int kmax) {
  if (!c || (mode != BD_NOISE_CHOLESKY && mode != BD_NOISE_KRYLOV) ||
      (mode == BD_NOISE_KRYLOV && (!(tol > 0.0) || kmax < 2 || kmax > 512)))
    return set_error(BD_ERR_ARG, "bd_set_noise_mode: mode 0 or 1; Krylov: tol > 0, 2 <= kmax <= 512");
  if (c->in_batch) return set_error(BD_ERR_STATE, "bd_set_noise_mode: the context belongs to a batch");
  CK(cudaStreamSynchronize(c->stream));
  if (c->graph) cudaGraphExecDestroy(c->graph), c->graph = nullptr;
  if (mode == BD_NOISE_KRYLOV && (!c->kscratch || kmax > c->krylov_kmax)) {
    c->kgraphs.clear();
    if (c->kscratch) cudaFree(c->kscratch), c->kscratch = nullptr;
    if (cudaMalloc((void**)&c->kscratch, bdk::krylov_scratch_doubles(c->m_cap, kmax) * sizeof(double)) != cudaSuccess)
      return set_error(BD_ERR_NOMEM, "bd_set_noise_mode: Krylov workspace allocation failed");
  }
  c->noise_mode = mode;
  if (mode == BD_NOISE_KRYLOV) c->krylov_tol = tol, c->krylov_kmax = kmax;
  return BD_OK;
}

extern "C" int bd_krylov_stats(const bd_ctx* c, int* iters, double* change) {
  if (!c || !iters || !change) return set_error(BD_ERR_ARG, "bd_krylov_stats: null argument");
  *iters = c->krylov_iters;
  *change = c->krylov_change;
  return BD_OK;
}

extern "C" int bd_set_mixed_passes(bd_ctx* c, int passes) {
  if (!c || passes < 1 || passes > 3) return set_error(BD_ERR_ARG, "bd_set_mixed_passes: passes is 1, 2 or 3");
  if (c->in_batch) return set_error(BD_ERR_STATE, "bd_set_mixed_passes: the context belongs to a batch");
  if (c->mixed_passes != passes && c->graph) {
    CK(cudaStreamSynchronize(c->stream));
    cudaGraphExecDestroy(c->graph);  // the captured step holds the old schedule
    c->graph = nullptr;
  }
  c->mixed_passes = passes;
  return BD_OK;
}

extern "C" int bd_batch_set_mixed_passes(bd_batch* b, int passes) {
  if (!b || passes < 1 || passes > 3) return set_error(BD_ERR_ARG, "bd_batch_set_mixed_passes: passes is 1, 2 or 3");
  CK(cudaStreamSynchronize(b->stream));
  if (b->graph) cudaGraphExecDestroy(b->graph), b->graph = nullptr;
  bdk::mixed_batch_free(b->chol);  // the plan is built again at the next step
  b->chol = nullptr;
  for (bd_ctx* c : b->ctx) c->mixed_passes = passes;
  return BD_OK;
}

extern "C" int bd_batch_launch_count(const bd_batch* b, int* out) {
  if (!b || !out) return set_error(BD_ERR_ARG, "bd_batch_launch_count: null argument");
  *out = b->launches;
  return BD_OK;
}

extern "C" int bd_batch_phase_times(bd_batch* b, float* out3) {
  if (!b || !out3) return set_error(BD_ERR_ARG, "bd_batch_phase_times: null argument");
  for (int k = 0; k < 3; k++) out3[k] = 0.f;
  if (!b->timing) {
    for (auto& e : b->tev)
      if (!e) CK(cudaEventCreate(&e));
    b->timing = true;
    b->timed = false;
    return BD_OK;
  }
  if (!b->timed) return BD_OK;
  CK(cudaEventSynchronize(b->tev[3]));
  for (int k = 0; k < 3; k++) CK(cudaEventElapsedTime(&out3[k], b->tev[k], b->tev[k + 1]));
  return BD_OK;
}

extern "C" int bd_batch_context(bd_batch* b, int i, bd_ctx** out) {
  if (!b || !out || i < 0 || i >= (int)b->ctx.size()) return set_error(BD_ERR_ARG, "bd_batch_context: bad argument");
  *out = b->ctx[i];
  return BD_OK;
}

static int batch_finish(bd_batch* b, double* energies) {
  const int nr = (int)b->ctx.size();
  std::vector<double> e(nr, 0.0);
  std::vector<int> derr(nr, 0);
  for (int i = 0; i < nr; i++) {
    bd_ctx* c = b->ctx[i];
    CK(cudaMemcpyAsync(&e[i], c->F0.E, sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    if (c->d_err) CK(cudaMemcpyAsync(&derr[i], c->d_err, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  }
  CK(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < nr; i++) {
    if (derr[i]) return set_error(BD_ERR_CUDA, "bd_batch: a tensor-core kernel timed out");
    if (!std::isfinite(e[i])) return set_error(BD_ERR_NONFINITE, "bd_batch: non-finite energy");
    if (energies) energies[i] = e[i];
  }
  return BD_OK;
}

extern "C" int bd_batch_step(bd_batch* b, const double* const* rr, const double* const* p, double* energies) {
  if (!b || !rr || !p) return set_error(BD_ERR_ARG, "bd_batch_step: null argument");
  for (size_t i = 0; i < b->ctx.size(); i++) {
    bd_ctx* c = b->ctx[i];
    if (!rr[i] || !p[i]) return set_error(BD_ERR_ARG, "bd_batch_step: null noise pointer");
    CK(cudaMemcpyAsync(c->rr, rr[i], 3 * (size_t)c->M.n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    CK(cudaMemcpyAsync(c->p, p[i], (size_t)c->m * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  }
  int rc = batch_device_step(b);
  if (rc) return rc;
  return batch_finish(b, energies);
}

extern "C" int bd_batch_step_device(bd_batch* b, const double* const* d_rr, const double* const* d_p) {
  if (!b || !d_rr || !d_p) return set_error(BD_ERR_ARG, "bd_batch_step_device: null argument");
  for (size_t i = 0; i < b->ctx.size(); i++) {
    bd_ctx* c = b->ctx[i];
    if (!d_rr[i] || !d_p[i]) return set_error(BD_ERR_ARG, "bd_batch_step_device: null noise pointer");
    if (d_rr[i] != c->rr)
      CK(cudaMemcpyAsync(c->rr, d_rr[i], 3 * (size_t)c->M.n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
    if (d_p[i] != c->p)
      CK(cudaMemcpyAsync(c->p, d_p[i], (size_t)c->m * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  }
  return batch_device_step(b);
}

extern "C" int bd_batch_run(bd_batch* b, int nsteps, unsigned long seed_base, double* energies) {
  if (!b || nsteps < 0) return set_error(BD_ERR_ARG, "bd_batch_run: bad argument");
  const size_t nr = b->ctx.size();
  if (b->noise.empty()) {
    b->noise.resize(nr, nullptr);
    b->h_rr.resize(nr);
    b->h_p.resize(nr);
    for (size_t i = 0; i < nr; i++) {
      if (b->ctx[i]->h_rvar.empty()) return set_error(BD_ERR_ARG, "bd_batch_run: a replica's model has no r_var");
      int rc = bd_noise_create(seed_base + i, &b->noise[i]);
      if (rc) return rc;
      b->h_rr[i].resize(3 * (size_t)b->ctx[i]->M.n);
      b->h_p[i].resize(b->ctx[i]->m);
    }
  }
  std::vector<const double*> prr(nr), pp(nr);
  for (int s = 0; s < nsteps; s++) {
    for (size_t i = 0; i < nr; i++) {
      bd_ctx* c = b->ctx[i];
      int rc = bd_noise_step(b->noise[i], (int)c->step_count, 3 * c->M.n, c->h_rvar.data(), c->m, b->h_rr[i].data(),
                             b->h_p[i].data());
      if (rc) return rc;
      prr[i] = b->h_rr[i].data();
      pp[i] = b->h_p[i].data();
    }
    int rc = bd_batch_step(b, prr.data(), pp.data(), s + 1 == nsteps ? energies : nullptr);
    if (rc) return rc;
  }
  return BD_OK;
}

extern "C" int bd_batch_run_device(bd_batch* b, int nsteps, unsigned long seed_base, double* energies) {
  if (!b || nsteps < 0) return set_error(BD_ERR_ARG, "bd_batch_run_device: bad argument");
  const int nr = (int)b->ctx.size();
  if (nr == 0) return BD_OK;
  for (bd_ctx* c : b->ctx)
    if (c->step_count != b->ctx[0]->step_count)
      return set_error(BD_ERR_STATE, "bd_batch_run_device: the replicas are at different steps");
  if (!b->dnoise) {
    std::vector<unsigned long> seeds(nr);
    std::vector<int> n3(nr), nD3(nr);
    std::vector<const double*> rv(nr);
    std::vector<double*> rr(nr), p(nr);
    for (int i = 0; i < nr; i++) {
      bd_ctx* c = b->ctx[i];
      if (c->h_rvar.empty()) return set_error(BD_ERR_ARG, "bd_batch_run_device: a replica's model has no r_var");
      seeds[i] = seed_base + (unsigned long)i;
      n3[i] = 3 * c->M.n;
      nD3[i] = c->m;
      rv[i] = c->h_rvar.data();
      rr[i] = c->rr;  // the draws land in the contexts' own noise buffers
      p[i] = c->p;
    }
    int rc = bdk::noise_batch_create(nr, seeds.data(), n3.data(), nD3.data(), rv.data(), rr.data(), p.data(),
                                     &b->dnoise);
    if (rc) return rc;
  }
  // no host synchronisation between steps: the noise launch and the batch
  // step (one graph with use_graph) of every step are enqueued back to back
  for (int s = 0; s < nsteps; s++) {
    int rc = bdk::noise_batch_step(b->dnoise, (int)b->ctx[0]->step_count, b->stream);
    if (!rc) rc = batch_device_step(b);
    if (rc) return rc;
  }
  return batch_finish(b, energies);
}

extern "C" int bd_set_moduli(bd_ctx* c, double h, double g, double s, double debye_length) {
  if (!c || !(debye_length > 0.0)) return set_error(BD_ERR_ARG, "bd_set_moduli: bad argument");
  if (c->in_batch) return set_error(BD_ERR_STATE, "bd_set_moduli: the context belongs to a batch");
  DevModel& M = c->M;
  const double kap = 1.0 / debye_length;
  M.debyell = M.debyell * (kap / M.debye);
  M.debye = kap;
  M.h = h;
  M.g = g;
  M.s = s;
  // a captured graph holds the old constants in its kernel parameters
  if (c->graph) {
    CK(cudaStreamSynchronize(c->stream));
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
  return BD_OK;
}

// main.cpp:386-465 changes which cores carry a linker histone every 100
// steps and with it n_LH and the size of D.  The chain, tails, frames and
// angles stay on the device (as the reference keeps them,
// func_cuda.cu:3434-3490); the caller's LH positions (main.cpp rebuilds them
// on the host, main.cpp:418-447) and the new binding's tables go into the
// buffers bd_create sized for every core bound, so nothing is reallocated.
extern "C" int bd_set_lh_flags(bd_ctx* c, const int* nc_lh_flag, const double* r_lh, const double* lh_rad) {
  if (!c || !nc_lh_flag || !c->model) return set_error(BD_ERR_ARG, "bd_set_lh_flags: null argument");
  if (c->in_batch) return set_error(BD_ERR_STATE, "bd_set_lh_flags: the context belongs to a batch");
  DevModel& M = c->M;
  const int nc = M.n_c, n = M.n, nt = M.n_tail, nlh = M.nlh;
  int bound = 0;
  for (int k = 0; k < nc; k++) {
    if (nc_lh_flag[k] != 0 && nc_lh_flag[k] != 1) return set_error(BD_ERR_ARG, "bd_set_lh_flags: flags are 0 or 1");
    bound += nc_lh_flag[k];
  }
  const int nLH = bound * nlh;
  if (nLH > 0 && !r_lh) return set_error(BD_ERR_ARG, "bd_set_lh_flags: LH positions required");
  if (3 * (n + nt + nLH) > c->m_cap) return set_error(BD_ERR_STATE, "bd_set_lh_flags: more LH beads than the context holds");
  // the new binding's per-bead tables, as bd_create builds them
  bdh::ModelCopy& mc = *c->model;
  std::vector<double> rad(nLH);
  if (lh_rad) {
    rad.assign(lh_rad, lh_rad + nLH);
  } else {  // every linker histone has the same beads: repeat the first one's radii
    std::vector<double> one(nlh, 0.5);
    if ((int)mc.lh_rad.size() >= nlh) one.assign(mc.lh_rad.begin(), mc.lh_rad.begin() + nlh);
    for (int k = 0; k < nLH; k++) rad[k] = one[k % std::max(nlh, 1)];
  }
  std::vector<int> core_bead, core_lh(nc, -1), lh_core_bead, lhp(nLH);
  for (int i = 0; i < n; i++)
    if (c->h_type[i] == 1) core_bead.push_back(i);
  for (int k = 0; k < nc; k++)
    if (nc_lh_flag[k] == 1) core_lh[k] = (int)lh_core_bead.size(), lh_core_bead.push_back(core_bead[k]);
  for (int b = 0; b < nLH; b++) {
    const int idx = b % nlh;
    lhp[b] = idx < M.n_lh_n ? idx : idx + M.n_lh_g;
  }
  cudaStream_t st = c->stream;
  CK(cudaStreamSynchronize(st));  // no step of the old size in flight
  int rc;
  if ((rc = up(const_cast<int*>(M.core_lh), core_lh.data(), nc, st)) ||
      (rc = up(const_cast<int*>(M.lh_core_bead), lh_core_bead.data(), (int)lh_core_bead.size(), st)) ||
      (rc = up(const_cast<int*>(M.lh_p), lhp.data(), nLH, st)) ||
      (rc = up(const_cast<int*>(M.nc_lh_flag), nc_lh_flag, nc, st)) ||
      (rc = up(const_cast<double*>(M.rad_all) + n + nt, rad.data(), nLH, st)) ||
      (rc = up(c->X.r_lh, r_lh, 3 * nLH, st)))
    return rc;
  // logical sizes and the offsets that depend on them
  M.n_LH = nLH;
  M.n_D = n + nt + nLH;
  M.n_lhcore = (int)lh_core_bead.size();
  c->m = 3 * M.n_D;
  c->S.og = n + nt + nLH;
  c->S.npos = n + nt + nLH + M.n_lhcore * M.n_lh_g;
  c->S.nE = 8 * n + nt + nLH;
  // the LH bend angles of the new beads; the frame pass is left out, since
  // its re-orthonormalisation of b and c is not bit-idempotent
  bdk::frame_angles(M, c->X, st);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  // everything planned for the old size goes
  if (c->graph) cudaGraphExecDestroy(c->graph), c->graph = nullptr;
  bdh::adj_free(c->adj);
  c->adj = nullptr;
  c->a_holds_factor = false;
  c->need_rebuild = true;  // the next step assembles and factors the tensor of the new size
  // the host copy of the model follows
  mc.nc_lh_flag.assign(nc_lh_flag, nc_lh_flag + nc);
  mc.lh_rad = rad;
  mc.m.n_LH = nLH;
  mc.bind();
  return BD_OK;
}

extern "C" int bd_restart_from_context(bd_ctx* c, bd_restart* rs) {
  if (!c || !rs) return set_error(BD_ERR_ARG, "bd_restart_from_context: null argument");
  const DevState& X = c->X;
  const long n = c->M.n, nc = c->M.n_c, nt = c->M.n_tail, nl = c->M.n_LH;
  rs->n = (int)n, rs->n_c = (int)nc, rs->n_tail = (int)nt, rs->n_LH = (int)nl;
  const std::pair<double*, const double*> cp[] = {
      {rs->r, X.r},         {rs->a, X.a},         {rs->b, X.b},         {rs->c, X.c},         {rs->alpha, X.alpha},
      {rs->beta, X.beta},   {rs->gamma, X.gamma}, {rs->length, X.length}, {rs->a_dna, X.a_dna}, {rs->b_dna, X.b_dna},
      {rs->c_dna, X.c_dna}, {rs->alpha_p, X.alpha_p}, {rs->beta_p, X.beta_p}, {rs->gamma_p, X.gamma_p},
      {rs->r_t, X.r_t},     {rs->r_lh, X.r_lh}};
  const long cnt[] = {3 * n, 3 * n, 3 * n, 3 * n, n, n, n, n, 3 * nc, 3 * nc, 3 * nc, nc, nc, nc, 3 * nt, 3 * nl};
  for (int k = 0; k < 16; k++) {
    if (!cnt[k]) continue;
    if (!cp[k].first) return set_error(BD_ERR_ARG, "bd_restart_from_context: missing array");
    CK(cudaMemcpyAsync(cp[k].first, cp[k].second, cnt[k] * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return BD_OK;
}

// One Ermak-McCammon move of the context's state with caller forces and
// noise: rotation_cal + rotate (func_cuda.cu:681-704, func.cpp:1607-1670),
// translation_cal with the species-block RPY drift (func_cuda.cu:650-679),
// then the frame refresh (update_Euler_Angle) - one half of main_cuda's
// predictor-corrector step.
extern "C" int bd_em_update(bd_ctx* c, const double* F, const double* T, const double* tF, const double* lF,
                            const double* rr, const double* rd) {
  if (!c || !F || !T || !rr || !rd || (c->M.n_tail && !tF) || (c->M.n_LH && !lF))
    return set_error(BD_ERR_ARG, "bd_em_update: null argument");
  const DevModel& M = c->M;
  cudaStream_t st = c->stream;
  const size_t d = sizeof(double), n3 = 3 * (size_t)M.n, nt3 = 3 * (size_t)M.n_tail, nl3 = 3 * (size_t)M.n_LH;
  CK(cudaMemcpyAsync(c->F0.F, F, n3 * d, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->F0.T, T, n3 * d, cudaMemcpyHostToDevice, st));
  if (nt3) CK(cudaMemcpyAsync(c->F0.tF, tF, nt3 * d, cudaMemcpyHostToDevice, st));
  if (nl3) CK(cudaMemcpyAsync(c->F0.lF, lF, nl3 * d, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->rr, rr, n3 * d, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->rd, rd, (size_t)c->m * d, cudaMemcpyHostToDevice, st));
  const bool mixed = c->precision == BD_PREC_MIXED;
  bdk::gather_rall(M, c->X, c->r_all, mixed ? &c->S : nullptr, st);
  bdk::rotate_translate(M, c->X, c->Y, c->F0, c->rr, c->rd, c->r_all, c->precision, c->S, st);
  CK(cudaMemcpyAsync(c->X.r, c->Y.r, n3 * d, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(c->X.a, c->Y.a, n3 * d, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(c->X.b, c->Y.b, n3 * d, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(c->X.c, c->Y.c, n3 * d, cudaMemcpyDeviceToDevice, st));
  if (nt3) CK(cudaMemcpyAsync(c->X.r_t, c->Y.r_t, nt3 * d, cudaMemcpyDeviceToDevice, st));
  if (nl3) CK(cudaMemcpyAsync(c->X.r_lh, c->Y.r_lh, nl3 * d, cudaMemcpyDeviceToDevice, st));
  bdk::frames(M, c->X, st);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));
  return BD_OK;
}

