// Internal declarations shared by the host code and the CUDA kernels of
// libbdgb300.so.  Not part of the public ABI (include/bd_capi.h is).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <memory>
#include <string>
#include <vector>

#include "../../include/bd_capi.h"

// core/core pairs: each pair's charge pairs over this many CTAs (both paths)
constexpr int kCCSplit = 4;

namespace bdh {

// error reporting (bd_capi.cpp)
int set_error(int code, const char* msg);

// ------------------------------------------------------------ host system
struct HostSystem {
  bd_model m{};
  std::vector<double> setup;
  std::vector<int> type, tail_fix, nc_t_flag, t_grp, t_fix, LH_conn, nc_lh_flag;
  std::vector<double> r, a, b, c, rad, phi_o, r_var, core_pos, core_q, tail_pos, r_t, h_t, g_t, lo_t, beta_o_t, t_q,
      t_rad, LH_g_pos, LH_q, LH_vdw_hh, LH_vdw_hc, LH_vdw_hl, LH_vdw_ht, LH_kstr, LH_kben, LH_streq, LH_betaeq,
      r_lh, lh_rad;
  std::vector<double> lh_tpos, lh_trad;  // LH template as build_LH places it: [3 nlh] core-frame positions, [nlh] radii
};

int load_system(const char* dir, const char* data_f, const char* core_f, const char* tail_f, const char* lh_f,
                const char* lhflag_f, HostSystem& S, std::string& err);
void refresh_model_pointers(HostSystem& S);
int write_xyz(const bd_model* m, const double* r, const double* a, const double* b, const double* c,
              const double* r_t, const double* r_lh, const char* path);

struct Mt19937 {
  uint32_t st[624];
  int idx = 625;
  double cached = 0.0;
  bool have = false;
  bool cr_log = false;  // polar transform: the C library's log (reference) or the correctly rounded one
  void seed(uint32_t s);
  uint32_t next();
  double real1() { return next() * (1.0 / 4294967295.0); }
  double normal(double mean, double sd);
};

}  // namespace bdh

// ------------------------------------------------------------ device model
// Everything a kernel needs about one fiber, passed by value.  Pointers are
// device pointers.  Bead classes: chain beads [0,n) (cores and linker DNA),
// tail beads [0,n_tail), mobile LH beads [0,n_LH); in the diffusion tensor
// they are stacked chain | tails | LH (n_D = n + n_tail + n_LH).
struct DevModel {
  int n, n_c, Nq, n_t, n_tail, n_lh_n, n_lh_g, n_lh_c, n_LH, n_D, nlh, n_dna, n_lhcore;
  double h, g, s, debyell, debye, q_l, k_e, k_ex;
  double sDD, sDC, sCC, sTT, sTL, sTC;
  double a1, a2, dt, del, s2dt;
  const int* type;         // [n]
  const int* core_rank;    // [n] cores in [0,i] minus 1
  const int* core_bead;    // [n_c] bead index of core k
  const int* dna_bead;     // [n_dna] bead index of the k-th linker bead
  const int* lh_core_bead; // [n_lhcore] bead index of the k-th LH-bearing core
  const int* core_lh;      // [n_c] LH ordinal of core k or -1
  const double* phi_o;     // [n]
  const double* rad_all;   // [n_D]
  const double* core_pos;  // [3 Nq]
  const double* core_q;    // [Nq]
  const double* tail_pos;  // [3 n_t]
  const int* tail_fix;     // [n_t]
  const int* nc_t_flag;    // [n_c]
  const double *h_t, *g_t, *lo_t, *beta_o_t, *t_q;  // [n_tail]
  const int *t_grp, *t_fix;                        // [n_tail]
  const int* t_core_bead;  // [n_tail] core bead of the tail's group ((t_grp-1)/10)
  const double* LH_g_pos;  // [3 n_lh_g]
  const int* LH_conn;      // [n_lh_n + n_lh_g + n_lh_c]
  const int* nc_lh_flag;   // [n_c]
  const double *LH_q, *LH_vdw_hh, *LH_vdw_hc, *LH_vdw_hl, *LH_vdw_ht, *LH_kstr, *LH_kben, *LH_streq, *LH_betaeq;
  double qmax_core;        // max |core_pos| (nm), for exact far-pair skipping
  double gmax;             // max |LH_g_pos|
  const float* t_qf;       // [n_tail] tail charges in FP32 (mixed path)
  const float* core_pf;    // [3 Nq] core_pos in FP32 (mixed path)
  const float* core_qf;    // [Nq] core_q in FP32 (mixed path)
  const int* lh_p;         // [n_LH] bead-type parameter index of each LH bead
  int tails_by_core;       // tail t belongs to core t / n_t (or to none): anchored-tail scans per core
};

// Configuration-dependent arrays of one state (current or predicted).
struct DevState {
  double *r, *a, *b, *c;          // [3n]
  double *r_t, *r_lh;             // [3 n_tail], [3 n_LH]
  double *alpha, *beta, *gamma, *length;   // [n]
  double *a_dna, *b_dna, *c_dna;           // [3 n_c]
  double *alpha_p, *beta_p, *gamma_p;      // [n_c]
  double *beta_t, *beta_lh;                // [n_tail], [n_LH]
  double* gpos;                            // [3 n_lhcore n_lh_g] G-head sites (per force pass)
};

struct DevForces {
  double *F, *T, *tF, *lF;   // [3n] [3n] [3 n_tail] [3 n_LH]
  double* E;                 // [1]
};

// Scratch for the deterministic two-stage pair sums (one slot per
// interacting object pair, reduced per bead in a fixed order).
struct DevScratch {
  double* cc;    // [n_c * n_c * 10]  core-core: F(3) T_i(3) T_j(3) E
  double* ccp;   // [kCCSplit * n_c * n_c * 10] core-core partials (a pair over kCCSplit CTAs)
  double* dc;    // [n_dna * n_c * 7] DNA-core: F_on_dna(3) T_core(3) E
  double* gc;    // [n_lhcore * n_c * 10] G-head(core I) - charges(core L): F_I(3) T_I(3) T_L(3) E
  double* ebuf;  // [nE] per-kernel energy partials
  int nE;
  // mixed path: every position of the force pass as a double-float pair
  // (hi, lo) of FP32 xyz, chain | tails | LH | G-heads
  float4 *ph, *pl;
  int ot, ol, og, npos;
  // mixed path: the move's start positions as double-float pairs (radius in
  // qh.w) and the move's forces in FP32, per bead of the tensor
  float4 *qh, *ql, *qf;
  double* bond;  // [4 (n_tail + n_LH)] mixed path: per-bead bonded force and energy of tails, LH beads
  double* bonds; // [37 n] per chain bond: forces and torques on both beads, energy
};

namespace bdk {
// frames.cu
void frames(const DevModel& M, DevState& S, cudaStream_t st);
// the angle pass alone: reads positions and frames, writes angles (and the
// tail and LH bend angles) without touching the frames
void frame_angles(const DevModel& M, DevState& S, cudaStream_t st);
// mixed: the drift from S.qh / S.ql (filled by gather_rall) and S.qf
void rotate_translate(const DevModel& M, const DevState& X, DevState& Y, const DevForces& Fo, const double* rr,
                      const double* rd, const double* r_all, int mixed, const DevScratch& S, cudaStream_t st);
void average_forces(const DevModel& M, const DevForces& A, const DevForces& B, DevForces& out, cudaStream_t st);
// r_all: every tensor bead's position; with S (mixed path) also S->qh / S->ql
void gather_rall(const DevModel& M, const DevState& X, double* r_all, const DevScratch* S, cudaStream_t st);
// forces.cu
// returns the number of kernels launched
int forces(const DevModel& M, DevState& X, DevForces& out, DevScratch& scr, int mixed, cudaStream_t st);
// rpy_chol.cu
// qh, ql (mixed path): the positions as double-float pairs (gather_rall's
// mirror); FP32 RPY blocks stored as double-float pairs (value, 0)
void rpy_assemble(int nD, const double* r_all, const double* rad, double a1, double a2, double* A, int lda,
                  cudaStream_t st, const float4* qh = nullptr, const float4* ql = nullptr);
int potrf_fp64(int m, double* A, int lda, double* rd_acc, const double* p, double s2dt, int* d_negpiv,
               cudaStream_t st);
size_t trmv_scratch_doubles(int m);
// k_tc_chol.cu (mixed precision: FP64 storage, FP32-class arithmetic, tcgen05 trailing updates)
size_t mixed_panel_bytes(int m);
int set_mixed_attributes();
// kev (optional): 2 events per launch that carries a bulk trailing update
// (the dominant kernel); *kev_pairs = how many were recorded, *kflop and
// *kbytes accumulate the tensor work those launches issue and their
// algorithmic HBM bytes.
// max_pass: at most this many panels (1..3) per bulk trailing pass.
int potrf_mixed(int m, double* A, int lda, unsigned char* PS, int* negpiv, int* err, cudaStream_t st,
                cudaEvent_t* kev = nullptr, int* kev_pairs = nullptr, double* kflop = nullptr,
                double* kbytes = nullptr, int max_pass = 3);
int mixed_tiles(int m);
// k_krylov.cu: rd = s2dt D^{1/2} p by Lanczos on the lower-stored tensor
size_t krylov_scratch_doubles(int m, int kmax);
// tc_gemm.cu: C = alpha A op(B) on tcgen05 (row-major FP32, three BF16
// slices, six products); M, N multiples of 128, K of 64; kmode limits each
// 128-tile's K range (1: k >= row0, 2: k >= col0, 4: k < col0 + 128);
// batch products zstride elements apart; a timed-out wait sets *err
int tc_gemm_f32(cudaStream_t st, int M, int N, int K, float alpha, const float* A, int lda, const float* B, int ldb,
                float* C, int ldc, bool tb, int kmode, int batch, long zstride, int* err);
int tc_gemm_attributes();
// k_noise.cu: the device noise stream of every replica of a batch, one launch per step
struct NoiseBatch;
int noise_batch_create(int nr, const unsigned long* seeds, const int* n3, const int* nD3,
                       const double* const* h_rvar, double* const* d_rr, double* const* d_p, NoiseBatch** out);
int noise_batch_step(NoiseBatch* b, int step, cudaStream_t st);
void noise_batch_free(NoiseBatch* b);
// A == nullptr: matrix-free products from the double-float position mirror qh/ql
// the Lanczos iterations of a context, kCheck at a time, as CUDA graphs
// (valid while the context's sizes, scratch and tensor pointer stay)
struct KrylovGraphs {
  int m = -1, kmax = -1;
  const double* scratch = nullptr;
  const double* A = nullptr;
  bool df = false;
  double a1 = 0.0, a2 = 0.0;
  std::vector<cudaGraphExec_t> blocks;
  void clear() {
    for (cudaGraphExec_t g : blocks)
      if (g) cudaGraphExecDestroy(g);
    blocks.clear();
  }
  ~KrylovGraphs() { clear(); }
};
int krylov_sqrt(int m, const double* A, int lda, bool df, const float4* qh, const float4* ql, double a1, double a2,
                const double* p, double s2dt, double tol, int kmax, double* rd, double* scratch, cudaStream_t st,
                int* iters, double* change, struct KrylovGraphs* graphs = nullptr);
int mixed_max_launches(int m);  // k_chol_step launches of one factorisation, at most
// Many mixed factorisations (replicas) advanced together: launch i runs step
// i of every factorisation's schedule (k_chol_step_multi), then one diagonal
// scatter for all.  The plan holds the matrices' addresses.
struct MixedBatch;
MixedBatch* mixed_batch_create(int nrep, const int* m, double* const* A, const int* lda, unsigned char* const* PS,
                               int* const* negpiv, int* const* err, int max_pass = 3);
int mixed_batch_run(const MixedBatch* b, cudaStream_t st);  // returns the launches issued
void mixed_batch_free(MixedBatch* b);

void trmv_lower_ws(int m, const double* A, int lda, const double* p, double s2dt, double* rd, double* part,
                   cudaStream_t st, bool df = false);
}  // namespace bdk

namespace bdh {
struct AdjWork;                 // k_adjoint.cu: buffers of the rollout gradient
void adj_free(AdjWork* w);

// A deep copy of a bd_model (arrays owned here), kept by every context so
// that it can be rebuilt for a new linker-histone binding (bd_set_lh_flags).
struct ModelCopy {
  bd_model m{};
  std::vector<int> type, tail_fix, nc_t_flag, t_grp, t_fix, LH_conn, nc_lh_flag;
  std::vector<double> rad, phi_o, r_var, core_pos, core_q, tail_pos, h_t, g_t, lo_t, beta_o_t, t_q, t_rad, LH_g_pos,
      LH_q, LH_vdw_hh, LH_vdw_hc, LH_vdw_hl, LH_vdw_ht, LH_kstr, LH_kben, LH_streq, LH_betaeq, lh_rad;
  void take(const bd_model& src);
  void bind();  // m's array pointers into the vectors (null for empty ones)
};
}  // namespace bdh

// One fiber on one device: every buffer is allocated at bd_create.
struct bd_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int precision = BD_PREC_FP64;
  int freq_rp = 1;
  int use_graph = 0;
  int mixed_passes = 3;  // panels per bulk trailing pass of the mixed factorisation (bd_set_mixed_passes)
  // noise displacement: 0 = L p (the reference's), 1 = D^{1/2} p by Lanczos (bd_set_noise_mode)
  int noise_mode = 0;
  double krylov_tol = 1e-6;
  int krylov_kmax = 64, krylov_iters = 0;
  double krylov_change = 0.0;
  double* kscratch = nullptr;
  bdk::KrylovGraphs kgraphs;  // the Lanczos iteration blocks, captured on first use
  bool a_holds_factor = false;  // A holds L (after a factorisation), not D
  bool need_rebuild = false;    // the next step assembles D whatever frequency_RP says (after a resize)
  long step_count = 0;
  DevModel M{};
  DevState X{}, Y{};
  DevForces F0{}, F1{}, Fa{};
  DevScratch S{};
  void* arena_base = nullptr;
  double* A = nullptr;   // m x lda, column-major; holds D then L (FP64 path)
  unsigned char* PS = nullptr;  // mixed path: BF16 panel slices
  int* d_err = nullptr;         // device error code of the tensor-core kernels
  int m = 0, lda = 0;  // 3 n_D now, and the leading dimension of A (for m_cap)
  int m_cap = 0;       // largest m the buffers hold: every core with a linker histone
  double *r_all = nullptr, *rd = nullptr, *p = nullptr, *rr = nullptr, *rd_part = nullptr, *energy = nullptr;
  int* negpiv = nullptr;
  cudaGraphExec_t graph = nullptr;
  int last_launches = 0;
  int host_negpiv = 0;
  cudaEvent_t ev[10] = {};
  bool timing = false;
  std::vector<cudaEvent_t> kev;   // events around every k_chol_step launch (timing steps only)
  int kev_pairs = 0;
  double kflop = 0.0;
  double kbytes = 0.0;
  // host copies for the drop-in paths
  std::vector<int> h_type;
  std::vector<double> h_rvar;  // rotational noise scale (bd_batch_run draws noise on the host)
  bdh::AdjWork* adj = nullptr;  // allocated by the first bd_adjoint / bd_rollout_loss
  std::shared_ptr<bdh::ModelCopy> model;  // the model it was created from
  bool in_batch = false;  // owned by a bd_batch (whose graph and plans hold its buffers and constants)
};

namespace bdh {
// An NVTX range around host-side phases, for profilers (nsys, ncu's NVTX
// filters); without a tool attached the calls do nothing.
struct Range {
  explicit Range(const char* name);
  ~Range();
};

// The device part of one step (bd_capi.cu).  With saves != nullptr the
// predictor state before and after its frame refresh and the corrector state
// before its refresh are copied to saves[0..2] ([r a b c r_t], 12n + 3 n_tail).
int step_device(bd_ctx* c, const double* d_rr, const double* d_p, double* const* saves = nullptr);
}  // namespace bdh
