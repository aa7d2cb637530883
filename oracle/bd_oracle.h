// Test infrastructure: the CPU oracle for the Brownian-dynamics step of the
// mesoscale chromatin fiber.  Only tests/, __graft_entry__.smoke() and the
// CPU-baseline legs of bench.py load it; the product never does.
//
// It restates, sequentially and in FP64, the reference's CPU physics
// (BD_cuda/func.cpp) composed in the order of the reference GPU step
// main_cuda (BD_cuda/func_cuda.cu:3434-3680).  Arithmetic is written in the
// reference's operation order so that, built without FMA contraction, it
// reproduces the reference bit for bit (pinned by tests against the
// reference compiled from its own sources, oracle/_ref).
#pragma once
#ifdef __cplusplus
extern "C" {
#endif

// Layout of every array follows the reference: xyz interleaved per bead
// (r[3*i+k]), row-major matrices.
typedef struct orc_system {
  int n, n_c, Nq, n_t, n_tail, n_lh_n, n_lh_g, n_lh_c, n_LH;
  double h, g, s, debyell, debye, q_l, k_e, k_ex;
  double sigma_DNA_DNA, sigma_DNA_Core, sigma_Core_Core, sigma_Tail_Tail, sigma_Tail_Linker, sigma_Tail_Core;
  double a1, a2, time_step, del, s2dt;
  const int* type;          // [n]
  const double* rad;        // [n]
  const double* phi_o;      // [n]
  const double* core_pos;   // [3*Nq] core frame, nm
  const double* core_q;     // [Nq]
  const double* tail_pos;   // [3*n_t] template, core frame, nm
  const int* tail_fix;      // [n_t] template
  const int* nc_t_flag;     // [n_c]
  const double* h_t; const double* g_t; const double* lo_t; const double* beta_o_t;
  const double* t_q; const double* t_rad;          // [n_tail]
  const int* t_grp; const int* t_fix;              // [n_tail]
  const double* LH_g_pos;   // [3*n_lh_g]
  const int* LH_conn;       // [n_lh_n+n_lh_g+n_lh_c]
  const int* nc_lh_flag;    // [n_c]
  const double* LH_q; const double* LH_vdw_hh; const double* LH_vdw_hc; const double* LH_vdw_hl;
  const double* LH_vdw_ht; const double* LH_kstr; const double* LH_kben; const double* LH_streq;
  const double* LH_betaeq;  // each [n_lh_n+n_lh_g+n_lh_c]
  const double* lh_rad;     // [n_LH]
} orc_system;

// Copies the system and the state.  With refresh != 0 the internal
// coordinates are computed from (r,a,b,c) as main.cpp:166 does at start-up,
// which re-orthonormalises the DNA frames.
void* orc_create(const orc_system* sys, const double* r, const double* a, const double* b, const double* c,
                 const double* r_t, const double* r_lh, int refresh);
void orc_destroy(void* h);
// Forces, torques and energy at the current state (func.cpp force functions,
// called in main_cuda's order); returns the energy.
double orc_forces(void* h, double* force, double* torque, double* t_force, double* LH_force);
// RPY tensor D and its Cholesky factor L at the current state, row-major.
void orc_tensor(void* h, double* D, double* L);
// One predictor-corrector step with the given noise; returns pass-1 energy.
double orc_step(void* h, const double* rr, const double* p);
int orc_em_update(void* h, const double* F, const double* T, const double* tF, const double* lF, const double* rr,
                  const double* rd);
// Named state arrays: r a b c r_t r_lh alpha beta gamma length a_dna b_dna
// c_dna alpha_p beta_p gamma_p beta_t beta_lh rd force torque t_force
// LH_force.  Returns the length, or -1 for an unknown name.
int orc_get(void* h, const char* name, double* out);
int orc_set(void* h, const char* name, const double* in);
// Reference Cholesky (func.cpp:806-836) of a row-major m x m matrix into
// L (row-major, upper part left untouched).  nthreads > 1 runs the same
// arithmetic column-parallel; results are bitwise identical.  Returns the
// number of negative pivots that were replaced by their absolute value.
int orc_cholesky(int m, const double* D, double* L, int nthreads);
// Host threads used by orc_step for the RPY assembly, the Cholesky and rd.
void orc_set_threads(int n);

// RPY assembly alone (func.cpp:737-804) for nD beads, row-major 3nD x 3nD.
void orc_rpy(int nD, const double* r, const double* rad, double a1, double a2, double* D);

// MT19937 + polar Box-Muller noise in the reference order (mt.cpp,
// utilities.cpp:304-336, main.cpp:386-388,479-486).
void* orc_noise_create(unsigned long seed);
void orc_noise_destroy(void* g);
unsigned int orc_noise_u32(void* g);
double orc_noise_real1(void* g);
double orc_noise_normal(void* g, double mean, double stddev);
// rr[n3] with per-DOF "stddev" r_var, then p[n_D3] ~ N(0,1).
void orc_noise_step(void* g, int step, int n3, const double* r_var, int n_D3, double* rr, double* p);

#ifdef __cplusplus
}
#endif
