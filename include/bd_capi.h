/*
 * bd_capi.h - C ABI of the GB300 Brownian-dynamics step for the mesoscale
 * chromatin fiber (libbdgb300.so).
 *
 * The reference (Schlicklab/Brownian_Dynamics_CUDA) exposes its GPU step as
 * four C++ functions (BD_cuda/func_cuda.h:37-52) backed by file-scope
 * globals.  This header replaces them with a handle-based C ABI: plain
 * pointers and sizes, host arrays in the reference's own layouts (xyz
 * interleaved per bead, row-major matrices), an int status from every call,
 * no globals and no C++ types.  A shim in the same library re-exports the
 * four reference symbols on top of it, so the
 * reference's main.cpp links against this library unchanged.
 *
 * Threading: a context is used by one host thread at a time; different
 * contexts are independent.  All device work of a context runs on the
 * stream given at creation (0 = a stream the context creates).
 */
#ifndef BD_CAPI_H
#define BD_CAPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
enum {
  BD_OK = 0,
  BD_ERR_ARG = 1,        /* bad pointer, size or name */
  BD_ERR_IO = 2,         /* input file missing or malformed */
  BD_ERR_CUDA = 3,       /* a CUDA runtime call failed (bd_last_error has it) */
  BD_ERR_NOMEM = 4,      /* device allocation failed */
  BD_ERR_NONFINITE = 5,  /* a NaN/Inf appeared in forces or positions */
  BD_ERR_NOT_SPD = 6,    /* reserved: strict-SPD mode found a non-positive pivot */
  BD_ERR_STATE = 7       /* call not valid in the context's current state */
};

/* Message of the last failing call on this thread (static storage). */
const char* bd_last_error(void);
/* Library version string. */
const char* bd_version(void);

/* --------------------------------------------------------------- precision */
enum {
  BD_PREC_FP64 = 0,   /* plain FP64 step: parity path against the FP64 oracle */
  BD_PREC_MIXED = 1   /* FP32-class: RPY tensor in FP32 into double-float storage, Cholesky with
                         FP32 panels and BF16x3 tensor-core (tcgen05) trailing updates, FP32
                         pair forces with compensated sums; no refinement.  Displacement
                         4e-7 to 8e-7 from the FP64 path on the benchmark fibers; up to
                         1.3e-6 on 3 of 256 uneven batch replicas (bd_set_mixed_passes) */
};

/* Noise displacement of a step (bd_set_noise_mode). */
enum {
  BD_NOISE_CHOLESKY = 0, /* rd = s2dt L p, L the Cholesky factor of D: the reference's */
  BD_NOISE_KRYLOV = 1    /* rd = s2dt D^{1/2} p by Lanczos: same covariance, another vector */
};

/* ------------------------------------------------------------ model (host)
 * Topology, parameters and per-bead constants of one fiber.  Field names and
 * meanings are those of cuda_application_init_data (func_cuda.cu:2676) and
 * main.cpp:38-372.  Arrays are borrowed: bd_create copies what it needs. */
typedef struct bd_model {
  int n, n_c;              /* beads on the chain (cores + linker DNA), cores   */
  int Nq;                  /* charges per core (300)                           */
  int n_t, n_tail;         /* tail beads per core (template), total tail beads */
  int n_lh_n, n_lh_g, n_lh_c, n_LH;  /* LH N-term / G-head / C-term per LH, total mobile LH beads */
  double h, g, s;          /* stretch, bend, twist constants (main.cpp:90-95)  */
  double debyell, debye, q_l, k_e, k_ex, k_h1;
  double sigma_DNA_DNA, sigma_DNA_Core, sigma_Core_Core;
  double sigma_Tail_Tail, sigma_Tail_Linker, sigma_Tail_Core;
  double a1, a2;           /* kT/(6 pi eta), kT/(8 pi eta)                      */
  double time_step, del, s2dt;  /* dt, dt/kT, sqrt(2 dt)                        */
  const int* type;         /* [n] 1 = core, 0 = linker DNA                      */
  const double* rad;       /* [n] hydrodynamic radius                           */
  const double* phi_o;     /* [n] intrinsic twist (update_phi_o)                */
  const double* r_var;     /* [3n] rotational noise "stddev" (main.cpp:292-303) */
  const double* core_pos;  /* [3 Nq] charge sites, core frame, nm               */
  const double* core_q;    /* [Nq]                                              */
  const double* tail_pos;  /* [3 n_t] tail template, core frame, nm             */
  const int* tail_fix;     /* [n_t] template anchor flags                       */
  const int* nc_t_flag;    /* [n_c] cores carrying tails                        */
  const double* h_t; const double* g_t; const double* lo_t; const double* beta_o_t;
  const double* t_q; const double* t_rad;   /* [n_tail]                          */
  const int* t_grp; const int* t_fix;       /* [n_tail]                          */
  const double* LH_g_pos;  /* [3 n_lh_g] globular head, core frame               */
  const int* LH_conn;      /* [n_lh_n+n_lh_g+n_lh_c]                             */
  const int* nc_lh_flag;   /* [n_c] cores carrying a linker histone              */
  const double* LH_q; const double* LH_vdw_hh; const double* LH_vdw_hc;
  const double* LH_vdw_hl; const double* LH_vdw_ht; const double* LH_kstr;
  const double* LH_kben; const double* LH_streq; const double* LH_betaeq;
  const double* lh_rad;    /* [n_LH]                                            */
} bd_model;

/* Configuration state.  With refresh_frames != 0 the internal coordinates
 * (Euler angles, exit frames, bend angles) are computed on the device from
 * r,a,b,c as main.cpp:166 does on the host, re-orthonormalising the DNA
 * frames; otherwise the angle arrays must be given (as init_data takes them). */
typedef struct bd_state {
  const double* r; const double* a; const double* b; const double* c;   /* [3n] */
  const double* r_t;       /* [3 n_tail] */
  const double* r_lh;      /* [3 n_LH]   */
  int refresh_frames;
  const double* alpha; const double* beta; const double* gamma; const double* length;  /* [n] */
  const double* a_dna; const double* b_dna; const double* c_dna;                       /* [3 n_c] */
  const double* alpha_p; const double* beta_p; const double* gamma_p;                  /* [n_c] */
} bd_state;

typedef struct bd_options {
  int precision;           /* BD_PREC_FP64 or BD_PREC_MIXED                      */
  int frequency_RP;        /* rebuild + refactor D every k steps (1 = every step,
                              as the reference does)                             */
  int use_graph;           /* capture the device part of a step in a CUDA graph  */
  int device;              /* CUDA device ordinal                                */
  void* stream;            /* cudaStream_t to run on, or NULL                    */
} bd_options;

/* ---------------------------------------------------- host system loader
 * Reads the reference's input files from dir exactly as main.cpp:38-372
 * does with readfile.cpp (setup.txt, data_mod, core charges, tail table,
 * LH table, LH.in) and builds tails, linker histones, phi_o, r_var and the
 * physical constants.  Frames are returned as read (not yet refreshed). */
typedef struct bd_system bd_system;
int bd_system_load(const char* dir, const char* data_file, const char* core_file, const char* tail_file,
                   const char* lh_file, const char* lh_flags_file, bd_system** out);
/* Model and state views that point into the system's own storage. */
int bd_system_model(const bd_system* sys, bd_model* out);
int bd_system_state(const bd_system* sys, bd_state* out);
/* setup.txt values: T steps freq freq_RP sigma x6 Mg Cs restart unbind Pbind (15) */
int bd_system_setup(const bd_system* sys, double* out15);
void bd_system_free(bd_system* sys);
/* The reference's text restart (write_restart, readfile.cpp:404-439):
 * restart_{r,a,b,c,Er,tail,lh}.txt in dir, one value per line with 15
 * decimals (Er NULL: zeros).  bd_system_load reads them back in place of
 * the start structure when setup.txt has restart = 1 (main.cpp:143-153,
 * :218-220, :279-281). */
int bd_write_restart_text(const char* dir, int n, int n_tail, int n_LH, const double* r, const double* a,
                          const double* b, const double* c, const double* Er, const double* r_t, const double* r_lh);
/* Appends one out.xyz frame (readfile.cpp:346-405 format). */
int bd_write_xyz(const bd_model* m, const double* r, const double* a, const double* b, const double* c,
                 const double* r_t, const double* r_lh, const char* path);

/* ------------------------------------------------------------ noise (host)
 * MT19937 + polar Box-Muller stream in the reference order (mt.cpp,
 * utilities.cpp:304-336, main.cpp:386-388 and :479-486). */
typedef struct bd_noise bd_noise;
int bd_noise_create(unsigned long seed, bd_noise** out);
/* Draws one step's noise: two uniforms when step % 100 == 0, then rr[n3]
 * with per-DOF scale r_var, then p[n_D3] ~ N(0,1). */
int bd_noise_step(bd_noise* g, int step, int n3, const double* r_var, int n_D3, double* rr, double* p);
int bd_noise_u32(bd_noise* g, int count, uint32_t* out);
void bd_noise_free(bd_noise* g);
/* The logarithm of the polar transform.  BD_LOG_LIBM (the default): the C
 * library's log, as the reference (utilities.cpp:304-336) - glibc's is
 * not correctly rounded (on ~1 in 1,400 of the transform's arguments it
 * differs from the correctly rounded value by one ulp), and its results may differ between machines.
 * BD_LOG_CR: a correctly rounded log (double-double atanh series), the one
 * the device stream (bd_dev_noise_*) uses, so the two streams are equal
 * bit for bit on every machine.  No counterpart in the reference. */
enum { BD_LOG_LIBM = 0, BD_LOG_CR = 1 };
int bd_noise_set_log(bd_noise* g, int mode);
/* The step's pieces separately, for a driver that runs the LH binding Monte
 * Carlo between them (bd_lh_mc): `count` uniforms genrand_real1 as main.cpp
 * draws them on steps with step % 100 == 0 (main.cpp:387-388), then the
 * step's normal draws.  bd_noise_step(g, step, ...) is exactly
 * bd_noise_uniforms(g, 2, u) when step % 100 == 0, then bd_noise_draws. */
int bd_noise_uniforms(bd_noise* g, int count, double* out);
int bd_noise_draws(bd_noise* g, int n3, const double* r_var, int n_D3, double* rr, double* p);
/* The generator's full state: the 624 MT19937 words, the index of the next
 * word, and the pending second deviate of the polar method. */
int bd_noise_get_state(const bd_noise* g, uint32_t* words624, int* index, int* have_cached, double* cached);
int bd_noise_set_state(bd_noise* g, const uint32_t* words624, int index, int have_cached, double cached);

/* ---------------------------------------------------------------- restart
 * Binary restart of one fiber: the step counter, positions, frames and the
 * internal coordinates (so that a context created from it with
 * refresh_frames = 0 continues bit for bit), the LH binding and, optionally,
 * the noise generator's state.  The reference's restart (readfile.cpp:346-441)
 * is text, positions only, and reseeds the generator.  Little-endian, file
 * magic "BDRST001".  Array sizes are those of bd_state and bd_model. */
typedef struct bd_restart {
  long step;
  int n, n_c, n_tail, n_LH;
  double *r, *a, *b, *c;                                /* [3n]            */
  double *alpha, *beta, *gamma, *length;                /* [n]             */
  double *a_dna, *b_dna, *c_dna;                        /* [3 n_c]         */
  double *alpha_p, *beta_p, *gamma_p;                   /* [n_c]           */
  double *r_t, *r_lh;                                   /* [3 n_tail] [3 n_LH] */
  int* nc_lh_flag;                                      /* [n_c]           */
} bd_restart;
/* Writes rs (all arrays given) and, if g is not NULL, g's state. */
int bd_restart_write(const char* path, const bd_restart* rs, const bd_noise* g);
/* Reads the header: step and sizes into rs (arrays untouched); *has_noise. */
int bd_restart_info(const char* path, bd_restart* rs, int* has_noise);
/* Reads everything into rs's arrays (sizes must match the file's) and, if g
 * is not NULL and the file has it, the generator's state into g. */
int bd_restart_read(const char* path, bd_restart* rs, bd_noise* g);
/* bd_restart_from_context (below, with the context calls) fills one from a
 * context. */
/* The same stream generated on the device (one CTA per generator; state in
 * device memory): bd_dev_noise_step writes step `step`'s draws into device
 * arrays d_rr [n3] (scaled by d_r_var) and d_p [n_D3], stream-ordered on
 * `stream` (a cudaStream_t, NULL for the legacy stream).  The 32-bit words
 * and the polar method's accept / reject decisions are those of
 * bd_noise_step bit for bit; the deviates equal those of a host stream set
 * to BD_LOG_CR bit for bit (the device log is the correctly rounded one),
 * and the reference's (the C library's log) except where that log rounds
 * differently (one ulp, ~1 in 1,400 of the polar transform's arguments). */
typedef struct bd_dev_noise bd_dev_noise;
int bd_dev_noise_create(unsigned long seed, bd_dev_noise** out);
int bd_dev_noise_step(bd_dev_noise* g, int step, int n3, const double* d_r_var, int n_D3, double* d_rr, double* d_p,
                      void* stream);
int bd_dev_noise_free(bd_dev_noise* g);

/* ------------------------------------------------------------ device step */
typedef struct bd_ctx bd_ctx;

/* Allocates device state and copies model + state to the device.
 * Replaces cuda_application_init_D_Chol + cuda_application_init_data
 * (func_cuda.cu:2665, :2676). */
int bd_create(const bd_model* m, const bd_state* s, const bd_options* opt, bd_ctx** out);
int bd_destroy(bd_ctx* ctx);

/* Sizes: n n_c n_tail n_LH n_D m(=3 n_D) lda(padded leading dim) precision */
int bd_sizes(const bd_ctx* ctx, int* out8);

/* One predictor-corrector BD step (main_cuda, func_cuda.cu:3434-3680).
 * rr[3n] and p[3 n_D] are host noise arrays; energy (may be NULL) receives
 * the pass-1 energy.  Host copies of the state are refreshed on return for
 * every non-NULL pointer in out_state-like arguments of bd_get_state.
 * Returns BD_ERR_NONFINITE, before launching anything, if rr or p holds a
 * NaN or Inf, and after the step if its energy is not finite (the reference
 * checks neither). */
int bd_step(bd_ctx* ctx, const double* rr, const double* p, double* energy);

/* Same step, noise already on the device (device pointers, stream-ordered). */
int bd_step_device(bd_ctx* ctx, const double* d_rr, const double* d_p, double* d_energy);

/* Drop-in form of main_cuda: runs bd_step and copies back exactly what
 * main_cuda copies back: r_lh every step; r, a, b, c, r_t when
 * step % frequency_of_sampling == 0 or step == number_of_steps - 1. */
int bd_step_reference(bd_ctx* ctx, int step, int number_of_steps, int frequency_of_sampling, const double* rr,
                      const double* p, double* energy, double* h_r, double* h_a, double* h_b, double* h_c,
                      double* h_r_t, double* h_r_lh);

/* Finer entry points (each works on the context's current state). */
/* Forces [3n], torques [3n], tail forces [3 n_tail], LH forces [3 n_LH], energy. */
int bd_forces(bd_ctx* ctx, double* force, double* torque, double* t_force, double* LH_force, double* energy);
/* Full symmetric RPY tensor, row-major m x m (m = 3 n_D). */
int bd_diffusion_tensor(bd_ctx* ctx, double* D);
/* Lower Cholesky factor of D, row-major m x m, upper triangle zero. */
int bd_cholesky(bd_ctx* ctx, double* L);
/* Noise displacement rd = sqrt(2 dt) L p for the current state, rd[m]. */
int bd_noise_displacement(bd_ctx* ctx, const double* p, double* rd);
/* One Ermak-McCammon move of the context's state with the caller's forces
 * (force, torque [3n], t_force [3 n_tail], LH_force [3 n_LH]) and noise
 * (rr [3n], rd [3 n_D]): frames rotated by dt tau / zeta + rr, positions
 * moved by rd + del D_blk F (rotation_cal, rotate, translation_cal:
 * func_cuda.cu:650-704, func.cpp:1607-1670), then the frames refreshed. */
int bd_em_update(bd_ctx* ctx, const double* force, const double* torque, const double* t_force,
                 const double* LH_force, const double* rr, const double* rd);

/* Named state arrays (host copies): r a b c r_t r_lh alpha beta gamma length
 * a_dna b_dna c_dna alpha_p beta_p gamma_p beta_t beta_lh rd force torque
 * t_force LH_force.  Returns BD_ERR_ARG for an unknown name. */
int bd_get_state(bd_ctx* ctx, const char* name, double* out, int* count);
/* Overwrites r a b c r_t or r_lh and refreshes the internal coordinates. */
int bd_set_state(bd_ctx* ctx, const char* name, const double* in);

/* Standalone dense kernels on caller-owned device buffers (stream-ordered on
 * the context's stream).  Matrices are column-major with leading dim lda. */
int bd_dev_rpy(bd_ctx* ctx, int n_beads, const double* d_r, const double* d_rad, double a1, double a2,
               double* d_D, int lda);
int bd_dev_potrf(bd_ctx* ctx, int m, double* d_A, int lda, int precision, int* d_info);

/* Allocation-free noise displacement: rd = s2dt * L p for a lower factor L
 * (column-major, leading dim lda) that the caller owns on the device, with
 * p and rd caller-owned device vectors of length m; stream-ordered on
 * `stream` (a cudaStream_t, NULL for the default stream).
 * No counterpart in the reference: it serves hosts that cannot let a
 * library call cudaMalloc/cudaFree (their device memory belongs to their own
 * pool allocator, or an allocation - which may synchronise the device -
 * would stall their step loop).  It calls no allocating routine: its
 * partial sums live in a fixed 4 MiB device array inside the library, so
 * m must not exceed 16384 (BD_ERR_ARG otherwise).  The first call on a
 * device looks that array's device address up (cudaGetSymbolAddress, with
 * the device current) and caches it with the device's current context; a
 * call in a new context (after cudaDeviceReset) looks it up again.  Under
 * lazy module loading (the CUDA default) that first look-up loads the
 * library's device code and commits the 4 MiB array, so the first call on a
 * device, and the first after a reset, allocates: make it once as a warm-up,
 * before the region that must not allocate and before any stream capture.
 * Later calls allocate nothing.  All calls share the array: calls whose
 * kernels overlap on the GPU race and must be ordered by the caller.
 * Nothing in the array needs to start at zero. */
int bd_noise_displacement_noalloc(int m, const double* d_L, int lda, const double* d_p, double s2dt, double* d_rd,
                                  void* stream);

/* ---------------------------------------------------------------- batches
 * Many independent fibers (replicas, e.g. of uneven size and salt) advanced
 * together.  All replicas share one stream; with use_graph one CUDA graph
 * holds every replica's step, run in turn (no two replicas' tensor-core
 * kernels overlap).  No counterpart in the reference, which runs one fiber
 * per process (main.cpp); each replica's step is the bd_step of its own
 * context.  Options apply to every replica (frequency_RP must be 1 for the
 * graph). */
typedef struct bd_batch bd_batch;
int bd_batch_create(int nrep, const bd_model* models, const bd_state* states, const bd_options* opt, bd_batch** out);
int bd_batch_destroy(bd_batch* b);
int bd_batch_size(const bd_batch* b, int* nrep);
/* The context of replica i (for bd_get_state, bd_set_state, bd_forces ...). */
int bd_batch_context(bd_batch* b, int i, bd_ctx** out);
/* Phase times of a batched mixed step, in ms: every replica's positions and
 * tensor, the batched factorisation, every replica's forces and moves.  The
 * first call switches timing on (zeros returned); while on, batch steps run
 * eagerly (no graph) with CUDA events around the phases, and later calls
 * return the last step's times.  Measurement only; no counterpart in the
 * reference. */
int bd_batch_phase_times(bd_batch* b, float* out3);
/* Kernel launches of the last batch step enqueued (a graph replays the same
 * launches).  No counterpart in the reference. */
int bd_batch_launch_count(const bd_batch* b, int* out);
/* Accuracy/speed setting of the mixed factorisation: at most `passes` (1, 2
 * or 3; default 3) panels per trailing read-modify-write pass.  Each pass
 * accumulates its panels' products in FP32 tensor memory before adding them
 * to the double-float tensor, so fewer panels per pass give a more accurate
 * factor at more HBM traffic (measured at 3N = 11,700: 3 -> 6.9 ms, noise
 * displacement 7.8e-7 from FP64; 2 -> 7.3 ms, 6.3e-7; 1 -> 9.4 ms, 5.4e-7).
 * The next step captures its graph again.  No counterpart in the reference
 * (its factorisation is FP64 cuSOLVER). */
int bd_set_mixed_passes(bd_ctx* ctx, int passes);
/* Noise displacement mode.  BD_NOISE_KRYLOV replaces the factorisation and
 * L p by the symmetric square root of D applied to p through the Lanczos
 * process (full re-orthogonalisation; stops when the relative change of the
 * approximation is <= tol, at most kmax iterations, 2 <= kmax <= 512): the
 * same covariance 2 dt D as the reference's noise, so a valid BD step, but a
 * different vector than L p, so not comparable step for step with the
 * reference (a fast mode for large fibers, where one tensor-vector product per
 * iteration replaces an O((3N)^3) factorisation).  D is rebuilt every
 * frequency_RP steps as before on FP64 contexts (products with the stored
 * tensor, FP64); mixed contexts compute every product matrix-free from the
 * current positions (FP32 RPY blocks, compensated sums), so they neither
 * assemble nor store the tensor.  A Krylov step reads the tridiagonal
 * coefficients back every 8 iterations: it is not stream-ordered and is never
 * captured in a graph.  Allocates its workspace ((kmax + 1) 3N + 3N doubles
 * + 64 (3N / 64)^2 doubles).  No counterpart in the reference
 * (its frequency_RP guard is commented out, func_cuda.cu:3504). */
int bd_set_noise_mode(bd_ctx* ctx, int mode, double tol, int kmax);
/* Iterations and last relative change of the most recent Krylov run. */
int bd_krylov_stats(const bd_ctx* ctx, int* iters, double* change);
int bd_batch_set_mixed_passes(bd_batch* b, int passes);
/* One step of every replica: rr[i], p[i] are replica i's host noise (as for
 * bd_step); energies[i] (optional) receives its energy. */
int bd_batch_step(bd_batch* b, const double* const* rr, const double* const* p, double* energies);
/* The same with device noise; stream-ordered, no host synchronisation. */
int bd_batch_step_device(bd_batch* b, const double* const* d_rr, const double* const* d_p);
/* nsteps steps with each replica's own host noise stream (MT19937 seeded
 * seed_base + i, draws as main.cpp:479-486); energies as bd_batch_step after
 * the last step. */
int bd_batch_run(bd_batch* b, int nsteps, unsigned long seed_base, double* energies);
/* The same run with each replica's stream generated on the device (the
 * bd_dev_noise_* stream, seeded seed_base + i; one launch per step for all
 * replicas, the draws written straight into the replicas' noise buffers):
 * nothing is copied from the host and the host does not wait between
 * steps; equal bit for bit to bd_batch_run with host streams set to
 * BD_LOG_CR.  energies as bd_batch_run.  No counterpart in the reference. */
int bd_batch_run_device(bd_batch* b, int nsteps, unsigned long seed_base, double* energies);

/* Timing of the last step's phases on the device (ms): rpy chol rd forces1
 * update1 frames forces2 update2 total.  Valid after a step with use_graph=0. */
int bd_phase_times(bd_ctx* ctx, float* out9);
/* Mixed path: total device time (CUDA events on the context's stream) of
 * the tensor-core trailing-update launches of the last step run with
 * timing enabled (see bd_phase_times), their number, and the BF16 tensor
 * work they issued (flop). */
int bd_kernel_time(bd_ctx* ctx, float* total_ms, int* launches, double* tensor_flop);
/* The same launches one by one: out_ms[i] for i < min(max, launches), in
 * panel order; *launches = their number. */
int bd_kernel_times(bd_ctx* ctx, float* out_ms, int max, int* launches);
/* Algorithmic HBM bytes of those launches: 16 B (double-float read + write)
 * per element of every trailing triangle they update. */
int bd_kernel_bytes(bd_ctx* ctx, double* bytes);
/* Count of kernel launches issued by the last bd_step (graph nodes count once each). */
int bd_launch_count(bd_ctx* ctx, int* out);
/* Pivots replaced by |pivot| in the last factorisation (func.cpp:827-833). */
int bd_negative_pivots(bd_ctx* ctx, int* out);

/* ------------------------------------------------------- LH binding (host)
 * main.cpp:386-465 in three calls: bd_lh_mc decides (core n_b =
 * (int)(n_c u_core), at most n_c - 1, releases its linker histone when
 * u_random <= unbind or binds one when u_random <= Pbind; *changed = 1 if
 * the flag changed); bd_lh_rebind places the beads for the new flags (cores
 * bound before keep old_r_lh's beads, newly bound ones get the template
 * tpos [3 nlh] in their frame: build_LH, func.cpp:2029-2059, and
 * main.cpp:414-447), with the template from bd_system_lh_template; then
 * bd_set_lh_flags resizes the context. */
int bd_lh_mc(int n_c, double u_random, double u_core, double unbind, double Pbind, int* nc_lh_flag, int* changed);
int bd_lh_rebind(int n, const int* type, int n_c, const double* r, const double* a, const double* b, const double* c,
                 int nlh, const double* tpos, const double* trad, const int* old_flags, const double* old_r_lh,
                 const int* new_flags, double* new_r_lh, double* new_lh_rad);
int bd_system_lh_template(const bd_system* sys, double* pos, double* rad);

/* A context's current state (device) into rs's arrays, which must be
 * allocated for the context's sizes (bd_sizes); rs's sizes are set from the
 * context, rs->step and rs->nc_lh_flag are left to the caller. */
int bd_restart_from_context(bd_ctx* ctx, bd_restart* rs);

/* Linker-histone binding changed (main.cpp:386-465: every 100 steps one
 * core may bind or release its linker histone, which changes n_LH and the
 * size of D): the context is resized on the device for the new flags [n_c],
 * with r_lh [3 n_LH] the new LH bead positions (bound cores in order, as
 * main.cpp:418-447 builds them) and lh_rad [n_LH] their radii (NULL: the
 * radii of the first linker histone the context holds, repeated; 0.5 nm for
 * every bead when it holds none).  Nothing is reallocated and no
 * state leaves the device: bd_create sizes every binding-dependent buffer
 * (D, its factor, the LH arrays, the mirrors) for every core bound, and the
 * call uploads the new LH tables and beads, sets the logical sizes, and makes
 * the next step assemble and factor the tensor of the new size (its graph is
 * captured again).  The handle stays valid; sizes (bd_sizes) change.  Not
 * for contexts inside a batch. */
int bd_set_lh_flags(bd_ctx* ctx, const int* nc_lh_flag, const double* r_lh, const double* lh_rad);

/* ---------------------------------------------------------------- gradients
 * No counterpart in the reference (main.cpp runs the dynamics forward only).
 *
 * Rollout observable: starting from the context's state, n_steps steps of
 * bd_step with the caller's noise (rr: n_steps rows of 3n, p: n_steps rows
 * of 3 n_D, the bd_noise_step stream), then
 *   loss = mean over the final `window` states of |r_{n-1} - r_0|^2 + Rg,
 * r the chain beads (cores and linker DNA), Rg their radius of gyration.
 * The context's state and step counter are left as they were.  Requires
 * n_LH == 0 and frequency_RP == 1.
 *
 * bd_adjoint: loss and its gradient grad4 = d loss / d (h, g, s, lambda_D)
 * (stretch, bend, twist moduli; Debye length lambda_D = 1 / debye, with
 * debyell scaled alongside), by the reverse-mode pass of the step with
 * recomputation checkpointing: the state is kept every checkpoint_every
 * steps and each segment is recomputed during the backward sweep.  The
 * forward arithmetic is the context's (FP32-class on a BD_PREC_MIXED
 * context, FP64 otherwise); the adjoint runs in FP32 or FP64 accordingly. */
int bd_adjoint(bd_ctx* ctx, int n_steps, int checkpoint_every, int window, const double* rr, const double* p,
               double* loss, double* grad4);
/* The loss alone (the forward sweep of bd_adjoint). */
int bd_rollout_loss(bd_ctx* ctx, int n_steps, int window, const double* rr, const double* p, double* loss);
/* Set h, g, s and the Debye length (debye = 1 / lambda_D, debyell scaled by
 * the same factor) of a context, e.g. for finite differences. */
int bd_set_moduli(bd_ctx* ctx, double h, double g, double s, double debye_length);
/* Kernel launches issued by the last bd_adjoint (forward sweep excluded). */
int bd_adjoint_launches(bd_ctx* ctx, long* out);

#ifdef __cplusplus
}
#endif
#endif /* BD_CAPI_H */
