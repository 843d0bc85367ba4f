/*
 * les_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the
 * les-model per-time-step hot path.
 *
 * One context owns a device mirror of one reference Field (src/field.h:9-41)
 * plus the pressure system (StencilMatrix A and IC factor L,
 * src/pressure.h:17-29) and all solver work vectors, on one GPU and one CUDA
 * stream.  Every entry point below replaces one reference function; the
 * comment on each names it (file:line in the les-model sources).  Array
 * layout is the reference's: idx = i*ny*nz + j*nz + k (src/field.h:40).
 *
 * Conventions
 *  - All functions return an les_status; nothing throws across the ABI.
 *  - Calls are asynchronous on the context's stream unless they return a
 *    host scalar (dt, iteration counts, lambda), which synchronise.
 *  - Host buffers passed in are read before the call returns; host buffers
 *    passed out are complete when the call returns.
 *  - One context per host thread; contexts share nothing.
 */
#ifndef LES_GB300_H
#define LES_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LES_ABI_VERSION 1

typedef enum les_status {
    LES_OK = 0,
    LES_NOT_CONVERGED = 1, /* iteration cap reached (the reference warns on stderr) */
    LES_NONFINITE = 2,     /* a residual or scalar became NaN/Inf */
    LES_BAD_ARG = 3,
    LES_CUDA_ERROR = 4,    /* les_last_error() has the CUDA message */
    LES_NO_DEVICE = 5,
    LES_TIMEOUT = 6        /* a bounded device-side wait gave up */
} les_status;

/* Mirrors Mesh, src/field.h:6. */
typedef struct les_mesh {
    int nx, ny, nz;
    double dx, dy, dz;
} les_mesh;

typedef struct les_ctx les_ctx;

/* Device arrays of the reference Field (src/field.h:13-20) plus the PCG
 * right-hand side b that src/main.cpp:135 allocates every step. */
typedef enum les_slot {
    LES_U = 0, LES_V, LES_W, LES_U_NEW, LES_V_NEW, LES_W_NEW,
    LES_P, LES_P_RHS, LES_NU_T, LES_B,
    LES_NSLOTS
} les_slot;

/* Pressure solvers, chosen at run time (the reference selects them by
 * commenting lines out, src/main.cpp:131-138). */
typedef enum les_solver {
    LES_SOLVER_PCG = 0,      /* src/pressure.cpp:342-414 / :762-835 */
    LES_SOLVER_JACOBI = 1,   /* src/pressure.cpp:106-172 */
    LES_SOLVER_GS_SOR = 2    /* src/pressure.cpp:186-247 */
} les_solver;

typedef enum les_precond {
    LES_PC_JACOBI = 0,     /* apply_jacobi_preconditioner, src/pressure.cpp:420-428 */
    LES_PC_IC = 1,         /* apply_ic_preconditioner with L from build_ic_preconditioner */
    LES_PC_CHEBYSHEV = 2,  /* apply_chebyshev_preconditioner, src/pressure.cpp:851-906 */
    LES_PC_IC_A = 3        /* as shipped: apply_ic_preconditioner(..., A, ...), :363, :396 */
} les_precond;

typedef enum les_precision {
    LES_FP64 = 0,   /* the reference's arithmetic */
    LES_MIXED = 1   /* FP32 inner PCG inside FP64 defect correction */
} les_precision;

typedef struct les_pcg_opts {
    int precond;          /* les_precond */
    int max_iter;         /* FP64: PCG iterations (reference: 1000, src/main.cpp:137);
                             MIXED: cap on the total inner iterations */
    double tol;           /* absolute tolerance on ||b - A x||_2 (reference semantics) */
    double lambda_min, lambda_max; /* Chebyshev bounds */
    int degree;           /* Chebyshev polynomial degree (reference default 5) */
    int precision;        /* les_precision */
    double inner_rtol;    /* MIXED: inner FP32 solve reduces its residual by this */
    int inner_max_iter;   /* MIXED: cap per inner solve */
    int max_outer;        /* MIXED: cap on defect-correction sweeps */
} les_pcg_opts;

typedef struct les_pcg_result {
    int iters;            /* FP64: reference iteration count; MIXED: total inner iterations */
    int outer;            /* MIXED: defect-correction sweeps (0 for FP64) */
    double residual;      /* final ||b - A x||_2 in FP64 */
} les_pcg_result;

typedef struct les_step_params {
    double nu, rho, cs;             /* reference: 1e-5, 1.2 (src/main.cpp:83-84), 0.18 (:425) */
    double cfl_conv, cfl_visc, dt_max; /* reference: 0.4, 0.2, 1e-4 (src/main.cpp:210-212) */
    double dt_fixed;                /* > 0: use this dt instead of compute_adaptive_dt */
    int solver;                     /* les_solver */
    les_pcg_opts pcg;               /* for LES_SOLVER_PCG; tol is absolute unless rel_tol > 0 */
    double rel_tol;                 /* > 0: PCG tol = rel_tol * ||b||_2 of this step */
    int stat_max_iter;              /* Jacobi (reference 100) / GS-SOR sweeps (reference 200) */
    double stat_tol;                /* max |dp| stop criterion (reference 1e-6) */
    double omega;                   /* GS-SOR relaxation (reference 1.7) */
    int want_tau;                   /* also store the (unused) SGS stress tensor */
} les_step_params;

typedef struct les_step_stats {
    double dt;
    int iters;            /* solver iterations / sweeps */
    int outer;            /* MIXED defect-correction sweeps */
    double residual;      /* PCG: final ||r||_2 */
    double b_norm;        /* PCG: ||b||_2 */
    int status;           /* les_status of the solve */
} les_step_stats;

/* ---- context ----------------------------------------------------------- */
les_status les_create(const les_mesh* mesh, int device, les_ctx** out);
void les_destroy(les_ctx* ctx);
const char* les_last_error(const les_ctx* ctx);
const char* les_status_string(int status);
int les_abi_version(void);
les_status les_sync(les_ctx* ctx);
/* The context's cudaStream_t (as void*), for callers that order their own
 * work or CUDA events against the library's. */
void* les_stream(les_ctx* ctx);
/* Device pointer of a slot (valid until the next les_momentum, which swaps
 * U<->U_NEW etc., or les_destroy). */
double* les_slot_ptr(les_ctx* ctx, int slot);
uint8_t* les_mask_ptr(les_ctx* ctx);

/* ---- host <-> device (the shim's Field sync points) --------------------- */
les_status les_upload(les_ctx* ctx, int slot, const double* host);
les_status les_download(les_ctx* ctx, int slot, double* host);
/* Several slots in one call: one asynchronous copy per slot on the
 * context's stream, one synchronisation at the end (the host buffers are
 * free again when the call returns).  Pinned host buffers let the copies run
 * at the link's bandwidth. */
les_status les_upload_many(les_ctx* ctx, int count, const int* slots, const double* const* hosts);
les_status les_download_many(les_ctx* ctx, int count, const int* slots, double* const* hosts);
/* is_solid (src/field.h:22) as one byte per cell, 0 or 1. */
les_status les_upload_mask(les_ctx* ctx, const uint8_t* solid);
les_status les_download_mask(les_ctx* ctx, uint8_t* solid);

/* ---- step physics, src/main.cpp ---------------------------------------- */
/* compute_adaptive_dt, src/main.cpp:208-250 (constants as arguments). */
les_status les_adaptive_dt(les_ctx* ctx, double nu, double cfl_conv, double cfl_visc,
                           double dt_max, double* dt);
/* apply_velocity_BCs, src/main.cpp:323-410. */
les_status les_velocity_bcs(les_ctx* ctx);
/* compute_sgs_stress, src/main.cpp:423-472 (Cs is an argument; the
 * reference hard-codes 0.18 at :425).  Writes nu_t on interior cells. */
les_status les_sgs(les_ctx* ctx, double cs, int want_tau);
/* apply_nut_BCs, src/main.cpp:483-547. */
les_status les_nut_bcs(les_ctx* ctx);
/* compute_sgs_stress + apply_nut_BCs fused into one pass. */
les_status les_sgs_nut(les_ctx* ctx, double cs, int want_tau);
/* tau_xx, xy, xz, yy, yz, zz (6*N doubles) of the last les_sgs(want_tau=1). */
les_status les_download_tau(les_ctx* ctx, double* host6n);
/* solve_momentum, src/main.cpp:563-659, including the u<->u_new swap. */
les_status les_momentum(les_ctx* ctx, double dt, double nu);
/* correct_velocity, src/main.cpp:671-714. */
les_status les_correct_velocity(les_ctx* ctx, double dt, double rho);

/* ---- pressure, src/pressure.cpp ---------------------------------------- */
/* calculate_divergence(p_rhs, ...), src/pressure.cpp:256-329 (reads U_NEW..). */
les_status les_divergence(les_ctx* ctx, double dt, double rho);
/* build_b_vector(b, p_rhs, ...), src/pressure.cpp:566-599. */
les_status les_build_b(les_ctx* ctx);
/* apply_pressure_BCs, src/pressure.cpp:14-93. */
les_status les_pressure_bcs(les_ctx* ctx);
/* solve_pressure_jacobi, src/pressure.cpp:106-172 (reference: max_iter 100,
 * tol 1e-6).  *sweeps gets the number of sweeps run. */
les_status les_solve_jacobi(les_ctx* ctx, double dt, double rho, int max_iter, double tol,
                            int* sweeps);
/* solve_pressure_GS, src/pressure.cpp:186-247 (reference: omega 1.7, tol 1e-6),
 * in hyperplane order, which reproduces the lexicographic update sequence. */
les_status les_solve_gs(les_ctx* ctx, double dt, double rho, int max_iter, double omega,
                        double tol, int* sweeps);
/* build_stencil, src/pressure.cpp:608-699, from the mask uploaded now (the
 * reference builds A before defining the obstacle, src/main.cpp:66-81; the
 * caller reproduces that by calling this before les_upload_mask). */
les_status les_build_stencil(les_ctx* ctx);
/* Install an arbitrary 7-diagonal A (order c, n, s, e, w, t, b). */
les_status les_set_stencil(les_ctx* ctx, const double* const* diag7);
les_status les_get_stencil(les_ctx* ctx, double* const* diag7);
/* build_ic_preconditioner, src/pressure.cpp:495-556, from the current A. */
les_status les_build_ic(les_ctx* ctx);
les_status les_set_ic_factor(les_ctx* ctx, const double* const* diag7);
les_status les_get_ic_factor(les_ctx* ctx, double* const* diag7);
/* estimate_lambda_max, src/pressure.cpp:917-955.  v0: start vector (N
 * doubles) or NULL for std::mt19937(1337)/uniform(-1,1) drawn in index
 * order (the reference's draw on one thread). */
les_status les_lambda_max(les_ctx* ctx, int n_iter, const double* v0, double* lambda);
/* solve_pressure_pcg (src/pressure.cpp:342-414) and
 * solve_pressure_pcg_chebyshev (:762-835): solves A p = b in place in P. */
les_status les_pcg(les_ctx* ctx, const les_pcg_opts* opts, les_pcg_result* res);

/* ---- operators on slots ------------------------------------------------- */
/* fast_apply_laplacian, src/pressure.cpp:709-746: out = A in. */
les_status les_spmv(les_ctx* ctx, int in_slot, int out_slot);
/* The preconditioner of opts applied once: out = M^-1 in
 * (src/pressure.cpp:420-428, :442-482, :851-906).  With an IC preconditioner
 * the call waits for the wavefront and returns LES_TIMEOUT if one of its
 * bounded waits gave up. */
les_status les_precond_apply(les_ctx* ctx, const les_pcg_opts* opts, int in_slot, int out_slot);
/* parallel_dot, src/pressure.cpp:962-970. */
les_status les_dot(les_ctx* ctx, int a_slot, int b_slot, double* out);
/* out = a*in1 + b*in2: parallel_saxpy (src/pressure.cpp:995-1002), and
 * parallel_axpy (:983-989) with a = 1, in1 = out.  Slots may alias. */
les_status les_axpby(les_ctx* ctx, int out_slot, double a, int in1_slot, double b, int in2_slot);

/* Dot product of two device vectors that allocates nothing (no counterpart
 * in the reference).  For callers that cannot call cudaMalloc -- code running
 * under a memory pool or arena that owns the process's device allocations, or
 * a thread that must not take the allocator's locks mid-step.  a, b: device
 * arrays of n doubles; out: device pointer that receives the result; stream:
 * a cudaStream_t (NULL for the default stream); the call is asynchronous on
 * it.  Scratch is a fixed 512 KiB array in device memory, which caps n at
 * LES_NOALLOC_MAX_CELLS; larger n is rejected with LES_BAD_ARG and a message
 * on stderr.  CUDA loads the library's modules lazily, so the array is
 * reserved on a device by the FIRST call there (which also looks up its
 * address) and held until the process exits: make that first call during
 * set-up, before reserving the rest of the device's memory and before any
 * stream capture; later calls reserve nothing.  All calls share the scratch,
 * so calls that overlap on the GPU race. */
#define LES_NOALLOC_MAX_CELLS 134217728LL
les_status les_dot_noalloc(const double* a, const double* b, long long n, double* out, void* stream);

/* ---- batched ensemble (no reference counterpart) ------------------------ */
/* Many independent cases (each its own mesh, fields, matrix and solver
 * state) advanced together: one CUDA graph launch per time step runs every
 * case's whole step as an independent branch.  Set each case up through its
 * context (les_ensemble_case: upload fields and mask, build the matrix, ...);
 * the contexts belong to the ensemble. */
typedef struct les_ensemble les_ensemble;
les_status les_ensemble_create(const les_mesh* meshes, int count, int device, les_ensemble** out);
void les_ensemble_destroy(les_ensemble* ens);
int les_ensemble_size(const les_ensemble* ens);
les_ctx* les_ensemble_case(les_ensemble* ens, int i);
const char* les_ensemble_last_error(const les_ensemble* ens);
/* One time step of every case: prm[i] for case i (each must be the
 * mixed-precision fused PCG, Jacobi or Chebyshev, on a device-built
 * matrix).  stats (count entries, or NULL for no host sync) as les_step. */
les_status les_ensemble_step(les_ensemble* ens, const les_step_params* prm, les_step_stats* stats);
les_status les_ensemble_sync(les_ensemble* ens);

/* ---- statistics (src/statistics.cpp) ------------------------------------ */
/* init_statistics (:80-96): zeroes the ten device-resident sums. */
les_status les_stats_begin(les_ctx* ctx, int start_step);
/* update_statistics (:98-131): adds the current u, v, w, p (and their
 * products) when current_step > start_step; no host copy. */
les_status les_stats_update(les_ctx* ctx, int current_step);
/* The raw sums (u, v, w, p, uu, vv, ww, uv, uw, vw; entries may be NULL). */
les_status les_stats_sums(les_ctx* ctx, double* const* out10, int* samples);
/* finalize_and_save (:133-186) without the file: means u, v, w, p and the
 * stresses uu, vv, ww, uv, uw, vw into out10 (entries may be NULL). */
les_status les_stats_finalize(les_ctx* ctx, double* const* out10, int* samples);
/* finalize_and_save: the statistics file (write_statistics_vtk, :11-71). */
les_status les_stats_save_vtk(les_ctx* ctx, const char* path);

/* ---- files (src/io.cpp) ---------------------------------------------------- */
/* write_field_vtk (:225-256) of the context's fields into `path` (the
 * reference's name is output/output_<step>.vtk).  Asynchronous: the fields
 * are snapshot on the device, staged to pinned memory on a copy stream and
 * formatted on host threads while the caller continues; les_io_wait joins. */
les_status les_write_vtk(les_ctx* ctx, int step, const char* path);
/* save_state (:14-58) into dir/checkpoint.meta and dir/checkpoint.data (the
 * reference's dir is "checkpoint"), asynchronous like les_write_vtk.
 * with_unew = 1 also writes u_new, v_new, w_new to dir/checkpoint.unew (not
 * in the reference's format: it makes a resume exact). */
les_status les_save_state(les_ctx* ctx, const char* dir, double time_simulated, double dt, int next_step,
                          int with_unew);
/* Waits for the last asynchronous file; returns its status. */
les_status les_io_wait(les_ctx* ctx);
/* load_state (:73-120): *step = 0 when dir holds no checkpoint. */
les_status les_load_state(les_ctx* ctx, const char* dir, double* time_simulated, double* dt, int* step,
                          int with_unew);
/* The same formats from host arrays (no device involved). */
les_status les_format_field_vtk(const les_mesh* mesh, int step, const double* u, const double* v, const double* w,
                                const double* p, const double* nu_t, const uint8_t* solid, const char* path);
les_status les_format_stats_vtk(const les_mesh* mesh, const double* const* mean4, const double* const* stress6,
                                const char* path);
les_status les_write_checkpoint_files(const les_mesh* mesh, const double* const* fields5, const uint8_t* solid,
                                      double time_simulated, double dt, int next_step, const char* dir,
                                      const double* const* unew3);
les_status les_read_checkpoint_files(const les_mesh* mesh, const char* dir, double* const* fields5, uint8_t* solid,
                                     double* time_simulated, double* dt, int* step, double* const* unew3);

/* ---- adjoint (no reference counterpart) --------------------------------- */
/* Inlet u profile (ny*nz values, index j*nz+k) applied by the velocity
 * boundary conditions in place of the reference's uniform u = 1
 * (src/main.cpp:334-345); NULL restores the uniform inlet. */
les_status les_set_inlet(les_ctx* ctx, const double* u_in);

/* Gradient of J = (1/N) sum_{n=1..N} sum_{probe box} |U_n|^2 / 2 (U_n the
 * velocity after step n) with respect to the inlet profile and Cs, by the
 * discrete adjoint of the time step (hand-written transposes of the SGS,
 * momentum, divergence, projection and boundary-condition kernels; the
 * adjoint pressure solve reuses the PCG through the symmetrising scaling of
 * the matrix).  The forward starts from the context's current fields with the
 * velocity boundary conditions applied (so the initial inlet values are the
 * profile too), stores (u, v, w, p) every checkpoint_every steps, and the
 * backward recomputes each segment from its checkpoint. */
typedef struct les_adjoint_params {
    les_step_params step;   /* PCG (Jacobi or Chebyshev; FP64, or mixed with its FP64
                               defect correction for tight tolerances), dt_fixed > 0;
                               the adjoint solves use the same solver */
    int steps;              /* N */
    int checkpoint_every;   /* steps per checkpoint segment */
    int box[6];             /* probe box i0, i1, j0, j1, k0, k1 (half-open) */
    double adj_rel_tol;     /* adjoint pressure solves: relative residual */
} les_adjoint_params;
les_status les_adjoint_forward(les_ctx* ctx, const les_adjoint_params* prm, double* J);
/* grad_inlet: ny*nz values (dJ/du_in), grad_cs: dJ/dCs.  Leaves the fields
 * at the first checkpoint's recomputation (restore them to continue). */
les_status les_adjoint_backward(les_ctx* ctx, double* grad_inlet, double* grad_cs);
/* Tangent-linear model (FP64): the directional derivative dJ along
 * (d_inlet, d_cs) by forward differentiation of the same steps from the first
 * checkpoint; with the backward's gradient g it must satisfy
 * dJ = g . d_inlet + grad_cs * d_cs (the dot-product test).  d_inlet may be
 * NULL.  Leaves the fields at step N. */
les_status les_adjoint_tangent(les_ctx* ctx, const double* d_inlet, double d_cs, double* dJ);

/* ---- autotuner (no reference counterpart) ------------------------------- */
/* Times the fused inner passes of the mixed-precision PCG for opts on the
 * context's current matrix over candidate strip shapes and march chunk
 * lengths (LES_OPT_ROWS_A/B, LES_OPT_CHUNK_A/B), with `share` the fraction
 * of the GPU the context gets while it runs (1 alone, 1/k beside k-1 other
 * cases), and sets the fastest.  best_us (optional) receives the time of one
 * inner iteration with the chosen shape.  The solver's work vectors are
 * overwritten; fields and matrix are not touched. */
les_status les_autotune(les_ctx* ctx, const les_pcg_opts* opts, double share, double* best_us);
/* The same over all cases of an ensemble at once (every case runs its
 * candidate concurrently, as in a step), choosing one setting per case
 * from the total time. */
les_status les_ensemble_autotune(les_ensemble* ens, const les_pcg_opts* opts, double* best_us);
/* In the batched form (les_ensemble_set_batched, default) les_ensemble_autotune
 * chooses instead how finely the batched passes split the cases' marches:
 * items up to `split` times the GPU's resident warps (2, 3, 4 or 6; 4 before
 * tuning), timed as batched inner iterations over all cases; best_us is then
 * the time of one such iteration.  This returns the split in use. */
int les_ensemble_batch_split(const les_ensemble* ens);
/* 1 (default): the cases' mixed-precision solves run batched -- every inner
 * pass, defect and update is one kernel over all cases, and the solver loops
 * run while any case iterates (used when all cases run the register-column
 * passes with one preconditioner; otherwise, and with 0, each case's step is
 * its own branch of the step graph). */
les_status les_ensemble_set_batched(les_ensemble* ens, int on);

/* ---- options (no reference counterpart) --------------------------------- */
typedef enum les_option {
    LES_OPT_FUSED = 0,  /* mixed-precision inner iteration (Jacobi, Chebyshev degree
                           2..7) as two fused passes: 1 (default) register-column
                           marches (device-built matrix; stored matrices use 2);
                           2 shared-memory tiles; 0: one kernel per vector operation */
    LES_OPT_TMA = 1,    /* 1: the shared-memory tile passes, with their planes staged
                           by TMA when nz % 16 == 0 and the matrix is device-built;
                           0 (default): no TMA */
    /* shape of the register-column passes (0 = built-in choice; les_autotune
       sets them by timing): */
    LES_OPT_ROWS_A = 2,   /* rows per strip of pass A: 8 or 16 */
    LES_OPT_ROWS_B = 3,   /* rows per strip of pass B: 16 (Jacobi), 4 or 8
                             (Chebyshev degree 2..4), 4 (degree 5..7) */
    LES_OPT_CHUNK_A = 4,  /* planes per march chunk of pass A */
    LES_OPT_CHUNK_B = 5,  /* planes per march chunk of pass B */
    LES_OPT_GRAPH = 6,    /* 1 (default): les_step with the mixed-precision fused PCG
                             runs as one CUDA graph launch (captured per velocity
                             buffer parity, both solver loops as conditional nodes;
                             not while les_profile records); 0: launch by launch */
    LES_OPT_PDL = 7,      /* 1 (default; 0 for ensemble cases): the register-column
                             passes are launched as programmatic dependents of the
                             kernel before them (their blocks become resident while it
                             drains); 0: plain stream order */
    LES_OPT_PHYS32 = 8,   /* 1 (default): a les_step whose pressure solve is the
                             mixed-precision PCG computes nu_t and the momentum update
                             in FP32 (FP64 fields, FP64 velocity update; not with
                             want_tau); 0: the reference-order FP64 kernels */
    LES_OPT_TEST_STALL = 9, /* test hook, 0 (default) off.  1: the first tile of the
                             IC(0) and GS-SOR wavefronts withholds its progress, so
                             the tiles after it wait in vain until their bounded wait
                             (about 2 s) gives up; the solve then returns LES_TIMEOUT
                             and the context stays usable.  For testing the failure
                             path only. */
    LES_OPT_COL_STRIDE = 10 /* 1 (default): the register-column passes of a grid with
                             nz = 32, 64, 128 or 256 run kernels compiled for that row
                             stride (row offsets as immediates); 0: the kernels that
                             read the stride at run time.  Same results either way. */
} les_option;
les_status les_set_option(les_ctx* ctx, int option, int value);
/* The current value of an option: the last one set, the default, or for the
 * strip shapes (LES_OPT_ROWS_A/B, LES_OPT_CHUNK_A/B) what les_autotune chose
 * (0 = the built-in choice). */
les_status les_get_option(const les_ctx* ctx, int option, int* value);

/* ---- accounting (no reference counterpart) ------------------------------ */
/* Number of kernels this context has launched so far. */
unsigned long long les_launch_count(const les_ctx* ctx);
/* CUDA-event timing of the solver's hot kernels: enable=1 starts a fresh
 * record, 0 stops recording. */
les_status les_profile(les_ctx* ctx, int enable);
/* Launch count and summed device time (ms) of one profiled kernel id
 * (0..7, names from les_profile_name). */
les_status les_profile_read(les_ctx* ctx, int kernel_id, int* launches, double* total_ms);
const char* les_profile_name(int kernel_id);
/* Measured FP64 arithmetic rate of the context's GPU: independent multiply
 * and add chains (one DMUL + one DADD per a*b+c, as the reference-order FP64
 * kernels execute them), best of three timed launches; *ops_per_s counts
 * each multiply and each add.  The denominator of the FP64 path's roofline. */
les_status les_fp64_rate(les_ctx* ctx, double* ops_per_s);
/* Records CUDA event slot `mark` (0..63) on the context's stream. */
les_status les_mark(les_ctx* ctx, int mark);
/* Device time between two recorded marks, in ms (waits for mark1). */
les_status les_elapsed(les_ctx* ctx, int mark0, int mark1, double* ms);

/* ---- one full time step, src/main.cpp:115-144 --------------------------- */
les_status les_step(les_ctx* ctx, const les_step_params* prm, les_step_stats* stats);
/* One step with host fields, for a host that keeps its fields in host memory
 * (the drop-in use of src/main.cpp:108-165): the n_in host arrays are
 * uploaded into their slots, the step runs, and the n_out slots are
 * downloaded -- the result of les_upload_many + les_step +
 * les_download_many, bit for bit.  With the PCG solver the downloads of
 * LES_U_NEW/V_NEW/W_NEW, LES_NU_T and LES_P_RHS, final before the pressure
 * solve, overlap it (from a second stream, released by an event after the
 * step's physics); the rest follow the step.  Host arrays should be pinned.
 * step_ms (optional): the step's own device time, CUDA events on the
 * context's stream around it (not the copies).  Returns after the last
 * download. */
les_status les_step_io(les_ctx* ctx, const les_step_params* prm, les_step_stats* stats, int n_in,
                       const int* in_slots, const double* const* in_hosts, int n_out, const int* out_slots,
                       double* const* out_hosts, double* step_ms);

#ifdef __cplusplus
}
#endif
#endif
