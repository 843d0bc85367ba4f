/*
 * les_oracle.h -- CPU oracle for the les-model per-time-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithms (les-model src/main.cpp and src/pressure.cpp), used as the
 * checker for the CUDA path and as the CPU baseline in bench.py.  It is never
 * linked into, loaded by or called from the product library.
 *
 * Layout follows the reference Field (src/field.h:40): idx = i*ny*nz + j*nz + k,
 * k contiguous.  The reference's std::vector<bool> is_solid becomes one uint8
 * (0/1) per cell.  The StencilMatrix (src/pressure.h:17-29) becomes seven
 * separate double arrays.
 *
 * Threading: loops the reference runs under `omp parallel for` carry the same
 * pragma here.  Reductions (dot/norm) use `reduction(+:...)` like
 * src/pressure.cpp:962-970, so with one thread they are a plain left-to-right
 * sum, bit-identical to the reference built with OMP_NUM_THREADS=1.
 */
#ifndef LES_ORACLE_H
#define LES_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { int nx, ny, nz; double dx, dy, dz; } lo_mesh;

/* Seven-diagonal stencil, one array each (src/pressure.h:17-29). */
typedef struct {
    double *c, *n, *s, *e, *w, *t, *b;
} lo_stencil;

enum { LO_PC_JACOBI = 0, LO_PC_IC = 1, LO_PC_CHEB = 2, LO_PC_NONE = 3 };

void   lo_set_threads(int n);
int    lo_get_threads(void);

/* --- BLAS-1 helpers, src/pressure.cpp:962-1013 --- */
double lo_dot(int64_t n, const double* a, const double* b);
double lo_norm(int64_t n, const double* a);
void   lo_axpy(int64_t n, double* out, double a, const double* in);
void   lo_saxpy(int64_t n, double* out, double a, const double* in1, double b, const double* in2);
void   lo_copy(int64_t n, double* out, const double* in);

/* --- step physics, src/main.cpp --- */
double lo_compute_adaptive_dt(const lo_mesh* m, const double* u, const double* v, const double* w,
                              const double* nu_t, double nu, double cfl_conv, double cfl_visc,
                              double dt_max);
void   lo_define_obstacle_mask(const lo_mesh* m, uint8_t* solid);
void   lo_apply_velocity_bcs(const lo_mesh* m, double* u, double* v, double* w, const uint8_t* solid);
double lo_smagorinsky_coef(const lo_mesh* m, double cs);
void   lo_compute_sgs(const lo_mesh* m, double cs_delta_sq, const double* u, const double* v,
                      const double* w, double* nu_t, double* tau /* 6*N or NULL */);
void   lo_apply_nut_bcs(const lo_mesh* m, double* nu_t, const uint8_t* solid);
void   lo_solve_momentum(const lo_mesh* m, double dt, double nu, const double* u, const double* v,
                         const double* w, const double* nu_t, double* u_new, double* v_new,
                         double* w_new);
void   lo_correct_velocity(const lo_mesh* m, double dt, double rho, const double* p, double* u,
                           double* v, double* w);

/* --- pressure, src/pressure.cpp --- */
void   lo_apply_pressure_bcs(const lo_mesh* m, double* p, const uint8_t* solid);
int    lo_solve_jacobi(const lo_mesh* m, double dt, double rho, const double* u, const double* v,
                       const double* w, double* p, const uint8_t* solid, int max_iter, double tol);
int    lo_solve_gs(const lo_mesh* m, double dt, double rho, const double* u, const double* v,
                   const double* w, double* p, const uint8_t* solid, int max_iter, double omega,
                   double tol);
void   lo_calculate_divergence(const lo_mesh* m, double dt, double rho, const double* u_new,
                               const double* v_new, const double* w_new, const uint8_t* solid,
                               double* rhs);
void   lo_build_b(const lo_mesh* m, const double* div, const uint8_t* solid, double* b);
void   lo_build_stencil(const lo_mesh* m, const uint8_t* solid, lo_stencil* A);
void   lo_spmv(const lo_mesh* m, const lo_stencil* A, const double* p, double* q);
void   lo_jacobi_precond(int64_t n, const lo_stencil* A, const double* r, double* z);
void   lo_ic_build(const lo_mesh* m, const lo_stencil* A, lo_stencil* L);
void   lo_ic_apply(const lo_mesh* m, const lo_stencil* L, const double* r, double* z);
void   lo_cheb_apply(const lo_mesh* m, const lo_stencil* A, double lmin, double lmax, int degree,
                     const double* r, double* z, double* work_p, double* work_res);
double lo_lambda_max(const lo_mesh* m, const lo_stencil* A, const double* v0, int n_iter,
                     double* work_v, double* work_w);
/* PCG, src/pressure.cpp:342-414 (and :762-835 for pc=LO_PC_CHEB).  pc selects
 * the preconditioner; for LO_PC_IC, L holds the factor (pass A itself for the
 * as-shipped behaviour).  work: 4*N doubles.  Returns the iteration count with
 * the reference's conventions (0 if already converged, max_iter if not). */
int    lo_pcg(const lo_mesh* m, const lo_stencil* A, const double* b, double* x, int pc,
              const lo_stencil* L, double lmin, double lmax, int degree, int max_iter, double tol,
              double* work, double* final_norm);

/* --- one full time step, src/main.cpp:108-165 (without I/O and statistics) --- */
typedef struct {
    double nu, rho, cs, cfl_conv, cfl_visc, dt_max;
    int    solver;       /* 0 PCG, 1 stationary Jacobi, 2 GS-SOR */
    int    pc;           /* LO_PC_* for PCG */
    int    max_iter;
    double tol;          /* absolute tolerance (PCG) */
    double rel_tol;      /* >0: tol = rel_tol*||b|| each step */
    double omega;        /* GS-SOR */
    double lmin, lmax;   /* Chebyshev */
    int    degree;
    double dt_fixed;     /* >0: use this dt instead of compute_adaptive_dt */
} lo_step_params;

typedef struct {
    double *u, *v, *w, *u_new, *v_new, *w_new, *p, *p_rhs, *nu_t;
    uint8_t* solid;
} lo_field;

/* Advances one step in place; swaps u<->u_new like src/main.cpp:656-658 by
 * swapping the pointers inside *f.  Returns solver iterations; *dt_out gets dt. */
int    lo_step(const lo_mesh* m, lo_field* f, const lo_stencil* A, const lo_stencil* L,
               const lo_step_params* prm, double* b_work, double* pcg_work, double* dt_out);

/* src/statistics.cpp:98-131: sums[10] = u, v, w, p, uu, vv, ww, uv, uw, vw */
void   lo_stats_update(int64_t n, const double* u, const double* v, const double* w, const double* p,
                       double* const* sums);
/* src/statistics.cpp:133-186 (without the file): out[10] = means of u, v, w,
 * p and the stresses uu, vv, ww, uv, uw, vw */
void   lo_stats_finalize(int64_t n, int samples, const double* const* sums, double* const* out);

#ifdef __cplusplus
}
#endif
#endif
