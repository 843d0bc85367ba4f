/*
 * les_oracle.c -- CPU oracle for the les-model per-time-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path (tests/), the
 * smoke check and the CPU-baseline leg of bench.py.  The product library
 * never links or calls this file.
 *
 * Every function restates one reference function, cited by file:line of the
 * les-model sources, keeping the reference's floating-point operation order
 * (no FMA: this file is compiled with -ffp-contract=off, matching the
 * reference's x86-64 -O2 build which has no FMA instructions available).
 * Deviations from the reference, all intentional and behaviour-preserving:
 *   - is_solid is one uint8 per cell instead of std::vector<bool>;
 *   - the caller owns every buffer (the reference allocates temporaries in
 *     src/pressure.cpp:111-112, :191, :348-351, :859-860, :922-923);
 *   - the Chebyshev/PCG functions take the preconditioner as an argument
 *     instead of having it chosen by commented-out lines (src/main.cpp:131-138,
 *     src/pressure.cpp:362-363);
 *   - the lambda_max start vector is an input (the reference fills it from a
 *     shared std::mt19937 inside an omp loop, src/pressure.cpp:926-931, which
 *     races for more than one thread).
 */
#include "les_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(i, j, k) ((int64_t)(i) * ny * nz + (int64_t)(j) * nz + (k))

void lo_set_threads(int n)
{
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int lo_get_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* BLAS-1, src/pressure.cpp:962-1013                                         */
/* ------------------------------------------------------------------------ */

/* src/pressure.cpp:962-970 */
double lo_dot(int64_t n, const double* a, const double* b)
{
    double sum = 0.0;
#pragma omp parallel for reduction(+ : sum)
    for (int64_t i = 0; i < n; ++i) sum += a[i] * b[i];
    return sum;
}

/* src/pressure.cpp:975-978 */
double lo_norm(int64_t n, const double* a) { return sqrt(lo_dot(n, a, a)); }

/* src/pressure.cpp:983-989: out += a*in */
void lo_axpy(int64_t n, double* out, double a, const double* in)
{
#pragma omp parallel for
    for (int64_t i = 0; i < n; ++i) out[i] += a * in[i];
}

/* src/pressure.cpp:995-1002: out = a*in1 + b*in2 (out may alias in2) */
void lo_saxpy(int64_t n, double* out, double a, const double* in1, double b, const double* in2)
{
#pragma omp parallel for
    for (int64_t i = 0; i < n; ++i) out[i] = a * in1[i] + b * in2[i];
}

/* src/pressure.cpp:1007-1012 */
void lo_copy(int64_t n, double* out, const double* in)
{
#pragma omp parallel for
    for (int64_t i = 0; i < n; ++i) out[i] = in[i];
}

/* ------------------------------------------------------------------------ */
/* Step physics, src/main.cpp                                                */
/* ------------------------------------------------------------------------ */

/* src/main.cpp:208-250, with the three constants as arguments (the reference
 * hard-codes CFL_CONV=0.4, CFL_VISC=0.2, DT_MAX=1e-4 at :210-212). */
double lo_compute_adaptive_dt(const lo_mesh* m, const double* u, const double* v, const double* w,
                              const double* nu_t, double nu, double cfl_conv, double cfl_visc,
                              double dt_max)
{
    const int64_t n = (int64_t)m->nx * m->ny * m->nz;
    double u_max_sq = 0.0;
#pragma omp parallel for reduction(max : u_max_sq)
    for (int64_t i = 0; i < n; ++i) {
        double mag_sq = u[i] * u[i] + v[i] * v[i] + w[i] * w[i];
        u_max_sq = (u_max_sq < mag_sq) ? mag_sq : u_max_sq;
    }
    double u_max = sqrt(u_max_sq);
    double min_dx = m->dx;
    if (m->dy < min_dx) min_dx = m->dy;
    if (m->dz < min_dx) min_dx = m->dz;
    double dt_conv = DBL_MAX;
    if (u_max > 1e-12) dt_conv = cfl_conv * min_dx / u_max;
    double nu_t_max = 0.0;
#pragma omp parallel for reduction(max : nu_t_max)
    for (int64_t i = 0; i < n; ++i) nu_t_max = (nu_t_max < nu_t[i]) ? nu_t[i] : nu_t_max;
    double min_dx_sq = min_dx * min_dx;
    double dt_visc = cfl_visc * min_dx_sq / (nu + nu_t_max);
    double r = dt_conv;
    if (dt_visc < r) r = dt_visc;
    if (dt_max < r) r = dt_max;
    return r;
}

/* src/main.cpp:256-313: the reference's two boxes. */
void lo_define_obstacle_mask(const lo_mesh* m, uint8_t* solid)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    int box[2][6] = {
        {nx / 5, nx / 4, ny * 2 / 5, ny * 3 / 5, nz * 2 / 5, nz * 3 / 5},
        {nx / 5 + nx / 2, (int)(nx / 4.5 + nx / 2), ny * 2 / 5, ny * 3 / 5, nz * 2 / 5, nz * 4 / 5},
    };
    for (int b = 0; b < 2; ++b)
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j)
                for (int k = 0; k < nz; ++k)
                    if (i >= box[b][0] && i < box[b][1] && j >= box[b][2] && j < box[b][3] &&
                        k >= box[b][4] && k < box[b][5])
                        solid[IDX(i, j, k)] = 1;
}

/* src/main.cpp:323-410, phases in the reference's order. */
void lo_apply_velocity_bcs(const lo_mesh* m, double* u, double* v, double* w, const uint8_t* solid)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    /* inlet i=0, Dirichlet u=1, skipping solid cells (:334-345) */
    for (int j = 0; j < ny; ++j)
        for (int k = 0; k < nz; ++k) {
            int64_t id = IDX(0, j, k);
            if (solid[id]) continue;
            u[id] = 1.0; v[id] = 0.0; w[id] = 0.0;
        }
    /* outlet i=nx-1, zero gradient (:348-360) */
    for (int j = 0; j < ny; ++j)
        for (int k = 0; k < nz; ++k) {
            int64_t a = IDX(nx - 1, j, k), b = IDX(nx - 2, j, k);
            u[a] = u[b]; v[a] = v[b]; w[a] = w[b];
        }
    /* y walls (:364-377) */
    for (int i = 0; i < nx; ++i)
        for (int k = 0; k < nz; ++k) {
            int64_t a = IDX(i, 0, k), b = IDX(i, ny - 1, k);
            u[a] = 0.0; v[a] = 0.0; w[a] = 0.0;
            u[b] = 0.0; v[b] = 0.0; w[b] = 0.0;
        }
    /* z walls (:381-392) */
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j) {
            int64_t a = IDX(i, j, 0), b = IDX(i, j, nz - 1);
            u[a] = 0.0; v[a] = 0.0; w[a] = 0.0;
            u[b] = 0.0; v[b] = 0.0; w[b] = 0.0;
        }
    /* interior obstacle overwrite (:395-409) */
#pragma omp parallel for
    for (int i = 1; i < nx - 1; ++i)
        for (int j = 1; j < ny - 1; ++j)
            for (int k = 1; k < nz - 1; ++k) {
                int64_t id = IDX(i, j, k);
                if (solid[id]) { u[id] = 0.0; v[id] = 0.0; w[id] = 0.0; }
            }
}

/* pow(Cs*delta, 2) with delta = pow(dx*dy*dz, 1/3), src/main.cpp:425-426, :461 */
double lo_smagorinsky_coef(const lo_mesh* m, double cs)
{
    double delta = pow(m->dx * m->dy * m->dz, 1.0 / 3.0);
    return pow(cs * delta, 2);
}

/* src/main.cpp:423-472 (interior cells only; tau optional: the reference
 * writes it but nothing reads it). */
void lo_compute_sgs(const lo_mesh* m, double cs_delta_sq, const double* u, const double* v,
                    const double* w, double* nu_t, double* tau)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    const int64_t n = (int64_t)nx * ny * nz;
    const double dx = m->dx, dy = m->dy, dz = m->dz;
#pragma omp parallel for
    for (int i = 1; i < nx - 1; i++)
        for (int j = 1; j < ny - 1; j++)
            for (int k = 1; k < nz - 1; k++) {
                int64_t id = IDX(i, j, k);
                double du_dx = (u[IDX(i + 1, j, k)] - u[IDX(i - 1, j, k)]) / (2 * dx);
                double du_dy = (u[IDX(i, j + 1, k)] - u[IDX(i, j - 1, k)]) / (2 * dy);
                double du_dz = (u[IDX(i, j, k + 1)] - u[IDX(i, j, k - 1)]) / (2 * dz);
                double dv_dx = (v[IDX(i + 1, j, k)] - v[IDX(i - 1, j, k)]) / (2 * dx);
                double dv_dy = (v[IDX(i, j + 1, k)] - v[IDX(i, j - 1, k)]) / (2 * dy);
                double dv_dz = (v[IDX(i, j, k + 1)] - v[IDX(i, j, k - 1)]) / (2 * dz);
                double dw_dx = (w[IDX(i + 1, j, k)] - w[IDX(i - 1, j, k)]) / (2 * dx);
                double dw_dy = (w[IDX(i, j + 1, k)] - w[IDX(i, j - 1, k)]) / (2 * dy);
                double dw_dz = (w[IDX(i, j, k + 1)] - w[IDX(i, j, k - 1)]) / (2 * dz);
                double Sxx = du_dx, Syy = dv_dy, Szz = dw_dz;
                double Sxy = 0.5 * (du_dy + dv_dx);
                double Sxz = 0.5 * (du_dz + dw_dx);
                double Syz = 0.5 * (dv_dz + dw_dy);
                double Smag = sqrt(2.0 * (Sxx * Sxx + Syy * Syy + Szz * Szz) +
                                   4.0 * (Sxy * Sxy + Sxz * Sxz + Syz * Syz));
                double nt = cs_delta_sq * Smag;
                nu_t[id] = nt;
                if (tau) {
                    tau[0 * n + id] = -2.0 * nt * Sxx;
                    tau[1 * n + id] = -2.0 * nt * Sxy;
                    tau[2 * n + id] = -2.0 * nt * Sxz;
                    tau[3 * n + id] = -2.0 * nt * Syy;
                    tau[4 * n + id] = -2.0 * nt * Syz;
                    tau[5 * n + id] = -2.0 * nt * Szz;
                }
            }
}

/* src/main.cpp:483-547, phases in order. */
void lo_apply_nut_bcs(const lo_mesh* m, double* nu_t, const uint8_t* solid)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    for (int j = 0; j < ny; ++j)
        for (int k = 0; k < nz; ++k) nu_t[IDX(0, j, k)] = 0.0;
    for (int j = 0; j < ny; ++j)
        for (int k = 0; k < nz; ++k) nu_t[IDX(nx - 1, j, k)] = nu_t[IDX(nx - 2, j, k)];
    for (int i = 0; i < nx; ++i)
        for (int k = 0; k < nz; ++k) { nu_t[IDX(i, 0, k)] = 0.0; nu_t[IDX(i, ny - 1, k)] = 0.0; }
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j) { nu_t[IDX(i, j, 0)] = 0.0; nu_t[IDX(i, j, nz - 1)] = 0.0; }
#pragma omp parallel for
    for (int i = 1; i < nx - 1; ++i)
        for (int j = 1; j < ny - 1; ++j)
            for (int k = 1; k < nz - 1; ++k)
                if (solid[IDX(i, j, k)]) nu_t[IDX(i, j, k)] = 0.0;
}

/* src/main.cpp:563-659, interior only; the caller performs the swap of
 * :656-658. */
void lo_solve_momentum(const lo_mesh* m, double dt, double nu, const double* u, const double* v,
                       const double* w, const double* nu_t, double* u_new, double* v_new,
                       double* w_new)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    const double inv_dx2 = 1.0 / (m->dx * m->dx);
    const double inv_dy2 = 1.0 / (m->dy * m->dy);
    const double inv_dz2 = 1.0 / (m->dz * m->dz);
    const double inv_2dx = 1.0 / (2.0 * m->dx);
    const double inv_2dy = 1.0 / (2.0 * m->dy);
    const double inv_2dz = 1.0 / (2.0 * m->dz);
    const double* comp[3] = {u, v, w};
    double* outc[3] = {u_new, v_new, w_new};
    for (int c = 0; c < 3; ++c) {
        const double* f = comp[c];
        double* o = outc[c];
#pragma omp parallel for
        for (int i = 1; i < nx - 1; ++i)
            for (int j = 1; j < ny - 1; ++j)
                for (int k = 1; k < nz - 1; ++k) {
                    int64_t id = IDX(i, j, k);
                    double nu_eff = nu + nu_t[id];
                    double fe = f[IDX(i + 1, j, k)], fw = f[IDX(i - 1, j, k)];
                    double fn = f[IDX(i, j + 1, k)], fs = f[IDX(i, j - 1, k)];
                    double ft = f[IDX(i, j, k + 1)], fb = f[IDX(i, j, k - 1)];
                    double fc = f[id];
                    double d_dx = (fe - fw) * inv_2dx;
                    double d_dy = (fn - fs) * inv_2dy;
                    double d_dz = (ft - fb) * inv_2dz;
                    double adv = u[id] * d_dx + v[id] * d_dy + w[id] * d_dz;
                    double lap = (fe - 2 * fc + fw) * inv_dx2 + (fn - 2 * fc + fs) * inv_dy2 +
                                 (ft - 2 * fc + fb) * inv_dz2;
                    o[id] = fc + dt * (-adv + nu_eff * lap);
                }
    }
}

/* src/main.cpp:671-714 */
void lo_correct_velocity(const lo_mesh* m, double dt, double rho, const double* p, double* u,
                         double* v, double* w)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    const double dt_over_rho = dt / rho;
    const double inv_2dx = 1.0 / (2.0 * m->dx);
    const double inv_2dy = 1.0 / (2.0 * m->dy);
    const double inv_2dz = 1.0 / (2.0 * m->dz);
#pragma omp parallel for
    for (int i = 1; i < nx - 1; ++i)
        for (int j = 1; j < ny - 1; ++j)
            for (int k = 1; k < nz - 1; ++k) {
                int64_t id = IDX(i, j, k);
                u[id] -= dt_over_rho * ((p[IDX(i + 1, j, k)] - p[IDX(i - 1, j, k)]) * inv_2dx);
                v[id] -= dt_over_rho * ((p[IDX(i, j + 1, k)] - p[IDX(i, j - 1, k)]) * inv_2dy);
                w[id] -= dt_over_rho * ((p[IDX(i, j, k + 1)] - p[IDX(i, j, k - 1)]) * inv_2dz);
            }
}

/* ------------------------------------------------------------------------ */
/* Pressure, src/pressure.cpp                                                */
/* ------------------------------------------------------------------------ */

/* src/pressure.cpp:14-93 */
void lo_apply_pressure_bcs(const lo_mesh* m, double* p, const uint8_t* solid)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    const int64_t si = (int64_t)ny * nz, sj = nz;
    for (int j = 0; j < ny; ++j)
        for (int k = 0; k < nz; ++k) p[IDX(0, j, k)] = p[IDX(1, j, k)];
    for (int j = 0; j < ny; ++j)
        for (int k = 0; k < nz; ++k) p[IDX(nx - 1, j, k)] = 0.0;
    for (int i = 0; i < nx; ++i)
        for (int k = 0; k < nz; ++k) {
            p[IDX(i, 0, k)] = p[IDX(i, 1, k)];
            p[IDX(i, ny - 1, k)] = p[IDX(i, ny - 2, k)];
        }
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j) {
            p[IDX(i, j, 0)] = p[IDX(i, j, 1)];
            p[IDX(i, j, nz - 1)] = p[IDX(i, j, nz - 2)];
        }
#pragma omp parallel for
    for (int i = 1; i < nx - 1; ++i)
        for (int j = 1; j < ny - 1; ++j)
            for (int k = 1; k < nz - 1; ++k) {
                int64_t id = IDX(i, j, k);
                if (!solid[id]) continue;
                if (!solid[id + si]) p[id] = p[id + si];
                else if (!solid[id - si]) p[id] = p[id - si];
                else if (!solid[id + sj]) p[id] = p[id + sj];
                else if (!solid[id - sj]) p[id] = p[id - sj];
                else if (!solid[id + 1]) p[id] = p[id + 1];
                else if (!solid[id - 1]) p[id] = p[id - 1];
            }
}

/* Interior RHS (rho/dt)*div(u) with central differences, shared by the two
 * stationary solvers (src/pressure.cpp:119-132 and :197-210). */
static void stationary_rhs(const lo_mesh* m, double coef, const double* u, const double* v,
                           const double* w, double* rhs)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
#pragma omp parallel for
    for (int i = 1; i < nx - 1; ++i)
        for (int j = 1; j < ny - 1; ++j)
            for (int k = 1; k < nz - 1; ++k) {
                double div = (u[IDX(i + 1, j, k)] - u[IDX(i - 1, j, k)]) / (2 * m->dx) +
                             (v[IDX(i, j + 1, k)] - v[IDX(i, j - 1, k)]) / (2 * m->dy) +
                             (w[IDX(i, j, k + 1)] - w[IDX(i, j, k - 1)]) / (2 * m->dz);
                rhs[IDX(i, j, k)] = coef * div;
            }
}

/* src/pressure.cpp:106-172.  Returns the number of sweeps performed (the
 * reference returns void).  max_iter/tol are 100/1e-6 in the reference. */
int lo_solve_jacobi(const lo_mesh* m, double dt, double rho, const double* u, const double* v,
                    const double* w, double* p, const uint8_t* solid, int max_iter, double tol)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    const int64_t n = (int64_t)nx * ny * nz;
    double* rhs = (double*)calloc((size_t)n, sizeof(double));
    double* pn = (double*)calloc((size_t)n, sizeof(double));
    double* cur = p;
    double* nxt = pn;
    const double dx2 = m->dx * m->dx, dy2 = m->dy * m->dy, dz2 = m->dz * m->dz;
    const double denom = 2 * (1.0 / dx2 + 1.0 / dy2 + 1.0 / dz2);
    stationary_rhs(m, rho / dt, u, v, w, rhs);
    int it_done = max_iter;
    for (int iter = 0; iter < max_iter; ++iter) {
        double maxr = 0.0;
#pragma omp parallel for reduction(max : maxr)
        for (int i = 1; i < nx - 1; ++i)
            for (int j = 1; j < ny - 1; ++j)
                for (int k = 1; k < nz - 1; ++k) {
                    int64_t id = IDX(i, j, k);
                    double p_old = cur[id];
                    nxt[id] = ((cur[IDX(i + 1, j, k)] + cur[IDX(i - 1, j, k)]) / dx2 +
                               (cur[IDX(i, j + 1, k)] + cur[IDX(i, j - 1, k)]) / dy2 +
                               (cur[IDX(i, j, k + 1)] + cur[IDX(i, j, k - 1)]) / dz2 - rhs[id]) /
                              denom;
                    double res = fabs(nxt[id] - p_old);
                    if (res > maxr) maxr = res;
                }
        double* t = cur; cur = nxt; nxt = t;   /* f.p.swap(p_new), :160 */
        lo_apply_pressure_bcs(m, cur, solid);
        if (maxr < tol) { it_done = iter + 1; break; }
    }
    if (cur != p) memcpy(p, cur, (size_t)n * sizeof(double));
    free(rhs);
    free(pn);
    return it_done;
}

/* src/pressure.cpp:186-247 (serial lexicographic SOR).  Returns sweeps. */
int lo_solve_gs(const lo_mesh* m, double dt, double rho, const double* u, const double* v,
                const double* w, double* p, const uint8_t* solid, int max_iter, double omega,
                double tol)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    const int64_t n = (int64_t)nx * ny * nz;
    double* rhs = (double*)calloc((size_t)n, sizeof(double));
    const double dx2 = m->dx * m->dx, dy2 = m->dy * m->dy, dz2 = m->dz * m->dz;
    const double coef = 1.0 / (2.0 * (1.0 / dx2 + 1.0 / dy2 + 1.0 / dz2));
    stationary_rhs(m, rho / dt, u, v, w, rhs);
    int it_done = max_iter;
    for (int iter = 0; iter < max_iter; ++iter) {
        double maxr = 0.0;
        for (int i = 1; i < nx - 1; ++i)
            for (int j = 1; j < ny - 1; ++j)
                for (int k = 1; k < nz - 1; ++k) {
                    int64_t id = IDX(i, j, k);
                    double p_old = p[id];
                    p[id] = (1 - omega) * p[id] +
                            omega * coef *
                                ((p[IDX(i + 1, j, k)] + p[IDX(i - 1, j, k)]) / dx2 +
                                 (p[IDX(i, j + 1, k)] + p[IDX(i, j - 1, k)]) / dy2 +
                                 (p[IDX(i, j, k + 1)] + p[IDX(i, j, k - 1)]) / dz2 - rhs[id]);
                    double res = fabs(p[id] - p_old);
                    if (res > maxr) maxr = res;
                }
        lo_apply_pressure_bcs(m, p, solid);
        if (maxr < tol) { it_done = iter + 1; break; }
    }
    free(rhs);
    return it_done;
}

/* src/pressure.cpp:256-329 (reads the u_new arrays). */
void lo_calculate_divergence(const lo_mesh* m, double dt, double rho, const double* u_new,
                             const double* v_new, const double* w_new, const uint8_t* solid,
                             double* rhs)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    const double scale = rho / dt;
    const double idx = 1.0 / (2.0 * m->dx), idy = 1.0 / (2.0 * m->dy), idz = 1.0 / (2.0 * m->dz);
    const double idx1 = 1.0 / m->dx, idy1 = 1.0 / m->dy, idz1 = 1.0 / m->dz;
#pragma omp parallel for
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                int64_t id = IDX(i, j, k);
                if (solid[id] || i == nx - 1) { rhs[id] = 0.0; continue; }
                double du_dx, dv_dy, dw_dz;
                if (i == 0) du_dx = (u_new[IDX(i + 1, j, k)] - u_new[id]) * idx1;
                else du_dx = (u_new[IDX(i + 1, j, k)] - u_new[IDX(i - 1, j, k)]) * idx;
                if (j == 0) dv_dy = (v_new[IDX(i, j + 1, k)] - v_new[id]) * idy1;
                else if (j == ny - 1) dv_dy = (v_new[id] - v_new[IDX(i, j - 1, k)]) * idy1;
                else dv_dy = (v_new[IDX(i, j + 1, k)] - v_new[IDX(i, j - 1, k)]) * idy;
                if (k == 0) dw_dz = (w_new[IDX(i, j, k + 1)] - w_new[id]) * idz1;
                else if (k == nz - 1) dw_dz = (w_new[id] - w_new[IDX(i, j, k - 1)]) * idz1;
                else dw_dz = (w_new[IDX(i, j, k + 1)] - w_new[IDX(i, j, k - 1)]) * idz;
                rhs[id] = scale * (du_dx + dv_dy + dw_dz);
            }
}

/* src/pressure.cpp:566-599 */
void lo_build_b(const lo_mesh* m, const double* div, const uint8_t* solid, double* b)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
#pragma omp parallel for
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                int64_t id = IDX(i, j, k);
                b[id] = (solid[id] || i == nx - 1) ? 0.0 : -div[id];
            }
}

/* src/pressure.cpp:608-699.  Writes all seven diagonals (the reference leaves
 * the off-diagonals of solid/outlet rows at the zeros of a fresh matrix). */
void lo_build_stencil(const lo_mesh* m, const uint8_t* solid, lo_stencil* A)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    const double idx2 = 1.0 / (m->dx * m->dx), idy2 = 1.0 / (m->dy * m->dy),
                 idz2 = 1.0 / (m->dz * m->dz);
    const double e0 = -idx2, w0 = -idx2, n0 = -idy2, s0 = -idy2, t0 = -idz2, b0 = -idz2;
    const double c0 = (2.0 * idx2 + 2.0 * idy2 + 2.0 * idz2);
#pragma omp parallel for
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                int64_t id = IDX(i, j, k);
                A->n[id] = A->s[id] = A->e[id] = A->w[id] = A->t[id] = A->b[id] = 0.0;
                if (solid[id] || i == nx - 1) { A->c[id] = 1.0; continue; }
                A->c[id] = c0;
                A->e[id] = e0; A->w[id] = w0; A->n[id] = n0; A->s[id] = s0;
                A->t[id] = t0; A->b[id] = b0;
                if (i == 0 || solid[IDX(i - 1, j, k)]) { A->e[id] += w0; A->w[id] = 0.0; }
                if (i == nx - 2) A->e[id] = 0.0;
                else if (solid[IDX(i + 1, j, k)]) { A->w[id] += e0; A->e[id] = 0.0; }
                if (j == 0 || solid[IDX(i, j - 1, k)]) { A->n[id] += s0; A->s[id] = 0.0; }
                if (j == ny - 1 || solid[IDX(i, j + 1, k)]) { A->s[id] += n0; A->n[id] = 0.0; }
                if (k == 0 || solid[IDX(i, j, k - 1)]) { A->t[id] += b0; A->b[id] = 0.0; }
                if (k == nz - 1 || solid[IDX(i, j, k + 1)]) { A->b[id] += t0; A->t[id] = 0.0; }
            }
}

/* src/pressure.cpp:709-746 */
void lo_spmv(const lo_mesh* m, const lo_stencil* A, const double* p, double* q)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    const int64_t si = (int64_t)ny * nz, sj = nz;
#pragma omp parallel for
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                int64_t id = IDX(i, j, k);
                double val = A->c[id] * p[id];
                if (i > 0) val += A->w[id] * p[id - si];
                if (i < nx - 1) val += A->e[id] * p[id + si];
                if (j > 0) val += A->s[id] * p[id - sj];
                if (j < ny - 1) val += A->n[id] * p[id + sj];
                if (k > 0) val += A->b[id] * p[id - 1];
                if (k < nz - 1) val += A->t[id] * p[id + 1];
                q[id] = val;
            }
}

/* src/pressure.cpp:420-428 */
void lo_jacobi_precond(int64_t n, const lo_stencil* A, const double* r, double* z)
{
#pragma omp parallel for
    for (int64_t i = 0; i < n; ++i) z[i] = r[i] / A->c[i];
}

/* src/pressure.cpp:495-556 (serial, lexicographic).  Zeroes L first, like
 * the fresh StencilMatrix the reference builds into. */
void lo_ic_build(const lo_mesh* m, const lo_stencil* A, lo_stencil* L)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    const int64_t n = (int64_t)nx * ny * nz, si = (int64_t)ny * nz, sj = nz;
    const double small_val = 1e-30;
    double* arrs[7] = {L->c, L->n, L->s, L->e, L->w, L->t, L->b};
    for (int a = 0; a < 7; ++a) memset(arrs[a], 0, (size_t)n * sizeof(double));
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                int64_t id = IDX(i, j, k);
                double sum_sq = 0.0;
                if (i > 0) {
                    double lc = L->c[id - si];
                    if (fabs(lc) > small_val) { L->w[id] = A->w[id] / lc; sum_sq += L->w[id] * L->w[id]; }
                }
                if (j > 0) {
                    double lc = L->c[id - sj];
                    if (fabs(lc) > small_val) { L->s[id] = A->s[id] / lc; sum_sq += L->s[id] * L->s[id]; }
                }
                if (k > 0) {
                    double lc = L->c[id - 1];
                    if (fabs(lc) > small_val) { L->b[id] = A->b[id] / lc; sum_sq += L->b[id] * L->b[id]; }
                }
                double diag = A->c[id] - sum_sq;
                L->c[id] = (diag <= small_val) ? 1.0 : sqrt(diag);
            }
}

/* src/pressure.cpp:442-482 (serial forward then backward substitution). */
void lo_ic_apply(const lo_mesh* m, const lo_stencil* L, const double* r, double* z)
{
    const int nx = m->nx, ny = m->ny, nz = m->nz;
    const int64_t si = (int64_t)ny * nz, sj = nz;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                int64_t id = IDX(i, j, k);
                double sum = r[id];
                if (i > 0) sum -= L->w[id] * z[id - si];
                if (j > 0) sum -= L->s[id] * z[id - sj];
                if (k > 0) sum -= L->b[id] * z[id - 1];
                z[id] = sum / L->c[id];
            }
    for (int i = nx - 1; i >= 0; --i)
        for (int j = ny - 1; j >= 0; --j)
            for (int k = nz - 1; k >= 0; --k) {
                int64_t id = IDX(i, j, k);
                double sum = z[id];
                if (i < nx - 1) sum -= L->w[id + si] * z[id + si];
                if (j < ny - 1) sum -= L->s[id + sj] * z[id + sj];
                if (k < nz - 1) sum -= L->b[id + 1] * z[id + 1];
                z[id] = sum / L->c[id];
            }
}

/* src/pressure.cpp:851-906 (work_p/work_res replace the per-call
 * allocations of :859-860). */
void lo_cheb_apply(const lo_mesh* m, const lo_stencil* A, double lmin, double lmax, int degree,
                   const double* r, double* z, double* p, double* res)
{
    const int64_t n = (int64_t)m->nx * m->ny * m->nz;
    const double d = (lmax + lmin) / 2.0;
    const double c = (lmax - lmin) / 2.0;
    double alpha, beta;
#pragma omp parallel for
    for (int64_t i = 0; i < n; ++i) z[i] = 0.0;
    lo_copy(n, res, r);
    alpha = 2.0 / d;
    lo_copy(n, p, res);
    lo_axpy(n, z, alpha, p);
    for (int k = 1; k < degree; ++k) {
        lo_spmv(m, A, z, res);
        lo_saxpy(n, res, 1.0, r, -1.0, res);
        beta = (c * alpha / 2.0) * (c * alpha / 2.0);
        alpha = 1.0 / (d - beta);
        lo_saxpy(n, p, 1.0, res, beta, p);
        lo_axpy(n, z, alpha, p);
    }
}

/* src/pressure.cpp:917-955 with an explicit start vector v0 (the reference
 * draws it from std::mt19937(1337) / uniform(-1,1) in index order when run on
 * one thread). */
double lo_lambda_max(const lo_mesh* m, const lo_stencil* A, const double* v0, int n_iter,
                     double* v, double* w)
{
    const int64_t n = (int64_t)m->nx * m->ny * m->nz;
    lo_copy(n, v, v0);
    lo_copy(n, w, v);
    double lambda = 0.0;
    for (int it = 0; it < n_iter; ++it) {
        lo_spmv(m, A, v, w);
        lambda = lo_dot(n, v, w);
        double nrm = lo_norm(n, w);
        lo_copy(n, v, w);
#pragma omp parallel for
        for (int64_t i = 0; i < n; ++i) v[i] /= nrm;
    }
    return lambda;
}

static void apply_pc(const lo_mesh* m, int pc, const lo_stencil* A, const lo_stencil* L,
                     double lmin, double lmax, int degree, const double* r, double* z,
                     double* wp, double* wres)
{
    const int64_t n = (int64_t)m->nx * m->ny * m->nz;
    switch (pc) {
    case LO_PC_JACOBI: lo_jacobi_precond(n, A, r, z); break;
    case LO_PC_IC: lo_ic_apply(m, L, r, z); break;
    case LO_PC_CHEB: lo_cheb_apply(m, A, lmin, lmax, degree, r, z, wp, wres); break;
    default: lo_copy(n, z, r); break;
    }
}

/* src/pressure.cpp:342-414 (and the identical loop of :762-835). */
int lo_pcg(const lo_mesh* m, const lo_stencil* A, const double* b, double* x, int pc,
           const lo_stencil* L, double lmin, double lmax, int degree, int max_iter, double tol,
           double* work, double* final_norm)
{
    const int64_t n = (int64_t)m->nx * m->ny * m->nz;
    double *r = work, *z = work + n, *p = work + 2 * n, *q = work + 3 * n;
    double *cp = NULL, *cres = NULL;
    if (pc == LO_PC_CHEB) {
        cp = (double*)malloc((size_t)n * sizeof(double));
        cres = (double*)malloc((size_t)n * sizeof(double));
    }
    int ret = max_iter;
    lo_spmv(m, A, x, q);
    lo_saxpy(n, r, 1.0, b, -1.0, q);
    double err = lo_norm(n, r);
    if (err < tol) { ret = 0; goto done; }
    apply_pc(m, pc, A, L, lmin, lmax, degree, r, p, cp, cres);
    double rho = lo_dot(n, r, p);
    for (int k = 1; k <= max_iter; ++k) {
        lo_spmv(m, A, p, q);
        double alpha = rho / lo_dot(n, p, q);
        lo_axpy(n, x, alpha, p);
        lo_axpy(n, r, -alpha, q);
        err = lo_norm(n, r);
        if (err < tol) { ret = k; goto done; }
        apply_pc(m, pc, A, L, lmin, lmax, degree, r, z, cp, cres);
        double rho_new = lo_dot(n, r, z);
        double beta = rho_new / rho;
        lo_saxpy(n, p, 1.0, z, beta, p);
        rho = rho_new;
    }
done:
    if (final_norm) *final_norm = err;
    free(cp);
    free(cres);
    return ret;
}

/* One time step in the order of src/main.cpp:115-144. */
int lo_step(const lo_mesh* m, lo_field* f, const lo_stencil* A, const lo_stencil* L,
            const lo_step_params* prm, double* b, double* pcg_work, double* dt_out)
{
    const int64_t n = (int64_t)m->nx * m->ny * m->nz;
    double dt = prm->dt_fixed > 0
                    ? prm->dt_fixed
                    : lo_compute_adaptive_dt(m, f->u, f->v, f->w, f->nu_t, prm->nu, prm->cfl_conv,
                                             prm->cfl_visc, prm->dt_max);
    lo_compute_sgs(m, lo_smagorinsky_coef(m, prm->cs), f->u, f->v, f->w, f->nu_t, NULL);
    lo_apply_nut_bcs(m, f->nu_t, f->solid);
    lo_solve_momentum(m, dt, prm->nu, f->u, f->v, f->w, f->nu_t, f->u_new, f->v_new, f->w_new);
    double* t;
    t = f->u; f->u = f->u_new; f->u_new = t;
    t = f->v; f->v = f->v_new; f->v_new = t;
    t = f->w; f->w = f->w_new; f->w_new = t;
    lo_apply_velocity_bcs(m, f->u, f->v, f->w, f->solid);
    int iters = 0;
    if (prm->solver == 0) {
        lo_calculate_divergence(m, dt, prm->rho, f->u_new, f->v_new, f->w_new, f->solid, f->p_rhs);
        lo_build_b(m, f->p_rhs, f->solid, b);
        double tol = prm->rel_tol > 0 ? prm->rel_tol * lo_norm(n, b) : prm->tol;
        iters = lo_pcg(m, A, b, f->p, prm->pc, L, prm->lmin, prm->lmax, prm->degree,
                       prm->max_iter, tol, pcg_work, NULL);
    } else if (prm->solver == 1) {
        iters = lo_solve_jacobi(m, dt, prm->rho, f->u, f->v, f->w, f->p, f->solid, prm->max_iter,
                                prm->tol);
    } else {
        iters = lo_solve_gs(m, dt, prm->rho, f->u, f->v, f->w, f->p, f->solid, prm->max_iter,
                            prm->omega, prm->tol);
    }
    lo_correct_velocity(m, dt, prm->rho, f->p, f->u, f->v, f->w);
    lo_apply_velocity_bcs(m, f->u, f->v, f->w, f->solid);
    if (dt_out) *dt_out = dt;
    return iters;
}

/* ------------------------------------------------------------------------ */
/* Statistics, src/statistics.cpp                                           */
/* ------------------------------------------------------------------------ */

/* src/statistics.cpp:110-130 */
void lo_stats_update(int64_t n, const double* u, const double* v, const double* w, const double* p,
                     double* const* s)
{
#pragma omp parallel for
    for (int64_t i = 0; i < n; ++i) {
        const double a = u[i], b = v[i], c = w[i], d = p[i];
        s[0][i] += a;
        s[1][i] += b;
        s[2][i] += c;
        s[3][i] += d;
        s[4][i] += a * a;
        s[5][i] += b * b;
        s[6][i] += c * c;
        s[7][i] += a * b;
        s[8][i] += a * c;
        s[9][i] += b * c;
    }
}

/* src/statistics.cpp:143-184 */
void lo_stats_finalize(int64_t n, int samples, const double* const* s, double* const* o)
{
    const double n_inv = 1.0 / (double)samples;
#pragma omp parallel for
    for (int64_t i = 0; i < n; ++i) {
        const double um = s[0][i] * n_inv, vm = s[1][i] * n_inv, wm = s[2][i] * n_inv;
        o[0][i] = um;
        o[1][i] = vm;
        o[2][i] = wm;
        o[3][i] = s[3][i] * n_inv;
        o[4][i] = (s[4][i] * n_inv) - (um * um);
        o[5][i] = (s[5][i] * n_inv) - (vm * vm);
        o[6][i] = (s[6][i] * n_inv) - (wm * wm);
        o[7][i] = (s[7][i] * n_inv) - (um * vm);
        o[8][i] = (s[8][i] * n_inv) - (um * wm);
        o[9][i] = (s[9][i] * n_inv) - (vm * wm);
    }
}
