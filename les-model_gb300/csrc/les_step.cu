// les_step.cu -- one time step of les-model's loop body (src/main.cpp:115-144)
// on the device: dt, SGS + nu_t BCs, momentum (+ swap), velocity BCs,
// pressure solve, projection, velocity BCs.  Statistics and VTK output
// (:152-164) stay with the caller.
#include <cmath>

#include "les_internal.cuh"

using namespace les;

namespace les {
les_status velocity_bcs_dev(les_ctx* c);
les_status sgs_nut_dev(les_ctx* c, double cs, int want_tau);
les_status momentum_dev(les_ctx* c, double dt, double nu, const double* dtp);
les_status correct_dev(les_ctx* c, double dt, double rho, const double* dtp);
les_status adaptive_dt_dev(les_ctx* c, double nu, double cfl_conv, double cfl_visc, double dt_max);
les_status div_b_dev(les_ctx* c, double dt, double rho, double rel_tol, const double* dtp);
les_status pcg_fp64(les_ctx* c, const les_pcg_opts* o, les_pcg_result* res, int keep_tol);
les_status pcg_mixed_impl(les_ctx* c, const les_pcg_opts* o, les_pcg_result* res, int keep_tol);
les_status solve_jacobi_dev(les_ctx* c, double dt, double rho, int max_iter, double tol, int* sweeps);
les_status solve_gs_dev(les_ctx* c, double dt, double rho, int max_iter, double omega, double tol, int* sweeps);
}

extern "C" les_status les_step(les_ctx* c, const les_step_params* prm, les_step_stats* stats)
{
    if (!c || !prm) return LES_BAD_ARG;
    if (prm->solver < LES_SOLVER_PCG || prm->solver > LES_SOLVER_GS_SOR) return LES_BAD_ARG;
    if (prm->solver == LES_SOLVER_PCG && !c->stencil_mode)
        return fail(c, LES_BAD_ARG, "PCG needs a matrix: call les_build_stencil first");
    cudaSetDevice(c->device);
    les_status st;
    double dt = prm->dt_fixed;
    if (!(dt > 0)) {
        st = adaptive_dt_dev(c, prm->nu, prm->cfl_conv, prm->cfl_visc, prm->dt_max);
        if (st) return st;
        st = read_state(c);
        if (st) return st;
        dt = c->h_state[0].scal[0];
    }
    if ((st = sgs_nut_dev(c, prm->cs, prm->want_tau))) return st;
    if ((st = momentum_dev(c, dt, prm->nu, nullptr))) return st;
    if ((st = velocity_bcs_dev(c))) return st;
    les_status solve = LES_OK;
    les_step_stats s{};
    s.dt = dt;
    if (prm->solver == LES_SOLVER_PCG) {
        if ((st = div_b_dev(c, dt, prm->rho, prm->rel_tol, nullptr))) return st;
        les_pcg_result r{};
        const int keep = prm->rel_tol > 0 ? 1 : 0;
        if (prm->pcg.precision == LES_MIXED) solve = pcg_mixed_impl(c, &prm->pcg, &r, keep);
        else solve = pcg_fp64(c, &prm->pcg, &r, keep);
        if (solve != LES_OK && solve != LES_NOT_CONVERGED && solve != LES_NONFINITE) return solve;
        s.iters = r.iters;
        s.outer = r.outer;
        s.residual = r.residual;
        s.b_norm = c->h_state[0].bnorm;
    } else if (prm->solver == LES_SOLVER_JACOBI) {
        solve = solve_jacobi_dev(c, dt, prm->rho, prm->stat_max_iter, prm->stat_tol, &s.iters);
        if (solve != LES_OK) return solve;
    } else {
        solve = solve_gs_dev(c, dt, prm->rho, prm->stat_max_iter, prm->omega, prm->stat_tol, &s.iters);
        if (solve != LES_OK) return solve;
    }
    if ((st = correct_dev(c, dt, prm->rho, nullptr))) return st;
    if ((st = velocity_bcs_dev(c))) return st;
    s.status = solve;
    if (stats) *stats = s;
    return LES_OK;
}
