// ref_harness.cpp -- C entry points around the compiled les-model reference.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.sh together with the
// reference's own src/main.cpp (renamed entry point), src/pressure.cpp,
// src/io.cpp and src/statistics.cpp into oracle/_ref/libles_ref.so.  It is
// used in the development container to (a) generate the golden fixtures under
// tests/golden/ and (b) check the C restatement in oracle/les_oracle.c against
// the real reference.  Nothing on the GPU path loads it.
//
// Each entry point copies flat arrays into the reference's Field /
// StencilMatrix types, calls the reference function unchanged and copies the
// results back out.  The only new logic is ref_pcg_restated(), which runs the
// reference's PCG loop (src/pressure.cpp:342-414) statement by statement with
// the preconditioner chosen at run time, because the reference wires only the
// IC-with-A preconditioner into solve_pressure_pcg (:362-363, :395-396).
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include <omp.h>
#include <unistd.h>

#include "field.h"
#include "io.h"
#include "pressure.h"
#include "statistics.h"

// Defined in the reference's src/main.cpp (prototypes at src/main.cpp:20-29).
double compute_adaptive_dt(const Field& field, const Mesh& mesh, double nu);
void define_obstacle_mask(Field& f, const Mesh& m);
void compute_sgs_stress(Field& f, Stress& sgs, const Mesh& m);
void apply_nut_BCs(Field& f, const Mesh& m);
void solve_momentum(Field& f, const Mesh& m, double dt, double nu);
void apply_velocity_BCs(Field& f, const Mesh& m);
void correct_velocity(Field& f, const Mesh& m, double dt, double rho);

namespace {

size_t ncell(const Mesh& m) { return (size_t)m.nx * m.ny * m.nz; }

void put(std::vector<double>& dst, const double* src, size_t n)
{
    if (src) std::memcpy(dst.data(), src, n * sizeof(double));
}
void get(double* dst, const std::vector<double>& src, size_t n)
{
    if (dst) std::memcpy(dst, src.data(), n * sizeof(double));
}
void put_mask(Field& f, const uint8_t* s, size_t n)
{
    if (s)
        for (size_t i = 0; i < n; ++i) f.is_solid[i] = s[i] != 0;
}

Mesh mk(int nx, int ny, int nz, double dx, double dy, double dz) { return Mesh{nx, ny, nz, dx, dy, dz}; }

void put_st(StencilMatrix& A, const double* const* d, size_t n)
{
    Vector* a[7] = {&A.A_c, &A.A_n, &A.A_s, &A.A_e, &A.A_w, &A.A_t, &A.A_b};
    for (int q = 0; q < 7; ++q) put(*a[q], d[q], n);
}
void get_st(double* const* d, const StencilMatrix& A, size_t n)
{
    const Vector* a[7] = {&A.A_c, &A.A_n, &A.A_s, &A.A_e, &A.A_w, &A.A_t, &A.A_b};
    for (int q = 0; q < 7; ++q) get(d[q], *a[q], n);
}

}  // namespace

#define MESH_ARGS int nx, int ny, int nz, double dx, double dy, double dz
#define MESH mk(nx, ny, nz, dx, dy, dz)

extern "C" {

void ref_set_threads(int n) { omp_set_num_threads(n); }

void ref_define_obstacle_mask(MESH_ARGS, uint8_t* solid)
{
    Mesh m = MESH;
    Field f(nx, ny, nz);
    define_obstacle_mask(f, m);
    for (size_t i = 0; i < ncell(m); ++i) solid[i] = f.is_solid[i] ? 1 : 0;
}

double ref_adaptive_dt(MESH_ARGS, const double* u, const double* v, const double* w,
                       const double* nu_t, double nu)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    put(f.u, u, n); put(f.v, v, n); put(f.w, w, n); put(f.nu_t, nu_t, n);
    return compute_adaptive_dt(f, m, nu);
}

void ref_velocity_bcs(MESH_ARGS, double* u, double* v, double* w, const uint8_t* solid)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    put(f.u, u, n); put(f.v, v, n); put(f.w, w, n); put_mask(f, solid, n);
    apply_velocity_BCs(f, m);
    get(u, f.u, n); get(v, f.v, n); get(w, f.w, n);
}

// compute_sgs_stress with the reference's hard-coded Cs = 0.18.  nu_t is
// in/out (the reference writes only interior cells).  tau: 6*N or NULL,
// order xx, xy, xz, yy, yz, zz.
void ref_sgs(MESH_ARGS, const double* u, const double* v, const double* w, double* nu_t, double* tau)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    Stress s(n);
    put(f.u, u, n); put(f.v, v, n); put(f.w, w, n); put(f.nu_t, nu_t, n);
    compute_sgs_stress(f, s, m);
    get(nu_t, f.nu_t, n);
    if (tau) {
        get(tau + 0 * n, s.tau_xx, n); get(tau + 1 * n, s.tau_xy, n); get(tau + 2 * n, s.tau_xz, n);
        get(tau + 3 * n, s.tau_yy, n); get(tau + 4 * n, s.tau_yz, n); get(tau + 5 * n, s.tau_zz, n);
    }
}

void ref_nut_bcs(MESH_ARGS, double* nu_t, const uint8_t* solid)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    put(f.nu_t, nu_t, n); put_mask(f, solid, n);
    apply_nut_BCs(f, m);
    get(nu_t, f.nu_t, n);
}

// solve_momentum: inputs u,v,w,nu_t and the u_new buffers' prior contents;
// outputs (after the reference's swap) go to out_u/v/w = f.u etc., and the
// swapped-out old velocities to out_un/vn/wn = f.u_new etc.
void ref_momentum(MESH_ARGS, double dt, double nu, const double* u, const double* v,
                  const double* w, const double* un, const double* vn, const double* wn,
                  const double* nu_t, double* out_u, double* out_v, double* out_w, double* out_un,
                  double* out_vn, double* out_wn)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    put(f.u, u, n); put(f.v, v, n); put(f.w, w, n);
    put(f.u_new, un, n); put(f.v_new, vn, n); put(f.w_new, wn, n);
    put(f.nu_t, nu_t, n);
    solve_momentum(f, m, dt, nu);
    get(out_u, f.u, n); get(out_v, f.v, n); get(out_w, f.w, n);
    get(out_un, f.u_new, n); get(out_vn, f.v_new, n); get(out_wn, f.w_new, n);
}

void ref_correct_velocity(MESH_ARGS, double dt, double rho, const double* p, double* u, double* v, double* w)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    put(f.u, u, n); put(f.v, v, n); put(f.w, w, n); put(f.p, p, n);
    correct_velocity(f, m, dt, rho);
    get(u, f.u, n); get(v, f.v, n); get(w, f.w, n);
}

void ref_pressure_bcs(MESH_ARGS, double* p, const uint8_t* solid)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    put(f.p, p, n); put_mask(f, solid, n);
    apply_pressure_BCs(f, m);
    get(p, f.p, n);
}

void ref_solve_jacobi(MESH_ARGS, double dt, double rho, const double* u, const double* v,
                      const double* w, double* p, const uint8_t* solid)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    put(f.u, u, n); put(f.v, v, n); put(f.w, w, n); put(f.p, p, n); put_mask(f, solid, n);
    solve_pressure_jacobi(f, m, dt, rho);
    get(p, f.p, n);
}

void ref_solve_gs(MESH_ARGS, double dt, double rho, const double* u, const double* v,
                  const double* w, double* p, const uint8_t* solid, int max_iter)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    put(f.u, u, n); put(f.v, v, n); put(f.w, w, n); put(f.p, p, n); put_mask(f, solid, n);
    solve_pressure_GS(f, m, dt, rho, max_iter);
    get(p, f.p, n);
}

void ref_divergence(MESH_ARGS, double dt, double rho, const double* un, const double* vn,
                    const double* wn, const uint8_t* solid, double* rhs)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    put(f.u_new, un, n); put(f.v_new, vn, n); put(f.w_new, wn, n); put_mask(f, solid, n);
    Vector out(n, 0.0);
    calculate_divergence(out, f, m, dt, rho);
    get(rhs, out, n);
}

void ref_build_b(MESH_ARGS, const double* div, const uint8_t* solid, double* b)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    put_mask(f, solid, n);
    Vector d(div, div + n), out(n, 0.0);
    build_b_vector(out, d, f, m);
    get(b, out, n);
}

// diag: 7 output arrays in the order c, n, s, e, w, t, b.
void ref_build_stencil(MESH_ARGS, const uint8_t* solid, double* const* diag)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    put_mask(f, solid, n);
    StencilMatrix A(n);
    build_stencil(A, f, m);
    get_st(diag, A, n);
}

void ref_spmv(MESH_ARGS, const double* const* diag, const double* p, double* q)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    StencilMatrix A(n);
    put_st(A, diag, n);
    Vector pv(p, p + n), qv(n, 0.0);
    fast_apply_laplacian(qv, pv, A, f);
    get(q, qv, n);
}

void ref_jacobi_precond(MESH_ARGS, const double* const* diag, const double* r, double* z)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    StencilMatrix A(n);
    put_st(A, diag, n);
    Vector rv(r, r + n), zv(n, 0.0);
    apply_jacobi_preconditioner(zv, rv, A);
    get(z, zv, n);
}

void ref_ic_build(MESH_ARGS, const double* const* diag, double* const* ldiag)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    StencilMatrix A(n), L(n);
    put_st(A, diag, n);
    build_ic_preconditioner(L, A, f, m);
    get_st(ldiag, L, n);
}

void ref_ic_apply(MESH_ARGS, const double* const* ldiag, const double* r, double* z)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    StencilMatrix L(n);
    put_st(L, ldiag, n);
    Vector rv(r, r + n), zv(n, 0.0);
    apply_ic_preconditioner(zv, rv, L, f);
    get(z, zv, n);
}

void ref_cheb_apply(MESH_ARGS, const double* const* diag, double lmin, double lmax, int degree,
                    const double* r, double* z)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    StencilMatrix A(n);
    put_st(A, diag, n);
    Vector rv(r, r + n), zv(n, 0.0);
    apply_chebyshev_preconditioner(zv, rv, A, f, lmin, lmax, degree);
    get(z, zv, n);
}

double ref_lambda_max(MESH_ARGS, const double* const* diag, int n_iter)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    StencilMatrix A(n);
    put_st(A, diag, n);
    return estimate_lambda_max(A, f, n_iter);
}

// solve_pressure_pcg exactly as shipped (IC apply with A as the factor).
int ref_pcg_shipped(MESH_ARGS, const double* const* diag, const double* b, double* x, int max_iter, double tol)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    StencilMatrix A(n);
    put_st(A, diag, n);
    Vector bv(b, b + n), xv(x, x + n);
    int it = solve_pressure_pcg(A, bv, xv, f, max_iter, tol);
    get(x, xv, n);
    return it;
}

int ref_pcg_cheb(MESH_ARGS, const double* const* diag, const double* b, double* x, double lmin,
                 double lmax, int degree, int max_iter, double tol)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    StencilMatrix A(n);
    put_st(A, diag, n);
    Vector bv(b, b + n), xv(x, x + n);
    int it = solve_pressure_pcg_chebyshev(A, bv, xv, f, lmin, lmax, degree, max_iter, tol);
    get(x, xv, n);
    return it;
}

// The PCG loop of src/pressure.cpp:342-414, statement for statement, with the
// preconditioner selected by pc: 0 = apply_jacobi_preconditioner (:420),
// 1 = apply_ic_preconditioner with the factor in ldiag (:442).
int ref_pcg_restated(MESH_ARGS, const double* const* diag, const double* const* ldiag, int pc,
                     const double* b, double* x, int max_iter, double tol)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field field(nx, ny, nz);
    StencilMatrix A(n), L(n);
    put_st(A, diag, n);
    if (ldiag) put_st(L, ldiag, n);
    Vector bv(b, b + n), xv(x, x + n);
    Vector r(n), z(n), p(n), q(n);
    auto precond = [&](Vector& out, const Vector& in) {
        if (pc == 0) apply_jacobi_preconditioner(out, in, A);
        else apply_ic_preconditioner(out, in, L, field);
    };
    int ret = max_iter;
    fast_apply_laplacian(q, xv, A, field);
    parallel_saxpy(r, 1.0, bv, -1.0, q);
    double initial_error = parallel_norm(r);
    if (initial_error < tol) {
        ret = 0;
    } else {
        precond(p, r);
        double rho = parallel_dot(r, p);
        for (int k = 1; k <= max_iter; ++k) {
            fast_apply_laplacian(q, p, A, field);
            double alpha = rho / parallel_dot(p, q);
            parallel_axpy(xv, alpha, p);
            parallel_axpy(r, -alpha, q);
            double error = parallel_norm(r);
            if (error < tol) { ret = k; break; }
            precond(z, r);
            double rho_new = parallel_dot(r, z);
            double beta = rho_new / rho;
            parallel_saxpy(p, 1.0, z, beta, p);
            rho = rho_new;
        }
    }
    get(x, xv, n);
    return ret;
}

// One step of the src/main.cpp:108-165 loop body with a fixed dt (dt>0) or
// compute_adaptive_dt (dt<=0), Cs fixed at the reference's 0.18.
// solver: 0 = PCG as shipped, 1 = PCG restated with Jacobi, 2 = PCG restated
// with IC(L), 3 = Chebyshev PCG, 4 = stationary Jacobi, 5 = GS-SOR.
// Fields are in/out; the u_new buffers hold what the swap leaves in them.
int ref_step(MESH_ARGS, double* u, double* v, double* w, double* un, double* vn, double* wn,
             double* p, double* p_rhs, double* nu_t, const uint8_t* solid,
             const double* const* diag, const double* const* ldiag, int solver, double dt,
             double nu, double rho, int max_iter, double rel_tol, double lmin, double lmax,
             int degree, int gs_iter, double* dt_out)
{
    Mesh m = MESH;
    size_t n = ncell(m);
    Field f(nx, ny, nz);
    Stress sgs(n);
    put(f.u, u, n); put(f.v, v, n); put(f.w, w, n);
    put(f.u_new, un, n); put(f.v_new, vn, n); put(f.w_new, wn, n);
    put(f.p, p, n); put(f.p_rhs, p_rhs, n); put(f.nu_t, nu_t, n); put_mask(f, solid, n);
    StencilMatrix A(n), L(n);
    put_st(A, diag, n);
    if (ldiag) put_st(L, ldiag, n);
    if (dt <= 0) dt = compute_adaptive_dt(f, m, nu);
    compute_sgs_stress(f, sgs, m);
    apply_nut_BCs(f, m);
    solve_momentum(f, m, dt, nu);
    apply_velocity_BCs(f, m);
    int it = 0;
    if (solver <= 3) {
        calculate_divergence(f.p_rhs, f, m, dt, rho);
        Vector b(n);
        build_b_vector(b, f.p_rhs, f, m);
        double tol = rel_tol * parallel_norm(b);
        if (solver == 0) it = solve_pressure_pcg(A, b, f.p, f, max_iter, tol);
        else if (solver == 3)
            it = solve_pressure_pcg_chebyshev(A, b, f.p, f, lmin, lmax, degree, max_iter, tol);
        else {
            std::vector<const double*> dv(7), lv(7);
            Vector* a[7] = {&A.A_c, &A.A_n, &A.A_s, &A.A_e, &A.A_w, &A.A_t, &A.A_b};
            Vector* l[7] = {&L.A_c, &L.A_n, &L.A_s, &L.A_e, &L.A_w, &L.A_t, &L.A_b};
            for (int q = 0; q < 7; ++q) { dv[q] = a[q]->data(); lv[q] = l[q]->data(); }
            it = ref_pcg_restated(nx, ny, nz, dx, dy, dz, dv.data(), lv.data(), solver == 1 ? 0 : 1,
                                  b.data(), f.p.data(), max_iter, tol);
        }
    } else if (solver == 4) {
        solve_pressure_jacobi(f, m, dt, rho);
    } else {
        solve_pressure_GS(f, m, dt, rho, gs_iter);
    }
    correct_velocity(f, m, dt, rho);
    apply_velocity_BCs(f, m);
    get(u, f.u, n); get(v, f.v, n); get(w, f.w, n);
    get(un, f.u_new, n); get(vn, f.v_new, n); get(wn, f.w_new, n);
    get(p, f.p, n); get(p_rhs, f.p_rhs, n); get(nu_t, f.nu_t, n);
    if (dt_out) *dt_out = dt;
    return it;
}

// ---- statistics and I/O (src/statistics.cpp, src/io.cpp) --------------------
// The reference writes into paths relative to the working directory
// (output/, checkpoint/); these wrappers run it inside `dir` and come back.
namespace {
struct InDir {
    std::string old;
    explicit InDir(const char* dir)
    {
        char buf[4096];
        if (getcwd(buf, sizeof buf)) old = buf;
        if (chdir(dir) != 0) old.clear();
    }
    ~InDir()
    {
        if (!old.empty() && chdir(old.c_str()) != 0) {}
    }
};
}  // namespace

// Runs init_statistics(start_step), then update_statistics for steps
// 0..nsteps-1 with fields (u, v, w, p) of each step, copies out the ten sums
// (u, v, w, p, uu, vv, ww, uv, uw, vw) and the sample count, and writes the
// final statistics file with finalize_and_save(dir/filename).
int ref_statistics(MESH_ARGS, int nsteps, int start_step, const double* const* uvwp, double* const* sums,
                   const char* dir, const char* filename)
{
    Mesh m = MESH;
    const size_t n = ncell(m);
    Statistics st;
    init_statistics(st, m, start_step);
    Field f;
    f.u.resize(n); f.v.resize(n); f.w.resize(n); f.p.resize(n);
    for (int s = 0; s < nsteps; ++s) {
        put(f.u, uvwp[4 * s + 0], n); put(f.v, uvwp[4 * s + 1], n);
        put(f.w, uvwp[4 * s + 2], n); put(f.p, uvwp[4 * s + 3], n);
        update_statistics(st, f, s);
    }
    const std::vector<double>* src[10] = {&st.sum_field.u, &st.sum_field.v, &st.sum_field.w, &st.sum_field.p,
                                          &st.uu_sum, &st.vv_sum, &st.ww_sum, &st.uv_sum, &st.uw_sum, &st.vw_sum};
    for (int q = 0; q < 10; ++q) get(sums[q], *src[q], n);
    {
        InDir d(dir);
        finalize_and_save(st, m, filename);
    }
    return st.num_samples;
}

// write_field_vtk into dir/output/output_<step>.vtk
void ref_write_field_vtk(MESH_ARGS, const double* u, const double* v, const double* w, const double* p,
                         const double* nu_t, const uint8_t* solid, int step, const char* dir)
{
    Mesh m = MESH;
    const size_t n = ncell(m);
    Field f;
    f.u.resize(n); f.v.resize(n); f.w.resize(n); f.p.resize(n); f.nu_t.resize(n); f.is_solid.assign(n, false);
    put(f.u, u, n); put(f.v, v, n); put(f.w, w, n); put(f.p, p, n); put(f.nu_t, nu_t, n);
    put_mask(f, solid, n);
    InDir d(dir);
    write_field_vtk(f, m, step);
}

// save_state into dir/checkpoint/checkpoint.{meta,data}
void ref_save_state(MESH_ARGS, const double* u, const double* v, const double* w, const double* p,
                    const double* nu_t, const uint8_t* solid, double time_simulated, double dt, int next_step,
                    const char* dir)
{
    Mesh m = MESH;
    const size_t n = ncell(m);
    Field f;
    f.u.resize(n); f.v.resize(n); f.w.resize(n); f.p.resize(n); f.nu_t.resize(n); f.is_solid.assign(n, false);
    put(f.u, u, n); put(f.v, v, n); put(f.w, w, n); put(f.p, p, n); put(f.nu_t, nu_t, n);
    put_mask(f, solid, n);
    InDir d(dir);
    save_state(f, m, time_simulated, dt, next_step);
}

}  // extern "C"
