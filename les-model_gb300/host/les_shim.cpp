// les_shim.cpp -- the les-model host API (src/pressure.h:31-63 and the step
// functions of src/main.cpp) implemented on the GB300 C ABI.
//
// Drop-in mode: every function keeps the reference's signature and in-place
// semantics on host std::vectors.  Each call uploads the arrays it reads into a
// device context (one per grid size, created on first use), runs the CUDA
// kernels and downloads the arrays it writes, so a caller's step loop,
// checkpoint, VTK and statistics code run unchanged.  Errors throw
// std::runtime_error (the reference has no error returns).
//
// Resident mode (les_shim::DeviceField in les_shim.hpp) keeps the Field on the
// device across steps and copies only at the caller's I/O points; that is the
// fast path.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <initializer_list>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "les_gb300.h"
#include "les_reference_api.h"

namespace {

std::mutex g_mu;
int g_device = -1;
std::string g_err;

struct Dev {
    les_ctx* c = nullptr;
    int nx, ny, nz;
    ~Dev() { les_destroy(c); }
};

using Key = std::tuple<int, int, int, double, double, double>;
std::map<Key, std::unique_ptr<Dev>> g_ctx;
Dev* g_last = nullptr;

int device()
{
    if (g_device < 0) {
        const char* e = std::getenv("LES_DEVICE");
        g_device = e ? std::atoi(e) : 0;
    }
    return g_device;
}

void check(les_ctx* c, les_status st, const char* what)
{
    if (st == LES_OK) return;
    g_err = std::string(what) + ": " + les_status_string(st) + (c ? std::string(" (") + les_last_error(c) + ")" : "");
    throw std::runtime_error(g_err);
}

// Context for a grid with known spacing.
Dev& dev_for(int nx, int ny, int nz, double dx, double dy, double dz)
{
    Key k{nx, ny, nz, dx, dy, dz};
    auto it = g_ctx.find(k);
    if (it == g_ctx.end()) {
        les_mesh m{nx, ny, nz, dx, dy, dz};
        auto d = std::make_unique<Dev>();
        d->nx = nx; d->ny = ny; d->nz = nz;
        check(nullptr, les_create(&m, device(), &d->c), "les_create");
        it = g_ctx.emplace(k, std::move(d)).first;
    }
    g_last = it->second.get();
    return *it->second;
}

Dev& dev_for(const Mesh& m) { return dev_for(m.nx, m.ny, m.nz, m.dx, m.dy, m.dz); }

// Context for a Field only (the call does not use the spacing): any context
// of the same shape, else one with unit spacing.
Dev& dev_for(const Field& f)
{
    for (auto& kv : g_ctx)
        if (kv.second->nx == f.nx && kv.second->ny == f.ny && kv.second->nz == f.nz) {
            g_last = kv.second.get();
            return *kv.second;
        }
    return dev_for(f.nx, f.ny, f.nz, 1.0, 1.0, 1.0);
}

// Context for a bare vector (BLAS-1 helpers, Jacobi preconditioner): the last
// context whose grid has that many cells.
Dev& dev_for_n(size_t n)
{
    if (g_last && (size_t)g_last->nx * g_last->ny * g_last->nz == n) return *g_last;
    for (auto& kv : g_ctx)
        if ((size_t)kv.second->nx * kv.second->ny * kv.second->nz == n) return *kv.second;
    g_err = "no device context of this size: call a Field-based function first";
    throw std::runtime_error(g_err);
}

void up(Dev& d, int slot, const std::vector<double>& v) { check(d.c, les_upload(d.c, slot, v.data()), "upload"); }
void down(Dev& d, int slot, std::vector<double>& v) { check(d.c, les_download(d.c, slot, v.data()), "download"); }

// several fields in one call (one synchronisation)
void ups(Dev& d, std::initializer_list<std::pair<int, const std::vector<double>*>> fs)
{
    std::vector<int> sl;
    std::vector<const double*> p;
    for (auto& f : fs) { sl.push_back(f.first); p.push_back(f.second->data()); }
    check(d.c, les_upload_many(d.c, (int)sl.size(), sl.data(), p.data()), "upload");
}

void downs(Dev& d, std::initializer_list<std::pair<int, std::vector<double>*>> fs)
{
    std::vector<int> sl;
    std::vector<double*> p;
    for (auto& f : fs) { sl.push_back(f.first); p.push_back(f.second->data()); }
    check(d.c, les_download_many(d.c, (int)sl.size(), sl.data(), p.data()), "download");
}

void up_mask(Dev& d, const Field& f)
{
    std::vector<uint8_t> m(f.is_solid.size());
    for (size_t i = 0; i < m.size(); ++i) m[i] = f.is_solid[i] ? 1 : 0;
    check(d.c, les_upload_mask(d.c, m.data()), "upload mask");
}

void up_matrix(Dev& d, const StencilMatrix& A, bool as_factor)
{
    const double* p[7] = {A.A_c.data(), A.A_n.data(), A.A_s.data(), A.A_e.data(),
                          A.A_w.data(), A.A_t.data(), A.A_b.data()};
    if (as_factor) check(d.c, les_set_ic_factor(d.c, p), "set IC factor");
    else check(d.c, les_set_stencil(d.c, p), "set stencil");
}

void down_matrix(Dev& d, StencilMatrix& A, bool factor)
{
    double* p[7] = {A.A_c.data(), A.A_n.data(), A.A_s.data(), A.A_e.data(), A.A_w.data(), A.A_t.data(), A.A_b.data()};
    if (factor) check(d.c, les_get_ic_factor(d.c, p), "get IC factor");
    else check(d.c, les_get_stencil(d.c, p), "get stencil");
}

int pcg_call(const StencilMatrix& A, const Vector& b, Vector& x, const Field& field, les_pcg_opts o)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(field);
    up_matrix(d, A, false);
    up(d, LES_B, b);
    up(d, LES_P, x);
    les_pcg_result r{};
    les_status st = les_pcg(d.c, &o, &r);
    if (st != LES_OK && st != LES_NOT_CONVERGED && st != LES_NONFINITE) check(d.c, st, "les_pcg");
    down(d, LES_P, x);
    if (st != LES_OK) {
        // src/pressure.cpp:411-413 / :832-834
        std::fprintf(stderr, "Warning: PCG did not converge after %d iterations.\n", o.max_iter);
        return o.max_iter;
    }
    return r.iters;
}

}  // namespace

// ---- step physics, src/main.cpp ----------------------------------------

double compute_adaptive_dt(const Field& f, const Mesh& m, double nu)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(m);
    ups(d, {{LES_U, &f.u}, {LES_V, &f.v}, {LES_W, &f.w}, {LES_NU_T, &f.nu_t}});
    double dt = 0;
    check(d.c, les_adaptive_dt(d.c, nu, 0.4, 0.2, 1e-4, &dt), "les_adaptive_dt");   // src/main.cpp:210-212
    return dt;
}

void compute_sgs_stress(Field& f, Stress& sgs, const Mesh& m)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(m);
    ups(d, {{LES_U, &f.u}, {LES_V, &f.v}, {LES_W, &f.w}, {LES_NU_T, &f.nu_t}});
    check(d.c, les_sgs(d.c, 0.18, 1), "les_sgs");   // Cs of src/main.cpp:425
    down(d, LES_NU_T, f.nu_t);
    const size_t n = f.u.size();
    std::vector<double> tau(6 * n);
    check(d.c, les_download_tau(d.c, tau.data()), "download tau");
    std::vector<double>* dst[6] = {&sgs.tau_xx, &sgs.tau_xy, &sgs.tau_xz, &sgs.tau_yy, &sgs.tau_yz, &sgs.tau_zz};
    for (int q = 0; q < 6; ++q) std::copy(tau.begin() + q * n, tau.begin() + (q + 1) * n, dst[q]->begin());
}

void apply_nut_BCs(Field& f, const Mesh& m)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(m);
    up(d, LES_NU_T, f.nu_t);
    up_mask(d, f);
    check(d.c, les_nut_bcs(d.c), "les_nut_bcs");
    down(d, LES_NU_T, f.nu_t);
}

void solve_momentum(Field& f, const Mesh& m, double dt, double nu)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(m);
    ups(d, {{LES_U, &f.u}, {LES_V, &f.v}, {LES_W, &f.w}, {LES_U_NEW, &f.u_new}, {LES_V_NEW, &f.v_new},
            {LES_W_NEW, &f.w_new}, {LES_NU_T, &f.nu_t}});
    check(d.c, les_momentum(d.c, dt, nu), "les_momentum");   // includes the swap of :656-658
    downs(d, {{LES_U, &f.u}, {LES_V, &f.v}, {LES_W, &f.w}, {LES_U_NEW, &f.u_new}, {LES_V_NEW, &f.v_new},
              {LES_W_NEW, &f.w_new}});
}

void apply_velocity_BCs(Field& f, const Mesh& m)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(m);
    ups(d, {{LES_U, &f.u}, {LES_V, &f.v}, {LES_W, &f.w}});
    up_mask(d, f);
    check(d.c, les_velocity_bcs(d.c), "les_velocity_bcs");
    downs(d, {{LES_U, &f.u}, {LES_V, &f.v}, {LES_W, &f.w}});
}

void correct_velocity(Field& f, const Mesh& m, double dt, double rho)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(m);
    ups(d, {{LES_U, &f.u}, {LES_V, &f.v}, {LES_W, &f.w}, {LES_P, &f.p}});
    check(d.c, les_correct_velocity(d.c, dt, rho), "les_correct_velocity");
    downs(d, {{LES_U, &f.u}, {LES_V, &f.v}, {LES_W, &f.w}});
}

// ---- pressure, src/pressure.cpp ------------------------------------------

void apply_pressure_BCs(Field& f, const Mesh& m)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(m);
    up(d, LES_P, f.p);
    up_mask(d, f);
    check(d.c, les_pressure_bcs(d.c), "les_pressure_bcs");
    down(d, LES_P, f.p);
}

void solve_pressure_jacobi(Field& f, const Mesh& m, double dt, double rho)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(m);
    ups(d, {{LES_U, &f.u}, {LES_V, &f.v}, {LES_W, &f.w}, {LES_P, &f.p}});
    up_mask(d, f);
    int sweeps = 0;
    check(d.c, les_solve_jacobi(d.c, dt, rho, 100, 1e-6, &sweeps), "les_solve_jacobi");   // :134, :165
    down(d, LES_P, f.p);
}

void solve_pressure_GS(Field& f, const Mesh& m, double dt, double rho, int maxIter)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(m);
    ups(d, {{LES_U, &f.u}, {LES_V, &f.v}, {LES_W, &f.w}, {LES_P, &f.p}});
    up_mask(d, f);
    int sweeps = 0;
    check(d.c, les_solve_gs(d.c, dt, rho, maxIter, 1.7, 1e-6, &sweeps), "les_solve_gs");   // :195, :240
    down(d, LES_P, f.p);
    if (sweeps < maxIter) std::printf("Pressure converged in %d iterations\n", sweeps);
}

void calculate_divergence(Vector& rhs, const Field& f, const Mesh& m, double dt, double rho)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(m);
    ups(d, {{LES_U_NEW, &f.u_new}, {LES_V_NEW, &f.v_new}, {LES_W_NEW, &f.w_new}});
    up_mask(d, f);
    check(d.c, les_divergence(d.c, dt, rho), "les_divergence");
    down(d, LES_P_RHS, rhs);
}

void build_b_vector(Vector& b, const Vector& div, const Field& f, const Mesh& m)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(m);
    up(d, LES_P_RHS, div);
    up_mask(d, f);
    check(d.c, les_build_b(d.c), "les_build_b");
    down(d, LES_B, b);
}

void build_stencil(StencilMatrix& A, const Field& f, const Mesh& m)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(m);
    up_mask(d, f);
    check(d.c, les_build_stencil(d.c), "les_build_stencil");
    down_matrix(d, A, false);
}

void fast_apply_laplacian(Vector& q, const Vector& p, const StencilMatrix& A, const Field& f)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(f);
    up_matrix(d, A, false);
    up(d, LES_P, p);
    check(d.c, les_spmv(d.c, LES_P, LES_B), "les_spmv");
    down(d, LES_B, q);
}

void apply_jacobi_preconditioner(Vector& z, const Vector& r, const StencilMatrix& A)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for_n(r.size());
    up_matrix(d, A, false);
    up(d, LES_P, r);
    les_pcg_opts o{};
    o.precond = LES_PC_JACOBI;
    check(d.c, les_precond_apply(d.c, &o, LES_P, LES_B), "jacobi preconditioner");
    down(d, LES_B, z);
}

void apply_ic_preconditioner(Vector& z, const Vector& r, const StencilMatrix& L, const Field& f)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(f);
    up_matrix(d, L, true);
    up(d, LES_P, r);
    les_pcg_opts o{};
    o.precond = LES_PC_IC;
    check(d.c, les_precond_apply(d.c, &o, LES_P, LES_B), "IC preconditioner");
    down(d, LES_B, z);
}

void build_ic_preconditioner(StencilMatrix& L, const StencilMatrix& A, const Field& f, const Mesh& m)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(m);
    up_matrix(d, A, false);
    check(d.c, les_build_ic(d.c), "les_build_ic");
    down_matrix(d, L, true);
}

int solve_pressure_pcg(const StencilMatrix& A, const Vector& b, Vector& x, const Field& field, int max_iter,
                       double tol)
{
    les_pcg_opts o{};
    o.precond = LES_PC_IC_A;   // as shipped: A passed as the IC factor, src/pressure.cpp:363, :396
    o.max_iter = max_iter;
    o.tol = tol;
    return pcg_call(A, b, x, field, o);
}

int solve_pressure_pcg_chebyshev(const StencilMatrix& A, const Vector& b, Vector& x, const Field& field,
                                 double lambda_min, double lambda_max, int poly_degree, int max_iter, double tol)
{
    les_pcg_opts o{};
    o.precond = LES_PC_CHEBYSHEV;
    o.max_iter = max_iter;
    o.tol = tol;
    o.lambda_min = lambda_min;
    o.lambda_max = lambda_max;
    o.degree = poly_degree;
    return pcg_call(A, b, x, field, o);
}

void apply_chebyshev_preconditioner(Vector& z, const Vector& r, const StencilMatrix& A, const Field& f,
                                    double lambda_min, double lambda_max, int poly_degree)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(f);
    up_matrix(d, A, false);
    up(d, LES_P, r);
    les_pcg_opts o{};
    o.precond = LES_PC_CHEBYSHEV;
    o.lambda_min = lambda_min;
    o.lambda_max = lambda_max;
    o.degree = poly_degree;
    check(d.c, les_precond_apply(d.c, &o, LES_P, LES_B), "chebyshev preconditioner");
    down(d, LES_B, z);
}

double estimate_lambda_max(const StencilMatrix& A, const Field& f, int n_iter)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for(f);
    up_matrix(d, A, false);
    double lam = 0;
    check(d.c, les_lambda_max(d.c, n_iter, nullptr, &lam), "les_lambda_max");
    return lam;
}

// ---- BLAS-1 helpers, src/pressure.cpp:962-1013 ---------------------------

double parallel_dot(const Vector& a, const Vector& b)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for_n(a.size());
    up(d, LES_P, a);
    up(d, LES_B, b);
    double r = 0;
    check(d.c, les_dot(d.c, LES_P, LES_B, &r), "les_dot");
    return r;
}

double parallel_norm(const Vector& v) { return std::sqrt(parallel_dot(v, v)); }

void parallel_axpy(Vector& out, double a, const Vector& in)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for_n(out.size());
    up(d, LES_P, out);
    up(d, LES_B, in);
    check(d.c, les_axpby(d.c, LES_P, 1.0, LES_P, a, LES_B), "les_axpby");
    down(d, LES_P, out);
}

void parallel_saxpy(Vector& out, double a, const Vector& in1, double b, const Vector& in2)
{
    std::lock_guard<std::mutex> lk(g_mu);
    Dev& d = dev_for_n(out.size());
    up(d, LES_P, in1);
    up(d, LES_B, in2);
    check(d.c, les_axpby(d.c, LES_P_RHS, a, LES_P, b, LES_B), "les_axpby");
    down(d, LES_P_RHS, out);
}

void parallel_copy(Vector& out, const Vector& in) { out = in; }

namespace les_shim {
void set_device(int dev)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_device = dev;
}
void reset()
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_ctx.clear();
    g_last = nullptr;
}
const char* last_error() { return g_err.c_str(); }
}  // namespace les_shim
